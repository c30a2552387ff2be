// keys_sort.cu -- bounding box, 63-bit octant-path keys, stable LSD radix
// sort of (key, slot) pairs, device-wide exclusive scan and the gather that
// puts the particle state into key order.
//
// Bit-exactness with the reference tree (projects/nbody_core/src/Tree.cpp):
//  * the root cube is the FP64 bounding box of the positions, centre
//    0.5*(lo+hi), half = max half extent (1.0 if <= 1e-12) times 1.001
//    (Tree.cpp:54-88);
//  * at each level the octant bit per axis is (p >= centre) (Tree.cpp:11-20)
//    and the child centre is centre +/- 0.5*half, rounded in FP64 exactly as
//    NewChild does (Tree.cpp:90-112).
// Key digit l (bits 3*(20-l)..+2) is the octant (x:1, y:2, z:4) of the
// particle's level-l ancestor, so ascending keys enumerate leaves in the
// reference's DFS ascending-octant order (Tree.cpp:157-175).
#include "engine.cuh"

#include <cstdio>

namespace ngrav {

// ---------------------------------------------------------------------------
// FP64 bounding box with order-preserving integer atomics
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long enc_f64(double d) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

__device__ __forceinline__ double dec_f64(unsigned long long u) {
    u = (u & 0x8000000000000000ull) ? (u & 0x7FFFFFFFFFFFFFFFull) : ~u;
    return __longlong_as_double((long long)u);
}

__device__ __forceinline__ double pos_d(const float4& hi, const float4* plo, long long i, int axis) {
    const float h = axis == 0 ? hi.x : (axis == 1 ? hi.y : hi.z);
    if (!plo) return (double)h;
    const float4 lo = plo[i];
    const float l = axis == 0 ? lo.x : (axis == 1 ? lo.y : lo.z);
    return (double)h + (double)l;
}

constexpr int kBoxThreads = 256;

__global__ void __launch_bounds__(kBoxThreads) bbox_kernel(const float4* __restrict__ pos,
                                                           const float4* __restrict__ plo, long long n,
                                                           Counters* C) {
    double lo[3] = {1.0 / 0.0, 1.0 / 0.0, 1.0 / 0.0};
    double hi[3] = {-1.0 / 0.0, -1.0 / 0.0, -1.0 / 0.0};
    bool bad = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        bad |= !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(p.w));
        for (int a = 0; a < 3; ++a) {
            const double v = pos_d(p, plo, i, a);
            lo[a] = fmin(lo[a], v);
            hi[a] = fmax(hi[a], v);
        }
    }
    __shared__ double slo[3][kBoxThreads / 32], shi[3][kBoxThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int a = 0; a < 3; ++a) {
        double l = lo[a], h = hi[a];
        for (int o = 16; o > 0; o >>= 1) {
            l = fmin(l, __shfl_xor_sync(0xffffffffu, l, o));
            h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
        }
        if (lane == 0) {
            slo[a][w] = l;
            shi[a][w] = h;
        }
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        double l = slo[a][0], h = shi[a][0];
        for (int k = 1; k < kBoxThreads / 32; ++k) {
            l = fmin(l, slo[a][k]);
            h = fmax(h, shi[a][k]);
        }
        atomicMin(&C->bbox_min[a], enc_f64(l));
        atomicMax(&C->bbox_max[a], enc_f64(h));
    }
    if (threadIdx.x == 0 && bad) atomicOr(&C->status, kStNonFinite);
}

// Root cube of BuildRoot (Tree.cpp:54-88), once per evaluation.
__global__ void root_kernel(Counters* C, long long n) {
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = n > 0 ? dec_f64(C->bbox_min[a]) : 0.0;
        hi[a] = n > 0 ? dec_f64(C->bbox_max[a]) : 0.0;
    }
    double half = __dmul_rn(0.5, __dsub_rn(hi[0], lo[0]));
    const double hy = __dmul_rn(0.5, __dsub_rn(hi[1], lo[1]));
    const double hz = __dmul_rn(0.5, __dsub_rn(hi[2], lo[2]));
    if (half < hy) half = hy;
    if (half < hz) half = hz;
    if (!(half > 1e-12)) half = 1.0;
    for (int a = 0; a < 3; ++a) C->root_center[a] = __dmul_rn(0.5, __dadd_rn(lo[a], hi[a]));
    C->root_half = __dmul_rn(half, 1.001);
}

void launch_bbox(const float4* pos, const float4* plo, long long n, Counters* C, cudaStream_t s) {
    long long blocks = (n + kBoxThreads - 1) / kBoxThreads;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) blocks = 1;
    bbox_kernel<<<(unsigned)blocks, kBoxThreads, 0, s>>>(pos, plo, n, C);
}

void launch_root(Counters* C, long long n, cudaStream_t s) { root_kernel<<<1, 1, 0, s>>>(C, n); }

// Ensemble: per-system FP64 bounding boxes.  Slots are grouped by system, so a
// warp whose 32 slots share one system reduces in registers first; mixed warps
// fall back to per-lane atomics.
__global__ void __launch_bounds__(kBoxThreads) forest_bbox_kernel(const float4* __restrict__ pos,
                                                                  const float4* __restrict__ plo, long long n,
                                                                  Forest F, Counters* C) {
    const int lane = threadIdx.x & 31;
    bool bad = false;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const long long i = base + lane;
        const bool has = i < n;
        int sys = has ? forest_system(F, i) : -1;
        double v[3] = {0.0, 0.0, 0.0};
        if (has) {
            const float4 p = pos[i];
            bad |= !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(p.w));
            for (int a = 0; a < 3; ++a) v[a] = pos_d(p, plo, i, a);
        }
        const int s0 = __shfl_sync(0xffffffffu, sys, 0);
        const bool uniform = __all_sync(0xffffffffu, !has || sys == s0);
        for (int a = 0; a < 3; ++a) {
            double l = has ? v[a] : 1.0 / 0.0, h = has ? v[a] : -1.0 / 0.0;
            if (uniform) {
                for (int o = 16; o > 0; o >>= 1) {
                    l = fmin(l, __shfl_xor_sync(0xffffffffu, l, o));
                    h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
                }
                if (lane == 0) {
                    atomicMin(&F.bbox[6 * s0 + a], enc_f64(l));
                    atomicMax(&F.bbox[6 * s0 + 3 + a], enc_f64(h));
                }
            } else if (has) {
                atomicMin(&F.bbox[6 * sys + a], enc_f64(l));
                atomicMax(&F.bbox[6 * sys + 3 + a], enc_f64(h));
            }
        }
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&C->status, kStNonFinite);
}

// BuildRoot (Tree.cpp:54-88) of every system; resets the boxes for the next
// evaluation.
__global__ void forest_root_kernel(Forest F) {
    for (int sys = blockIdx.x * blockDim.x + threadIdx.x; sys < F.nsys; sys += gridDim.x * blockDim.x) {
        const bool empty = F.off[sys + 1] <= F.off[sys];
        double lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = empty ? 0.0 : dec_f64(F.bbox[6 * sys + a]);
            hi[a] = empty ? 0.0 : dec_f64(F.bbox[6 * sys + 3 + a]);
            F.bbox[6 * sys + a] = ~0ull;
            F.bbox[6 * sys + 3 + a] = 0ull;
        }
        double half = __dmul_rn(0.5, __dsub_rn(hi[0], lo[0]));
        const double hy = __dmul_rn(0.5, __dsub_rn(hi[1], lo[1]));
        const double hz = __dmul_rn(0.5, __dsub_rn(hi[2], lo[2]));
        if (half < hy) half = hy;
        if (half < hz) half = hz;
        if (!(half > 1e-12)) half = 1.0;
        for (int a = 0; a < 3; ++a) F.root[4 * sys + a] = __dmul_rn(0.5, __dadd_rn(lo[a], hi[a]));
        F.root[4 * sys + 3] = __dmul_rn(half, 1.001);
    }
}

void launch_forest_bbox(const float4* pos, const float4* plo, long long n, const Forest& F, Counters* C,
                        cudaStream_t s) {
    long long blocks = (n + kBoxThreads - 1) / kBoxThreads;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) blocks = 1;
    forest_bbox_kernel<<<(unsigned)blocks, kBoxThreads, 0, s>>>(pos, plo, n, F, C);
}

void launch_forest_root(const Forest& F, cudaStream_t s) {
    forest_root_kernel<<<(F.nsys + 127) / 128, 128, 0, s>>>(F);
}

// SPLIT -> PLAIN: fold the low halves into FP32 positions.
__global__ void collapse_split_kernel(float4* __restrict__ pos, float4* __restrict__ plo, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 p = pos[i];
        const float4 l = plo[i];
        p.x = (float)((double)p.x + (double)l.x);
        p.y = (float)((double)p.y + (double)l.y);
        p.z = (float)((double)p.z + (double)l.z);
        pos[i] = p;
        plo[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

void launch_collapse_split(float4* pos, float4* plo, long long n, cudaStream_t s) {
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    collapse_split_kernel<<<(unsigned)blocks, 256, 0, s>>>(pos, plo, n);
}

// ---------------------------------------------------------------------------
// 63-bit keys by the reference's FP64 centre recurrence
// ---------------------------------------------------------------------------

__device__ __forceinline__ long long ordered_bits(double x) {
    // Integer image of a finite double that orders like the double (-0
    // taken as +0): one 64-bit compare replaces the FP64 comparison.
    long long b = __double_as_longlong(x);
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFll);
}

template <int LEVELS>
__device__ __forceinline__ unsigned axis_bits(double p, double c, double h) {
    // Returns LEVELS octant bits of one axis, level 0 in the highest bit:
    // bit = p >= c, then h = h / 2 and c = c +- h rounded in FP64 (NewChild).
    // GB300's FP64 pipe is narrow, so only the centre add stays FP64: the
    // comparison is an integer compare of ordered bit images, the halving an
    // exponent decrement (exact: h >= 1e-12 stays normal over 21 levels) and
    // c - h the addition of -h (the same IEEE result).
    const long long op = ordered_bits(p);
    long long hb = __double_as_longlong(h);
    unsigned bits = 0;
#pragma unroll
    for (int l = 0; l < LEVELS; ++l) {
        const bool b = op >= ordered_bits(c);
        bits = (bits << 1) | (b ? 1u : 0u);
        hb -= 1ll << 52;
        c = __dadd_rn(c, __longlong_as_double(b ? hb : (hb | (long long)0x8000000000000000ull)));
    }
    return bits;
}

constexpr int kKeyTabLevels = 17;                // key levels whose centres are tabulated per build
constexpr int kKeyTabSize = 1 << kKeyTabLevels;  // table entries per axis (entry 0 unused)
constexpr int kKeySub = 4;                       // levels a table thread fills below its own entry
constexpr int kKeyTop = kKeyTabLevels - 1 - kKeySub;  // level of those threads' entries
static_assert(kKeyTop >= 0, "the table is deeper than one thread's subtree");

long long key_table_entries() { return 3LL * kKeyTabSize; }

__device__ __forceinline__ double centre_step(double c, long long hb, bool up) {
    return __dadd_rn(c, __longlong_as_double(up ? hb : (hb | (long long)0x8000000000000000ull)));
}

// The centre recurrence of an axis depends only on that axis's own octant
// bits, so the centres of levels 0 .. kKeyTabLevels-1 are tabulated once per
// build: an implicit binary tree per axis, entry 1 the root centre and entry
// 2e + b the child of entry e on side b (b = 1: p >= c).  Every entry is the
// exact FP64 sequence of additions of the walk down to it, so the keys kernel
// looks the top levels up and adds in FP64 only below them.  One thread per
// entry of level kKeyTop replays the walk to it and derives its subtree
// kKeySub levels down, one addition per entry from the parent's value (the
// same operands and rounding as the walk); one thread per entry above
// kKeyTop replays its own walk.  Entries are stored as their ordered bit
// images (ordered_bits), the form the keys kernel compares.
__global__ void __launch_bounds__(256) key_table_kernel(const Counters* __restrict__ C, long long* __restrict__ tab) {
    constexpr int nroot = 1 << kKeyTop;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool sub = i < 3 * nroot;
    const int j = sub ? i : i - 3 * nroot;
    if (j >= 3 * nroot) return;
    const int axis = j / nroot;
    const int e = sub ? nroot + j % nroot : j % nroot;  // an entry of level kKeyTop, or one above it
    if (e == 0) return;
    const int l = 31 - __clz(e);  // level of entry e: its bits below the leading one are levels 0 .. l-1
    double c = C->root_center[axis];
    long long hb = __double_as_longlong(C->root_half);
    for (int k = l - 1; k >= 0; --k) {
        hb -= 1ll << 52;
        c = centre_step(c, hb, (e >> k) & 1);
    }
    long long* t = tab + (long long)axis * kKeyTabSize;
    t[e] = ordered_bits(c);
    if (!sub) return;
    double lv[1 << kKeySub];  // the subtree's centres of one level, left to right
    lv[0] = c;
#pragma unroll
    for (int d = 1; d <= kKeySub; ++d) {
        hb -= 1ll << 52;
#pragma unroll
        for (int q = (1 << d) - 1; q >= 0; --q) lv[q] = centre_step(lv[q >> 1], hb, q & 1);
#pragma unroll
        for (int q = 0; q < (1 << d); ++q) t[(e << d) + q] = ordered_bits(lv[q]);
    }
}

// The double of an ordered bit image (a -0 centre comes back as +0, which
// gives the same sums with the nonzero halves added to it).
__device__ __forceinline__ double from_ordered(long long o) {
    return __longlong_as_double(o ^ ((o >> 63) & 0x7FFFFFFFFFFFFFFFll));
}

// axis_bits over all kKeyLevels levels with the top kKeyTabLevels looked up
// in the axis's table of ordered images.
__device__ __forceinline__ unsigned axis_bits_tab(double p, const long long* __restrict__ tab, double h0) {
    const long long op = ordered_bits(p);
    unsigned e = 1;
#pragma unroll
    for (int l = 0; l < kKeyTabLevels; ++l) e = 2 * e + (op >= __ldg(tab + e) ? 1u : 0u);
    // continue from the centre of level kKeyTabLevels: the last tabulated
    // centre plus or minus h / 2^kKeyTabLevels, as the recurrence would
    long long hb = __double_as_longlong(h0) - ((long long)kKeyTabLevels << 52);
    double c = __dadd_rn(from_ordered(__ldg(tab + (e >> 1))),
                         __longlong_as_double(e & 1 ? hb : (hb | (long long)0x8000000000000000ull)));
    unsigned bits = e - (1u << kKeyTabLevels);
#pragma unroll
    for (int l = kKeyTabLevels; l < kKeyLevels; ++l) {
        const bool b = op >= ordered_bits(c);
        bits = (bits << 1) | (b ? 1u : 0u);
        if (l + 1 < kKeyLevels) {
            hb -= 1ll << 52;
            c = __dadd_rn(c, __longlong_as_double(b ? hb : (hb | (long long)0x8000000000000000ull)));
        }
    }
    return bits;
}

// Spread 21 bits so bit k lands at 3k.
__device__ __forceinline__ unsigned long long spread3(unsigned v) {
    unsigned long long x = v & 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__global__ void __launch_bounds__(256) keys_kernel(const float4* __restrict__ pos, const float4* __restrict__ plo,
                                                   long long n, const Counters* __restrict__ C,
                                                   const long long* __restrict__ tab,
                                                   unsigned long long* __restrict__ keys,
                                                   unsigned* __restrict__ vals) {
    const double h0 = C->root_half;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        double px = p.x, py = p.y, pz = p.z;
        if (plo) {
            const float4 l = plo[i];
            px += (double)l.x;
            py += (double)l.y;
            pz += (double)l.z;
        }
        const unsigned bx = axis_bits_tab(px, tab, h0);
        const unsigned by = axis_bits_tab(py, tab + kKeyTabSize, h0);
        const unsigned bz = axis_bits_tab(pz, tab + 2 * kKeyTabSize, h0);
        keys[i] = spread3(bx) | (spread3(by) << 1) | (spread3(bz) << 2);
        vals[i] = (unsigned)i;
    }
}

// Ensemble keys: the system id in the top SYSL digits, then 21 - SYSL levels
// of octant path from the system's own root cube.
template <int SYSL>
__global__ void __launch_bounds__(256) forest_keys_kernel(const float4* __restrict__ pos,
                                                          const float4* __restrict__ plo, long long n, Forest F,
                                                          unsigned long long* __restrict__ keys,
                                                          unsigned* __restrict__ vals) {
    constexpr int L = kKeyLevels - SYSL;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int sys = forest_system(F, i);
        const double cx = F.root[4 * sys], cy = F.root[4 * sys + 1], cz = F.root[4 * sys + 2];
        const double h0 = F.root[4 * sys + 3];
        const float4 p = pos[i];
        double px = p.x, py = p.y, pz = p.z;
        if (plo) {
            const float4 l = plo[i];
            px += (double)l.x;
            py += (double)l.y;
            pz += (double)l.z;
        }
        const unsigned bx = axis_bits<L>(px, cx, h0);
        const unsigned by = axis_bits<L>(py, cy, h0);
        const unsigned bz = axis_bits<L>(pz, cz, h0);
        keys[i] = ((unsigned long long)sys << (3 * L)) | spread3(bx) | (spread3(by) << 1) | (spread3(bz) << 2);
        vals[i] = (unsigned)i;
    }
}

int launch_keys(const float4* pos, const float4* plo, long long n, Counters* C, const Forest& F, long long* ktab,
                unsigned long long* keys, unsigned* vals, cudaStream_t s) {
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    const unsigned g = (unsigned)blocks;
    switch (F.sys_levels) {
        case 0:
            key_table_kernel<<<(6 * (1 << kKeyTop) + 255) / 256, 256, 0, s>>>(C, ktab);
            keys_kernel<<<g, 256, 0, s>>>(pos, plo, n, C, ktab, keys, vals);
            return 2;
        case 1: forest_keys_kernel<1><<<g, 256, 0, s>>>(pos, plo, n, F, keys, vals); break;
        case 2: forest_keys_kernel<2><<<g, 256, 0, s>>>(pos, plo, n, F, keys, vals); break;
        case 3: forest_keys_kernel<3><<<g, 256, 0, s>>>(pos, plo, n, F, keys, vals); break;
        case 4: forest_keys_kernel<4><<<g, 256, 0, s>>>(pos, plo, n, F, keys, vals); break;
        case 5: forest_keys_kernel<5><<<g, 256, 0, s>>>(pos, plo, n, F, keys, vals); break;
        default: forest_keys_kernel<6><<<g, 256, 0, s>>>(pos, plo, n, F, keys, vals); break;
    }
    return 1;
}

// ---------------------------------------------------------------------------
// Device-wide exclusive scan of unsigned (reduce / scan partials / downsweep)
// ---------------------------------------------------------------------------

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

long long scan_tmp_size(long long n) { return (n + kScanTile - 1) / kScanTile + 1; }

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* s_warp, unsigned& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    if (w == 0) {
        unsigned t = lane < nw ? s_warp[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) s_warp[lane] = t;
    }
    __syncthreads();
    total = s_warp[nw - 1];
    const unsigned before = w > 0 ? s_warp[w - 1] : 0u;
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const unsigned* __restrict__ in, long long n,
                                                                   unsigned* __restrict__ partial) {
    const long long base = blockIdx.x * (long long)kScanTile;
    unsigned s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long i = base + k * kScanThreads + threadIdx.x;
        if (i < n) s += in[i];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ unsigned ws[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int k = 0; k < kScanThreads / 32; ++k) t += ws[k];
        partial[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) scan_partials_kernel(unsigned* partial, int nb) {
    __shared__ unsigned s_warp[32];
    unsigned carry = 0;
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const unsigned v = i < nb ? partial[i] : 0u;
        unsigned total;
        const unsigned ex = block_exclusive_scan(v, s_warp, total);
        if (i < nb) partial[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_down_kernel(const unsigned* __restrict__ in, long long n,
                                                                 const unsigned* __restrict__ partial,
                                                                 unsigned* __restrict__ out) {
    __shared__ unsigned s_warp[32];
    const long long base = blockIdx.x * (long long)kScanTile + (long long)threadIdx.x * kScanItems;
    unsigned v[kScanItems];
    unsigned sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long i = base + k;
        v[k] = i < n ? in[i] : 0u;
        sum += v[k];
    }
    unsigned total;
    unsigned run = block_exclusive_scan(sum, s_warp, total) + partial[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

void device_exclusive_scan(const unsigned* in, unsigned* out, long long n, unsigned* tmp, cudaStream_t s) {
    if (n <= 0) return;
    const int nb = (int)((n + kScanTile - 1) / kScanTile);
    scan_reduce_kernel<<<nb, kScanThreads, 0, s>>>(in, n, tmp);
    scan_partials_kernel<<<1, 1024, 0, s>>>(tmp, nb);
    scan_down_kernel<<<nb, kScanThreads, 0, s>>>(in, n, tmp, out);
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 9-bit digits (seven passes cover the 63-bit keys),
// tiles of 4096 keys (512 threads x 8); three kernels per pass (tile
// histograms, per-digit scans over the tiles, scatter)
// ---------------------------------------------------------------------------

constexpr int kRsThreads = 512;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsItems = 8;
constexpr int kRsTile = kRsThreads * kRsItems;   // 4096
constexpr int kRsWarpSpan = 32 * kRsItems;       // consecutive keys per warp
constexpr int kRsScatterMinBlocks = 2;
constexpr unsigned kRsMask = kRsBins - 1;
constexpr int kRsDpt = kRsBins / kRsThreads;     // digits per thread in the digit scans
static_assert(kRsDpt * kRsThreads == kRsBins, "whole digits per thread in the digit scans");

// Lanes of the warp holding the same digit as this lane (the invalid lanes of
// a ragged last tile form a group of their own): the AND of one ballot per
// digit bit, cheaper than a warp match.
__device__ __forceinline__ unsigned digit_peers(unsigned d, bool valid) {
    const unsigned vb = __ballot_sync(0xffffffffu, valid);
    unsigned peers = valid ? vb : ~vb;
#pragma unroll
    for (int b = 0; b < kRsDigitBits; ++b) {
        const bool bit = (d >> b) & 1u;
        const unsigned bb = __ballot_sync(0xffffffffu, bit);
        peers &= bit ? bb : ~bb;
    }
    return peers;
}

// Histogram of one digit per tile, digit-major: hist[d * nblocks + b].  All
// keys of a thread are loaded before the first is counted; plain shared
// atomics (a warp match to combine equal digits costs more than the
// conflicts it saves).
__global__ void __launch_bounds__(kRsThreads) rs_hist_kernel(const unsigned long long* __restrict__ keys,
                                                             long long n, int shift, unsigned* __restrict__ hist) {
    __shared__ unsigned h[kRsBins];
#pragma unroll
    for (int j = 0; j < kRsDpt; ++j) h[threadIdx.x + j * kRsThreads] = 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long base = blockIdx.x * (long long)kRsTile + w * kRsWarpSpan + lane;
    unsigned d[kRsItems];
#pragma unroll
    for (int k = 0; k < kRsItems; ++k) {
        const long long i = base + k * 32;
        d[k] = i < n ? (unsigned)(__ldg(keys + i) >> shift) & kRsMask : (unsigned)kRsBins;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kRsItems; ++k) {
        if (d[k] < (unsigned)kRsBins) atomicAdd(&h[d[k]], 1u);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRsDpt; ++j)
        hist[(threadIdx.x + j * kRsThreads) * gridDim.x + blockIdx.x] = h[threadIdx.x + j * kRsThreads];
}

// One block per digit d: exclusive scan over the tiles of row d of the
// histogram, in place, and the row's total into totals[d].  The scatter adds
// the digit's own offset (the exclusive scan of the totals) itself.
__global__ void __launch_bounds__(kRsThreads) rs_scan_kernel(unsigned* __restrict__ hist, int nb,
                                                             unsigned* __restrict__ totals) {
    __shared__ unsigned s_warp[32];
    unsigned* row = hist + (long long)blockIdx.x * nb;
    constexpr int kPer = 4;
    unsigned carry = 0;
    for (int c0 = 0; c0 < nb; c0 += kRsThreads * kPer) {
        const int i0 = c0 + threadIdx.x * kPer;
        unsigned v[kPer];
        unsigned sum = 0;
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            v[k] = i0 + k < nb ? row[i0 + k] : 0u;
            sum += v[k];
        }
        unsigned total;
        unsigned run = carry + block_exclusive_scan(sum, s_warp, total);
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            if (i0 + k < nb) row[i0 + k] = run;
            run += v[k];
        }
        carry += total;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

// The tile's keys are ranked by digit in shared memory and written out in
// digit runs.  The per-warp digit counters share the tile buffer (they are
// dead once every key holds its rank), so a CTA holds 53 KB; at 64 registers
// two CTAs of 512 threads share an SM.
constexpr size_t kRsScatterSmem = (size_t)kRsTile * (sizeof(unsigned long long) + sizeof(unsigned));
static_assert(kRsWarps * kRsBins * sizeof(unsigned) <= kRsScatterSmem, "digit counters fit the tile buffer");

__global__ void __launch_bounds__(kRsThreads, kRsScatterMinBlocks) rs_scatter_kernel(const unsigned long long* __restrict__ kin,
                                                                const unsigned* __restrict__ vin,
                                                                unsigned long long* __restrict__ kout,
                                                                unsigned* __restrict__ vout, long long n, int shift,
                                                                const unsigned* __restrict__ hist_scan,
                                                                const unsigned* __restrict__ totals) {
    extern __shared__ unsigned long long rs_smem[];
    unsigned long long* skeys = rs_smem;                             // kRsTile
    unsigned* svals = reinterpret_cast<unsigned*>(skeys + kRsTile);  // kRsTile
    unsigned (*warp_cnt)[kRsBins] = reinterpret_cast<unsigned (*)[kRsBins]>(rs_smem);  // aliases skeys
    __shared__ unsigned digit_start[kRsBins];   // block-local exclusive prefix over digits
    __shared__ unsigned digit_base[kRsBins];    // global output offset of (digit, block)
    __shared__ unsigned s_warp[32];

    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < kRsWarps * kRsBins; k += kRsThreads) (&warp_cnt[0][0])[k] = 0;

    const long long tile = blockIdx.x * (long long)kRsTile;
    const long long base = tile + w * kRsWarpSpan + lane;
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned long long key[kRsItems];
    unsigned val[kRsItems];
    unsigned short rank[kRsItems];
#pragma unroll
    for (int k = 0; k < kRsItems; ++k) {
        const long long i = base + k * 32;
        const bool valid = i < n;
        key[k] = valid ? kin[i] : 0ull;
        val[k] = valid ? vin[i] : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kRsItems; ++k) {
        const bool valid = base + k * 32 < n;
        const unsigned d = valid ? (unsigned)(key[k] >> shift) & kRsMask : (unsigned)kRsBins;
        const unsigned peers = digit_peers(d, valid);
        unsigned before = 0;
        if (valid) before = warp_cnt[w][d];
        __syncwarp();
        if (valid) {
            rank[k] = (unsigned short)(before + __popc(peers & lt_mask));
            if ((__ffs(peers) - 1) == lane) warp_cnt[w][d] = before + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    // Per digit (thread t: digits kRsDpt t ...): exclusive prefix over warps
    // (stable: warp w precedes w+1), then over digits; the digit's global
    // offset is the scan of the digit totals plus this tile's row prefix.
    unsigned run[kRsDpt], tot[kRsDpt];
    unsigned rsum = 0, tsum = 0;
#pragma unroll
    for (int j = 0; j < kRsDpt; ++j) {
        const unsigned d = kRsDpt * threadIdx.x + j;
        run[j] = 0;
#pragma unroll
        for (int ww = 0; ww < kRsWarps; ++ww) {
            const unsigned c = warp_cnt[ww][d];
            warp_cnt[ww][d] = run[j];
            run[j] += c;
        }
        tot[j] = __ldg(totals + d);
        rsum += run[j];
        tsum += tot[j];
    }
    unsigned total;
    unsigned ds = block_exclusive_scan(rsum, s_warp, total);
    unsigned gs = block_exclusive_scan(tsum, s_warp, total);
#pragma unroll
    for (int j = 0; j < kRsDpt; ++j) {
        const unsigned d = kRsDpt * threadIdx.x + j;
        digit_start[d] = ds;
        digit_base[d] = gs + hist_scan[d * gridDim.x + blockIdx.x];
        ds += run[j];
        gs += tot[j];
    }
    __syncthreads();
    // every key's place in the tile, then (counters dead) the tile itself
#pragma unroll
    for (int k = 0; k < kRsItems; ++k) {
        if (base + k * 32 < n) {
            const unsigned dd = (unsigned)(key[k] >> shift) & kRsMask;
            rank[k] = (unsigned short)(digit_start[dd] + warp_cnt[w][dd] + rank[k]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kRsItems; ++k) {
        if (base + k * 32 < n) {
            skeys[rank[k]] = key[k];
            svals[rank[k]] = val[k];
        }
    }
    __syncthreads();
    long long nvalid = n - tile;
    if (nvalid > kRsTile) nvalid = kRsTile;
    for (int j = threadIdx.x; j < nvalid; j += kRsThreads) {
        const unsigned long long kk = skeys[j];
        const unsigned dd = (unsigned)(kk >> shift) & kRsMask;
        const unsigned o = digit_base[dd] + (unsigned)j - digit_start[dd];
        kout[o] = kk;
        vout[o] = svals[j];
    }
}

long long radix_hist_size(long long n) { return ((n + kRsTile - 1) / kRsTile + 1) * kRsBins; }

void radix_sort_pairs(SortBuffers& sb, long long n, int passes, int shift0, cudaStream_t s) {
    if (n <= 1) return;
    const int nb = (int)((n + kRsTile - 1) / kRsTile);
    static bool attr_done = false;
    if (!attr_done) {
        cudaFuncSetAttribute(rs_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRsScatterSmem);
        attr_done = true;
    }
    unsigned* totals = sb.hist + (long long)nb * kRsBins;
    unsigned long long* kin = sb.keys;
    unsigned long long* kout = sb.keys_alt;
    unsigned* vin = sb.vals;
    unsigned* vout = sb.vals_alt;
    for (int p = 0; p < passes; ++p) {
        const int shift = shift0 + kRsDigitBits * p;
        rs_hist_kernel<<<nb, kRsThreads, 0, s>>>(kin, n, shift, sb.hist);
        rs_scan_kernel<<<kRsBins, kRsThreads, 0, s>>>(sb.hist, nb, totals);
        rs_scatter_kernel<<<nb, kRsThreads, kRsScatterSmem, s>>>(kin, vin, kout, vout, n, shift, sb.hist, totals);
        unsigned long long* tk = kin;
        kin = kout;
        kout = tk;
        unsigned* tv = vin;
        vin = vout;
        vout = tv;
    }
    if (passes & 1) {
        cudaMemcpyAsync(sb.keys, kin, sizeof(unsigned long long) * n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(sb.vals, vin, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, s);
    }
}

// ---------------------------------------------------------------------------
// Gather the state into key order: new[k] = old[perm[k]] (into the *2 buffers)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) permute_kernel(const unsigned* __restrict__ perm, long long n,
                                                      const float4* __restrict__ pos, const float4* __restrict__ plo,
                                                      const float4* __restrict__ vel, const float4* __restrict__ vlo,
                                                      const float4* __restrict__ acc,
                                                      const int* __restrict__ id, float4* __restrict__ pos2,
                                                      float4* __restrict__ plo2, float4* __restrict__ vel2,
                                                      float4* __restrict__ vlo2, float4* __restrict__ acc2,
                                                      int* __restrict__ id2) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const unsigned j = perm[k];
        pos2[k] = pos[j];
        if (plo) plo2[k] = plo[j];
        vel2[k] = vel[j];
        if (vlo) vlo2[k] = vlo[j];
        acc2[k] = acc[j];
        id2[k] = id[j];
    }
}

void launch_permute(const Particles& P, const unsigned* perm, long long n, bool split, cudaStream_t s) {
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    permute_kernel<<<(unsigned)blocks, 256, 0, s>>>(perm, n, P.pos, split ? P.plo : nullptr, P.vel,
                                                     split ? P.vlo : nullptr, P.acc, P.id, P.pos2,
                                                     split ? P.plo2 : nullptr, P.vel2, split ? P.vlo2 : nullptr,
                                                     P.acc2, P.id2);
}

}  // namespace ngrav
