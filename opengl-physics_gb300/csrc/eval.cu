// eval.cu -- force evaluation from the walk's interaction lists: P2C over
// each group's far list, P2P over its near list, and the closing half-kick.
//
// Arithmetic restates the reference (projects/nbody_core/src/Solvers.cpp):
//   P2P  a += G m d / (|d|^2 + eps^2)^(3/2)                 (AccumPairPlummer, :19-38)
//   P2C  the same softened monopole of the node's mass at its COM, plus the
//        unsoftened traceless quadrupole
//        a += -G Q.d / r^5 + 2.5 G (d.Q.d) d / r^7       (AddQuadrupole, :147-179)
// with the group's own members included as a near leaf (the self term is
// zero for eps > 0 and masked for eps == 0).
//
// GB300 mapping.  One warp per group (dynamic scheduling), lane = (target t,
// slice s): nt targets x floor(32/nt) source slices, each slice a contiguous
// run of the staged sources (odd length, so the slices of a quarter-warp
// read distinct bank groups), walked four at a time; slices are summed at
// the end of the group.  A group's targets run in blocks of up to 64, each
// in one or two passes over every staged chunk (split to keep the lanes
// busy: 20 targets as 4 x 8 + 16 x 2 slices), the second pass's sums parked
// in shared memory; 80 registers and about 9 KiB of shared memory per warp
// keep 6 CTAs of 4 warps per SM.
// Far records are staged 32 at a time into shared memory in the group's
// frame; the records of the next batch and the node ids of the one after
// are loaded while a batch is evaluated, so no batch waits on a list-id ->
// record load chain.  Near leaves are staged by TMA bulk copies
// (cp.async.bulk completing on an mbarrier with a bounded wait), one copy
// per run of leaves whose particles are contiguous (leaves are in key order,
// so siblings met together form one run), into a 5 KiB shared-memory
// buffer, each batch as many leaves (up to 32) as fit by their actual
// counts; the first near batch is in flight during the far field, and each
// next batch's leaf records load while a batch is evaluated.  (A second
// buffer would overlap copy and compute within the warp, but halves the
// resident warps; measured slower.)  In SPLIT precision the staged sources
// then move from their leaves' frames into the group's (each slot knows its
// leaf from a byte map written at staging), and each lane's partial sums
// are Kahan compensated once per staged chunk.
#include "engine.cuh"
#include "softening.cuh"

namespace ngrav {

constexpr int kEvalWarps = 4;
constexpr int kEvalThreads = kEvalWarps * 32;
constexpr int kSrcCap = 320;                  // sources per staging buffer (5 KiB)
constexpr int kBuffers = 1;                   // staging buffers per warp (2 halves occupancy)
constexpr unsigned kWaitLimit = 1u << 26;     // bounded mbarrier polling

struct __align__(128) EvalSmem {
    float4 src[kBuffers][kSrcCap];            // TMA destinations
    float4 farA[32];                          // far batch: COM in the group frame, mass
    float4 farB[32];                          //   Qxx Qyy Qxy Qxz
    float2 farQ[32];                          //   Qyz, Qzz = -(Qxx + Qyy)
    float red[3][32];                         // slice reduction
    float4 pass_tgt[32];                      // second pass of a target block: target, packed lane map
    float4 pass_acc[32];                      //   running sums ax ay az, compensation cx
    float2 pass_cmp[32];                      //   compensation cy cz
    float4 shift[kBuffers][32];               // near-leaf frame shift (SPLIT)
    int start[kBuffers][32];
    int pre[kBuffers][33];
    unsigned long long bar[2];
    unsigned char owner[kSrcCap];             // staged slot -> its leaf's lane in the batch (SPLIT)
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait for the phase with parity `phase`; false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned phase) {
    const unsigned b = smem_u32(bar);
    for (unsigned it = 0; it < kWaitLimit; ++it) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(b), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ int excl_scan(int v, int lane, int& total) {
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

// Lane mapping for a block of nt <= 32 targets: lane = (target t, slice s),
// t = lane % nt, s = lane / nt, S = floor(32 / nt) slices.  All lanes of a
// slice read the same source (shared-memory broadcast).  P2P slices are
// contiguous runs of the staged sources (p2p_chunk); P2C slices take records
// s, s + S, s + 2S, ... of a 32-record batch.
struct Lane {
    float tx, ty, tz;
    int sl, S, nt;
    bool active;
    float ax, ay, az, cx, cy, cz;
};

// Adds one chunk's partial sum; in SPLIT precision Kahan-compensated (the
// compensation costs four adds per component per chunk, not per pair).
template <bool SPLIT>
__device__ __forceinline__ void accumulate(Lane& g, float px, float py, float pz) {
    if (SPLIT) {
        float y = px - g.cx, t = g.ax + y;
        g.cx = (t - g.ax) - y;
        g.ax = t;
        y = py - g.cy;
        t = g.ay + y;
        g.cy = (t - g.ay) - y;
        g.ay = t;
        y = pz - g.cz;
        t = g.az + y;
        g.cz = (t - g.az) - y;
        g.az = t;
    } else {
        g.ax += px;
        g.ay += py;
        g.az += pz;
    }
}

// Target blocks of up to 64 targets run in one or two passes over each
// staged chunk: pass 0 takes the first `first[n]` targets, pass 1 the rest,
// each with floor(32 / targets) source slices.  The split minimises the
// source steps per staged source, 1/S0 + 1/S1 (plus 0.03 per extra pass for
// its loop and accumulator traffic), against one pass of all n (1/S, n <= 32):
// a block of 20 targets runs as 4 x 8 slices + 16 x 2 slices (0.625 steps
// per source) instead of 20 lanes with 12 idle (1 step), and a block of 40
// as 8 x 4 + 32 x 1 without staging its lists twice.
constexpr int kBlockTargets = 64;
struct PassSplit {
    unsigned char first[kBlockTargets + 1];
};
constexpr PassSplit make_pass_split() {
    PassSplit t{};
    for (int n = 1; n <= kBlockTargets; ++n) {
        float best = n <= 32 ? 1.f / (float)(32 / n) : 1e30f;
        int b0 = n <= 32 ? n : 32;
        for (int a = 1; a < n && a <= 32; ++a) {
            const int b = n - a;
            if (b > 32) continue;
            const float c = 1.f / (float)(32 / a) + 1.f / (float)(32 / b) + 0.03f;
            if (c < best) {
                best = c;
                b0 = a;
            }
        }
        t.first[n] = (unsigned char)b0;
    }
    return t;
}
__constant__ PassSplit kPassSplit = make_pass_split();

// Lane map of nt <= 32 targets starting at slot `first`, sums zeroed.
__device__ __forceinline__ Lane make_lane(const float4* __restrict__ src, int first, int nt, int lane) {
    Lane g;
    g.nt = nt;
    g.S = 32 / nt;
    g.active = lane < nt * g.S;
    g.sl = lane / nt;
    const float4 tp = src[first + lane % nt];
    g.tx = tp.x;
    g.ty = tp.y;
    g.tz = tp.z;
    g.ax = g.ay = g.az = g.cx = g.cy = g.cz = 0.f;
    return g;
}

__device__ __forceinline__ void save_pass(EvalSmem& sm, const Lane& g, int lane) {
    const int map = g.sl | (g.S << 8) | (g.nt << 16) | ((int)g.active << 24);
    sm.pass_tgt[lane] = make_float4(g.tx, g.ty, g.tz, __int_as_float(map));
    sm.pass_acc[lane] = make_float4(g.ax, g.ay, g.az, g.cx);
    sm.pass_cmp[lane] = make_float2(g.cy, g.cz);
}

__device__ __forceinline__ Lane load_pass(const EvalSmem& sm, int lane) {
    Lane g;
    const float4 t = sm.pass_tgt[lane], a = sm.pass_acc[lane];
    const float2 c = sm.pass_cmp[lane];
    const int map = __float_as_int(t.w);
    g.tx = t.x;
    g.ty = t.y;
    g.tz = t.z;
    g.sl = map & 0xFF;
    g.S = (map >> 8) & 0xFF;
    g.nt = (map >> 16) & 0xFF;
    g.active = (map >> 24) != 0;
    g.ax = a.x;
    g.ay = a.y;
    g.az = a.z;
    g.cx = a.w;
    g.cy = c.x;
    g.cz = c.y;
    return g;
}

// Applies `f` (one chunk's evaluation) to pass 0 (registers) and, for a
// two-pass block, to pass 1 (shared memory).
template <class F>
__device__ __forceinline__ void for_passes(Lane& g, bool two, EvalSmem& sm, int lane, F&& f) {
    f(g);
    if (two) {
        Lane h = load_pass(sm, lane);
        f(h);
        sm.pass_acc[lane] = make_float4(h.ax, h.ay, h.az, h.cx);
        sm.pass_cmp[lane] = make_float2(h.cy, h.cz);
    }
}

// SOFT: 0 Plummer, 1 Plummer with eps = 0 (the self pair gives 0), 2 spline.
template <int SOFT>
__device__ __forceinline__ void p2p_pair(const float4& a, float tx, float ty, float tz, float eps2, float ih,
                                         float& px, float& py, float& pz) {
    const float dx = a.x - tx, dy = a.y - ty, dz = a.z - tz;
    float f;
    if (SOFT == 2) {
        f = pair_factor<kSoftSpline>(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), a.w, 0.f, ih);
    } else {
        const float r = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
        const float ir = rsqrtf(r);
        f = a.w * (ir * ir * ir);
        if (SOFT == 1) f = r > 0.f ? f : 0.f;
    }
    px = fmaf(f, dx, px);
    py = fmaf(f, dy, py);
    pz = fmaf(f, dz, pz);
}

// One staged chunk of ns sources against the lane's target.  Slice s takes a
// contiguous run of len = ceil(ns / S) sources (rounded up to odd: the S
// slices of a quarter-warp then read distinct shared-memory bank groups in
// the same LDS.128), walked four at a time with immediate offsets from one
// pointer, in two independent accumulation chains.
template <bool SPLIT, int SOFT>
__device__ __forceinline__ void p2p_chunk(Lane& g, const float4* __restrict__ s_src, int ns, float eps2, float ih) {
    if (!g.active) return;
    float px = 0.f, py = 0.f, pz = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;
    const float tx = g.tx, ty = g.ty, tz = g.tz;
    const int len = ((ns + g.S - 1) / g.S) | 1;
    const int b = min(ns, g.sl * len);
    const float4* p = s_src + b;
    const float4* const pe = s_src + min(ns, b + len);
    for (; p + 4 <= pe; p += 4) {
        const float4 a0 = p[0], a1 = p[1], a2 = p[2], a3 = p[3];
        p2p_pair<SOFT>(a0, tx, ty, tz, eps2, ih, px, py, pz);
        p2p_pair<SOFT>(a1, tx, ty, tz, eps2, ih, qx, qy, qz);
        p2p_pair<SOFT>(a2, tx, ty, tz, eps2, ih, px, py, pz);
        p2p_pair<SOFT>(a3, tx, ty, tz, eps2, ih, qx, qy, qz);
    }
    for (; p < pe; ++p) p2p_pair<SOFT>(p[0], tx, ty, tz, eps2, ih, px, py, pz);
    accumulate<SPLIT>(g, px + qx, py + qy, pz + qz);
}

template <bool SPLIT, bool QUAD, int SOFT>
__device__ __forceinline__ void p2c_chunk(Lane& g, const float4* __restrict__ fA, const float4* __restrict__ fB,
                                          const float2* __restrict__ fQ, int nf, float eps2, float ih) {
    if (!g.active) return;
    float px = 0.f, py = 0.f, pz = 0.f;
    const float tx = g.tx, ty = g.ty, tz = g.tz;
    for (int f = g.sl; f < nf; f += g.S) {
        const float4 A = fA[f];
        const float dx = A.x - tx, dy = A.y - ty, dz = A.z - tz;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float fm = pair_factor<SOFT == 2 ? kSoftSpline : kSoftPlummer>(r2, A.w, eps2, ih);
        if (QUAD) {
            const float4 B = fB[f];
            const float2 Q = fQ[f];  // Qyz, Qzz
            const float qdx = fmaf(B.x, dx, fmaf(B.z, dy, B.w * dz));
            const float qdy = fmaf(B.z, dx, fmaf(B.y, dy, Q.x * dz));
            const float qdz = fmaf(B.w, dx, fmaf(Q.x, dy, Q.y * dz));
            const float qd2 = fmaf(dx, qdx, fmaf(dy, qdy, dz * qdz));
            const float ir = rsqrtf(r2);
            const float ir2 = ir * ir;
            const float ir5 = ir2 * ir2 * ir;
            // monopole and the radial quadrupole term share one multiplier of d
            const float c = fm + 2.5f * qd2 * (ir5 * ir2);
            px = fmaf(-ir5, qdx, fmaf(c, dx, px));
            py = fmaf(-ir5, qdy, fmaf(c, dy, py));
            pz = fmaf(-ir5, qdz, fmaf(c, dz, pz));
        } else {
            px = fmaf(fm, dx, px);
            py = fmaf(fm, dy, py);
            pz = fmaf(fm, dz, pz);
        }
    }
    accumulate<SPLIT>(g, px, py, pz);
}

// One near leaf's info (lane = list entry), loaded into registers.  The
// leaf centre's double-float halves are kept as loaded: the frame shift is
// formed only when the batch is staged, a batch later, so these loads never
// stall the batch being computed.
struct NearInfo {
    int start, cnt;
    float4 h, l;
};

// Publish a batch's info to buffer `b` and start its TMA copies: one bulk
// copy per run of leaves whose particles are contiguous in memory (leaves
// are in key order, so siblings met together form one run), issued by the
// run's first lane.  In SPLIT precision each lane also forms its leaf's
// frame shift and marks the staged slots of its leaf in `owner`.  Returns
// the number of staged sources.
template <bool SPLIT>
__device__ __forceinline__ int stage_batch(EvalSmem& sm, int b, const NearInfo& in, int lane,
                                          const float4* __restrict__ src, const float4& gchi, const float4& gclo) {
    int tot;
    const int ex = excl_scan(in.cnt, lane, tot);
    sm.start[b][lane] = in.start;
    sm.pre[b][lane] = ex;
    if (lane == 31) sm.pre[b][32] = tot;
    if (SPLIT) {
        sm.shift[b][lane] = make_float4((in.h.x - gchi.x) + (in.l.x - gclo.x), (in.h.y - gchi.y) + (in.l.y - gclo.y),
                                        (in.h.z - gchi.z) + (in.l.z - gclo.z), 0.f);
        for (int k = 0; k < in.cnt; ++k) sm.owner[ex + k] = (unsigned char)lane;
    }
    if (tot > 0) {
        // run heads: a staged leaf that does not continue the previous lane's range
        const int pend = __shfl_up_sync(0xffffffffu, in.start + in.cnt, 1);
        const int pcnt = __shfl_up_sync(0xffffffffu, in.cnt, 1);
        const bool head = in.cnt > 0 && (lane == 0 || pcnt == 0 || pend != in.start);
        const unsigned heads = __ballot_sync(0xffffffffu, head);
        const unsigned later = heads & ~(0xFFFFFFFFu >> (31 - lane));  // heads after this lane
        const int nxt = later ? __ffs(later) - 1 : 31;
        const int ex_next = __shfl_sync(0xffffffffu, ex, nxt);
        const int run_end = later ? ex_next : tot;
        if (lane == 0) mbar_expect_tx(&sm.bar[b], (unsigned)tot * 16u);
        __syncwarp();
        if (head) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tma_load_1d(&sm.src[b][ex], src + in.start, (unsigned)(run_end - ex) * 16u, &sm.bar[b]);
        }
    }
    __syncwarp();
    return tot;
}

// A leaf's staging info from its node id (-1: past the list, count 0).
template <bool SPLIT>
__device__ __forceinline__ NearInfo near_info_of(const NodeArrays& T, int node) {
    NearInfo r;
    r.start = 0;
    r.cnt = 0;
    r.h = make_float4(0.f, 0.f, 0.f, 0.f);
    r.l = r.h;
    if (node >= 0) {
        const float4 Cw = T.wC[node];
        r.start = __float_as_int(Cw.z);
        r.cnt = __float_as_int(Cw.w) & 0xFFFFFF;
        if (SPLIT) {
            r.h = T.chi[node];
            r.l = T.clo[node];
        }
    }
    return r;
}

// The near list's node ids of entries pos .. pos+63 held in registers (w0:
// pos + lane, w1: pos + 32 + lane; -1 past the list), so a batch's leaf
// records load from ids that arrived a batch earlier.  A batch takes at most
// 32 entries, so the ids still needed after it are in the window and only
// its tail is refilled from memory; the window spans at most two of the
// list's 128-entry chunks (ca holds pos, cb is the next one).
struct NearWindow {
    int pos, w0, w1, ca, cb;
};

__device__ __forceinline__ int near_entry(const ListBuffers& LB, const NearWindow& W, int e, int nnear) {
    if (e >= nnear) return -1;
    const int c = (e >> 7) == (W.pos >> 7) ? W.ca : W.cb;
    return LB.near[(long long)c * kListChunk + (e & (kListChunk - 1))];
}

__device__ __forceinline__ NearWindow near_window(const ListBuffers& LB, int first, int nnear, int lane) {
    NearWindow W;
    W.pos = 0;
    W.ca = first;
    W.cb = nnear > kListChunk ? LB.near_next[first] : -1;
    W.w0 = lane < nnear ? LB.near[(long long)first * kListChunk + lane] : -1;
    W.w1 = 32 + lane < nnear ? LB.near[(long long)first * kListChunk + 32 + lane] : -1;
    return W;
}

// Move the window forward by nb <= 32 entries.
__device__ __forceinline__ void near_advance(const ListBuffers& LB, NearWindow& W, int nb, int nnear, int lane) {
    const int i0 = nb + lane, i1 = nb + 32 + lane;  // old-window indices of the new w0, w1
    const int a0 = __shfl_sync(0xffffffffu, W.w0, i0 & 31);
    const int a1 = __shfl_sync(0xffffffffu, W.w1, i0 & 31);
    const int b1 = __shfl_sync(0xffffffffu, W.w1, i1 & 31);
    const int n0 = i0 < 32 ? a0 : a1;
    const int n1 = i1 < 64 ? b1 : near_entry(LB, W, W.pos + i1, nnear);
    W.w0 = n0;
    W.w1 = n1;
    const int np = W.pos + nb;
    if ((np >> 7) != (W.pos >> 7)) {  // the window now starts in the next chunk
        W.ca = W.cb;
        W.cb = ((np >> 7) + 1) * kListChunk < nnear ? LB.near_next[W.ca] : -1;
    }
    W.pos = np;
}

// Stage the longest prefix of the 32 leaves in `in` whose sources fit `cap`
// (at least one: every leaf fits the buffer outside the big-leaf path).
// Returns the staged source count; nb = leaves staged.
template <bool SPLIT>
__device__ __forceinline__ int stage_fitting(EvalSmem& sm, const NearInfo& in, int lane,
                                             const float4* __restrict__ src, int cap, int& nb,
                                             const float4& gchi, const float4& gclo) {
    int tot;
    const int ex = excl_scan(in.cnt, lane, tot);
    const bool fits = ex + in.cnt <= cap || lane == 0;
    nb = __popc(__ballot_sync(0xffffffffu, fits));  // counts are >= 0: a prefix of lanes
    NearInfo mine = in;
    if (lane >= nb) mine.cnt = 0;
    return stage_batch<SPLIT>(sm, 0, mine, lane, src, gchi, gclo);
}

// Moves a staged batch of ns sources from their leaves' frames into the
// group's frame: source j adds the shift of the leaf that owns its slot.
// The iterations are independent, so their shared-memory loads overlap.
__device__ __forceinline__ void shift_batch(EvalSmem& sm, int ns, int lane) {
#pragma unroll 4
    for (int j = lane; j < ns; j += 32) {
        const float4 sh = sm.shift[0][sm.owner[j]];
        float4 v = sm.src[0][j];
        v.x += sh.x;
        v.y += sh.y;
        v.z += sh.z;
        sm.src[0][j] = v;
    }
}

// Sums the slices of each of a pass's targets (slots first .. first+nt-1),
// writes the accelerations and applies the closing half kick.
template <bool SPLIT>
__device__ __forceinline__ void finish_targets(EvalSmem& sm, const Lane& g, int first, int lane,
                                               const WalkParams& wp, float4* __restrict__ acc,
                                               float4* __restrict__ vel, float4* __restrict__ vlo) {
    if (g.active) {
        sm.red[0][lane] = g.ax;
        sm.red[1][lane] = g.ay;
        sm.red[2][lane] = g.az;
    }
    __syncwarp();
    if (lane < g.nt) {
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int s = 0; s < g.S; ++s) {
            sx += sm.red[0][lane + s * g.nt];
            sy += sm.red[1][lane + s * g.nt];
            sz += sm.red[2][lane + s * g.nt];
        }
        const float ax = wp.G * sx, ay = wp.G * sy, az = wp.G * sz;
        const int slot = first + lane;
        acc[slot] = make_float4(ax, ay, az, 0.f);
        if (wp.kick) {
            float4 v = vel[slot];
            float4 vl = SPLIT ? vlo[slot] : make_float4(0.f, 0.f, 0.f, 0.f);
            kick_v(v, SPLIT ? &vl : nullptr, wp.hdt, make_float4(ax, ay, az, 0.f));
            vel[slot] = v;
            if (SPLIT) vlo[slot] = vl;
        }
    }
    __syncwarp();
}

template <bool SPLIT, bool QUAD, int SOFT>
__global__ void __launch_bounds__(kEvalThreads, 6) eval_kernel(NodeArrays T, Counters* C,
                                                            const float4* __restrict__ src,
                                                            float4* __restrict__ acc, float4* __restrict__ vel,
                                                            float4* __restrict__ vlo,
                                                            const int* __restrict__ leaf_list, WalkParams wp,
                                                            ListBuffers LB) {
    extern __shared__ __align__(128) unsigned char eval_smem_raw[];
    const int lane = threadIdx.x & 31;
    EvalSmem& sm = reinterpret_cast<EvalSmem*>(eval_smem_raw)[threadIdx.x >> 5];
    if (C->status & kStFatal) return;
    if (lane == 0) {
        mbar_init(&sm.bar[0]);
        mbar_init(&sm.bar[1]);
    }
    __syncwarp();
    unsigned phase[2] = {0u, 0u};
    const int nleaves = C->nleaves;
    // Sources per near batch: the tuned cap (at most one staging buffer).
    const int maxleaf = max(1, C->max_leaf_count);
    const int tile = wp.p2p_tile > 0 && wp.p2p_tile < kSrcCap ? wp.p2p_tile : kSrcCap;
    const bool big_leaves = maxleaf > kSrcCap;
    unsigned long long pairs = 0, p2c = 0;
    bool timeout = false;

    for (;;) {
        int gi = 0;
        if (lane == 0) gi = atomicAdd(&C->eval_next, 1);
        gi = __shfl_sync(0xffffffffu, gi, 0);
        if (gi >= nleaves) break;
        const int leaf = leaf_list[gi];
        const float4 gC = T.wC[leaf];
        const int gstart = __float_as_int(gC.z);
        const int gcount = __float_as_int(gC.w) & 0xFFFFFF;
        const int4 gin = LB.ginfo[gi];
        const int far_first = gin.x, near_first = gin.y, nfar = gin.z, nnear = gin.w;
        float4 gchi = make_float4(0.f, 0.f, 0.f, 0.f), gclo = gchi;
        if (SPLIT) {
            gchi = T.chi[leaf];
            gclo = T.clo[leaf];
        }
        for (int t0 = 0; t0 < gcount; t0 += kBlockTargets) {
            const int nblk = min(kBlockTargets, gcount - t0);
            const int b0 = kPassSplit.first[nblk];
            const bool two = b0 < nblk;
            // Far records come in batches of 32 list entries.  The records of
            // batch k are loaded during batch k-1 and the node ids of batch
            // k+1 during batch k-1 as well (chunk links one chunk ahead), so
            // no batch waits on a list-id -> record load chain of its own.
            // The first near batch's leaf records load alongside the first
            // far batch, and its copies are in flight during the far field.
            int fcur = far_first;                                    // chunk of the next ids to load
            int fnxt = nfar > kListChunk ? LB.far_next[far_first] : -1;
            float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A, D = A;
            {
                const int id0 = lane < nfar ? LB.far[(long long)fcur * kListChunk + lane] : -1;
                if (id0 >= 0) {
                    A = T.wA[id0];
                    D = T.wD[id0];
                    if (QUAD) B = T.wB[id0];
                }
            }
            int fid = 32 + lane < nfar ? LB.far[(long long)fcur * kListChunk + 32 + lane] : -1;  // batch 1
            int nb = 0, ns_cur = 0;
            NearWindow W = {0, -1, -1, -1, -1};
            NearInfo info;
            if (!big_leaves) {
                W = near_window(LB, near_first, nnear, lane);
                info = near_info_of<SPLIT>(T, W.w0);
            }
            Lane g = make_lane(src, gstart + t0, b0, lane);
            if (two) save_pass(sm, make_lane(src, gstart + t0 + b0, nblk - b0, lane), lane);
            if (!big_leaves) {
                ns_cur = stage_fitting<SPLIT>(sm, info, lane, src, tile, nb, gchi, gclo);
                near_advance(LB, W, nb, nnear, lane);
            }

            // ---- far field ----
            for (int b = 0, k = 0; b < nfar; b += 32, ++k) {
                if (b + lane < nfar) {
                    float4 rA = A;
                    if (SPLIT) {
                        rA.x = (A.x - gchi.x) + (D.x - gclo.x);
                        rA.y = (A.y - gchi.y) + (D.y - gclo.y);
                        rA.z = (A.z - gchi.z) + (D.z - gclo.z);
                    }
                    sm.farA[lane] = rA;
                    if (QUAD) {
                        sm.farB[lane] = B;
                        sm.farQ[lane] = make_float2(D.w, -(B.x + B.y));
                    }
                }
                __syncwarp();
                if (fid >= 0) {  // records of batch k+1
                    A = T.wA[fid];
                    D = T.wD[fid];
                    if (QUAD) B = T.wB[fid];
                }
                fid = -1;
                const int e2 = b + 64;  // first entry of batch k+2
                if (e2 < nfar) {
                    if ((e2 & (kListChunk - 1)) == 0) {  // batch k+2 opens the next chunk
                        fcur = fnxt;
                        fnxt = e2 + kListChunk < nfar ? LB.far_next[fcur] : -1;
                    }
                    if (e2 + lane < nfar) fid = LB.far[(long long)fcur * kListChunk + (e2 & (kListChunk - 1)) + lane];
                }
                const int nrec = min(32, nfar - b);
                for_passes(g, two, sm, lane, [&](Lane& x) {
                    p2c_chunk<SPLIT, QUAD, SOFT>(x, sm.farA, sm.farB, sm.farQ, nrec, wp.eps2, wp.ih);
                });
                __syncwarp();
            }
            p2c += (unsigned long long)nblk * (unsigned long long)nfar;

            // ---- near field: batches of up to 32 leaves (as many as fit the
            // staging buffer, by their actual counts) staged by TMA ----
            int total = 0;
            if (!big_leaves) {
                // batch 0 was staged before the far field
                if (W.pos < nnear) info = near_info_of<SPLIT>(T, W.w0);
                while (ns_cur > 0) {
                    if (!mbar_wait(&sm.bar[0], phase[0])) {
                        timeout = true;
                        break;
                    }
                    phase[0] ^= 1u;
                    if (SPLIT) shift_batch(sm, ns_cur, lane);  // into the group's frame
                    __syncwarp();
                    for_passes(g, two, sm, lane,
                               [&](Lane& x) { p2p_chunk<SPLIT, SOFT>(x, sm.src[0], ns_cur, wp.eps2, wp.ih); });
                    __syncwarp();
                    total += ns_cur;
                    // stage the next batch (its info is in registers), then fetch
                    // the info of the one after
                    int ns_next = 0;
                    if (W.pos < nnear) {
                        ns_next = stage_fitting<SPLIT>(sm, info, lane, src, tile, nb, gchi, gclo);
                        near_advance(LB, W, nb, nnear, lane);
                        if (W.pos < nnear) info = near_info_of<SPLIT>(T, W.w0);
                    }
                    ns_cur = ns_next;
                }
                if (timeout) {
                    // give copies still in flight a bounded chance to land
                    mbar_wait(&sm.bar[0], phase[0]);
                    if (kBuffers == 2) mbar_wait(&sm.bar[1], phase[1]);
                }
            } else {
                // Leaves larger than a staging buffer (depth-limited): plain loads, piecewise.
                int c = near_first;
                for (int b = 0; b < nnear; ++b) {
                    if (b > 0 && (b & (kListChunk - 1)) == 0) c = LB.near_next[c];
                    const int node = LB.near[(long long)c * kListChunk + (b & (kListChunk - 1))];
                    const float4 Cw = T.wC[node];
                    const int st = __float_as_int(Cw.z), cn = __float_as_int(Cw.w) & 0xFFFFFF;
                    float4 sh = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (SPLIT) {
                        const float4 h = T.chi[node], l = T.clo[node];
                        sh = make_float4((h.x - gchi.x) + (l.x - gclo.x), (h.y - gchi.y) + (l.y - gclo.y),
                                         (h.z - gchi.z) + (l.z - gclo.z), 0.f);
                    }
                    for (int off = 0; off < cn; off += kSrcCap) {
                        const int ns = min(kSrcCap, cn - off);
                        __syncwarp();
                        for (int j = lane; j < ns; j += 32) {
                            float4 v = src[st + off + j];
                            v.x += sh.x;
                            v.y += sh.y;
                            v.z += sh.z;
                            sm.src[0][j] = v;
                        }
                        __syncwarp();
                        for_passes(g, two, sm, lane,
                                   [&](Lane& x) { p2p_chunk<SPLIT, SOFT>(x, sm.src[0], ns, wp.eps2, wp.ih); });
                    }
                    __syncwarp();
                    total += cn;
                }
            }
            if (timeout) break;
            pairs += (unsigned long long)nblk * (unsigned long long)total - (unsigned long long)nblk;

            // ---- sum the slices of each target, write a, closing kick ----
            finish_targets<SPLIT>(sm, g, gstart + t0, lane, wp, acc, vel, vlo);
            if (two) finish_targets<SPLIT>(sm, load_pass(sm, lane), gstart + t0 + b0, lane, wp, acc, vel, vlo);
            __syncwarp();
        }
        if (timeout) break;
    }
    if (timeout && lane == 0) atomicOr(&C->status, kStTimeout);
    if (lane == 0) {
        atomicAdd(&C->p2p_pairs, pairs);
        atomicAdd(&C->p2c_terms, p2c);
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

size_t eval_smem_bytes() { return sizeof(EvalSmem) * kEvalWarps; }
int eval_warps_per_block() { return kEvalWarps; }

#define NGRAV_EVAL_INSTANCES(X)                                                       \
    X(true, true, 0) X(true, true, 1) X(true, true, 2) X(true, false, 0) X(true, false, 1) \
    X(true, false, 2) X(false, true, 0) X(false, true, 1) X(false, true, 2) X(false, false, 0) \
    X(false, false, 1) X(false, false, 2)

void eval_set_attributes() {
    const int bytes = (int)eval_smem_bytes();
#define NGRAV_ATTR(SP, Q, Z) \
    cudaFuncSetAttribute(eval_kernel<SP, Q, Z>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    NGRAV_EVAL_INSTANCES(NGRAV_ATTR)
#undef NGRAV_ATTR
}

int eval_blocks_per_sm() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, eval_kernel<true, true, 0>, kEvalThreads,
                                                  eval_smem_bytes());
    return nb > 0 ? nb : 1;
}

void launch_eval(const NodeArrays& T, Counters* C, const Particles& P, const int* leaf_list, const WalkParams& wp,
                 const ListBuffers& LB, int nwarps, cudaStream_t s) {
    const int blocks = (nwarps + kEvalWarps - 1) / kEvalWarps;
    const int soft = wp.soft == kSoftSpline ? 2 : (!(wp.eps2 > 0.f) ? 1 : 0);
    const size_t smem = eval_smem_bytes();
#define NGRAV_LAUNCH(SP, Q, Z)                                                                             \
    if (wp.split == (SP) && (wp.quadrupole != 0) == (Q) && soft == (Z))                                   \
        eval_kernel<SP, Q, Z><<<blocks, kEvalThreads, smem, s>>>(T, C, P.src, P.acc, P.vel, P.vlo, leaf_list, wp, LB);
    NGRAV_EVAL_INSTANCES(NGRAV_LAUNCH)
#undef NGRAV_LAUNCH
}

}  // namespace ngrav
