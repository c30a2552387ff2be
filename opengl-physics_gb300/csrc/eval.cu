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
// slice s): nt targets x floor(32/nt) source slices; slices are summed at
// the end of the group.  A group's targets run in blocks of up to 64, each
// in one or two passes over every staged chunk (split to keep the lanes
// busy: 20 targets as 4 x 8 + 16 x 2 slices), the second pass's sums parked
// in shared memory.  The pair arithmetic runs on Blackwell's packed FP32
// pipe (add / mul / fma .f32x2): each lane takes two sources per step, so
// twelve pair operations issue as six instructions and the kernel is bound
// by the FMA pipe rather than by issue slots, leaving the staging work its
// own issue slots.  Staged sources are therefore kept as pairs, {x0 x1 y0
// y1}{z0 z1 m0 m1}, and far records as pairs of records likewise.
// Far records are staged 32 at a time into shared memory in the group's
// frame; the records of the next batch and the node ids of the one after
// are loaded while a batch is evaluated, so no batch waits on a list-id ->
// record load chain.  Near leaves are staged by TMA bulk copies
// (cp.async.bulk completing on an mbarrier with a bounded wait), one copy
// per run of leaves whose particles are contiguous (leaves are in key order,
// so siblings met together form one run), into a 6 KiB shared-memory
// buffer, each batch as many leaves (up to 32) as fit by their actual
// counts; the first near batch is in flight during the far field, and the
// next batch's leaf records are copied into shared memory (cp.async) while
// a batch is evaluated.  A pass over each landed batch then pairs the
// sources up in place and, in SPLIT precision, moves them from their
// leaves' frames into the group's (each slot finds its leaf from a bit mask
// of the leaves' first slots), and each lane's partial sums are Kahan
// compensated once per staged chunk.
#include "engine.cuh"
#include "softening.cuh"

namespace ngrav {

constexpr int kEvalWarps = 4;
constexpr int kEvalThreads = kEvalWarps * 32;
constexpr int kEvalMinBlocks = 5;             // CTAs per SM (96 registers per thread)
constexpr int kSrcCap = 384;                  // sources per staging buffer (6 KiB; even: a pad slot for odd counts)
constexpr unsigned kWaitLimit = 1u << 26;     // bounded mbarrier polling
constexpr float kFarPad = 1e18f;              // position of the zero record that pads an odd far batch

struct __align__(128) EvalSmem {
    float4 src[kSrcCap];                      // TMA destination; then source pairs {x0 x1 y0 y1}{z0 z1 m0 m1}
    float4 farX[16];                          // far record pairs in the group frame: x0 x1 y0 y1
    float4 farZ[16];                          //   z0 z1 m0 m1
    float4 farQ0[16];                         //   Qxx0 Qxx1 Qyy0 Qyy1
    float4 farQ1[16];                         //   Qxy0 Qxy1 Qxz0 Qxz1
    float4 farQ2[16];                         //   Qyz0 Qyz1 Qzz0 Qzz1 (Qzz = -(Qxx + Qyy))
    float red[3][32];                         // slice reduction
    float4 pass_tgt[32];                      // second pass of a target block: target, packed lane map
    float4 pass_acc[32];                      //   running sums ax ay az, compensation cx
    float2 pass_cmp[32];                      //   compensation cy cz
    float4 shift[32];                         // staged leaves' frame shifts (SPLIT), by rank
    float4 nwc[32];                           // next near batch's leaf records (cp.async): wC
    float4 nhi[32];                           //   centre hi (SPLIT)
    float4 nlo[32];                           //   centre lo (SPLIT)
    float4 gch, gcl;                          // the group leaf's centre, hi and lo (SPLIT)
    int first[32];                            // staged leaves' first slots, by rank
    int nleaf;                                // non-empty leaves in the staged batch
    unsigned long long bar;
    unsigned long long npairs, nterms;        // interaction counters of this warp
};
// kEvalMinBlocks CTAs of kEvalWarps warps fit one SM's 228 KiB of shared
// memory (1 KiB of it reserved per CTA).
static_assert(kEvalMinBlocks * (kEvalWarps * sizeof(EvalSmem) + 1024) <= 228 * 1024, "eval smem per SM");

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
// slice read the same source pair (shared-memory broadcast).  P2P slices are
// contiguous runs of the staged source pairs (p2p_chunk); P2C slices take
// record pairs s, s + S, s + 2S, ... of a 32-record batch.
struct Lane {
    float tx, ty, tz;
    float rS;                                 // 1 / S, scaled up (slice_recip)
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

// 1 / S from the hardware reciprocal, scaled up by 2^-18 so that
// floor(n * rS) is the exact quotient n / S for every n <= 255 (the scaled
// error stays far below the 1 / S gap to the next integer).
__device__ __forceinline__ float slice_recip(int S) { return __fdividef(1.f, (float)S) * 1.000003814697265625f; }

// Lane map of nt <= 32 targets starting at slot `first`, sums zeroed.
__device__ __forceinline__ Lane make_lane(const float4* __restrict__ src, int first, int nt, int lane) {
    Lane g;
    g.nt = nt;
    g.S = 32 / nt;
    g.rS = slice_recip(g.S);
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
    g.rS = slice_recip(g.S);
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

// Packed FP32 pair arithmetic (two lanes of one register pair per op).
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// Two sources {x0 x1 y0 y1}{z0 z1 m0 m1} against one target (given negated
// and duplicated): the reference's softened pair
// (Solvers.cpp:19-38, AccumPairPlummer) for each, FP32.
// SOFT: 0 Plummer, 1 Plummer with eps = 0 (the self pair gives 0), 2 spline.
template <int SOFT>
__device__ __forceinline__ void p2p_pair2(const float4& P, const float4& Q, float2 ntx, float2 nty, float2 ntz,
                                          float2 e2, float ih, float2& ax, float2& ay, float2& az) {
    const float2 dx = add2(make_float2(P.x, P.y), ntx);
    const float2 dy = add2(make_float2(P.z, P.w), nty);
    const float2 dz = add2(make_float2(Q.x, Q.y), ntz);
    const float2 m = make_float2(Q.z, Q.w);
    float2 f;
    if (SOFT == 2) {
        const float2 r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
        f = make_float2(pair_factor<kSoftSpline>(r2.x, m.x, 0.f, ih), pair_factor<kSoftSpline>(r2.y, m.y, 0.f, ih));
    } else {
        const float2 r2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
        const float2 ir = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
        f = mul2(m, mul2(mul2(ir, ir), ir));
        if (SOFT == 1) {
            f.x = r2.x > 0.f ? f.x : 0.f;
            f.y = r2.y > 0.f ? f.y : 0.f;
        }
    }
    ax = fma2(f, dx, ax);
    ay = fma2(f, dy, ay);
    az = fma2(f, dz, az);
}

// One staged chunk of np source pairs against the lane's target.  Slice s
// takes a contiguous run of len = ceil(np / S) pairs (rounded up to odd: the
// slices of a quarter-warp then read distinct shared-memory bank groups in
// the same LDS.128), walked eight (then four) pairs at a time with immediate
// offsets from one pointer, in two independent accumulation chains.
template <bool SPLIT, int SOFT>
__device__ __forceinline__ void p2p_chunk(Lane& g, const float4* __restrict__ s2, int np, float eps2, float ih) {
    if (!g.active) return;
    const float2 ntx = dup2(-g.tx), nty = dup2(-g.ty), ntz = dup2(-g.tz), e2 = dup2(eps2);
    float2 ax = dup2(0.f), ay = ax, az = ax, bx = ax, by = ax, bz = ax;
    const int len = __float2int_rz((float)(np + g.S - 1) * g.rS) | 1;  // ceil(np / S), odd
    const int b = min(np, g.sl * len);
    const float4* p = s2 + 2 * b;
    const float4* const pe = s2 + 2 * min(np, b + len);
    for (; p + 16 <= pe; p += 16) {  // eight pairs in flight
        const float4 a0 = p[0], a1 = p[1], a2 = p[2], a3 = p[3], a4 = p[4], a5 = p[5], a6 = p[6], a7 = p[7];
        const float4 a8 = p[8], a9 = p[9], a10 = p[10], a11 = p[11], a12 = p[12], a13 = p[13], a14 = p[14], a15 = p[15];
        p2p_pair2<SOFT>(a0, a1, ntx, nty, ntz, e2, ih, ax, ay, az);
        p2p_pair2<SOFT>(a2, a3, ntx, nty, ntz, e2, ih, bx, by, bz);
        p2p_pair2<SOFT>(a4, a5, ntx, nty, ntz, e2, ih, ax, ay, az);
        p2p_pair2<SOFT>(a6, a7, ntx, nty, ntz, e2, ih, bx, by, bz);
        p2p_pair2<SOFT>(a8, a9, ntx, nty, ntz, e2, ih, ax, ay, az);
        p2p_pair2<SOFT>(a10, a11, ntx, nty, ntz, e2, ih, bx, by, bz);
        p2p_pair2<SOFT>(a12, a13, ntx, nty, ntz, e2, ih, ax, ay, az);
        p2p_pair2<SOFT>(a14, a15, ntx, nty, ntz, e2, ih, bx, by, bz);
    }
    for (; p + 8 <= pe; p += 8) {
        const float4 a0 = p[0], a1 = p[1], a2 = p[2], a3 = p[3], a4 = p[4], a5 = p[5], a6 = p[6], a7 = p[7];
        p2p_pair2<SOFT>(a0, a1, ntx, nty, ntz, e2, ih, ax, ay, az);
        p2p_pair2<SOFT>(a2, a3, ntx, nty, ntz, e2, ih, bx, by, bz);
        p2p_pair2<SOFT>(a4, a5, ntx, nty, ntz, e2, ih, ax, ay, az);
        p2p_pair2<SOFT>(a6, a7, ntx, nty, ntz, e2, ih, bx, by, bz);
    }
    for (; p < pe; p += 2) p2p_pair2<SOFT>(p[0], p[1], ntx, nty, ntz, e2, ih, ax, ay, az);
    const float2 sx = add2(ax, bx), sy = add2(ay, by), sz = add2(az, bz);
    accumulate<SPLIT>(g, sx.x + sx.y, sy.x + sy.y, sz.x + sz.y);
}

// One far batch of np record pairs against the lane's target: the softened
// monopole of each node's mass at its COM plus the unsoftened quadrupole
// (Solvers.cpp:147-179, AddQuadrupole), the two sharing one multiplier of
// the offset.  Packed FP32 over the two records of a pair.
template <bool SPLIT, bool QUAD, int SOFT>
__device__ __forceinline__ void p2c_chunk(Lane& g, const EvalSmem& sm, int np, float eps2, float ih) {
    if (!g.active) return;
    const float2 ntx = dup2(-g.tx), nty = dup2(-g.ty), ntz = dup2(-g.tz), e2 = dup2(eps2);
    float2 ax = dup2(0.f), ay = ax, az = ax;
    for (int k = g.sl; k < np; k += g.S) {
        const float4 X = sm.farX[k], Z = sm.farZ[k];
        const float2 dx = add2(make_float2(X.x, X.y), ntx);
        const float2 dy = add2(make_float2(X.z, X.w), nty);
        const float2 dz = add2(make_float2(Z.x, Z.y), ntz);
        const float2 m = make_float2(Z.z, Z.w);
        const float2 r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
        float2 fm;
        if (SOFT == 2) {
            fm = make_float2(pair_factor<kSoftSpline>(r2.x, m.x, eps2, ih), pair_factor<kSoftSpline>(r2.y, m.y, eps2, ih));
        } else {
            const float2 re = add2(r2, e2);
            const float2 is = make_float2(rsqrtf(re.x), rsqrtf(re.y));
            fm = mul2(m, mul2(mul2(is, is), is));
        }
        if (QUAD) {
            const float4 Q0 = sm.farQ0[k], Q1 = sm.farQ1[k], Q2 = sm.farQ2[k];
            const float2 qxx = make_float2(Q0.x, Q0.y), qyy = make_float2(Q0.z, Q0.w);
            const float2 qxy = make_float2(Q1.x, Q1.y), qxz = make_float2(Q1.z, Q1.w);
            const float2 qyz = make_float2(Q2.x, Q2.y), qzz = make_float2(Q2.z, Q2.w);
            const float2 qdx = fma2(qxx, dx, fma2(qxy, dy, mul2(qxz, dz)));
            const float2 qdy = fma2(qxy, dx, fma2(qyy, dy, mul2(qyz, dz)));
            const float2 qdz = fma2(qxz, dx, fma2(qyz, dy, mul2(qzz, dz)));
            const float2 qd2 = fma2(dx, qdx, fma2(dy, qdy, mul2(dz, qdz)));
            const float2 ir = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
            const float2 ir2 = mul2(ir, ir);
            const float2 ir5 = mul2(mul2(ir2, ir2), ir);
            const float2 nir5 = make_float2(-ir5.x, -ir5.y);
            // monopole and the radial quadrupole term share one multiplier of d
            const float2 c = fma2(mul2(dup2(2.5f), qd2), mul2(ir5, ir2), fm);
            ax = fma2(nir5, qdx, fma2(c, dx, ax));
            ay = fma2(nir5, qdy, fma2(c, dy, ay));
            az = fma2(nir5, qdz, fma2(c, dz, az));
        } else {
            ax = fma2(fm, dx, ax);
            ay = fma2(fm, dy, ay);
            az = fma2(fm, dz, az);
        }
    }
    accumulate<SPLIT>(g, ax.x + ax.y, ay.x + ay.y, az.x + az.y);
}

// Far record of lane `lane` (the batch's entry b + lane; a zero record far
// away when past the list) into its half of record pair lane / 2, in the
// group frame.
template <bool SPLIT, bool QUAD>
__device__ __forceinline__ void stage_far(EvalSmem& sm, int lane, bool valid, const float4& A, const float4& B,
                                          const float4& D) {
    float x = kFarPad, y = kFarPad, z = kFarPad, m = 0.f;
    float qxx = 0.f, qyy = 0.f, qxy = 0.f, qxz = 0.f, qyz = 0.f;
    if (valid) {
        x = A.x;
        y = A.y;
        z = A.z;
        if (SPLIT) {
            const float4 gh = sm.gch, gl = sm.gcl;
            x = (A.x - gh.x) + (D.x - gl.x);
            y = (A.y - gh.y) + (D.y - gl.y);
            z = (A.z - gh.z) + (D.z - gl.z);
        }
        m = A.w;
        if (QUAD) {
            qxx = B.x;
            qyy = B.y;
            qxy = B.z;
            qxz = B.w;
            qyz = D.w;
        }
    }
    const int k = lane >> 1, h = lane & 1;
    float* fx = reinterpret_cast<float*>(&sm.farX[k]);
    float* fz = reinterpret_cast<float*>(&sm.farZ[k]);
    fx[h] = x;
    fx[2 + h] = y;
    fz[h] = z;
    fz[2 + h] = m;
    if (QUAD) {
        float* q0 = reinterpret_cast<float*>(&sm.farQ0[k]);
        float* q1 = reinterpret_cast<float*>(&sm.farQ1[k]);
        float* q2 = reinterpret_cast<float*>(&sm.farQ2[k]);
        q0[h] = qxx;
        q0[2 + h] = qyy;
        q1[h] = qxy;
        q1[2 + h] = qxz;
        q2[h] = qyz;
        q2[2 + h] = -(qxx + qyy);
    }
}

// Leaf records of the next near batch (lane = list entry; node < 0: past
// the list) copied into shared memory by cp.async, so they cost no
// registers while the batch before is evaluated and land long before they
// are read.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

template <bool SPLIT>
__device__ __forceinline__ void prefetch_near(EvalSmem& sm, const NodeArrays& T, int node, int lane) {
    if (node >= 0) {
        cp_async16(&sm.nwc[lane], &T.wC[node]);
        if (SPLIT) {
            cp_async16(&sm.nhi[lane], &T.chi[node]);
            cp_async16(&sm.nlo[lane], &T.clo[node]);
        }
    } else {
        sm.nwc[lane] = make_float4(0.f, 0.f, 0.f, 0.f);  // count 0
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void prefetch_wait() {
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncwarp();
}

// Publish a batch (lane = leaf; cnt = 0 for lanes not staged; ex = the
// leaf's first slot, tot = the staged total) and start its TMA copies: one
// bulk copy per run of leaves whose particles are contiguous in memory
// (leaves are in key order, so siblings met together form one run), issued
// by the run's first lane.  The non-empty leaves' first slots and, in SPLIT
// precision, frame shifts are stored by rank for the pairing pass.
template <bool SPLIT>
__device__ __forceinline__ void stage_batch(EvalSmem& sm, int start, int cnt, int ex, int tot, int lane,
                                           const float4* __restrict__ src) {
    const unsigned nz = __ballot_sync(0xffffffffu, cnt > 0);
    if (cnt > 0) {
        const int r = __popc(nz & ((1u << lane) - 1u));
        sm.first[r] = ex;
        if (SPLIT) {
            const float4 h = sm.nhi[lane], l = sm.nlo[lane], gh = sm.gch, gl = sm.gcl;
            sm.shift[r] = make_float4((h.x - gh.x) + (l.x - gl.x), (h.y - gh.y) + (l.y - gl.y),
                                      (h.z - gh.z) + (l.z - gl.z), 0.f);
        }
    }
    if (lane == 0) sm.nleaf = __popc(nz);
    if (tot > 0) {
        // run heads: a staged leaf that does not continue the previous lane's range
        const int pend = __shfl_up_sync(0xffffffffu, start + cnt, 1);
        const int pcnt = __shfl_up_sync(0xffffffffu, cnt, 1);
        const bool head = cnt > 0 && (lane == 0 || pcnt == 0 || pend != start);
        const unsigned heads = __ballot_sync(0xffffffffu, head);
        const unsigned later = heads & ~(0xFFFFFFFFu >> (31 - lane));  // heads after this lane
        const int nxt = later ? __ffs(later) - 1 : 31;
        const int ex_next = __shfl_sync(0xffffffffu, ex, nxt);
        const int run_end = later ? ex_next : tot;
        if (lane == 0) mbar_expect_tx(&sm.bar, (unsigned)tot * 16u);
        __syncwarp();
        if (head) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tma_load_1d(&sm.src[ex], src + start, (unsigned)(run_end - ex) * 16u, &sm.bar);
        }
    }
    __syncwarp();
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

// Stage the longest prefix of the 32 prefetched leaves whose sources fit
// `cap` (at least one: every leaf fits the buffer outside the big-leaf
// path).  Returns the staged source count; nb = leaves staged.
template <bool SPLIT>
__device__ __forceinline__ int stage_fitting(EvalSmem& sm, int lane, const float4* __restrict__ src, int cap,
                                             int& nb) {
    prefetch_wait();
    const float4 Cw = sm.nwc[lane];
    const int start = __float_as_int(Cw.z), c = __float_as_int(Cw.w) & 0xFFFFFF;
    int tot;
    const int ex = excl_scan(c, lane, tot);
    const bool fits = ex + c <= cap || lane == 0;
    nb = __popc(__ballot_sync(0xffffffffu, fits));  // counts are >= 0: a prefix of lanes
    const int cnt = lane < nb ? c : 0;
    const int staged = __shfl_sync(0xffffffffu, ex + cnt, nb - 1);
    stage_batch<SPLIT>(sm, start, cnt, ex, staged, lane, src);
    return staged;
}

// Pairs up a landed batch of ns sources in place: slots 2k and 2k + 1
// become {x0 x1 y0 y1}{z0 z1 m0 m1} (an odd count pads slot ns with a zero
// mass at the group's origin, which adds nothing); lane l takes pair l of
// each window of 64 slots.  In SPLIT precision each source first moves from
// its leaf's frame into the group's: bit i of a window's mask is set where
// a staged leaf starts at slot i of the window (one OR-reduction per half),
// so a slot's leaf rank is the leaves started before the window plus the
// mask bits up to the slot, minus one.
template <bool SPLIT>
__device__ __forceinline__ void pair_batch(EvalSmem& sm, int ns, int lane) {
    const float4 pad = make_float4(0.f, 0.f, 0.f, 0.f);
    const int f = SPLIT && lane < sm.nleaf ? sm.first[lane] : 0x7fffffff;
    const unsigned long long upto = ~0ull >> (63 - 2 * lane);  // mask bits 0 .. 2 lane
    int before = -1;
#pragma unroll 2
    for (int base = 0; base < ns; base += 64) {
        int l0 = 0, l1 = 0;
        if (SPLIT) {
            const unsigned o = (unsigned)(f - base);
            const unsigned lo = __reduce_or_sync(0xffffffffu, o < 32u ? 1u << o : 0u);
            const unsigned hi = __reduce_or_sync(0xffffffffu, o - 32u < 32u ? 1u << (o - 32u) : 0u);
            const unsigned long long starts = ((unsigned long long)hi << 32) | lo;
            l0 = before + __popcll(starts & upto);
            l1 = l0 + (int)((starts >> (2 * lane + 1)) & 1ull);
            before += __popc(lo) + __popc(hi);
        }
        const int j0 = base + 2 * lane;
        if (j0 < ns) {
            const bool two = j0 + 1 < ns;
            float4 a = sm.src[j0];
            float4 b = two ? sm.src[j0 + 1] : pad;
            if (SPLIT) {
                const float4 sa = sm.shift[l0], sb = sm.shift[l1];
                a.x += sa.x;
                a.y += sa.y;
                a.z += sa.z;
                if (two) {
                    b.x += sb.x;
                    b.y += sb.y;
                    b.z += sb.z;
                }
            }
            sm.src[j0] = make_float4(a.x, b.x, a.y, b.y);
            sm.src[j0 + 1] = make_float4(a.z, b.z, a.w, b.w);
        }
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
__global__ void __launch_bounds__(kEvalThreads, kEvalMinBlocks) eval_kernel(NodeArrays T, Counters* C,
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
        mbar_init(&sm.bar);
        sm.npairs = sm.nterms = 0ull;
    }
    __syncwarp();
    unsigned phase = 0u;
    const int nleaves = C->nleaves;
    // Sources per near batch: the tuned cap (at most one staging buffer).
    const int maxleaf = max(1, C->max_leaf_count);
    const int tile = wp.p2p_tile > 0 && wp.p2p_tile < kSrcCap ? wp.p2p_tile : kSrcCap;
    const bool big_leaves = maxleaf > kSrcCap;
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
        if (SPLIT) {
            __syncwarp();
            if (lane == 0) {
                sm.gch = T.chi[leaf];
                sm.gcl = T.clo[leaf];
            }
            __syncwarp();
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
            if (!big_leaves) {
                W = near_window(LB, near_first, nnear, lane);
                prefetch_near<SPLIT>(sm, T, W.w0, lane);
            }
            Lane g = make_lane(src, gstart + t0, b0, lane);
            if (two) save_pass(sm, make_lane(src, gstart + t0 + b0, nblk - b0, lane), lane);
            if (!big_leaves) {
                ns_cur = stage_fitting<SPLIT>(sm, lane, src, tile, nb);
                near_advance(LB, W, nb, nnear, lane);
            }

            // ---- far field ----
            for (int b = 0, k = 0; b < nfar; b += 32, ++k) {
                stage_far<SPLIT, QUAD>(sm, lane, b + lane < nfar, A, B, D);
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
                const int npr = (min(32, nfar - b) + 1) >> 1;
                for_passes(g, two, sm, lane,
                           [&](Lane& x) { p2c_chunk<SPLIT, QUAD, SOFT>(x, sm, npr, wp.eps2, wp.ih); });
                __syncwarp();
            }
            if (lane == 0) sm.nterms += (unsigned long long)nblk * (unsigned long long)nfar;

            // ---- near field: batches of up to 32 leaves (as many as fit the
            // staging buffer, by their actual counts) staged by TMA ----
            int total = 0;
            if (!big_leaves) {
                // batch 0 was staged before the far field
                if (W.pos < nnear) prefetch_near<SPLIT>(sm, T, W.w0, lane);
                while (ns_cur > 0) {
                    if (!mbar_wait(&sm.bar, phase)) {
                        timeout = true;
                        break;
                    }
                    phase ^= 1u;
                    pair_batch<SPLIT>(sm, ns_cur, lane);  // source pairs, in the group's frame
                    __syncwarp();
                    const int np = (ns_cur + 1) >> 1;
                    for_passes(g, two, sm, lane,
                               [&](Lane& x) { p2p_chunk<SPLIT, SOFT>(x, sm.src, np, wp.eps2, wp.ih); });
                    __syncwarp();
                    total += ns_cur;
                    // stage the next batch (its info is in registers), then fetch
                    // the info of the one after
                    int ns_next = 0;
                    if (W.pos < nnear) {
                        ns_next = stage_fitting<SPLIT>(sm, lane, src, tile, nb);
                        near_advance(LB, W, nb, nnear, lane);
                        if (W.pos < nnear) prefetch_near<SPLIT>(sm, T, W.w0, lane);
                    }
                    ns_cur = ns_next;
                }
                if (timeout) mbar_wait(&sm.bar, phase);  // give copies in flight a bounded chance to land
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
                        const float4 h = T.chi[node], l = T.clo[node], gh = sm.gch, gl = sm.gcl;
                        sh = make_float4((h.x - gh.x) + (l.x - gl.x), (h.y - gh.y) + (l.y - gl.y),
                                         (h.z - gh.z) + (l.z - gl.z), 0.f);
                    }
                    for (int off = 0; off < cn; off += kSrcCap) {
                        const int ns = min(kSrcCap, cn - off);
                        __syncwarp();
                        for (int j0 = 2 * lane; j0 < ns; j0 += 64) {  // pairs, in the group's frame
                            float4 a = src[st + off + j0];
                            float4 c = j0 + 1 < ns ? src[st + off + j0 + 1] : make_float4(-sh.x, -sh.y, -sh.z, 0.f);
                            a.x += sh.x;
                            a.y += sh.y;
                            a.z += sh.z;
                            c.x += sh.x;
                            c.y += sh.y;
                            c.z += sh.z;
                            sm.src[j0] = make_float4(a.x, c.x, a.y, c.y);
                            sm.src[j0 + 1] = make_float4(a.z, c.z, a.w, c.w);
                        }
                        __syncwarp();
                        const int np = (ns + 1) >> 1;
                        for_passes(g, two, sm, lane,
                                   [&](Lane& x) { p2p_chunk<SPLIT, SOFT>(x, sm.src, np, wp.eps2, wp.ih); });
                    }
                    __syncwarp();
                    total += cn;
                }
            }
            if (timeout) break;
            if (lane == 0) sm.npairs += (unsigned long long)nblk * (unsigned long long)total - (unsigned long long)nblk;

            // ---- sum the slices of each target, write a, closing kick ----
            finish_targets<SPLIT>(sm, g, gstart + t0, lane, wp, acc, vel, vlo);
            if (two) finish_targets<SPLIT>(sm, load_pass(sm, lane), gstart + t0 + b0, lane, wp, acc, vel, vlo);
            __syncwarp();
        }
        if (timeout) break;
    }
    if (timeout && lane == 0) atomicOr(&C->status, kStTimeout);
    if (lane == 0) {
        atomicAdd(&C->p2p_pairs, sm.npairs);
        atomicAdd(&C->p2c_terms, sm.nterms);
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
