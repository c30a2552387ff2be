// walk_pp.cu -- the per-particle walk of the reference (WalkBH,
// projects/nbody_core/src/Solvers.cpp:181-227), used by the relative
// (GADGET-2) opening test (ComputeAccelBarnesHutPerParticle, :359-382) and by
// the block-timestep integrator's target subsets (ComputeAccelBarnesHutTargets,
// :384-405).
//
// Every target decides every node on its own path:
//   leaf:      exact pairs with each member but itself;
//   internal:  accepted (softened monopole + unsoftened quadrupole) iff
//              geometric: (2h)^2 < theta^2 d^2, d = |com - x_target|;
//              relative:  M (2h)^2 < alpha |a_old| d^4 / G when |a_old| > 0,
//                         the geometric test otherwise (Mac.hpp:31-42);
//              otherwise its children are visited.
// GPU mapping: one warp per leaf, one lane per member (leaves above 32 members
// run in slices of 32).  The warp walks the union of its members' paths; each
// stack entry carries the mask of members still on that path, so a member that
// accepts a node stops there while the others descend, and the result of every
// member is exactly its own walk.  Sums are FP32 with Kahan compensation;
// differences use the double-float positions; a test within a relative 1e-5 of
// its threshold is re-taken in FP64 on the FP64 moments.
#include "engine.cuh"
#include "softening.cuh"
#include "walk_common.cuh"

namespace ngrav {

constexpr int kPpWarps = 4;
constexpr int kPpThreads = kPpWarps * 32;
constexpr int kPpStack = 1024;  // union of the members' paths: levels x 8 at most

struct PpParams {
    int relative;                     // relative MAC (else geometric)
    float alpha;                      // relative MAC tolerance
    double alpha_d;
    const unsigned char* targets;     // per slot: compute this particle (NULL: all)
    // block timesteps (System::BlockStep): only particles whose rung step
    // (rung in vel.w) ends at finest substep `sub` + 1, each closing with its
    // own half-kick 0.5 base / 2^rung
    int block, sub, rmax;
    double base;
};

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

template <bool SPLIT, bool QUAD, int SOFT>
__global__ void __launch_bounds__(kPpThreads) walk_pp_kernel(NodeArrays T, Counters* C, Particles P,
                                                             const int* __restrict__ leaf_list, WalkParams wp,
                                                             PpParams pp) {
    __shared__ int s_node[kPpWarps * kPpStack];
    __shared__ unsigned s_mask[kPpWarps * kPpStack];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    int* snode = s_node + w * kPpStack;
    unsigned* smask = s_mask + w * kPpStack;
    if (C->status & kStFatal) return;
    const int nleaves = C->nleaves;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    unsigned long long pairs = 0, p2c = 0, tests = 0;
    unsigned bad = 0;
    for (;;) {
        int gi = 0;
        if (lane == 0) gi = atomicAdd(&C->work_next, 1);
        gi = __shfl_sync(0xffffffffu, gi, 0);
        if (gi >= nleaves) break;
        const int leaf = leaf_list[gi];
        const int ls = T.start[leaf], lc = T.count[leaf];
        const int root = T.sysroot[leaf];
        for (int base = 0; base < lc; base += 32) {
            const int slot = ls + base + lane;
            bool mine = base + lane < lc;
            if (mine && pp.targets) mine = pp.targets[slot] != 0;
            float hdt_mine = wp.hdt;
            if (mine && pp.block) {
                const int rung = (int)P.vel[slot].w;
                mine = ((pp.sub + 1) % (1 << (pp.rmax - rung))) == 0;
                hdt_mine = (float)(0.5 * pp.base / (double)(1 << rung));
            }
            const unsigned active = __ballot_sync(0xffffffffu, mine);
            if (pp.block && lane == 0) atomicAdd(&C->targets, (unsigned long long)__popc(active));
            if (active == 0) continue;
            const float4 tp = mine ? P.pos[slot] : zero;
            const float4 tl = (mine && SPLIT) ? P.plo[slot] : zero;
            const float4 ao = mine ? P.acc[slot] : zero;
            const float aold = sqrtf(ao.x * ao.x + ao.y * ao.y + ao.z * ao.z);
            const double txd = (double)tp.x + tl.x, tyd = (double)tp.y + tl.y, tzd = (double)tp.z + tl.z;
            float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
            int size = 1;
            if (lane == 0) {
                snode[0] = root;
                smask[0] = active;
            }
            __syncwarp();
            int visits = 0;
            while (size > 0) {
                const int take = min(size, 32);
                size -= take;
                visits += take;
                if (visits > wp.node_limit) {
                    bad |= kStCorrupt;
                    break;
                }
                const int my_node = lane < take ? snode[size + lane] : -1;
                const unsigned my_mask = lane < take ? smask[size + lane] : 0u;
                __syncwarp();
                float4 A = zero, B = zero, Cw = zero, D = zero;
                if (my_node >= 0) {
                    A = T.wA[my_node];
                    Cw = T.wC[my_node];
                    D = T.wD[my_node];
                    if (QUAD) B = T.wB[my_node];
                }
                for (int e = 0; e < take; ++e) {
                    const int nd = __shfl_sync(0xffffffffu, my_node, e);
                    const unsigned m = __shfl_sync(0xffffffffu, my_mask, e);
                    const float mass = __shfl_sync(0xffffffffu, A.w, e);
                    if (m == 0u || !(mass > 0.f)) continue;
                    const bool on = (m >> lane) & 1u;
                    const int meta = __shfl_sync(0xffffffffu, __float_as_int(Cw.w), e);
                    const int link = __shfl_sync(0xffffffffu, __float_as_int(Cw.z), e);
                    if (meta < 0) {  // leaf: exact pairs for the members on this path
                        const int cnt = meta & 0xFFFFFF;
                        for (int j = link; j < link + cnt; ++j) {
                            const float4 q = P.pos[j];
                            const float4 ql = SPLIT ? P.plo[j] : zero;
                            if (!on || j == slot) continue;
                            const float dx = (q.x - tp.x) + (ql.x - tl.x);
                            const float dy = (q.y - tp.y) + (ql.y - tl.y);
                            const float dz = (q.z - tp.z) + (ql.z - tl.z);
                            const float f = pair_factor<SOFT>(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), q.w, wp.eps2, wp.ih);
                            kahan_add(sx, cx, f * dx);
                            kahan_add(sy, cy, f * dy);
                            kahan_add(sz, cz, f * dz);
                        }
                        if (lane == 0) {
                            // members on the path, each with every leaf member but itself
                            unsigned long long k = 0;
                            for (unsigned mm = m; mm; mm &= mm - 1) {
                                const int t = __ffs(mm) - 1;
                                const int ts = ls + base + t;
                                k += (unsigned long long)cnt - ((ts >= link && ts < link + cnt) ? 1u : 0u);
                            }
                            pairs += k;
                        }
                        continue;
                    }
                    const float ax_ = __shfl_sync(0xffffffffu, A.x, e), ay_ = __shfl_sync(0xffffffffu, A.y, e),
                                az_ = __shfl_sync(0xffffffffu, A.z, e);
                    const float dxl = __shfl_sync(0xffffffffu, D.x, e), dyl = __shfl_sync(0xffffffffu, D.y, e),
                                dzl = __shfl_sync(0xffffffffu, D.z, e);
                    const float sz_ = __shfl_sync(0xffffffffu, Cw.y, e);
                    float qxx = 0.f, qyy = 0.f, qxy = 0.f, qxz = 0.f;
                    const float qyz = __shfl_sync(0xffffffffu, D.w, e);
                    if (QUAD) {  // every lane takes part in the broadcast
                        qxx = __shfl_sync(0xffffffffu, B.x, e);
                        qyy = __shfl_sync(0xffffffffu, B.y, e);
                        qxy = __shfl_sync(0xffffffffu, B.z, e);
                        qxz = __shfl_sync(0xffffffffu, B.w, e);
                    }
                    bool accept = false;
                    float dx = 0.f, dy = 0.f, dz = 0.f, d2 = 0.f;
                    if (on) {
                        dx = (ax_ - tp.x) + (dxl - tl.x);
                        dy = (ay_ - tp.y) + (dyl - tl.y);
                        dz = (az_ - tp.z) + (dzl - tl.z);
                        d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        const bool rel = pp.relative && aold > 0.f;
                        float lhs, rhs;
                        if (rel) {
                            lhs = mass * sz_ * sz_;
                            rhs = pp.alpha * aold * d2 * d2 / wp.G;
                        } else {
                            lhs = sz_ * sz_;
                            rhs = wp.theta2 * d2;
                        }
                        accept = lhs < rhs;
                        if (wp.retest && fabsf(lhs - rhs) <= 1e-5f * (lhs + rhs)) {
                            const double ex = T.comx[nd] - txd, ey = T.comy[nd] - tyd, ez = T.comz[nd] - tzd;
                            const double dd2 = ex * ex + ey * ey + ez * ez;
                            const double s2 = 4.0 * T.half[nd] * T.half[nd];
                            accept = rel ? T.mass[nd] * s2 < pp.alpha_d * (double)aold * dd2 * dd2 / (double)wp.G
                                         : s2 < wp.theta2_d * dd2;
                        }
                    }
                    const unsigned open = __ballot_sync(0xffffffffu, on && !accept);
                    const unsigned acc_m = __ballot_sync(0xffffffffu, on && accept);
                    tests += lane == 0 ? (unsigned long long)__popc(m) : 0ull;
                    p2c += lane == 0 ? (unsigned long long)__popc(acc_m) : 0ull;
                    if (on && accept) {
                        const float f = pair_factor<SOFT>(d2, mass, wp.eps2, wp.ih);
                        float px = f * dx, py = f * dy, pz = f * dz;
                        if (QUAD) {
                            const float qzz = -(qxx + qyy);
                            const float qdx = fmaf(qxx, dx, fmaf(qxy, dy, qxz * dz));
                            const float qdy = fmaf(qxy, dx, fmaf(qyy, dy, qyz * dz));
                            const float qdz = fmaf(qxz, dx, fmaf(qyz, dy, qzz * dz));
                            const float qd2 = fmaf(dx, qdx, fmaf(dy, qdy, dz * qdz));
                            const float ir = rsqrtf(d2);
                            const float ir2 = ir * ir;
                            const float ir5 = ir2 * ir2 * ir;
                            const float c2 = 2.5f * qd2 * (ir5 * ir2);
                            px = fmaf(-ir5, qdx, fmaf(c2, dx, px));
                            py = fmaf(-ir5, qdy, fmaf(c2, dy, py));
                            pz = fmaf(-ir5, qdz, fmaf(c2, dz, pz));
                        }
                        kahan_add(sx, cx, px);
                        kahan_add(sy, cy, py);
                        kahan_add(sz, cz, pz);
                    }
                    if (open) {
                        const int nch = meta & 0xFFFFFF;
                        if (size + nch > kPpStack) {
                            bad |= kStStackOverflow;
                            size = 0;
                            break;
                        }
                        if (lane < nch) {
                            snode[size + lane] = link + lane;
                            smask[size + lane] = open;
                        }
                        size += nch;
                    }
                }
                __syncwarp();
            }
            if (mine) {
                const float ax = wp.G * (sx - cx), ay = wp.G * (sy - cy), az = wp.G * (sz - cz);
                P.acc[slot] = make_float4(ax, ay, az, 0.f);
                if (wp.kick) {
                    float4 v = P.vel[slot];
                    float4 vl = SPLIT ? P.vlo[slot] : make_float4(0.f, 0.f, 0.f, 0.f);
                    kick_v(v, SPLIT ? &vl : nullptr, hdt_mine, make_float4(ax, ay, az, 0.f));
                    P.vel[slot] = v;
                    if (SPLIT) P.vlo[slot] = vl;
                }
            }
            if (bad & (kStStackOverflow | kStCorrupt)) break;
        }
        if (bad & (kStStackOverflow | kStCorrupt)) break;
    }
    for (int o = 16; o > 0; o >>= 1) bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    if (lane == 0) {
        if (bad) atomicOr(&C->status, bad);
        atomicAdd(&C->p2p_pairs, pairs);
        atomicAdd(&C->p2c_terms, p2c);
        atomicAdd(&C->mac_tests, tests);
    }
}

#define NGRAV_PP_INSTANCES(X) \
    X(true, true, 0) X(true, true, 1) X(true, false, 0) X(true, false, 1) X(false, true, 0) X(false, true, 1) \
    X(false, false, 0) X(false, false, 1)

void launch_walk_pp(const NodeArrays& T, Counters* C, const Particles& P, const int* leaf_list, const WalkParams& wp,
                    int relative, double alpha, const unsigned char* targets, const int* block, double block_base,
                    int nwarps, cudaStream_t s) {
    PpParams pp;
    pp.relative = relative;
    pp.alpha = (float)alpha;
    pp.alpha_d = alpha;
    pp.targets = targets;
    pp.block = block ? 1 : 0;
    pp.sub = block ? block[0] : 0;
    pp.rmax = block ? block[1] : 0;
    pp.base = block_base;
    const int blocks = (nwarps + kPpWarps - 1) / kPpWarps;
    const int soft = wp.soft == kSoftSpline ? 1 : 0;
#define NGRAV_PP_LAUNCH(SP, Q, SO)                                                                  \
    if (wp.split == (SP) && (wp.quadrupole != 0) == (Q) && soft == (SO))                          \
        walk_pp_kernel<SP, Q, (SO) ? kSoftSpline : kSoftPlummer><<<blocks, kPpThreads, 0, s>>>(T, C, P, leaf_list, wp, pp);
    NGRAV_PP_INSTANCES(NGRAV_PP_LAUNCH)
#undef NGRAV_PP_LAUNCH
}

}  // namespace ngrav
