// walk.cu -- the grouped Barnes-Hut walk and the force evaluation, as two
// kernels: a traversal that writes per-group interaction lists, and a dense
// FP32 evaluation (P2C over the far list, P2P over the near list with source
// leaf tiles brought into shared memory by TMA bulk copies) that ends with
// the closing half-kick.
//
// Semantics restate the reference's grouped walk
// (projects/nbody_core/src/Solvers.cpp:248-355):
//  * each leaf is a target group; the group sphere is the leaf COM with
//    radius maxRadius;
//  * an internal node is accepted (far, P2C) iff
//      worst = |com_node - com_group| - maxRadius_group > 0  and
//      (2 half)^2 < theta^2 worst^2                       (:261-271)
//    otherwise its children are visited;
//  * every leaf reached is near (exact P2P), however far away (:256-258);
//  * the group's own members interact exactly, self excluded (:340-348);
//  * nodes with mass <= 0 are skipped (:254).
// P2P: a += G m d / (|d|^2 + eps^2)^(3/2)  (AccumPairPlummer, :19-38).
// P2C: softened monopole plus the unsoftened traceless quadrupole
//      a += -G Q.d / r^5 + 2.5 G (d.Q.d) d / r^7  (AddQuadrupole, :147-179).
//
// Walk: one warp per group, groups taken dynamically in key order.  Each
// iteration tests up to 32 nodes (one per lane); near leaves and far nodes
// are appended (ballot + prefix) to per-warp staging lists in global memory
// with coalesced stores, opened children are pushed on a per-warp stack.  The
// opening test runs in FP32 on double-float COMs; decisions within a
// relative band of 1e-5 of the threshold are re-taken in FP64 on the FP64
// moments.  At the end of a group its lists are copied to a contiguous slot
// of the list pool (one atomic per list).
//
// Evaluation: one warp per group, lane = (target t, slice s) with nt targets
// and floor(32/nt) source slices; slices are summed at the end.  Far records
// are staged (shifted to the group's frame) into shared memory 32 at a time.
// Near leaves are staged up to 256 sources at a time: lane e issues a
// cp.async.bulk for leaf e's contiguous float4 range, all completing on one
// mbarrier (bounded wait).
#include "engine.cuh"

namespace ngrav {

// ---------------------------------------------------------------------------
// Walk
// ---------------------------------------------------------------------------

constexpr int kWalkWarps = 4;
constexpr int kWalkThreads = kWalkWarps * 32;

__device__ __forceinline__ int warp_excl_scan(int v, int lane, int& total) {
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

__global__ void __launch_bounds__(kWalkThreads) walk_kernel(NodeArrays T, Counters* C,
                                                            const int* __restrict__ leaf_list, WalkParams wp,
                                                            ListBuffers LB) {
    const int lane = threadIdx.x & 31;
    const int gwarp = blockIdx.x * kWalkWarps + (threadIdx.x >> 5);
    if (C->status & kStFatal) return;
    int* stack = LB.stack + (long long)gwarp * LB.stack_cap;
    int* sfar = LB.scratch + (long long)gwarp * 2 * LB.scratch_cap;
    int* snear = sfar + LB.scratch_cap;
    const int nleaves = C->nleaves;
    const double root_half = C->root_half;
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned long long tests = 0, retests = 0, groups = 0;
    int stack_max = 0, list_max = 0;
    unsigned bad = 0;

    for (;;) {
        int gi = 0;
        if (lane == 0) gi = atomicAdd(&C->work_next, 1);
        gi = __shfl_sync(0xffffffffu, gi, 0);
        if (gi >= nleaves) break;
        const int leaf = leaf_list[gi];
        const float4 gA = T.wA[leaf];
        const float4 gC = T.wC[leaf];
        const float4 gD = T.wD[leaf];
        const float gR = gC.x;
        double gcx_d = 0.0, gcy_d = 0.0, gcz_d = 0.0, gr_d = 0.0;
        if (wp.retest) {
            gcx_d = T.comx[leaf];
            gcy_d = T.comy[leaf];
            gcz_d = T.comz[leaf];
            gr_d = T.maxr[leaf];
        }
        ++groups;
        int nfar = 0, nnear = 1;
        if (lane == 0) snear[0] = leaf;  // own members first (the self term is zero)
        int size = 0;
        if (leaf != 0) {
            if (lane == 0) stack[0] = 0;
            size = 1;
        }
        int visits = 0;
        __syncwarp();
        while (size > 0) {
            const int take = min(size, 32);
            size -= take;
            visits += take;
            if (visits > wp.node_limit) {
                bad |= kStCorrupt;
                break;
            }
            int node = -1;
            if (lane < take) node = stack[size + lane];
            int kind = 0;  // 0 none, 1 near, 2 far, 3 open
            int nch = 0, link = 0;
            bool tested = false;
            if (node >= 0 && node != leaf) {
                const float4 A = T.wA[node];
                const float4 Cw = T.wC[node];
                const int meta = __float_as_int(Cw.w);
                link = __float_as_int(Cw.z);
                if (A.w > 0.f) {
                    if (meta < 0) {
                        kind = 1;
                    } else {
                        tested = true;
                        const float4 D = T.wD[node];
                        const float dx = (A.x - gA.x) + (D.x - gD.x);
                        const float dy = (A.y - gA.y) + (D.y - gD.y);
                        const float dz = (A.z - gA.z) + (D.z - gD.z);
                        const float dist = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                        const float worst = dist - gR;
                        const float size_n = Cw.y;
                        bool accept = worst > 0.f && size_n * size_n < wp.theta2 * worst * worst;
                        if (wp.retest) {
                            const float margin = wp.theta * worst - size_n;
                            if (fabsf(margin) <= 1e-5f * (wp.theta * (dist + gR) + size_n)) {
                                ++retests;
                                const double ex = T.comx[node] - gcx_d, ey = T.comy[node] - gcy_d,
                                             ez = T.comz[node] - gcz_d;
                                const double d2 = ex * ex + ey * ey + ez * ez;
                                const double sz = 2.0 * ldexp(root_half, -((meta >> 24) & 31));
                                const double w = sqrt(d2) - gr_d;
                                accept = w > 0.0 && sz * sz < wp.theta2_d * w * w;
                            }
                        }
                        if (accept) {
                            kind = 2;
                        } else {
                            kind = 3;
                            nch = meta & 0xFFFFFF;
                        }
                    }
                }
            }
            tests += __popc(__ballot_sync(0xffffffffu, tested));
            const unsigned mnear = __ballot_sync(0xffffffffu, kind == 1);
            const unsigned mfar = __ballot_sync(0xffffffffu, kind == 2);
            const int add_near = __popc(mnear), add_far = __popc(mfar);
            if (nnear + add_near > LB.scratch_cap || nfar + add_far > LB.scratch_cap) {
                bad |= kStListOverflow;
                break;
            }
            if (kind == 1) snear[nnear + __popc(mnear & lt_mask)] = node;
            if (kind == 2) sfar[nfar + __popc(mfar & lt_mask)] = node;
            nnear += add_near;
            nfar += add_far;
            int tot;
            const int off = warp_excl_scan(nch, lane, tot);
            if (size + tot > LB.stack_cap) {
                bad |= kStStackOverflow;
                break;
            }
            for (int k = 0; k < nch; ++k) stack[size + off + k] = link + k;
            size += tot;
            stack_max = max(stack_max, size);
            __syncwarp();
        }
        if (bad) break;
        // Copy the group's lists to contiguous slots of the pool.
        unsigned long long fbase = 0, nbase = 0;
        if (lane == 0) {
            fbase = atomicAdd(&C->far_total, (unsigned long long)nfar);
            nbase = atomicAdd(&C->near_total, (unsigned long long)nnear);
        }
        fbase = __shfl_sync(0xffffffffu, fbase, 0);
        nbase = __shfl_sync(0xffffffffu, nbase, 0);
        if ((long long)(fbase + nfar) > LB.far_cap || (long long)(nbase + nnear) > LB.near_cap) {
            bad |= kStListOverflow;
            break;
        }
        for (int i = lane; i < nfar; i += 32) LB.far[fbase + i] = sfar[i];
        for (int i = lane; i < nnear; i += 32) LB.near[nbase + i] = snear[i];
        if (lane == 0) {
            LB.goff[2 * gi] = (long long)fbase;
            LB.goff[2 * gi + 1] = (long long)nbase;
            LB.gcnt[2 * gi] = nfar;
            LB.gcnt[2 * gi + 1] = nnear;
        }
        list_max = max(list_max, max(nfar, nnear));
        __syncwarp();
    }
    if (lane == 0) {
        if (bad) atomicOr(&C->status, bad);
        atomicAdd(&C->mac_tests, tests);
        atomicAdd(&C->groups, groups);
        atomicMax(&C->stack_max, stack_max);
        atomicMax(&C->list_max, list_max);
    }
    for (int o = 16; o > 0; o >>= 1) retests += __shfl_xor_sync(0xffffffffu, retests, o);
    if (lane == 0 && retests) atomicAdd(&C->mac_retests, retests);
}

// ---------------------------------------------------------------------------
// Evaluation
// ---------------------------------------------------------------------------

constexpr int kEvalWarps = 4;
constexpr int kEvalThreads = kEvalWarps * 32;
constexpr int kSrcCap = 256;                  // staged sources per chunk (4 KiB)
constexpr unsigned kWaitLimit = 1u << 26;     // bounded mbarrier polling

struct __align__(128) EvalSmem {
    float4 src[kSrcCap];                      // TMA destination (16-byte multiples)
    float4 farA[32];                          // relative COM, mass
    float4 farB[32];                          // Qxx Qyy Qxy Qxz
    float farQyz[32];
    float4 shift[32];                         // near-leaf frame shift
    int pre[33];                              // exclusive prefix of source counts
    int cnt[32];
    int start[32];
    float red[3][32];
    unsigned long long bar;                   // mbarrier
};

struct Lane {
    float tx, ty, tz;
    int sl, S, nt;
    bool active;
    float ax, ay, az, cx, cy, cz;
};

template <bool SPLIT>
__device__ __forceinline__ void accumulate(Lane& g, float px, float py, float pz) {
    if (SPLIT) {  // blocked Kahan: compensate once per staged chunk
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

template <bool SPLIT, bool ZEROSOFT>
__device__ __forceinline__ void p2p_chunk(Lane& g, const float4* __restrict__ s_src, int ns, float eps2) {
    if (!g.active) return;
    float px = 0.f, py = 0.f, pz = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;
    const float tx = g.tx, ty = g.ty, tz = g.tz;
    const int S = g.S;
    int j = g.sl;
    // two independent accumulator sets for ILP
    for (; j + S < ns; j += 2 * S) {
        const float4 a = s_src[j];
        const float4 b = s_src[j + S];
        const float ax_ = a.x - tx, ay_ = a.y - ty, az_ = a.z - tz;
        const float bx_ = b.x - tx, by_ = b.y - ty, bz_ = b.z - tz;
        const float ra = fmaf(ax_, ax_, fmaf(ay_, ay_, fmaf(az_, az_, eps2)));
        const float rb = fmaf(bx_, bx_, fmaf(by_, by_, fmaf(bz_, bz_, eps2)));
        const float ia = rsqrtf(ra), ib = rsqrtf(rb);
        float fa = a.w * (ia * ia * ia), fb = b.w * (ib * ib * ib);
        if (ZEROSOFT) {
            fa = ra > 0.f ? fa : 0.f;
            fb = rb > 0.f ? fb : 0.f;
        }
        px = fmaf(fa, ax_, px);
        py = fmaf(fa, ay_, py);
        pz = fmaf(fa, az_, pz);
        qx = fmaf(fb, bx_, qx);
        qy = fmaf(fb, by_, qy);
        qz = fmaf(fb, bz_, qz);
    }
    if (j < ns) {
        const float4 a = s_src[j];
        const float ax_ = a.x - tx, ay_ = a.y - ty, az_ = a.z - tz;
        const float ra = fmaf(ax_, ax_, fmaf(ay_, ay_, fmaf(az_, az_, eps2)));
        const float ia = rsqrtf(ra);
        float fa = a.w * (ia * ia * ia);
        if (ZEROSOFT) fa = ra > 0.f ? fa : 0.f;
        px = fmaf(fa, ax_, px);
        py = fmaf(fa, ay_, py);
        pz = fmaf(fa, az_, pz);
    }
    accumulate<SPLIT>(g, px + qx, py + qy, pz + qz);
}

template <bool SPLIT, bool QUAD>
__device__ __forceinline__ void p2c_chunk(Lane& g, const EvalSmem& sm, int nf, float eps2) {
    if (!g.active) return;
    float px = 0.f, py = 0.f, pz = 0.f;
    const float tx = g.tx, ty = g.ty, tz = g.tz;
    for (int f = g.sl; f < nf; f += g.S) {
        const float4 A = sm.farA[f];
        const float dx = A.x - tx, dy = A.y - ty, dz = A.z - tz;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float rs = rsqrtf(r2 + eps2);
        const float fm = A.w * (rs * rs * rs);
        px = fmaf(fm, dx, px);
        py = fmaf(fm, dy, py);
        pz = fmaf(fm, dz, pz);
        if (QUAD) {
            const float4 B = sm.farB[f];
            const float qyz = sm.farQyz[f];
            const float qzz = -(B.x + B.y);
            const float qdx = fmaf(B.x, dx, fmaf(B.z, dy, B.w * dz));
            const float qdy = fmaf(B.z, dx, fmaf(B.y, dy, qyz * dz));
            const float qdz = fmaf(B.w, dx, fmaf(qyz, dy, qzz * dz));
            const float qd2 = fmaf(dx, qdx, fmaf(dy, qdy, dz * qdz));
            const float ir = rsqrtf(r2);
            const float ir2 = ir * ir;
            const float ir5 = ir2 * ir2 * ir;
            const float c1 = -ir5;
            const float c2 = 2.5f * qd2 * (ir5 * ir2);
            px = fmaf(c1, qdx, fmaf(c2, dx, px));
            py = fmaf(c1, qdy, fmaf(c2, dy, py));
            pz = fmaf(c1, qdz, fmaf(c2, dz, pz));
        }
    }
    accumulate<SPLIT>(g, px, py, pz);
}

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait for the phase with parity `phase`; returns false on timeout.
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

// Stage entries [e0, e1) of the current batch (all of them fit kSrcCap) by
// TMA, wait, shift to the group frame, evaluate.  Returns false on timeout.
template <bool SPLIT, bool ZEROSOFT>
__device__ __forceinline__ bool stage_and_p2p(Lane& g, EvalSmem& sm, const float4* __restrict__ src, int e0,
                                              int e1, int lane, unsigned& phase, float eps2) {
    const int base = sm.pre[e0];
    const int ns = sm.pre[e1] - base;
    if (ns <= 0) return true;
    if (lane == 0) mbar_expect_tx(&sm.bar, (unsigned)ns * 16u);
    __syncwarp();
    const int e = e0 + lane;
    if (e < e1) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tma_load_1d(&sm.src[sm.pre[e] - base], src + sm.start[e], (unsigned)sm.cnt[e] * 16u, &sm.bar);
    }
    const bool ok = mbar_wait(&sm.bar, phase);
    phase ^= 1u;
    if (!ok) return false;
    if (SPLIT && e < e1) {
        const float4 sh = sm.shift[e];
        float4* q = &sm.src[sm.pre[e] - base];
        for (int k = 0; k < sm.cnt[e]; ++k) {
            float4 v = q[k];
            v.x += sh.x;
            v.y += sh.y;
            v.z += sh.z;
            q[k] = v;
        }
    }
    __syncwarp();
    p2p_chunk<SPLIT, ZEROSOFT>(g, sm.src, ns, eps2);
    __syncwarp();
    return true;
}

template <bool SPLIT, bool QUAD, bool ZEROSOFT>
__global__ void __launch_bounds__(kEvalThreads) eval_kernel(NodeArrays T, Counters* C,
                                                            const float4* __restrict__ src,
                                                            float4* __restrict__ acc, float4* __restrict__ vel,
                                                            const int* __restrict__ leaf_list, WalkParams wp,
                                                            ListBuffers LB) {
    extern __shared__ __align__(128) unsigned char eval_smem_raw[];
    const int lane = threadIdx.x & 31;
    EvalSmem& sm = reinterpret_cast<EvalSmem*>(eval_smem_raw)[threadIdx.x >> 5];
    if (C->status & kStFatal) return;
    if (lane == 0) mbar_init(&sm.bar);
    __syncwarp();
    unsigned phase = 0;
    const int nleaves = C->nleaves;
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
        const long long foff = LB.goff[2 * gi], noff = LB.goff[2 * gi + 1];
        const int nfar = LB.gcnt[2 * gi], nnear = LB.gcnt[2 * gi + 1];
        float4 gchi = make_float4(0.f, 0.f, 0.f, 0.f), gclo = gchi;
        if (SPLIT) {
            gchi = T.chi[leaf];
            gclo = T.clo[leaf];
        }
        for (int t0 = 0; t0 < gcount; t0 += 32) {
            Lane g;
            g.nt = min(32, gcount - t0);
            g.S = 32 / g.nt;
            g.active = lane < g.nt * g.S;
            const int t = lane % g.nt;
            g.sl = lane / g.nt;
            const float4 tp = src[gstart + t0 + t];
            g.tx = tp.x;
            g.ty = tp.y;
            g.tz = tp.z;
            g.ax = g.ay = g.az = g.cx = g.cy = g.cz = 0.f;

            // ---- far field ----
            for (int b = 0; b < nfar; b += 32) {
                const int e = b + lane;
                if (e < nfar) {
                    const int node = LB.far[foff + e];
                    const float4 A = T.wA[node];
                    const float4 D = T.wD[node];
                    float rx = A.x, ry = A.y, rz = A.z;
                    if (SPLIT) {
                        rx = (A.x - gchi.x) + (D.x - gclo.x);
                        ry = (A.y - gchi.y) + (D.y - gclo.y);
                        rz = (A.z - gchi.z) + (D.z - gclo.z);
                    }
                    sm.farA[lane] = make_float4(rx, ry, rz, A.w);
                    if (QUAD) {
                        sm.farB[lane] = T.wB[node];
                        sm.farQyz[lane] = D.w;
                    }
                }
                __syncwarp();
                p2c_chunk<SPLIT, QUAD>(g, sm, min(32, nfar - b), wp.eps2);
                __syncwarp();
            }
            p2c += (unsigned long long)g.nt * (unsigned long long)nfar;

            // ---- near field: batches of 32 leaves, chunks of <= kSrcCap sources ----
            int total = 0;
            for (int b = 0; b < nnear && !timeout; b += 32) {
                const int e = b + lane;
                int cnt = 0;
                if (e < nnear) {
                    const int node = LB.near[noff + e];
                    const float4 Cw = T.wC[node];
                    cnt = __float_as_int(Cw.w) & 0xFFFFFF;
                    sm.start[lane] = __float_as_int(Cw.z);
                    if (SPLIT) {
                        const float4 h = T.chi[node], l = T.clo[node];
                        sm.shift[lane] = make_float4((h.x - gchi.x) + (l.x - gclo.x), (h.y - gchi.y) + (l.y - gclo.y),
                                                     (h.z - gchi.z) + (l.z - gclo.z), 0.f);
                    }
                }
                sm.cnt[lane] = cnt;
                int tot;
                const int ex = warp_excl_scan(cnt, lane, tot);
                sm.pre[lane] = ex;
                if (lane == 31) sm.pre[32] = tot;
                __syncwarp();
                total += tot;
                const int ne = min(32, nnear - b);
                int e0 = 0;
                while (e0 < ne) {
                    // largest e1 with pre[e1] - pre[e0] <= kSrcCap (uniform across the warp)
                    int e1 = e0 + 1;
                    while (e1 < ne && sm.pre[e1 + 1] - sm.pre[e0] <= kSrcCap) ++e1;
                    if (sm.pre[e1] - sm.pre[e0] > kSrcCap) {
                        // one leaf larger than the staging buffer (depth-limited): plain loads
                        const int st = sm.start[e0], c = sm.cnt[e0];
                        const float4 sh = sm.shift[e0];
                        for (int off = 0; off < c; off += kSrcCap) {
                            const int ns = min(kSrcCap, c - off);
                            __syncwarp();
                            for (int k = lane; k < ns; k += 32) {
                                float4 v = src[st + off + k];
                                if (SPLIT) {
                                    v.x += sh.x;
                                    v.y += sh.y;
                                    v.z += sh.z;
                                }
                                sm.src[k] = v;
                            }
                            __syncwarp();
                            p2p_chunk<SPLIT, ZEROSOFT>(g, sm.src, ns, wp.eps2);
                        }
                        __syncwarp();
                    } else if (!stage_and_p2p<SPLIT, ZEROSOFT>(g, sm, src, e0, e1, lane, phase, wp.eps2)) {
                        timeout = true;
                        break;
                    }
                    e0 = e1;
                }
                __syncwarp();
            }
            pairs += (unsigned long long)g.nt * (unsigned long long)total - (unsigned long long)g.nt;

            // ---- reduce the slices, write a, closing kick ----
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
                const int slot = gstart + t0 + lane;
                acc[slot] = make_float4(ax, ay, az, 0.f);
                if (wp.kick) {
                    float4 v = vel[slot];
                    v.x = fmaf(wp.hdt, ax, v.x);
                    v.y = fmaf(wp.hdt, ay, v.y);
                    v.z = fmaf(wp.hdt, az, v.z);
                    vel[slot] = v;
                }
            }
            __syncwarp();
            if (timeout) break;
        }
        if (timeout) break;
    }
    if (timeout) {
        // a bulk copy never completed: flag it and give in-flight copies a
        // bounded chance to land before the block retires
        mbar_wait(&sm.bar, phase);
        if (lane == 0) atomicOr(&C->status, kStTimeout);
    }
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
int walk_warps_per_block() { return kWalkWarps; }

#define NGRAV_EVAL_INSTANCES(X) \
    X(true, true, true) X(true, true, false) X(true, false, true) X(true, false, false) \
    X(false, true, true) X(false, true, false) X(false, false, true) X(false, false, false)

void walk_set_attributes() {
    const int bytes = (int)eval_smem_bytes();
#define NGRAV_ATTR(SP, Q, Z) \
    cudaFuncSetAttribute(eval_kernel<SP, Q, Z>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    NGRAV_EVAL_INSTANCES(NGRAV_ATTR)
#undef NGRAV_ATTR
}

int walk_blocks_per_sm() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, walk_kernel, kWalkThreads, 0);
    return nb > 0 ? nb : 1;
}

int eval_blocks_per_sm() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, eval_kernel<true, true, false>, kEvalThreads,
                                                  eval_smem_bytes());
    return nb > 0 ? nb : 1;
}

void launch_walk(const NodeArrays& T, Counters* C, const int* leaf_list, const WalkParams& wp,
                 const ListBuffers& LB, cudaStream_t s) {
    const int blocks = (LB.nwarps + kWalkWarps - 1) / kWalkWarps;
    walk_kernel<<<blocks, kWalkThreads, 0, s>>>(T, C, leaf_list, wp, LB);
}

void launch_eval(const NodeArrays& T, Counters* C, const Particles& P, const int* leaf_list, const WalkParams& wp,
                 const ListBuffers& LB, int nwarps, cudaStream_t s) {
    const int blocks = (nwarps + kEvalWarps - 1) / kEvalWarps;
    const bool zs = !(wp.eps2 > 0.f);
    const size_t smem = eval_smem_bytes();
#define NGRAV_LAUNCH(SP, Q, Z)                                                                             \
    if (wp.split == (SP) && (wp.quadrupole != 0) == (Q) && zs == (Z))                                     \
        eval_kernel<SP, Q, Z><<<blocks, kEvalThreads, smem, s>>>(T, C, P.src, P.acc, P.vel, leaf_list, wp, LB);
    NGRAV_EVAL_INSTANCES(NGRAV_LAUNCH)
#undef NGRAV_LAUNCH
}

}  // namespace ngrav
