// walk.cu -- warp-cooperative grouped Barnes-Hut walk with interaction lists
// staged in shared memory, softened P2P and monopole+quadrupole P2C, and the
// closing half-kick fused into the epilogue.
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
// GB300 mapping: one warp per target group, dynamic group scheduling in key
// order (like OpenMP dynamic,32 over leaves).  The warp tests up to 32 nodes
// per iteration (one per lane), appends near leaves / far nodes to per-warp
// lists in shared memory and pushes opened children on a per-warp stack; when
// a list fills it is flushed: sources are staged into shared memory (shifted
// to the group's frame in SPLIT precision) and evaluated with lane =
// (target t, slice s): nt targets x floor(32/nt) source slices.  The opening
// test runs in FP32 on double-float COMs; decisions within a relative band
// of 1e-5 of the threshold are re-taken in FP64 on the FP64 moments.
#include "engine.cuh"

namespace ngrav {

constexpr int kWalkWarps = 4;
constexpr int kWalkThreads = kWalkWarps * 32;
constexpr int kNearCap = 64;
constexpr int kFarCap = 64;
constexpr int kSrcCap = 512;

struct WarpSmem {
    float4 src[kSrcCap];
    float4 farA[kFarCap];
    float4 farB[kFarCap];
    float farQyz[kFarCap];
    float4 nearShift[kNearCap];      // shift.xyz, start (int bits)
    int nearPre[kNearCap + 1];       // exclusive prefix of source counts
    int nearIds[kNearCap];
    int farIds[kFarCap];
    float red[3][32];
};

struct GroupCtx {
    // target of this lane
    float tx, ty, tz;
    int t, sl, S, nt;
    bool active;
    // group frame
    float4 gchi, gclo;
    // accumulators (Kahan compensated in SPLIT)
    float ax, ay, az, cx, cy, cz;
};

template <bool SPLIT>
__device__ __forceinline__ void accumulate(GroupCtx& g, float px, float py, float pz) {
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

template <bool SPLIT, bool ZEROSOFT>
__device__ __forceinline__ void p2p_chunk(GroupCtx& g, const float4* __restrict__ s_src, int ns, float eps2) {
    if (!g.active) return;
    float px = 0.f, py = 0.f, pz = 0.f;
    const float tx = g.tx, ty = g.ty, tz = g.tz;
    int j = g.sl;
    const int S = g.S;
#pragma unroll 4
    for (; j < ns; j += S) {
        const float4 q = s_src[j];
        const float dx = q.x - tx, dy = q.y - ty, dz = q.z - tz;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
        const float inv = rsqrtf(r2);
        float f = q.w * (inv * inv * inv);
        if (ZEROSOFT) f = r2 > 0.f ? f : 0.f;
        px = fmaf(f, dx, px);
        py = fmaf(f, dy, py);
        pz = fmaf(f, dz, pz);
    }
    accumulate<SPLIT>(g, px, py, pz);
}

template <bool SPLIT, bool QUAD>
__device__ __forceinline__ void p2c_chunk(GroupCtx& g, const WarpSmem& sm, int nf, float eps2) {
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
            const float ir7 = ir5 * ir2;
            const float c1 = -ir5;
            const float c2 = 2.5f * qd2 * ir7;
            px = fmaf(c1, qdx, fmaf(c2, dx, px));
            py = fmaf(c1, qdy, fmaf(c2, dy, py));
            pz = fmaf(c1, qdz, fmaf(c2, dz, pz));
        }
    }
    accumulate<SPLIT>(g, px, py, pz);
}

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

template <bool SPLIT, bool ZEROSOFT>
__device__ __forceinline__ void flush_near(GroupCtx& g, WarpSmem& sm, int nnear, const NodeArrays& T,
                           const float4* __restrict__ src, float eps2, int lane,
                           unsigned long long& pairs) {
    // Per-entry source counts, starts and frame shifts.
    for (int e0 = 0; e0 < nnear; e0 += 32) {
        const int e = e0 + lane;
        int cnt = 0;
        if (e < nnear) {
            const int node = sm.nearIds[e];
            const float4 Cw = T.wC[node];
            const int start = __float_as_int(Cw.z);
            cnt = __float_as_int(Cw.w) & 0xFFFFFF;
            float sx = 0.f, sy = 0.f, sz = 0.f;
            if (SPLIT) {
                const float4 h = T.chi[node], l = T.clo[node];
                sx = (h.x - g.gchi.x) + (l.x - g.gclo.x);
                sy = (h.y - g.gchi.y) + (l.y - g.gclo.y);
                sz = (h.z - g.gchi.z) + (l.z - g.gclo.z);
            }
            sm.nearShift[e] = make_float4(sx, sy, sz, __int_as_float(start));
        }
        int tot;
        const int ex = warp_excl_scan(cnt, lane, tot);
        const int carry = e0 == 0 ? 0 : sm.nearPre[e0];
        __syncwarp();
        if (e < nnear) sm.nearPre[e] = carry + ex;
        if (lane == 31) sm.nearPre[min(e0 + 32, nnear)] = carry + tot;
        __syncwarp();
    }
    const int total = sm.nearPre[nnear];
    pairs += (unsigned long long)g.nt * (unsigned long long)total;
    // Greedy chunks of whole entries that fit the staging buffer.
    int e0 = 0;
    while (e0 < nnear) {
        const int base = sm.nearPre[e0];
        // largest e1 with nearPre[e1] - base <= kSrcCap
        int lo = e0 + 1, hi = nnear;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sm.nearPre[mid] - base <= kSrcCap)
                lo = mid;
            else
                hi = mid - 1;
        }
        int e1 = lo;
        if (sm.nearPre[e1] - base > kSrcCap) {
            // One oversized leaf (depth-limited): stage it in pieces.
            const float4 sh = sm.nearShift[e0];
            const int start = __float_as_int(sh.w);
            const int cnt = sm.nearPre[e0 + 1] - base;
            for (int off = 0; off < cnt; off += kSrcCap) {
                const int ns = min(kSrcCap, cnt - off);
                for (int k = lane; k < ns; k += 32) {
                    float4 q = src[start + off + k];
                    q.x += sh.x;
                    q.y += sh.y;
                    q.z += sh.z;
                    sm.src[k] = q;
                }
                __syncwarp();
                p2p_chunk<SPLIT, ZEROSOFT>(g, sm.src, ns, eps2);
                __syncwarp();
            }
            e1 = e0 + 1;
        } else {
            for (int e = e0 + lane; e < e1; e += 32) {
                const float4 sh = sm.nearShift[e];
                const int start = __float_as_int(sh.w);
                const int o = sm.nearPre[e] - base;
                const int cnt = sm.nearPre[e + 1] - sm.nearPre[e];
                for (int k = 0; k < cnt; ++k) {
                    float4 q = src[start + k];
                    q.x += sh.x;
                    q.y += sh.y;
                    q.z += sh.z;
                    sm.src[o + k] = q;
                }
            }
            __syncwarp();
            p2p_chunk<SPLIT, ZEROSOFT>(g, sm.src, sm.nearPre[e1] - base, eps2);
            __syncwarp();
        }
        e0 = e1;
    }
}

template <bool SPLIT, bool QUAD>
__device__ __forceinline__ void flush_far(GroupCtx& g, WarpSmem& sm, int nfar, const NodeArrays& T, float eps2, int lane,
                          unsigned long long& p2c) {
    for (int f = lane; f < nfar; f += 32) {
        const int node = sm.farIds[f];
        const float4 A = T.wA[node];
        float rx = A.x, ry = A.y, rz = A.z;
        if (SPLIT) {
            const float4 D = T.wD[node];
            rx = (A.x - g.gchi.x) + (D.x - g.gclo.x);
            ry = (A.y - g.gchi.y) + (D.y - g.gclo.y);
            rz = (A.z - g.gchi.z) + (D.z - g.gclo.z);
        }
        sm.farA[f] = make_float4(rx, ry, rz, A.w);
        if (QUAD) {
            sm.farB[f] = T.wB[node];
            sm.farQyz[f] = T.wC[node].x;
        }
    }
    __syncwarp();
    p2c += (unsigned long long)g.nt * (unsigned long long)nfar;
    p2c_chunk<SPLIT, QUAD>(g, sm, nfar, eps2);
    __syncwarp();
}

template <bool SPLIT, bool QUAD, bool ZEROSOFT>
__global__ void __launch_bounds__(kWalkThreads) walk_kernel(NodeArrays T, Counters* C,
                                                            const float4* __restrict__ src,
                                                            float4* __restrict__ acc, float4* __restrict__ vel,
                                                            const int* __restrict__ leaf_list, WalkParams wp,
                                                            int* __restrict__ stack_pool) {
    extern __shared__ __align__(16) unsigned char walk_smem_raw[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    WarpSmem& sm = reinterpret_cast<WarpSmem*>(walk_smem_raw)[wib];
    const int gwarp = blockIdx.x * kWalkWarps + wib;
    int* stack = stack_pool + (long long)gwarp * wp.stack_cap;
    if (C->status & kStFatal) return;
    const int nleaves = C->nleaves;
    const double root_half = C->root_half;
    const unsigned lt_mask = (1u << lane) - 1u;

    unsigned long long pairs = 0, p2c = 0, tests = 0, retests = 0, groups = 0;
    int stack_max = 0;
    bool overflow = false;

    for (;;) {
        int gi = 0;
        if (lane == 0) gi = atomicAdd(&C->work_next, 1);
        gi = __shfl_sync(0xffffffffu, gi, 0);
        if (gi >= nleaves) break;
        const int leaf = leaf_list[gi];
        const float4 gA = T.wA[leaf];
        const float4 gC = T.wC[leaf];
        const float4 gD = T.wD[leaf];
        const int gstart = __float_as_int(gC.z);
        const int gcount = __float_as_int(gC.w) & 0xFFFFFF;
        const float gR = gD.w;
        double gcx_d = 0.0, gcy_d = 0.0, gcz_d = 0.0, gr_d = 0.0;
        if (wp.retest) {
            gcx_d = T.comx[leaf];
            gcy_d = T.comy[leaf];
            gcz_d = T.comz[leaf];
            gr_d = T.maxr[leaf];
        }
        GroupCtx g;
        if (SPLIT) {
            g.gchi = T.chi[leaf];
            g.gclo = T.clo[leaf];
        }
        ++groups;
        for (int t0 = 0; t0 < gcount; t0 += 32) {
            const int nt = min(32, gcount - t0);
            g.nt = nt;
            g.S = 32 / nt;
            g.active = lane < nt * g.S;
            g.t = lane % nt;
            g.sl = lane / nt;
            const float4 tp = src[gstart + t0 + g.t];
            g.tx = tp.x;
            g.ty = tp.y;
            g.tz = tp.z;
            g.ax = g.ay = g.az = 0.f;
            g.cx = g.cy = g.cz = 0.f;

            int nnear = 1, nfar = 0;
            if (lane == 0) sm.nearIds[0] = leaf;  // own members (self term is zero)
            int size = 0;
            if (leaf != 0) {
                if (lane == 0) stack[0] = 0;
                size = 1;
            }
            __syncwarp();
            int visits = 0;
            while (size > 0) {
                const int take = min(size, 32);
                visits += take;
                if (visits > wp.node_limit) {  // a node is visited at most once per group
                    overflow = true;
                    break;
                }
                size -= take;
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
                if (kind == 1) sm.nearIds[nnear + __popc(mnear & lt_mask)] = node;
                if (kind == 2) sm.farIds[nfar + __popc(mfar & lt_mask)] = node;
                nnear += __popc(mnear);
                nfar += __popc(mfar);
                int tot;
                const int off = warp_excl_scan(nch, lane, tot);
                if (size + tot > wp.stack_cap) {
                    overflow = true;
                    break;
                }
                for (int k = 0; k < nch; ++k) stack[size + off + k] = link + k;
                size += tot;
                stack_max = max(stack_max, size);
                __syncwarp();
                if (nnear > kNearCap - 32) {
                    flush_near<SPLIT, ZEROSOFT>(g, sm, nnear, T, src, wp.eps2, lane, pairs);
                    nnear = 0;
                }
                if (nfar > kFarCap - 32) {
                    flush_far<SPLIT, QUAD>(g, sm, nfar, T, wp.eps2, lane, p2c);
                    nfar = 0;
                }
            }
            if (overflow) break;
            if (nnear > 0) flush_near<SPLIT, ZEROSOFT>(g, sm, nnear, T, src, wp.eps2, lane, pairs);
            if (nfar > 0) flush_far<SPLIT, QUAD>(g, sm, nfar, T, wp.eps2, lane, p2c);
            pairs -= (unsigned long long)nt;  // self terms

            // Reduce the S slices of each target.
            if (g.active) {
                sm.red[0][lane] = g.ax;
                sm.red[1][lane] = g.ay;
                sm.red[2][lane] = g.az;
            }
            __syncwarp();
            if (lane < nt) {
                float sx = 0.f, sy = 0.f, sz = 0.f;
                for (int s = 0; s < g.S; ++s) {
                    sx += sm.red[0][lane + s * nt];
                    sy += sm.red[1][lane + s * nt];
                    sz += sm.red[2][lane + s * nt];
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
        }
        if (overflow) break;
    }
    if (overflow && lane == 0) atomicOr(&C->status, kStStackOverflow);  // or a visit-limit breach
    if (lane == 0) {
        atomicAdd(&C->p2p_pairs, pairs);
        atomicAdd(&C->p2c_terms, p2c);
        atomicAdd(&C->mac_tests, tests);
        atomicAdd(&C->groups, groups);
        atomicMax(&C->stack_max, stack_max);
    }
    // retests are counted per lane
    for (int o = 16; o > 0; o >>= 1) retests += __shfl_xor_sync(0xffffffffu, retests, o);
    if (lane == 0 && retests) atomicAdd(&C->mac_retests, retests);
}

int walk_blocks_for(int nwarps) { return (nwarps + kWalkWarps - 1) / kWalkWarps; }

size_t walk_smem_bytes() { return sizeof(WarpSmem) * kWalkWarps; }

int walk_warps_per_block() { return kWalkWarps; }

int walk_blocks_per_sm() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, walk_kernel<true, true, false>, kWalkThreads,
                                                  walk_smem_bytes());
    return nb > 0 ? nb : 1;
}

void walk_set_attributes() {
    const int bytes = (int)walk_smem_bytes();
#define NGRAV_ATTR(SP, Q, Z) \
    cudaFuncSetAttribute(walk_kernel<SP, Q, Z>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)
    NGRAV_ATTR(true, true, true);
    NGRAV_ATTR(true, true, false);
    NGRAV_ATTR(true, false, true);
    NGRAV_ATTR(true, false, false);
    NGRAV_ATTR(false, true, true);
    NGRAV_ATTR(false, true, false);
    NGRAV_ATTR(false, false, true);
    NGRAV_ATTR(false, false, false);
#undef NGRAV_ATTR
}

void launch_walk(const NodeArrays& T, Counters* C, const Particles& P, const int* leaf_list, int max_leaves,
                 const WalkParams& wp, int* stack_pool, int nwarps, cudaStream_t s) {
    const int blocks = walk_blocks_for(nwarps);
    const bool zs = !(wp.eps2 > 0.f);
    const size_t smem = walk_smem_bytes();
#define NGRAV_WALK(SP, Q, Z) \
    walk_kernel<SP, Q, Z><<<blocks, kWalkThreads, smem, s>>>(T, C, P.src, P.acc, P.vel, leaf_list, wp, stack_pool)
    if (wp.split) {
        if (wp.quadrupole) {
            if (zs) NGRAV_WALK(true, true, true); else NGRAV_WALK(true, true, false);
        } else {
            if (zs) NGRAV_WALK(true, false, true); else NGRAV_WALK(true, false, false);
        }
    } else {
        if (wp.quadrupole) {
            if (zs) NGRAV_WALK(false, true, true); else NGRAV_WALK(false, true, false);
        } else {
            if (zs) NGRAV_WALK(false, false, true); else NGRAV_WALK(false, false, false);
        }
    }
#undef NGRAV_WALK
}

}  // namespace ngrav
