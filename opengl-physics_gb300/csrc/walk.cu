// walk.cu -- the grouped Barnes-Hut walk: a traversal kernel that applies the
// reference's opening test per leaf group and writes each group's far and
// near interaction lists.
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
// iteration tests up to 64 nodes (two per lane); near leaves and far nodes
// are appended (ballot + prefix) to the group's lists with coalesced stores,
// opened children are pushed on a per-warp stack.  The
// opening test runs in FP32 on double-float COMs; decisions within a
// relative band of 1e-5 of the threshold are re-taken in FP64 on the FP64
// moments.  Lists are chains of 128-entry chunks taken from a pool with one
// atomic per chunk, so every entry is written once.
//
// The evaluation of the lists lives in eval.cu.
#include "engine.cuh"
#include "walk_common.cuh"

namespace ngrav {

// ---------------------------------------------------------------------------
// Walk
// ---------------------------------------------------------------------------

constexpr int kWalkWarps = 4;
constexpr int kWalkThreads = kWalkWarps * 32;
constexpr int kNPL = 2;  // nodes tested per lane per iteration (memory-level parallelism)

// STACK > 0: a per-warp traversal stack of STACK entries in shared memory
// (push -> pop never leaves the SM; the size trades occupancy against the
// frontier it holds, a tuned choice); STACK = 0: the global-memory stack, the
// fallback for trees whose frontier outgrows shared memory.
template <int STACK>
__global__ void __launch_bounds__(kWalkThreads) walk_kernel(NodeArrays T, Counters* C,
                                                            const int* __restrict__ leaf_list, WalkParams wp,
                                                            ListBuffers LB) {
    __shared__ int s_stack[STACK > 0 ? kWalkWarps * STACK : 1];
    const int lane = threadIdx.x & 31;
    const int gwarp = blockIdx.x * kWalkWarps + (threadIdx.x >> 5);
    if (C->status & kStFatal) return;
    int* stack = STACK > 0 ? s_stack + (threadIdx.x >> 5) * STACK : LB.stack + (long long)gwarp * LB.stack_cap;
    const int stack_cap = STACK > 0 ? STACK : LB.stack_cap;
    const int nleaves = C->nleaves;
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned long long tests = 0, retests = 0, groups = 0;
    int stack_max = 0, list_max = 0;
    unsigned bad = 0;
    int fres_next = 0, fres_end = 0, nres_next = 0, nres_end = 0;  // chunk reservoirs

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
        ChunkList far = {-1, -1, 0, 0, fres_next, fres_end}, near = {-1, -1, 0, 0, nres_next, nres_end};
        // own members first (the self term is zero)
        list_append(near, lane == 0, leaf, LB.near, LB.near_next, &C->near_chunks, LB.near_chunk_cap, lane,
                    lt_mask, bad);
        int size = 0, visits = 0;
        const int root = T.sysroot[leaf];
        if (leaf != root) {
            // The root's test, by every lane at once (the same arithmetic as
            // the loop's): when it opens, as it nearly always does, its
            // children start the stack, sparing an iteration that would test
            // one node; otherwise the root takes the loop's path.
            const float4 A = T.wA[root], Cw = T.wC[root], D = T.wD[root];
            const int meta = __float_as_int(Cw.w);
            bool open = false;
            if (A.w > 0.f && meta >= 0) {
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
                        if (lane == 0) ++retests;
                        const double ex = T.comx[root] - gcx_d, ey = T.comy[root] - gcy_d,
                                     ez = T.comz[root] - gcz_d;
                        const double d2 = ex * ex + ey * ey + ez * ez;
                        const double sz = 2.0 * T.half[root];
                        const double w = sqrt(d2) - gr_d;
                        accept = w > 0.0 && sz * sz < wp.theta2_d * w * w;
                    }
                }
                open = !accept;
            }
            if (open) {
                const int nch = meta & 0xFFFFFF, link = __float_as_int(Cw.z);
                if (lane < nch) stack[lane] = link + lane;
                size = nch;
                visits = 1;
                tests += 1;
            } else {
                if (lane == 0) stack[0] = root;
                size = 1;
            }
        }
        __syncwarp();
        while (size > 0) {
            const int take = min(size, 32 * kNPL);
            size -= take;
            visits += take;
            if (visits > wp.node_limit) {
                bad |= kStCorrupt;
                break;
            }
            int node[kNPL];
#pragma unroll
            for (int q = 0; q < kNPL; ++q) {
                const int idx = lane + 32 * q;
                node[q] = idx < take ? stack[size + idx] : -1;
            }
            float4 A[kNPL], Cw[kNPL], Dw[kNPL];
#pragma unroll
            for (int q = 0; q < kNPL; ++q) {  // all record loads in flight together
                if (node[q] >= 0) {
                    A[q] = T.wA[node[q]];
                    Cw[q] = T.wC[node[q]];
                    Dw[q] = T.wD[node[q]];
                } else {
                    A[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                    Cw[q] = A[q];
                    Dw[q] = A[q];
                }
            }
            int kind[kNPL], nch[kNPL], link[kNPL];
            bool tested_any[kNPL];
#pragma unroll
            for (int q = 0; q < kNPL; ++q) {
                kind[q] = 0;  // 0 none, 1 near, 2 far, 3 open
                nch[q] = 0;
                tested_any[q] = false;
                const int meta = __float_as_int(Cw[q].w);
                link[q] = __float_as_int(Cw[q].z);
                if (node[q] >= 0 && node[q] != leaf && A[q].w > 0.f) {
                    if (meta < 0) {
                        kind[q] = 1;
                    } else {
                        tested_any[q] = true;
                        const float4 D = Dw[q];
                        const float dx = (A[q].x - gA.x) + (D.x - gD.x);
                        const float dy = (A[q].y - gA.y) + (D.y - gD.y);
                        const float dz = (A[q].z - gA.z) + (D.z - gD.z);
                        const float dist = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                        const float worst = dist - gR;
                        const float size_n = Cw[q].y;
                        bool accept = worst > 0.f && size_n * size_n < wp.theta2 * worst * worst;
                        if (wp.retest) {
                            const float margin = wp.theta * worst - size_n;
                            if (fabsf(margin) <= 1e-5f * (wp.theta * (dist + gR) + size_n)) {
                                ++retests;
                                const int nd = node[q];
                                const double ex = T.comx[nd] - gcx_d, ey = T.comy[nd] - gcy_d,
                                             ez = T.comz[nd] - gcz_d;
                                const double d2 = ex * ex + ey * ey + ez * ez;
                                const double sz = 2.0 * T.half[nd];
                                const double w = sqrt(d2) - gr_d;
                                accept = w > 0.0 && sz * sz < wp.theta2_d * w * w;
                            }
                        }
                        if (accept) {
                            kind[q] = 2;
                        } else {
                            kind[q] = 3;
                            nch[q] = meta & 0xFFFFFF;
                        }
                    }
                }
            }
            static_assert(kNPL == 2, "the batched appends below take two nodes per lane");
            tests += __popc(__ballot_sync(0xffffffffu, tested_any[0])) +
                     __popc(__ballot_sync(0xffffffffu, tested_any[1]));
            list_append2(near, kind[0] == 1, node[0], kind[1] == 1, node[1], LB.near, LB.near_next, &C->near_chunks,
                         LB.near_chunk_cap, lane, lt_mask, bad);
            list_append2(far, kind[0] == 2, node[0], kind[1] == 2, node[1], LB.far, LB.far_next, &C->far_chunks,
                         LB.far_chunk_cap, lane, lt_mask, bad);
            {  // both nodes' children onto the stack with one scan
                int tot;
                const int off = warp_excl_scan(nch[0] + nch[1], lane, tot);
                if (size + tot > stack_cap) {
                    bad |= kStStackOverflow;
                    break;
                }
                for (int k = 0; k < nch[0]; ++k) stack[size + off + k] = link[0] + k;
                for (int k = 0; k < nch[1]; ++k) stack[size + off + nch[0] + k] = link[1] + k;
                size += tot;
            }
            stack_max = max(stack_max, size);
            __syncwarp();
        }
        fres_next = far.res_next;
        fres_end = far.res_end;
        nres_next = near.res_next;
        nres_end = near.res_end;
        if (lane == 0) LB.ginfo[gi] = make_int4(far.first, near.first, far.count, near.count);
        list_max = max(list_max, max(far.count, near.count));
        if (bad & (kStStackOverflow | kStCorrupt)) break;
    }
    for (int o = 16; o > 0; o >>= 1) bad |= __shfl_xor_sync(0xffffffffu, bad, o);
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
// Launchers
// ---------------------------------------------------------------------------

int walk_warps_per_block() { return kWalkWarps; }

int walk_blocks_per_sm() {
    int nb = 0, ng = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, walk_kernel<1024>, kWalkThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ng, walk_kernel<0>, kWalkThreads, 0);
    nb = nb > ng ? nb : ng;
    return nb > 0 ? nb : 1;
}

void launch_walk(const NodeArrays& T, Counters* C, const int* leaf_list, const WalkParams& wp,
                 const ListBuffers& LB, cudaStream_t s) {
    const int blocks = (LB.nwarps + kWalkWarps - 1) / kWalkWarps;
    if (wp.global_stack)
        walk_kernel<0><<<blocks, kWalkThreads, 0, s>>>(T, C, leaf_list, wp, LB);
    else if (wp.smem_stack == 1024)
        walk_kernel<1024><<<blocks, kWalkThreads, 0, s>>>(T, C, leaf_list, wp, LB);
    else if (wp.smem_stack == 4096)
        walk_kernel<4096><<<blocks, kWalkThreads, 0, s>>>(T, C, leaf_list, wp, LB);
    else
        walk_kernel<2048><<<blocks, kWalkThreads, 0, s>>>(T, C, leaf_list, wp, LB);
}

}  // namespace ngrav
