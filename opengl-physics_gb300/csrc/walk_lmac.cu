// walk_lmac.cu -- the grouped walk with the learned opening test (lmac.cuh).
//
// Same traversal and list output as walk_kernel (walk.cu; semantics of the
// reference's grouped walk, Solvers.cpp:248-355), with the opening decision of
// an internal node replaced:
//   worst <= 0 or 2h >= rho_hi * worst   -> open
//   2h <= rho_lo * worst                 -> accept (far)
//   otherwise                            -> ask the network
// Pairs for the network wait in a per-warp queue of 64 slots whose features sit
// in the CTA's shared operand tile; the four warps of a CTA advance in step and
// the CTA evaluates all queued pairs with one tensor-core flush (lmac_tc.cuh)
// whenever some warp's queue is full or some warp has nothing else to do.  A
// flushed pair is accepted iff its logit z > gate, opened iff z < -gate, and
// decided by the geometric test with the run's theta otherwise.
//
// lmac_tc_forward_kernel evaluates the same routine on given features (the
// unit test of the tensor-core path against the oracle).
#include "engine.cuh"
#include "lmac.cuh"
#include "lmac_tc.cuh"
#include "walk_common.cuh"

namespace ngrav {

constexpr int kLmWarps = 4;
constexpr int kLmThreads = kLmWarps * 32;
constexpr int kLmStack = 1024;  // per-warp shared-memory traversal stack
constexpr int kLmQueue = 64;

size_t walk_lmac_smem_bytes() {
    return sizeof(LmacTiles) + 1024 + sizeof(int) * (kLmWarps * kLmQueue + 8 + kLmWarps * kLmStack);
}

template <bool SMEM_STACK>
__global__ void __launch_bounds__(kLmThreads) walk_lmac_kernel(NodeArrays T, Counters* C,
                                                               const int* __restrict__ leaf_list, WalkParams wp,
                                                               ListBuffers LB, const LmacDev* __restrict__ model) {
    extern __shared__ unsigned char lm_dyn[];
    LmacTiles& S = *lmac_tiles_at(lm_dyn);
    int* pend_all = reinterpret_cast<int*>(&S + 1);
    int* flags = pend_all + kLmWarps * kLmQueue;
    int* s_stack = flags + 8;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int gwarp = blockIdx.x * kLmWarps + warp;
    lmac_tc_init(S, model);
    int* pend = pend_all + warp * kLmQueue;
    int* stack = SMEM_STACK ? s_stack + warp * kLmStack : LB.stack + (long long)gwarp * LB.stack_cap;
    const int stack_cap = SMEM_STACK ? kLmStack : LB.stack_cap;
    const int nleaves = C->nleaves;
    const unsigned lt_mask = (1u << lane) - 1u;
    const float eps = sqrtf(wp.eps2);
    unsigned long long tests = 0, groups = 0, queries = 0, accepts = 0, fallbacks = 0, flushes = 0;
    int stack_max = 0, list_max = 0;
    unsigned bad = 0;
    int fres_next = 0, fres_end = 0, nres_next = 0, nres_end = 0;
    bool active = false, exhausted = (C->status & kStFatal) != 0;
    int gi = 0, leaf = 0, size = 0, npend = 0, visits = 0;
    float4 gA = make_float4(0.f, 0.f, 0.f, 0.f), gD = gA;
    float gR = 0.f, amin = 0.f;
    ChunkList far = {-1, -1, 0, 0, 0, 0}, near = far;
    uint32_t phase = 0;
    int it = 0;

    for (;;) {
        // ---- take a new group ----
        if (!active && !exhausted) {
            int g = 0;
            if (lane == 0) g = atomicAdd(&C->work_next, 1);
            g = __shfl_sync(0xffffffffu, g, 0);
            if (g >= nleaves) {
                exhausted = true;
            } else {
                gi = g;
                leaf = leaf_list[gi];
                gA = T.wA[leaf];
                gD = T.wD[leaf];
                gR = T.wC[leaf].x;
                amin = T.amin[leaf];
                ++groups;
                far = {-1, -1, 0, 0, fres_next, fres_end};
                near = {-1, -1, 0, 0, nres_next, nres_end};
                list_append(near, lane == 0, leaf, LB.near, LB.near_next, &C->near_chunks, LB.near_chunk_cap,
                            lane, lt_mask, bad);
                size = 0;
                if (leaf != 0) {
                    if (lane == 0) stack[0] = 0;
                    size = 1;
                }
                visits = 0;
                npend = 0;
                active = true;
                __syncwarp();
            }
        }
        // ---- one traversal step: up to 64 nodes, as the queue allows ----
        if (active && size > 0 && npend < kLmQueue) {
            const int take = min(size, kLmQueue - npend);
            size -= take;
            visits += take;
            int node[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int idx = lane + 32 * q;
                node[q] = idx < take ? stack[size + idx] : -1;
            }
            __syncwarp();
            int kind[2], nch[2], link[2];
            float feat[2][kLmacIn];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                kind[q] = 0;  // 0 none, 1 near, 2 far, 3 open, 4 ask the network
                nch[q] = 0;
                link[q] = 0;
                const int nd = node[q];
                if (nd >= 0 && nd != leaf) {
                    const float4 A = T.wA[nd];
                    const float4 Cw = T.wC[nd];
                    const int meta = __float_as_int(Cw.w);
                    link[q] = __float_as_int(Cw.z);
                    if (A.w > 0.f) {
                        if (meta < 0) {
                            kind[q] = 1;
                        } else {
                            const float4 D = T.wD[nd];
                            const float dx = (A.x - gA.x) + (D.x - gD.x);
                            const float dy = (A.y - gA.y) + (D.y - gD.y);
                            const float dz = (A.z - gA.z) + (D.z - gD.z);
                            const float worst = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - gR;
                            const float sz = Cw.y;
                            if (!(worst > 0.f) || sz >= wp.lm_rho_hi * worst) {
                                kind[q] = 3;
                            } else if (sz <= wp.lm_rho_lo * worst) {
                                kind[q] = 2;
                            } else {
                                kind[q] = 4;
                                lmac_features(gA, gD, gR, amin, A, T.wB[nd], Cw, D, T.count[nd], wp.G, eps,
                                              wp.lm_log2b, feat[q]);
                            }
                            if (kind[q] == 3) nch[q] = meta & 0xFFFFFF;
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                tests += __popc(__ballot_sync(0xffffffffu, kind[q] >= 2));
                list_append(near, kind[q] == 1, node[q], LB.near, LB.near_next, &C->near_chunks,
                            LB.near_chunk_cap, lane, lt_mask, bad);
                list_append(far, kind[q] == 2, node[q], LB.far, LB.far_next, &C->far_chunks, LB.far_chunk_cap,
                            lane, lt_mask, bad);
                const unsigned m = __ballot_sync(0xffffffffu, kind[q] == 4);
                if (kind[q] == 4) {
                    const int slot = npend + __popc(m & lt_mask);
                    lmac_put_features(S, warp, slot, feat[q]);
                    pend[slot] = node[q];
                }
                npend += __popc(m);
            }
            bool ovf = false;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                int tot;
                const int off = warp_excl_scan(nch[q], lane, tot);
                if (size + tot > stack_cap) {
                    ovf = true;
                    break;
                }
                for (int k = 0; k < nch[q]; ++k) stack[size + off + k] = link[q] + k;
                size += tot;
            }
            if (ovf || visits > wp.node_limit) {
                bad |= ovf ? kStStackOverflow : kStCorrupt;
                active = false;  // the host re-runs the evaluation (larger stack) or reports
                exhausted = true;
                npend = 0;
            }
            stack_max = max(stack_max, size);
            __syncwarp();
        }
        // ---- CTA step: flush when some warp needs the network ----
        const bool need = active && npend > 0 && (npend == kLmQueue || size == 0);
        const bool done = exhausted && !active;
        if (lane == 0) flags[(it & 1) * 4 + warp] = (need ? 1 : 0) | (done ? 2 : 0);
        __syncthreads();
        int any_need = 0, all_done = 2;
#pragma unroll
        for (int w = 0; w < kLmWarps; ++w) {
            const int f = flags[(it & 1) * 4 + w];
            any_need |= f & 1;
            all_done &= f & 2;
        }
        ++it;
        if (all_done) break;
        if (any_need) {
            float z0 = 0.f, z1 = 0.f;
            const bool ok = lmac_tc_flush(S, warp, lane, phase, z0, z1);
            ++flushes;
            if (!ok) {
                bad |= kStTimeout;
                active = false;
                exhausted = true;
                npend = 0;
            }
            if (npend > 0) {
                int kind[2], nch[2], link[2], node[2];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int slot = lane + 32 * q;
                    node[q] = slot < npend ? pend[slot] : -1;
                    kind[q] = 0;
                    nch[q] = 0;
                    link[q] = 0;
                    if (node[q] >= 0) {
                        const float z = q ? z1 : z0;
                        const float4 Cw = T.wC[node[q]];
                        bool acc;
                        if (fabsf(z) >= wp.lm_gate) {
                            acc = z > 0.f;
                        } else {  // low confidence: the geometric test decides
                            const float4 A = T.wA[node[q]], D = T.wD[node[q]];
                            const float dx = (A.x - gA.x) + (D.x - gD.x);
                            const float dy = (A.y - gA.y) + (D.y - gD.y);
                            const float dz = (A.z - gA.z) + (D.z - gD.z);
                            const float worst = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - gR;
                            acc = worst > 0.f && Cw.y * Cw.y < wp.theta2 * worst * worst;
                            ++fallbacks;
                        }
                        kind[q] = acc ? 2 : 3;
                        if (acc) ++accepts;
                        if (!acc) {
                            nch[q] = __float_as_int(Cw.w) & 0xFFFFFF;
                            link[q] = __float_as_int(Cw.z);
                        }
                    }
                }
                queries += npend;
                bool ovf = false;
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    list_append(far, kind[q] == 2, node[q], LB.far, LB.far_next, &C->far_chunks,
                                LB.far_chunk_cap, lane, lt_mask, bad);
                    int tot;
                    const int off = warp_excl_scan(nch[q], lane, tot);
                    if (size + tot > stack_cap) {
                        ovf = true;
                        break;
                    }
                    for (int k = 0; k < nch[q]; ++k) stack[size + off + k] = link[q] + k;
                    size += tot;
                }
                npend = 0;
                if (ovf) {
                    bad |= kStStackOverflow;
                    active = false;
                    exhausted = true;
                }
                stack_max = max(stack_max, size);
                __syncwarp();
            }
        }
        // ---- group finished ----
        if (active && size == 0 && npend == 0) {
            fres_next = far.res_next;
            fres_end = far.res_end;
            nres_next = near.res_next;
            nres_end = near.res_end;
            if (lane == 0) LB.ginfo[gi] = make_int4(far.first, near.first, far.count, near.count);
            list_max = max(list_max, max(far.count, near.count));
            active = false;
        }
    }
    lmac_tc_release(S);
    for (int o = 16; o > 0; o >>= 1) {
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
        fallbacks += __shfl_xor_sync(0xffffffffu, fallbacks, o);
        accepts += __shfl_xor_sync(0xffffffffu, accepts, o);
    }
    if (lane == 0) {
        if (bad) atomicOr(&C->status, bad);
        atomicAdd(&C->mac_tests, tests);
        atomicAdd(&C->groups, groups);
        atomicAdd(&C->lm_queries, queries);
        atomicAdd(&C->lm_accepts, accepts);
        atomicAdd(&C->lm_fallbacks, fallbacks);
        atomicMax(&C->stack_max, stack_max);
        atomicMax(&C->list_max, list_max);
    }
    if (threadIdx.x == 0) atomicAdd(&C->lm_flushes, flushes);
}

// Logits of n pairs from raw features X[n][8] (standardised with the model's
// statistics inside), 256 pairs per CTA flush: pair base + 64 w + p sits in
// slot p of warp w.  status |= kStTimeout if a wait ran out.
__global__ void __launch_bounds__(kLmThreads) lmac_tc_forward_kernel(const LmacDev* __restrict__ model,
                                                                     const float* __restrict__ X, int n,
                                                                     float* __restrict__ z,
                                                                     unsigned* __restrict__ status) {
    extern __shared__ unsigned char lm_dyn[];
    LmacTiles& S = *lmac_tiles_at(lm_dyn);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    lmac_tc_init(S, model);
    uint32_t phase = 0;
    bool ok_all = true;
    for (long long base = (long long)blockIdx.x * 256; base < n; base += (long long)gridDim.x * 256) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const long long i = base + 64 * warp + 32 * q + lane;
            float f[kLmacIn];
#pragma unroll
            for (int k = 0; k < kLmacIn; ++k) f[k] = i < n ? X[i * kLmacIn + k] : 0.f;
            lmac_put_features(S, warp, 32 * q + lane, f);
        }
        float z0, z1;
        ok_all = lmac_tc_flush(S, warp, lane, phase, z0, z1) && ok_all;
        const long long i0 = base + 64 * warp + lane, i1 = i0 + 32;
        if (i0 < n) z[i0] = z0;
        if (i1 < n) z[i1] = z1;
    }
    lmac_tc_release(S);
    if (!ok_all) atomicOr(status, kStTimeout);
}

void launch_walk_lmac(const NodeArrays& T, Counters* C, const int* leaf_list, const WalkParams& wp,
                      const ListBuffers& LB, const LmacDev* model, cudaStream_t s) {
    const size_t smem = walk_lmac_smem_bytes();
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(walk_lmac_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(walk_lmac_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    const int blocks = (LB.nwarps + kLmWarps - 1) / kLmWarps;
    if (wp.global_stack)
        walk_lmac_kernel<false><<<blocks, kLmThreads, smem, s>>>(T, C, leaf_list, wp, LB, model);
    else
        walk_lmac_kernel<true><<<blocks, kLmThreads, smem, s>>>(T, C, leaf_list, wp, LB, model);
}

int walk_lmac_blocks_per_sm() {
    const size_t smem = walk_lmac_smem_bytes();
    cudaFuncSetAttribute(walk_lmac_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, walk_lmac_kernel<true>, kLmThreads, smem);
    // 64 tensor-memory columns per CTA: at most 8 CTAs share an SM's 512.
    nb = nb < 8 ? nb : 8;
    return nb > 0 ? nb : 1;
}

void launch_lmac_tc_forward(const LmacDev* model, const float* X, int n, float* z, unsigned* status, int sm_count,
                            cudaStream_t s) {
    if (n <= 0) return;
    const size_t smem = walk_lmac_smem_bytes();
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(lmac_tc_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    long long blocks = ((long long)n + 255) / 256;
    if (blocks > (long long)sm_count * 4) blocks = (long long)sm_count * 4;
    lmac_tc_forward_kernel<<<(unsigned)blocks, kLmThreads, smem, s>>>(model, X, n, z, status);
}

}  // namespace ngrav
