// walk_lmac.cu -- the grouped walk with the learned opening test (lmac.cuh),
// run in rounds.
//
// Same traversal and list output as walk_kernel (walk.cu; semantics of the
// reference's grouped walk, Solvers.cpp:248-355), with the opening decision of
// an internal node replaced:
//   worst <= 0 or 2h >= rho_hi * worst   -> open
//   2h <= rho_lo * worst                 -> accept (far)
//   quadrupole error bound within screen x budget x amin -> accept (far)
//   otherwise                            -> the network decides
// Round r of the walk (walk_lmac_round_kernel) resolves the group's deferred
// pairs of round r-1 (accept -> far list, open -> children onto the stack),
// then walks until its stack is empty, deferring every pair for the network
// (its node id, with the geometric decision in the top bit) into a chunked
// per-group pending list.  Between rounds, lmac_infer_kernel gathers the
// deferred pairs' records, computes their features and evaluates the network
// on the tensor cores (lmac_tc.cuh, 256 pairs per CTA flush), and stores the
// decision: accept iff the logit z > gate, open iff z < -gate, the geometric
// test with the run's theta otherwise.  The last round decides its band pairs
// by the bound and the geometric test, so every group's lists are complete
// after it.  Traversal warps never wait for the tensor cores, and the
// tensor-core kernel runs as a streaming batch.
//
// lmac_tc_forward_kernel evaluates the same network routine on given features
// (the unit test of the tensor-core path against the oracle).
#include "engine.cuh"
#include "lmac.cuh"
#include "lmac_internal.cuh"
#include "lmac_tc.cuh"
#include "walk_common.cuh"

namespace ngrav {

constexpr int kLwWarps = 4;
constexpr int kLwThreads = kLwWarps * 32;
// Per-warp shared-memory traversal stack: 2048 entries at 6 CTAs per SM, or
// 1024 at 8 (the walk_stack tuning knob picks; an overflow moves the run to
// the global-memory stack).

// Append to a group's deferred-pair list: chunks taken one at a time (so
// every chunk counted is owned and filled), owner and fill recorded for the
// tensor-core kernel.
__device__ __forceinline__ void pend_append(ChunkList& L, bool has, int val, const LmacRounds& R, int out,
                                            int* counter, int leaf, int lane, unsigned lt_mask, unsigned& bad) {
    const unsigned m = __ballot_sync(0xffffffffu, has);
    const int k = __popc(m);
    if (k == 0) return;
    const int cap = R.pend_chunk_cap;
    if (L.cur < 0) {
        int c = 0;
        if (lane == 0) {
            c = atomicAdd(counter, 1);
            if (c < cap) R.pend_owner[out][c] = leaf;
        }
        L.cur = L.first = __shfl_sync(0xffffffffu, c, 0);
        L.pos = 0;
    }
    int newc = -1;
    if (L.pos + k > kPendChunk) {
        if (lane == 0) {
            newc = atomicAdd(counter, 1);
            if (L.cur < cap) {
                R.pend_next[out][L.cur] = newc;
                R.pend_fill[out][L.cur] = kPendChunk;
            }
            if (newc < cap) R.pend_owner[out][newc] = leaf;
        }
        newc = __shfl_sync(0xffffffffu, newc, 0);
    }
    if (has) {
        const int i = L.pos + __popc(m & lt_mask);
        const int c = i < kPendChunk ? L.cur : newc;
        const int p = i < kPendChunk ? i : i - kPendChunk;
        if (c < cap) {
            R.pend_node[out][(long long)c * kPendChunk + p] = val;
        } else {
            bad |= kStPendOverflow;
        }
    }
    if (newc >= 0) {
        L.cur = newc;
        L.pos = L.pos + k - kPendChunk;
    } else {
        L.pos += k;
    }
    L.count += k;
}

// Standardised features as the tensor-core operand row: 8 x BF16.
__device__ __forceinline__ uint4 lmac_row(const float f[kLmacIn], const WalkParams& wp) {
    uint4 v;
    v.x = pack_bf16x2((f[0] - wp.lm_mu[0]) * wp.lm_isd[0], (f[1] - wp.lm_mu[1]) * wp.lm_isd[1]);
    v.y = pack_bf16x2((f[2] - wp.lm_mu[2]) * wp.lm_isd[2], (f[3] - wp.lm_mu[3]) * wp.lm_isd[3]);
    v.z = pack_bf16x2((f[4] - wp.lm_mu[4]) * wp.lm_isd[4], (f[5] - wp.lm_mu[5]) * wp.lm_isd[5]);
    v.w = pack_bf16x2((f[6] - wp.lm_mu[6]) * wp.lm_isd[6], (f[7] - wp.lm_mu[7]) * wp.lm_isd[7]);
    return v;
}

__device__ __forceinline__ bool geometric_accept(const float4 A, const float4 Cw, const float4 D, const float4 gA,
                                                 const float4 gD, float gR, float theta2) {
    const float dx = (A.x - gA.x) + (D.x - gD.x);
    const float dy = (A.y - gA.y) + (D.y - gD.y);
    const float dz = (A.z - gA.z) + (D.z - gD.z);
    const float worst = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - gR;
    return worst > 0.f && Cw.y * Cw.y < theta2 * worst * worst;
}

template <int STACK, int MINB>
__global__ void __launch_bounds__(kLwThreads, MINB) walk_lmac_round_kernel(NodeArrays T, Counters* C,
                                                                        const int* __restrict__ leaf_list,
                                                                        WalkParams wp, ListBuffers LB, LmacRounds R,
                                                                        int round) {
    // STACK = 0: the global-memory stack of LB
    __shared__ int s_stack[STACK > 0 ? kLwWarps * STACK : 1];
    const int lane = threadIdx.x & 31;
    const int gwarp = blockIdx.x * kLwWarps + (threadIdx.x >> 5);
    if (C->status & kStFatal) return;
    int* stack = STACK > 0 ? s_stack + (threadIdx.x >> 5) * STACK : LB.stack + (long long)gwarp * LB.stack_cap;
    const int stack_cap = STACK > 0 ? STACK : LB.stack_cap;
    const bool last = round == R.rounds - 1;
    const int in = (round + 1) & 1, out = round & 1;
    const int ngroups = round == 0 ? C->nleaves : R.ctr[4 * (round - 1) + 1];
    int* sched = R.ctr + 4 * round;
    int* active_out = R.active[out];
    int* pend_ctr = R.ctr + 4 * round + 2;
    const unsigned lt_mask = (1u << lane) - 1u;
    const float four_g = 4.f * wp.G;
    unsigned long long tests = 0, groups = 0, resolved = 0, screened = 0;
    int stack_max = 0, list_max = 0;
    unsigned bad = 0;
    int fres_next = 0, fres_end = 0, nres_next = 0, nres_end = 0;

    for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(sched, 1);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= ngroups) break;
        const int gi = round == 0 ? k : R.active[in][k];
        const int leaf = leaf_list[gi];
        const float4 gA = T.wA[leaf];
        const float4 gD = T.wD[leaf];
        const float gR = T.wC[leaf].x;
        const float amin = T.amin[leaf];
        const float screen_b = wp.lm_screen * wp.lm_budget * amin;  // 0: no screen
        ChunkList far, near, pend = {-1, -1, 0, 0, 0, 0};
        int size = 0;
        if (round == 0) {
            ++groups;
            far = {-1, -1, 0, 0, fres_next, fres_end};
            near = {-1, -1, 0, 0, nres_next, nres_end};
            list_append(near, lane == 0, leaf, LB.near, LB.near_next, &C->near_chunks, LB.near_chunk_cap, lane,
                        lt_mask, bad);
            const int root = T.sysroot[leaf];
            if (leaf != root) {
                // The root's first rule (open when worst <= 0 or 2h >= rho_hi
                // worst), by every lane at once: when it opens, as it nearly
                // always does, its children start the stack, sparing an
                // iteration that would test one node; otherwise the root takes
                // the loop's path.
                const float4 A = T.wA[root], Cw = T.wC[root], D = T.wD[root];
                const int meta = __float_as_int(Cw.w);
                bool open = false;
                if (A.w > 0.f && meta >= 0) {
                    const float dx = (A.x - gA.x) + (D.x - gD.x);
                    const float dy = (A.y - gA.y) + (D.y - gD.y);
                    const float dz = (A.z - gA.z) + (D.z - gD.z);
                    const float worst = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - gR;
                    open = !(worst > 0.f) || Cw.y >= wp.lm_rho_hi * worst;
                }
                if (open) {
                    const int nch = meta & 0xFFFFFF, link = __float_as_int(Cw.z);
                    if (lane < nch) stack[lane] = link + lane;
                    size = nch;
                    tests += 1;
                } else {
                    if (lane == 0) stack[0] = root;
                    size = 1;
                }
            }
            __syncwarp();
        } else {
            const LmacGroupState g = R.gs[gi];
            far = {g.far_first, g.far_cur, g.far_pos, g.far_count, fres_next, fres_end};
            near = {g.near_first, g.near_cur, g.near_pos, g.near_count, nres_next, nres_end};
            // resolve the deferred pairs of the previous round, 32 at a time
            int chunk = g.pend_first;
            for (int i0 = 0; i0 < g.pend_count; i0 += 32) {
                const int e = (i0 & (kPendChunk - 1)) + lane;
                const bool has = i0 + lane < g.pend_count;
                int node = -1, nch = 0, link = 0;
                bool acc = false;
                if (has) {
                    const long long slot = (long long)chunk * kPendChunk + e;
                    node = R.pend_node[in][slot] & 0x7FFFFFFF;
                    acc = R.dec[slot] != 0;
                    if (!acc) {
                        const float4 Cw = T.wC[node];
                        nch = __float_as_int(Cw.w) & 0xFFFFFF;
                        link = __float_as_int(Cw.z);
                    }
                }
                resolved += __popc(__ballot_sync(0xffffffffu, has));
                list_append(far, has && acc, node, LB.far, LB.far_next, &C->far_chunks, LB.far_chunk_cap, lane,
                            lt_mask, bad);
                int tot;
                const int off = warp_excl_scan(nch, lane, tot);
                if (size + tot > stack_cap) {
                    bad |= kStStackOverflow;
                    break;
                }
                for (int q = 0; q < nch; ++q) stack[size + off + q] = link + q;
                size += tot;
                if (((i0 + 32) & (kPendChunk - 1)) == 0 && i0 + 32 < g.pend_count) chunk = R.pend_next[in][chunk];
            }
            __syncwarp();
        }
        int visits = 0;
        while (size > 0 && !(bad & (kStStackOverflow | kStCorrupt))) {
            const int take = min(size, 64);
            size -= take;
            visits += take;
            if (visits > wp.node_limit) {
                bad |= kStCorrupt;
                break;
            }
            int node[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int idx = lane + 32 * q;
                node[q] = idx < take ? stack[size + idx] : -1;
            }
            float4 A[2], Cw[2], D[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {  // every record in flight at once
                if (node[q] >= 0) {
                    A[q] = T.wA[node[q]];
                    Cw[q] = T.wC[node[q]];
                    D[q] = T.wD[node[q]];
                } else {
                    A[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                    Cw[q] = A[q];
                    D[q] = A[q];
                }
            }
            __syncwarp();
            int kind[2], nch[2], link[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                kind[q] = 0;  // 0 none, 1 near, 2 far, 3 open, 4 deferred
                nch[q] = 0;
                link[q] = __float_as_int(Cw[q].z);
                const int meta = __float_as_int(Cw[q].w);
                if (node[q] >= 0 && node[q] != leaf && A[q].w > 0.f) {
                    if (meta < 0) {
                        kind[q] = 1;
                    } else {
                        const float dx = (A[q].x - gA.x) + (D[q].x - gD.x);
                        const float dy = (A[q].y - gA.y) + (D[q].y - gD.y);
                        const float dz = (A[q].z - gA.z) + (D[q].z - gD.z);
                        const float worst = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - gR;
                        const float sz = Cw[q].y;
                        if (!(worst > 0.f) || sz >= wp.lm_rho_hi * worst) {
                            kind[q] = 3;
                        } else if (sz <= wp.lm_rho_lo * worst) {
                            kind[q] = 2;
                        } else {
                            // the network (rounds before the last) or the geometric test
                            kind[q] = !last ? 4 : (sz * sz < wp.theta2 * worst * worst ? 2 : 3);
                            // Quadrupole truncation bound on every member (Salmon & Warren
                            // 1994, p = 2): |da| <= G M / w^2 * 4 x^3 / (1 - x)^2, x = r / w,
                            // r = maxR; tested as 4 G M r^3 <= screen b amin w^3 (w - r)^2.
                            const float r = Cw[q].x, wr = worst - r;
                            if (kind[q] != 2 && screen_b > 0.f && wr > 0.f &&
                                four_g * A[q].w * (r * r * r) <= screen_b * (worst * worst * worst) * (wr * wr)) {
                                kind[q] = 2;
                                ++screened;
                            }
                        }
                        if (kind[q] == 3) nch[q] = meta & 0xFFFFFF;
                        // the geometric decision rides in the deferred node id's top
                        // bit for the low-confidence fallback
                        if (kind[q] == 4 && sz * sz < wp.theta2 * worst * worst) node[q] |= (int)0x80000000u;
                    }
                }
            }
            tests += __popc(__ballot_sync(0xffffffffu, kind[0] >= 2)) + __popc(__ballot_sync(0xffffffffu, kind[1] >= 2));
            list_append2(near, kind[0] == 1, node[0], kind[1] == 1, node[1], LB.near, LB.near_next, &C->near_chunks,
                         LB.near_chunk_cap, lane, lt_mask, bad);
            list_append2(far, kind[0] == 2, node[0], kind[1] == 2, node[1], LB.far, LB.far_next, &C->far_chunks,
                         LB.far_chunk_cap, lane, lt_mask, bad);
#pragma unroll
            for (int q = 0; q < 2; ++q)
                pend_append(pend, kind[q] == 4, node[q], R, out, pend_ctr, leaf, lane, lt_mask, bad);
            {  // both nodes' children onto the stack with one scan
                int tot;
                const int off = warp_excl_scan(nch[0] + nch[1], lane, tot);
                if (size + tot > stack_cap) {
                    bad |= kStStackOverflow;
                } else {
                    for (int c = 0; c < nch[0]; ++c) stack[size + off + c] = link[0] + c;
                    for (int c = 0; c < nch[1]; ++c) stack[size + off + nch[0] + c] = link[1] + c;
                    size += tot;
                }
            }
            stack_max = max(stack_max, size);
            __syncwarp();
        }
        fres_next = far.res_next;
        fres_end = far.res_end;
        nres_next = near.res_next;
        nres_end = near.res_end;
        if (pend.count > 0) {
            // park the group until the network has decided its pairs
            if (lane == 0) {
                if (pend.cur < R.pend_chunk_cap) R.pend_fill[out][pend.cur] = pend.pos;
                LmacGroupState g;
                g.far_first = far.first;
                g.far_cur = far.cur;
                g.far_pos = far.pos;
                g.far_count = far.count;
                g.near_first = near.first;
                g.near_cur = near.cur;
                g.near_pos = near.pos;
                g.near_count = near.count;
                g.pend_first = pend.first;
                g.pend_count = pend.count;
                g.pad[0] = g.pad[1] = 0;
                R.gs[gi] = g;
                active_out[atomicAdd(R.ctr + 4 * round + 1, 1)] = gi;
            }
        } else {
            if (lane == 0) LB.ginfo[gi] = make_int4(far.first, near.first, far.count, near.count);
            list_max = max(list_max, max(far.count, near.count));
        }
        if (bad & (kStStackOverflow | kStCorrupt)) break;
    }
    for (int o = 16; o > 0; o >>= 1) {
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
        screened += __shfl_xor_sync(0xffffffffu, screened, o);
    }
    if (lane == 0) {
        if (bad) atomicOr(&C->status, bad);
        atomicAdd(&C->mac_tests, tests);
        if (screened) atomicAdd(&C->lm_screened, screened);
        if (groups) atomicAdd(&C->groups, groups);
        atomicMax(&C->stack_max, stack_max);
        atomicMax(&C->list_max, list_max);
    }
    (void)resolved;
}

// Decide every deferred pair of `round`: chunks 8t .. 8t+7 form tile t
// (entry l of chunk 8t + 2w + h is pair slot 32h + l of warp w).  Each
// thread gathers its two pairs' records (the node's, and its chunk's group
// leaf's), computes the features and writes the operand rows; the ids of the
// CTA's next tile are in flight meanwhile, and the CTAs sharing an SM overlap
// one another's gathers with their tensor-core work.
__global__ void __launch_bounds__(kLwThreads) lmac_infer_kernel(NodeArrays T, Counters* C, WalkParams wp,
                                                                LmacRounds R, int round,
                                                                const LmacDev* __restrict__ model) {
    extern __shared__ unsigned char lm_dyn[];
    LmacTiles& S = *lmac_tiles_at(lm_dyn);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    __shared__ unsigned s_status;
    if (threadIdx.x == 0) s_status = C->status;
    __syncthreads();
    if (s_status & kStFatal) return;  // uniform across the CTA
    const int pool = round & 1;
    int nchunks = R.ctr[4 * round + 2];
    nchunks = nchunks < R.pend_chunk_cap ? nchunks : R.pend_chunk_cap;
    const int ntiles = (nchunks + 7) / 8;  // a tile: 8 chunks, two per warp
    if ((int)blockIdx.x >= ntiles) return;
    lmac_tc_init(S, model);
    const int* pnode = R.pend_node[pool];
    const int* fill = R.pend_fill[pool];
    const int* owner = R.pend_owner[pool];
    const float eps = sqrtf(wp.eps2);
    unsigned char* a1 = reinterpret_cast<unsigned char*>(S.a2);
    uint32_t phase = 0;
    bool ok_all = true;
    unsigned long long queries = 0, accepts = 0, fallbacks = 0, flushes = 0;
    // ids of a tile: node (top bit: the geometric decision), owner leaf, or
    // -1 past a chunk's fill
    auto load_ids = [&](int t, int nd[2], int lf[2]) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int c = 8 * t + 2 * warp + h;
            const bool in = c < nchunks && lane < fill[c];
            nd[h] = in ? pnode[(long long)c * kPendChunk + lane] : 0;
            lf[h] = in ? owner[c] : -1;
        }
    };
    int nd[2], lf[2];
    int t = blockIdx.x;
    load_ids(t, nd, lf);
    for (; t < ntiles; t += gridDim.x) {
        const int cnd[2] = {nd[0], nd[1]}, clf[2] = {lf[0], lf[1]};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            uint4 row = make_uint4(0u, 0u, 0u, 0u);
            if (clf[h] >= 0) {
                const int node = cnd[h] & 0x7FFFFFFF, leaf = clf[h];
                float f[kLmacIn];
                lmac_features(T.wA[leaf], T.wD[leaf], T.wC[leaf].x, T.amin[leaf], T.wA[node], T.wB[node],
                              T.wC[node], T.wD[node], T.count[node], wp.G, eps, wp.lm_log2b, f);
                row = lmac_row(f, wp);
            }
            *reinterpret_cast<uint4*>(a1 + tc::kmajor_offset(32 * warp + lane, 8 * h, kA1Lbo, kA1Sbo)) = row;
        }
        if (t + (int)gridDim.x < ntiles) load_ids(t + gridDim.x, nd, lf);  // in flight during the MMAs
        float z[2];
        ok_all = lmac_tc_flush(S, warp, lane, phase, z[0], z[1]) && ok_all;
        ++flushes;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (clf[h] < 0) continue;
            const long long slot = (long long)(8 * t + 2 * warp + h) * kPendChunk + lane;
            bool acc;
            if (fabsf(z[h]) >= wp.lm_gate) {
                acc = z[h] > 0.f;
            } else {  // low confidence: the geometric test decides (recorded by the walk)
                acc = cnd[h] < 0;
                ++fallbacks;
            }
            ++queries;
            if (acc) ++accepts;
            R.dec[slot] = acc ? 1 : 0;
        }
    }
    lmac_tc_release(S);
    for (int o = 16; o > 0; o >>= 1) {
        queries += __shfl_xor_sync(0xffffffffu, queries, o);
        accepts += __shfl_xor_sync(0xffffffffu, accepts, o);
        fallbacks += __shfl_xor_sync(0xffffffffu, fallbacks, o);
    }
    if (lane == 0) {
        atomicAdd(&C->lm_queries, queries);
        atomicAdd(&C->lm_accepts, accepts);
        atomicAdd(&C->lm_fallbacks, fallbacks);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&C->lm_flushes, flushes);
        if (!ok_all) atomicOr(&C->status, kStTimeout);
    }
}

// Logits of n pairs from raw features X[n][8] (standardised with the model's
// statistics inside), 256 pairs per CTA flush: pair base + 64 w + p sits in
// slot p of warp w.  status |= kStTimeout if a wait ran out.
__global__ void __launch_bounds__(kLwThreads) lmac_tc_forward_kernel(const LmacDev* __restrict__ model,
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

static size_t tc_smem_bytes() { return sizeof(LmacTiles) + 1024; }

// Dynamic shared-memory limits of the tensor-core kernels, set once at
// context creation (never inside a graph capture).
void lmac_set_attributes() {
    const int smem = (int)tc_smem_bytes();
    cudaFuncSetAttribute(lmac_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(lmac_tc_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

void launch_walk_lmac_round(const NodeArrays& T, Counters* C, const int* leaf_list, const WalkParams& wp,
                            const ListBuffers& LB, const LmacRounds& R, int round, int sm_count, cudaStream_t s) {
    // persistent warps: one wave of resident CTAs (the global-stack variant
    // has one stack per warp of LB)
    if (wp.global_stack) {
        const int blocks = (LB.nwarps + kLwWarps - 1) / kLwWarps;
        walk_lmac_round_kernel<0, 6><<<blocks, kLwThreads, 0, s>>>(T, C, leaf_list, wp, LB, R, round);
    } else if (wp.smem_stack == 1024) {
        walk_lmac_round_kernel<1024, 8><<<sm_count * 8, kLwThreads, 0, s>>>(T, C, leaf_list, wp, LB, R, round);
    } else {
        walk_lmac_round_kernel<2048, 6><<<sm_count * 6, kLwThreads, 0, s>>>(T, C, leaf_list, wp, LB, R, round);
    }
}

void launch_lmac_infer(const NodeArrays& T, Counters* C, const WalkParams& wp, const LmacRounds& R, int round,
                       const LmacDev* model, int sm_count, cudaStream_t s) {
    const size_t smem = tc_smem_bytes();
    // 64 tensor-memory columns per CTA: up to 8 CTAs per SM.
    lmac_infer_kernel<<<sm_count * 7, kLwThreads, smem, s>>>(T, C, wp, R, round, model);
}

void launch_lmac_tc_forward(const LmacDev* model, const float* X, int n, float* z, unsigned* status, int sm_count,
                            cudaStream_t s) {
    if (n <= 0) return;
    const size_t smem = tc_smem_bytes();
    long long blocks = ((long long)n + 255) / 256;
    if (blocks > (long long)sm_count * 4) blocks = (long long)sm_count * 4;
    lmac_tc_forward_kernel<<<(unsigned)blocks, kLwThreads, smem, s>>>(model, X, n, z, status);
}

}  // namespace ngrav
