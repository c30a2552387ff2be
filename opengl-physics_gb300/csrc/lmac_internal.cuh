// lmac_internal.cuh -- launchers and parameter blocks of the learned opening
// test's data generation, training and inference (see lmac.cuh).
#pragma once

#include "engine.cuh"
#include "lmac.cuh"

namespace ngrav {

struct LmacRecordParams {
    float theta;                      // geometric test of the recording walk
    float rho_lo, rho_hi;             // band of 2h/worst that is sampled
    uint32_t seed;
    uint32_t threshold;               // keep a band pair iff hash < threshold
    int node_limit;
    int cap;                          // capacity of `pairs`
    int* work;                        // group scheduler (zeroed by the caller)
    int2* pairs;                      // (group leaf, node)
    unsigned long long* nkept;        // pairs kept (may exceed cap)
    unsigned long long* nband;        // band pairs met
    unsigned long long* ndropped;     // groups cut short (stack or visit limit)
};

// ---- round-based learned walk (walk_lmac.cu) ----
// A group between rounds: its interaction lists so far and its deferred pairs.
struct LmacGroupState {
    int far_first, far_cur, far_pos, far_count;
    int near_first, near_cur, near_pos, near_count;
    int pend_first, pend_count;
    int pad[2];
};

constexpr int kLmMaxRounds = 8;
// Deferred pairs are kept in chunks of one warp's width: a group that parks
// a few pairs wastes at most 31 slots of the tensor-core tiles.
constexpr int kPendChunk = 32;
// Per round r: ctr[4r] walk scheduler, ctr[4r+1] groups deferred, ctr[4r+2]
// pending chunks taken, ctr[4r+3] unused.
struct LmacRounds {
    int rounds;                        // rounds this evaluation runs (the last decides geometrically)
    LmacGroupState* gs;                // per group index
    int* active[2];                    // group indices with deferred pairs (ping-pong by round parity)
    int* pend_node[2];                 // deferred node ids, chunks of kPendChunk (ping-pong)
    int* pend_next[2];                 // chunk links
    int* pend_owner[2];                // chunk -> group leaf
    int* pend_fill[2];                 // chunk -> entries used
    unsigned char* dec;                // decisions for the pool being resolved (1 = accept)
    int pend_chunk_cap;
    int* ctr;                          // 4 * kLmMaxRounds counters, zeroed per evaluation
};

void launch_walk_lmac_round(const NodeArrays& T, Counters* C, const int* leaf_list, const WalkParams& wp,
                            const ListBuffers& LB, const LmacRounds& R, int round, int sm_count, cudaStream_t s);
void launch_lmac_infer(const NodeArrays& T, Counters* C, const WalkParams& wp, const LmacRounds& R, int round,
                       const LmacDev* model, int sm_count, cudaStream_t s);
void launch_lmac_tc_forward(const LmacDev* model, const float* X, int n, float* z, unsigned* status, int sm_count,
                            cudaStream_t s);

void launch_lmac_record(const NodeArrays& T, const Counters* C, const int* leaf_list, const LmacRecordParams& rp,
                        int blocks, cudaStream_t s);
void launch_lmac_amin(const NodeArrays& T, const Counters* C, const int* leaf_list, const float4* acc,
                      long long max_leaves, cudaStream_t s);
void launch_lmac_label(const NodeArrays& T, const float4* pos, const float4* plo, const float4* acc,
                       const int2* pairs, int npairs, float G, float eps2, float* r_out, cudaStream_t s);
void launch_lmac_features(const NodeArrays& T, const int2* pairs, int npairs, float G, float eps, float* X,
                          cudaStream_t s);

void launch_lmac_make_batch(const float* X, const float* r, long long n, const LmacNorm& norm, int nb,
                            uint32_t seed, float u_range, bool standardise, float* Xb, float* yb, float* wb,
                            cudaStream_t s);
int lmac_grad_blocks(int nb);
void launch_lmac_grad(const float* Xb, const float* yb, const float* wb, int nb, const float* P, float scale,
                      float* partial, float* stats, cudaStream_t s);
void launch_lmac_adam(const float* partial, int nblocks, float* grad, float* P, float* m, float* v, bool step,
                      float lr, float beta1, float beta2, float bc1, float bc2, float adam_eps, cudaStream_t s);
void launch_lmac_forward(const float* X, int n, const float* P, float* z, cudaStream_t s);

}  // namespace ngrav
