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
