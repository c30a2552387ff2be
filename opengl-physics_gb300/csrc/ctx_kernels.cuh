// ctx_kernels.cuh -- launchers of kdk.cu used by the context (internal).
#pragma once

#include "engine.cuh"

namespace ngrav {

void launch_upload_f64(long long n, const double* x, const double* y, const double* z, const double* vx,
                       const double* vy, const double* vz, const double* m, const Particles& P, bool split,
                       cudaStream_t s);
void launch_state_f64(long long n, const double* x, const double* y, const double* z, const double* vx,
                      const double* vy, const double* vz, const Particles& P, bool split, cudaStream_t s);
void launch_state_f32(long long n, const float* x, const float* y, const float* z, const float* vx,
                      const float* vy, const float* vz, const Particles& P, bool split, cudaStream_t s);
void launch_upload_f32(long long n, const float* x, const float* y, const float* z, const float* vx,
                       const float* vy, const float* vz, const float* m, const Particles& P, bool split,
                       cudaStream_t s);
void launch_download(long long n, const int* id, const float4* a, const float4* alo, double* ox, double* oy,
                     double* oz, cudaStream_t s);
void launch_inverse_id(long long n, const int* id, int* inv, cudaStream_t s);
int diag_blocks(long long n);
void launch_diag_pass1(long long n, const Particles& P, bool split, double* partial, cudaStream_t s);
void launch_diag_pass2(long long n, const Particles& P, bool split, double cx, double cy, double cz, double* partial,
                       cudaStream_t s);
int potential_blocks(long long n);
// Exact pair potential with FP32 pair terms and FP64 sums (Plummer).
int potential_f32_blocks(long long n, int sm_count);
void launch_potential_f32(long long n, const Particles& P, bool split, double eps2, int blocks, double* partial,
                          cudaStream_t s);
void launch_potential(long long n, const Particles& P, bool split, double eps2, double spline_h, double* partial,
                      cudaStream_t s);
int sampler_shares(long long n, int nslots, int sm_count);
// FP64 pairs (one block per target), or FP32 pairs tiled over `shares`
// source shares with FP64 totals (partial: shares * 3 * nslots doubles).
void launch_sampler(long long n, const Particles& P, bool split, const int* slots, int nslots, double eps2,
                    double spline_h, bool fp64_pairs, double* out, double* partial, int shares, cudaStream_t s);
void launch_reset_counters(Counters* C, cudaStream_t s);
void eval_set_attributes();
void lmac_set_attributes();
int walk_warps_per_block();
int walk_blocks_per_sm();
int eval_warps_per_block();
int eval_blocks_per_sm();
size_t eval_smem_bytes();
void launch_gather_slots(const int* inv, const int* targets, int nt, int* slots, cudaStream_t s);
double run_fma_probe(int sm_count, cudaStream_t s);

// ensemble.cu
void launch_forest_sampler(const Particles& P, bool split, const int* slots, int nslots, const Forest& F,
                           double eps2, double spline_h, double* out, cudaStream_t s);
void launch_gather_float4(const float4* a, const int* slots, int ns, float4* out, cudaStream_t s);
void launch_forest_diag(const Particles& P, bool split, const Forest& F, double* part, cudaStream_t s);
void launch_forest_potential(const Particles& P, bool split, const Forest& F, double eps2, int chunks, double* part,
                             cudaStream_t s);

// walk_pp.cu: the per-particle walk (relative MAC, target subsets), with the
// force sums and the closing kick.
// block = {sub, rmax}: block-timestep mode (nullptr: every particle).
void launch_walk_pp(const NodeArrays& T, Counters* C, const Particles& P, const int* leaf_list, const WalkParams& wp,
                    int relative, double alpha, const unsigned char* targets, const int* block, double block_base,
                    int nwarps, cudaStream_t s);
// kdk.cu: block timesteps
void launch_frame_download(long long n, const int* id, const float4* pos, const float4* plo, const float4* vel,
                           const float4* vlo, float* opos, float* ovel, cudaStream_t s);
void launch_amax(long long n, const float4* acc, unsigned long long* out, cudaStream_t s);
void launch_rung_download(long long n, const int* id, const float4* vel, int* out, cudaStream_t s);
void launch_rungs(long long n, const Particles& P, double base, double eta, double eps, int max_rung, int* rmax,
                  cudaStream_t s);
void launch_block_kick_drift(long long n, const Particles& P, bool split, double base, int sub, int rmax, float dtmin,
                             cudaStream_t s);

}  // namespace ngrav
