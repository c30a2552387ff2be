// ctx_internal.cuh -- the context behind the C-ABI handle and the host
// helpers shared by the translation units that implement include/ngrav_gpu.h
// (ctx.cu: state, force evaluation, KDK; lmac_host.cu: the learned opening
// test).
#pragma once

#include "ngrav_gpu.h"

#include "engine.cuh"

#include <string>
#include <vector>

using namespace ngrav;

namespace ngrav_ctx {
struct LmacState;  // lmac_host.cu
}

struct ngrav_gpu_ctx {
    ngrav_gpu_opts opts{};
    std::string err;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    long long n = 0;
    long long cap_n = 0;
    Particles P;
    SortBuffers SB;
    NodeArrays T;
    Counters* C = nullptr;
    Counters hc{};
    int* leaf_at = nullptr;
    unsigned* flags = nullptr;
    unsigned* scanbuf = nullptr;
    int* leaf_list = nullptr;
    ListBuffers LB;
    int eval_nwarps = 0;
    long long gi_cap = 0;
    bool walk_global_stack = false;
    double* stage = nullptr;          // 7 * cap_n doubles (upload / download staging)
    double* dpartial = nullptr;
    long long dpartial_cap = 0;
    int* inv = nullptr;
    int* dtargets = nullptr;
    int* dslots = nullptr;
    double* dsamp = nullptr;
    int samp_cap = 0;
    bool have = false;
    bool primed = false;
    long long force_evals = 0;
    cudaEvent_t ev[8] = {};
    cudaEvent_t sev[2] = {};
    bool events = false;
    double phase_ms[7] = {};
    // cumulative measurement counters (ngrav_gpu_reset_cumulative)
    long long launches = 0;
    long long cum_evals = 0, cum_pairs = 0, cum_p2c = 0;
    double cum_ms_walk = 0.0, cum_ms_force = 0.0, cum_ms_eval = 0.0, cum_ms_step = 0.0;
    bool acc_valid = false;           // P.acc holds a force evaluation of this particle set
    int walk_stack = 2048;            // tuned: per-warp shared-memory walk stack entries
    int sort_levels = kKeyLevels;     // key levels sorted and built (adapted to the tree's depth)
    int sort_passes = kRsPasses;      // radix-sort passes of the last evaluation enqueued
    int p2p_tile = 0;                 // tuned: sources per near batch (0: the kernel's maximum)
    int soft = 0;                     // kSoftPlummer / kSoftSpline (softening.cuh)
    double alpha = 0.001;             // relative opening test tolerance
    // block-timestep evaluation in progress: {finest substep, max rung}
    bool block_on = false;
    long long cum_particle_evals = 0;  // System::ParticleEvals: targets of every evaluation
    int block_args[2] = {0, 0};
    double block_base = 0.0;
    // ensemble of independent systems (Forest of engine.cuh); nsys = 1: one system
    Forest F;
    long long* f_off = nullptr;
    double* f_root = nullptr;
    unsigned long long* f_bbox = nullptr;
    std::vector<long long> h_off;
    // CUDA graphs of one KDK step (kick-drift + force evaluation), keyed by
    // every pointer and parameter the launches bake in; two slots because the
    // particle buffers alternate between steps.
    struct StepGraph {
        std::vector<unsigned char> key;
        cudaGraphExec_t exec = nullptr;
        long long launches = 0;
    };
    StepGraph graphs[2];
    int graph_next = 0;
    bool capturing = false;
    bool use_graphs = true;
    long long graph_captures = 0, graph_replays = 0;
    // learned opening test (model, training buffers, run-time control)
    ngrav_ctx::LmacState* lm = nullptr;
};

namespace ngrav_ctx {

#define NG_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                 \
            return (e_ == cudaErrorMemoryAllocation) ? NGRAV_ERR_OOM : NGRAV_ERR_CUDA;     \
        }                                                                                  \
    } while (0)

#define NG_TRY(expr)          \
    do {                      \
        int rc_ = (expr);     \
        if (rc_) return rc_;  \
    } while (0)

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

template <typename T>
cudaError_t dalloc(T*& p, long long count) {
    return cudaMalloc((void**)&p, sizeof(T) * (size_t)(count > 0 ? count : 1));
}

int fail(ngrav_gpu_ctx* ctx, int code, const std::string& msg);
bool split_of(const ngrav_gpu_ctx* ctx);
// Smoothing length of the spline softening, 0 with Plummer softening.
inline double spline_h(const ngrav_gpu_ctx* ctx) { return ctx->soft == 1 ? ctx->opts.eps : 0.0; }
ngrav::WalkParams walk_params(const ngrav_gpu_ctx* ctx, bool kick, float hdt);
// One force evaluation of the current state (retrying on capacity growth).
int evaluate(ngrav_gpu_ctx* ctx, bool bbox_ready, bool kick, float hdt);
int ensure_samp(ngrav_gpu_ctx* ctx, int ns);
int ensure_partial(ngrav_gpu_ctx* ctx, long long count);
void free_forest(ngrav_gpu_ctx* ctx);

// Learned opening test hooks (lmac_host.cu).
void lmac_destroy(ngrav_gpu_ctx* ctx);
// Decide whether the next walk uses the learned test and put its buffers in
// place (allocations happen here, never inside a graph capture).
bool lmac_prepare(ngrav_gpu_ctx* ctx);
// Fill the walk parameters of a prepared learned walk; false if not prepared.
bool lmac_walk_setup(ngrav_gpu_ctx* ctx, ngrav::WalkParams& wp, const void** model);
// Append what a captured step depends on to a graph key.
void lmac_key(const ngrav_gpu_ctx* ctx, std::vector<unsigned char>& key);
void lmac_launch_walk(ngrav_gpu_ctx* ctx, const ngrav::WalkParams& wp, const void* model);
// The deferred-pair pools overflowed: size them to what the walk counted.
int lmac_grow_pools(ngrav_gpu_ctx* ctx);
// Testing: free the deferred-pair pools; later walks start them at `chunks`.
int lmac_debug_shrink(ngrav_gpu_ctx* ctx, long long chunks);
// After a force evaluation: run the periodic FP64 check, revert on a breach.
int lmac_after_eval(ngrav_gpu_ctx* ctx);
void lmac_fill_stats(const ngrav_gpu_ctx* ctx, ngrav_gpu_stats* out);

}  // namespace ngrav_ctx
