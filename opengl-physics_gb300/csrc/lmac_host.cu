// lmac_host.cu -- host side of the learned opening test: training-data
// generation over snapshots of the run, training (Adam on the GPU), model
// packing for the tensor-core walk, the run-time check against the FP64
// direct sum with its revert to the geometric test, and the inspection
// entry points of include/ngrav_gpu.h.
#include "ctx_internal.cuh"
#include "ctx_kernels.cuh"
#include "lmac.cuh"
#include "lmac_internal.cuh"
#include "tc.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

namespace ngrav_ctx {

struct LmacState {
    ngrav_gpu_lmac_opts opts{};
    bool have_model = false;
    float hP[kLmacParams] = {};
    LmacNorm norm{};
    LmacDev* dModel = nullptr;
    float* dP = nullptr;       // FP32 master parameters
    float* dM = nullptr;       // Adam moments
    float* dV = nullptr;
    float* dGrad = nullptr;
    float* dPartial = nullptr;
    float* dStats = nullptr;
    int partial_blocks = 0;
    float* dXb = nullptr;
    float* dyb = nullptr;
    float* dwb = nullptr;
    int batch_cap = 0;
    float* dX = nullptr;       // training features (unit budget), ndata x 8
    float* dR = nullptr;       // labels r
    long long data_cap = 0;
    int2* dPairs = nullptr;
    int pair_cap = 0;
    unsigned long long* dCnt = nullptr;  // kept, band, dropped
    int* dWork = nullptr;
    unsigned* dStatus = nullptr;
    float* dZ = nullptr;
    int z_cap = 0;
    // round-based walk buffers
    LmacRounds R{};
    long long gs_cap = 0;
    // run-time control
    bool prepared = false;    // the next walk uses the learned test (buffers in place)
    bool used_last = false;
    int evals_since_check = 0;
    bool reverted = false;
    int checks = 0;
    double last_check_rms = -1.0;
    long long start_chunks = 0;  // > 0: deferred-pair pools start at this many chunks (testing)
};

namespace {

uint16_t bf16_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);  // round to nearest even
    return (uint16_t)(u >> 16);
}

int ensure_state(ngrav_gpu_ctx* ctx) {
    if (ctx->lm) return NGRAV_OK;
    ctx->lm = new (std::nothrow) LmacState();
    if (!ctx->lm) return fail(ctx, NGRAV_ERR_OOM, "learned MAC state");
    ngrav_gpu_lmac_default_opts(&ctx->lm->opts);
    LmacState& L = *ctx->lm;
    NG_CUDA(dalloc(L.dModel, 1));
    NG_CUDA(dalloc(L.dP, kLmacParams));
    NG_CUDA(dalloc(L.dM, kLmacParams));
    NG_CUDA(dalloc(L.dV, kLmacParams));
    NG_CUDA(dalloc(L.dGrad, kLmacParams));
    NG_CUDA(dalloc(L.dCnt, 4));
    NG_CUDA(dalloc(L.dWork, 1));
    NG_CUDA(dalloc(L.dStatus, 1));
    return NGRAV_OK;
}

int ensure_batch(ngrav_gpu_ctx* ctx, int nb) {
    LmacState& L = *ctx->lm;
    if (nb <= L.batch_cap) return NGRAV_OK;
    dfree(L.dXb);
    dfree(L.dyb);
    dfree(L.dwb);
    dfree(L.dPartial);
    dfree(L.dStats);
    NG_CUDA(dalloc(L.dXb, (long long)nb * kLmacIn));
    NG_CUDA(dalloc(L.dyb, nb));
    NG_CUDA(dalloc(L.dwb, nb));
    L.partial_blocks = lmac_grad_blocks(nb);
    NG_CUDA(dalloc(L.dPartial, (long long)L.partial_blocks * kLmacParams));
    NG_CUDA(dalloc(L.dStats, 2LL * L.partial_blocks));
    L.batch_cap = nb;
    return NGRAV_OK;
}

int ensure_pairs(ngrav_gpu_ctx* ctx, int cap) {
    LmacState& L = *ctx->lm;
    if (cap <= L.pair_cap) return NGRAV_OK;
    dfree(L.dPairs);
    NG_CUDA(dalloc(L.dPairs, cap));
    L.pair_cap = cap;
    return NGRAV_OK;
}

int ensure_data(ngrav_gpu_ctx* ctx, long long cap) {
    LmacState& L = *ctx->lm;
    if (cap <= L.data_cap) return NGRAV_OK;
    dfree(L.dX);
    dfree(L.dR);
    NG_CUDA(dalloc(L.dX, cap * kLmacIn));
    NG_CUDA(dalloc(L.dR, cap));
    L.data_cap = cap;
    return NGRAV_OK;
}

int ensure_z(ngrav_gpu_ctx* ctx, int n) {
    LmacState& L = *ctx->lm;
    if (n <= L.z_cap) return NGRAV_OK;
    dfree(L.dZ);
    NG_CUDA(dalloc(L.dZ, n));
    L.z_cap = n;
    return NGRAV_OK;
}

// Pack the FP32 model into the walk's layout and upload it.
int upload_model(ngrav_gpu_ctx* ctx) {
    LmacState& L = *ctx->lm;
    LmacDev h{};
    std::memcpy(h.mu, L.norm.mu, sizeof(h.mu));
    std::memcpy(h.isd, L.norm.isd, sizeof(h.isd));
    for (int j = 0; j < kLmacHidden; ++j) {
        h.b1[j] = L.hP[kLmacB1 + j];
        h.b2[j] = L.hP[kLmacB2 + j];
        h.w3[j] = L.hP[kLmacW3 + j];
    }
    h.b3 = L.hP[kLmacB3];
    unsigned char* w1 = reinterpret_cast<unsigned char*>(h.w1t);
    unsigned char* w2 = reinterpret_cast<unsigned char*>(h.w2t);
    for (int n = 0; n < 64; ++n)
        for (int k = 0; k < 16; ++k) {
            float v = 0.f;
            if (n < 32 && k < 8) v = L.hP[kLmacW1 + n * kLmacIn + k];
            if (n >= 32 && k >= 8) v = L.hP[kLmacW1 + (n - 32) * kLmacIn + (k - 8)];
            const uint16_t b = bf16_bits(v);
            std::memcpy(w1 + tc::kmajor_offset(n, k, kW1Lbo, kW1Sbo), &b, 2);
        }
    for (int n = 0; n < 64; ++n)
        for (int k = 0; k < 64; ++k) {
            float v = 0.f;
            if (n < 32 && k < 32) v = L.hP[kLmacW2 + n * kLmacHidden + k];
            if (n >= 32 && k >= 32) v = L.hP[kLmacW2 + (n - 32) * kLmacHidden + (k - 32)];
            const uint16_t b = bf16_bits(v);
            std::memcpy(w2 + tc::kmajor_offset(n, k, kW2Lbo, kW2Sbo), &b, 2);
        }
    NG_CUDA(cudaMemcpyAsync(L.dModel, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
    NG_CUDA(cudaMemcpyAsync(L.dP, L.hP, sizeof(L.hP), cudaMemcpyHostToDevice, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    L.have_model = true;
    return NGRAV_OK;
}

// Record, label and featurise band pairs of the current tree.  Appends up to
// `cap` pairs at (X, R); returns kept count and band count.
int collect_pairs(ngrav_gpu_ctx* ctx, float theta_rec, float rho_lo, float rho_hi, double keep, uint32_t seed,
                  int cap, float* X, float* R, int* nkept_out, long long* nband_out) {
    LmacState& L = *ctx->lm;
    cudaStream_t s = ctx->stream;
    NG_TRY(ensure_pairs(ctx, std::max(cap, 1)));
    launch_lmac_amin(ctx->T, ctx->C, ctx->leaf_list, ctx->P.acc, std::min<long long>(ctx->n, ctx->T.cap), s);
    NG_CUDA(cudaMemsetAsync(L.dCnt, 0, 4 * sizeof(unsigned long long), s));
    NG_CUDA(cudaMemsetAsync(L.dWork, 0, sizeof(int), s));
    LmacRecordParams rp{};
    rp.theta = theta_rec;
    rp.rho_lo = rho_lo;
    rp.rho_hi = rho_hi;
    rp.seed = seed;
    const double k = std::min(1.0, std::max(0.0, keep));
    rp.threshold = k >= 1.0 ? 0xFFFFFFFFu : (uint32_t)(k * 4294967296.0);
    rp.node_limit = ctx->T.cap + 32;
    rp.cap = cap;
    rp.work = L.dWork;
    rp.pairs = L.dPairs;
    rp.nkept = L.dCnt;
    rp.nband = L.dCnt + 1;
    rp.ndropped = L.dCnt + 2;
    launch_lmac_record(ctx->T, ctx->C, ctx->leaf_list, rp, ctx->sm_count * 4, s);
    unsigned long long cnt[3];
    NG_CUDA(cudaMemcpyAsync(cnt, L.dCnt, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    NG_CUDA(cudaStreamSynchronize(s));
    NG_CUDA(cudaGetLastError());
    const int np = (int)std::min<unsigned long long>(cnt[0], (unsigned long long)cap);
    ctx->launches += 2;
    if (np > 0) {
        launch_lmac_label(ctx->T, ctx->P.pos, split_of(ctx) ? ctx->P.plo : nullptr, ctx->P.acc, L.dPairs, np,
                          (float)ctx->opts.G, (float)(ctx->opts.eps * ctx->opts.eps), R, s);
        launch_lmac_features(ctx->T, L.dPairs, np, (float)ctx->opts.G, (float)ctx->opts.eps, X, s);
        ctx->launches += 2;
    }
    NG_CUDA(cudaStreamSynchronize(s));
    NG_CUDA(cudaGetLastError());
    *nkept_out = np;
    *nband_out = (long long)cnt[1];
    return NGRAV_OK;
}

// One pass of the gradient kernel over a batch already in dXb/dyb/dwb; with
// step, an Adam update.  Returns (loss sum, correct count) when `stats`.
int grad_pass(ngrav_gpu_ctx* ctx, const float* P, int nb, float scale, bool step, float lr, int t,
              double* loss_sum, double* correct) {
    LmacState& L = *ctx->lm;
    cudaStream_t s = ctx->stream;
    const int blocks = lmac_grad_blocks(nb);
    launch_lmac_grad(L.dXb, L.dyb, L.dwb, nb, P, scale, L.dPartial, L.dStats, s);
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - std::pow(b1, (float)std::max(t, 1)), bc2 = 1.f - std::pow(b2, (float)std::max(t, 1));
    launch_lmac_adam(L.dPartial, blocks, L.dGrad, L.dP, L.dM, L.dV, step, lr, b1, b2, bc1, bc2, 1e-8f, s);
    ctx->launches += 2;
    if (loss_sum || correct) {
        std::vector<float> st(2 * (size_t)blocks);
        NG_CUDA(cudaMemcpyAsync(st.data(), L.dStats, sizeof(float) * st.size(), cudaMemcpyDeviceToHost, s));
        NG_CUDA(cudaStreamSynchronize(s));
        double ls = 0.0, cs = 0.0;
        for (int b = 0; b < blocks; ++b) {
            ls += st[2 * b];
            cs += st[2 * b + 1];
        }
        if (loss_sum) *loss_sum = ls;
        if (correct) *correct = cs;
    }
    return NGRAV_OK;
}

void free_rounds(LmacState& L) {
    dfree(L.R.gs);
    for (int k = 0; k < 2; ++k) {
        dfree(L.R.active[k]);
        dfree(L.R.pend_node[k]);
        dfree(L.R.pend_next[k]);
        dfree(L.R.pend_owner[k]);
        dfree(L.R.pend_fill[k]);
    }
    dfree(L.R.dec);
    dfree(L.R.ctr);
    L.R.pend_chunk_cap = 0;
    L.gs_cap = 0;
}

// Group state and active lists for `groups` groups; deferred-pair pools of
// `chunks` chunks each.
int ensure_rounds(ngrav_gpu_ctx* ctx, long long groups, long long chunks) {
    LmacState& L = *ctx->lm;
    if (!L.R.ctr) NG_CUDA(dalloc(L.R.ctr, 4 * kLmMaxRounds));
    if (groups > L.gs_cap) {
        dfree(L.R.gs);
        dfree(L.R.active[0]);
        dfree(L.R.active[1]);
        NG_CUDA(dalloc(L.R.gs, groups));
        NG_CUDA(dalloc(L.R.active[0], groups));
        NG_CUDA(dalloc(L.R.active[1], groups));
        L.gs_cap = groups;
    }
    chunks = std::min<long long>(chunks, 0x7FFFFFF0LL / kPendChunk);
    if (chunks > L.R.pend_chunk_cap) {
        for (int k = 0; k < 2; ++k) {
            dfree(L.R.pend_node[k]);
            dfree(L.R.pend_next[k]);
            dfree(L.R.pend_owner[k]);
            dfree(L.R.pend_fill[k]);
            NG_CUDA(dalloc(L.R.pend_node[k], chunks * kPendChunk));
            NG_CUDA(dalloc(L.R.pend_next[k], chunks));
            NG_CUDA(dalloc(L.R.pend_owner[k], chunks));
            NG_CUDA(dalloc(L.R.pend_fill[k], chunks));
        }
        dfree(L.R.dec);
        NG_CUDA(dalloc(L.R.dec, chunks * kPendChunk));
        L.R.pend_chunk_cap = (int)chunks;
    }
    return NGRAV_OK;
}

}  // namespace

void lmac_destroy(ngrav_gpu_ctx* ctx) {
    if (!ctx->lm) return;
    LmacState& L = *ctx->lm;
    dfree(L.dModel); dfree(L.dP); dfree(L.dM); dfree(L.dV); dfree(L.dGrad); dfree(L.dPartial); dfree(L.dStats);
    dfree(L.dXb); dfree(L.dyb); dfree(L.dwb); dfree(L.dX); dfree(L.dR); dfree(L.dPairs); dfree(L.dCnt);
    dfree(L.dWork); dfree(L.dStatus); dfree(L.dZ);
    free_rounds(L);
    delete ctx->lm;
    ctx->lm = nullptr;
}

bool lmac_prepare(ngrav_gpu_ctx* ctx) {
    LmacState* L = ctx->lm;
    bool use = ctx->opts.mac == NGRAV_MAC_LEARNED && L && L->have_model && !L->reverted && ctx->acc_valid;
    if (use) {
        // every group may park once per round; pools start at 32 deferred
        // pairs per particle (grown to what a round needs if that is short)
        const long long groups = std::max<long long>(ctx->cap_n, 1);
        const long long est = L->start_chunks > 0 ? L->start_chunks : ctx->n + 1024;
        if (ensure_rounds(ctx, groups, std::max<long long>(L->R.pend_chunk_cap, est)) != NGRAV_OK) use = false;
        L->R.rounds = std::max(2, std::min(kLmMaxRounds, L->opts.rounds));
    }
    if (L) L->prepared = use;
    return use;
}

bool lmac_walk_setup(ngrav_gpu_ctx* ctx, WalkParams& wp, const void** model) {
    LmacState* L = ctx->lm;
    const bool use = L && L->prepared;
    if (L) L->used_last = use;
    if (!use) return false;
    wp.learned = 1;
    wp.lm_log2b = (float)std::log2(std::max(L->opts.budget, 1e-30));
    wp.lm_gate = (float)L->opts.gate;
    wp.lm_rho_lo = (float)L->opts.rho_lo;
    wp.lm_rho_hi = (float)L->opts.rho_hi;
    wp.lm_screen = (float)L->opts.screen;
    wp.lm_budget = (float)L->opts.budget;
    for (int i = 0; i < kLmacIn; ++i) {
        wp.lm_mu[i] = L->norm.mu[i];
        wp.lm_isd[i] = L->norm.isd[i];
    }
    *model = L->dModel;
    return true;
}

void lmac_key(const ngrav_gpu_ctx* ctx, std::vector<unsigned char>& key) {
    const LmacState* L = ctx->lm;
    const unsigned char on = (L && L->prepared) ? 1 : 0;
    key.push_back(on);
    if (!on) return;
    auto put = [&](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        key.insert(key.end(), b, b + n);
    };
    put(&L->R, sizeof(L->R));
    put(&L->dModel, sizeof(L->dModel));
    put(&L->opts, sizeof(L->opts));
    put(&L->norm, sizeof(L->norm));
}

void lmac_launch_walk(ngrav_gpu_ctx* ctx, const WalkParams& wp, const void* model) {
    LmacState& L = *ctx->lm;
    cudaStream_t s = ctx->stream;
    cudaMemsetAsync(L.R.ctr, 0, sizeof(int) * 4 * kLmMaxRounds, s);
    for (int r = 0; r < L.R.rounds; ++r) {
        launch_walk_lmac_round(ctx->T, ctx->C, ctx->leaf_list, wp, ctx->LB, L.R, r, ctx->sm_count, s);
        if (r + 1 < L.R.rounds)
            launch_lmac_infer(ctx->T, ctx->C, wp, L.R, r, static_cast<const LmacDev*>(model), ctx->sm_count, s);
    }
    ctx->launches += 2 * L.R.rounds - 2;  // beyond the one walk launch counted by the caller
}

int lmac_debug_shrink(ngrav_gpu_ctx* ctx, long long chunks) {
    NG_TRY(ensure_state(ctx));
    LmacState& L = *ctx->lm;
    // drop the pools (and group state) so the next prepared walk starts at `chunks`
    free_rounds(L);
    L.start_chunks = chunks;
    return NGRAV_OK;
}

int lmac_grow_pools(ngrav_gpu_ctx* ctx) {
    LmacState& L = *ctx->lm;
    int ctr[4 * kLmMaxRounds];
    NG_CUDA(cudaMemcpy(ctr, L.R.ctr, sizeof(ctr), cudaMemcpyDeviceToHost));
    long long need = 0;
    for (int r = 0; r < kLmMaxRounds; ++r) need = std::max<long long>(need, ctr[4 * r + 2]);
    if (need >= 0x7FFFFFF0LL / kPendChunk) return fail(ctx, NGRAV_ERR_CAPACITY, "deferred-pair pool exhausted");
    return ensure_rounds(ctx, L.gs_cap, std::max<long long>(need + need / 4 + 1024, 2LL * L.R.pend_chunk_cap));
}

int lmac_after_eval(ngrav_gpu_ctx* ctx) {
    LmacState* L = ctx->lm;
    if (!L || !L->used_last) return NGRAV_OK;
    L->used_last = false;
    if (L->opts.check_every <= 0) return NGRAV_OK;
    if (++L->evals_since_check < L->opts.check_every) return NGRAV_OK;
    L->evals_since_check = 0;
    const int ns = (int)std::min<long long>(L->opts.check_targets, ctx->n);
    if (ns <= 0) return NGRAV_OK;
    ngrav_gpu_ferr fe;
    NG_TRY(ngrav_gpu_force_error(ctx, ns, 0x5eed0000ull + (uint64_t)L->checks, 0, &fe));
    L->checks += 1;
    L->last_check_rms = fe.rms;
    if (!(fe.rms <= L->opts.revert_rms)) L->reverted = true;
    return NGRAV_OK;
}

void lmac_fill_stats(const ngrav_gpu_ctx* ctx, ngrav_gpu_stats* out) {
    const Counters& c = ctx->hc;
    out->lmac_queries = (long long)c.lm_queries;
    out->lmac_accepts = (long long)c.lm_accepts;
    out->lmac_fallbacks = (long long)c.lm_fallbacks;
    out->lmac_flushes = (long long)c.lm_flushes;
    out->lmac_screened = (long long)c.lm_screened;
    const LmacState* L = ctx->lm;
    out->lmac_active = (L && ctx->opts.mac == NGRAV_MAC_LEARNED && L->have_model && !L->reverted) ? 1 : 0;
    out->lmac_reverted = (L && L->reverted) ? 1 : 0;
    out->lmac_checks = L ? L->checks : 0;
    out->lmac_last_check_rms = L ? L->last_check_rms : -1.0;
}

}  // namespace ngrav_ctx

using namespace ngrav_ctx;

extern "C" {

int ngrav_gpu_lmac_default_opts(ngrav_gpu_lmac_opts* o) {
    if (!o) return NGRAV_ERR_INVALID_ARG;
    std::memset(o, 0, sizeof(*o));
    o->budget = 3e-5;
    o->gate = 0.25;
    o->rho_lo = 0.25;
    o->rho_hi = 1.25;
    o->check_every = 10;
    o->check_targets = 4096;
    o->revert_rms = 1e-3;
    o->rounds = 3;
    o->screen = 1000.0;
    return NGRAV_OK;
}

int ngrav_gpu_lmac_set_opts(ngrav_gpu_ctx* ctx, const ngrav_gpu_lmac_opts* o) {
    if (!ctx || !o) return NGRAV_ERR_INVALID_ARG;
    if (!(o->budget > 0.0) || !(o->gate >= 0.0) || !(o->rho_lo >= 0.0) || !(o->rho_hi > o->rho_lo) ||
        !(o->screen >= 0.0) ||
        o->check_every < 0 || o->check_targets < 0 || o->rounds < 2 || o->rounds > kLmMaxRounds)
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "learned MAC options out of range");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    NG_TRY(ensure_state(ctx));
    ctx->lm->opts = *o;
    return NGRAV_OK;
}

int ngrav_gpu_lmac_default_train_opts(ngrav_gpu_lmac_train_opts* o) {
    if (!o) return NGRAV_ERR_INVALID_ARG;
    std::memset(o, 0, sizeof(*o));
    o->snapshots = 16;
    o->steps_between = 2;
    o->dt = 0.0;
    o->pairs = 1LL << 22;
    o->theta_record = 0.3;
    o->u_range = 6.0;
    o->epochs = 4;
    o->batch = 8192;
    o->lr = 2e-3;
    o->seed = 1;
    return NGRAV_OK;
}

int ngrav_gpu_lmac_train(ngrav_gpu_ctx* ctx, const ngrav_gpu_lmac_train_opts* o, ngrav_gpu_lmac_report* out) {
    if (!ctx || !o) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    if (o->snapshots < 1 || o->pairs < 1024 || o->epochs < 1 || o->batch < 128 || (o->batch % 128) != 0 ||
        !(o->lr > 0.0) || !(o->theta_record > 0.0) || !(o->u_range > 0.0) || o->steps_between < 0)
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "learned MAC training options out of range");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    NG_TRY(ensure_state(ctx));
    LmacState& L = *ctx->lm;
    const auto t0 = std::chrono::steady_clock::now();
    // ---- data: pairs of every snapshot, generated with the geometric test ----
    const int saved_mac = ctx->opts.mac;
    ctx->opts.mac = NGRAV_MAC_GEOMETRIC;
    const long long total = o->pairs;
    NG_TRY(ensure_data(ctx, total));
    const long long per = (total + o->snapshots - 1) / o->snapshots;
    NG_TRY(ensure_pairs(ctx, (int)std::min<long long>(per, 0x7FFFFFF0LL)));
    long long have = 0, band_total = 0;
    double expect_band = 0.0;
    int rc = NGRAV_OK;
    for (int sshot = 0; sshot < o->snapshots && rc == NGRAV_OK; ++sshot) {
        if (sshot == 0 || !(o->dt > 0.0) || o->steps_between == 0) {
            if (sshot == 0 || !ctx->acc_valid) rc = ngrav_gpu_prime(ctx);
        } else {
            rc = ngrav_gpu_step(ctx, o->steps_between, o->dt);
        }
        if (rc) break;
        const int want = (int)std::min<long long>(per, total - have);
        if (want <= 0) break;
        const uint32_t seed = (uint32_t)(o->seed * 7919u + 104729u * (uint32_t)sshot);
        int kept = 0;
        long long band = 0;
        if (expect_band <= 0.0) {  // count the band once to set the keep rate
            rc = collect_pairs(ctx, (float)o->theta_record, (float)L.opts.rho_lo, (float)L.opts.rho_hi, 0.0, seed,
                               1, L.dX + have * kLmacIn, L.dR + have, &kept, &band);
            if (rc) break;
            expect_band = (double)std::max<long long>(band, 1);
        }
        const double keep = std::min(1.0, 1.05 * want / expect_band);
        rc = collect_pairs(ctx, (float)o->theta_record, (float)L.opts.rho_lo, (float)L.opts.rho_hi, keep, seed, want,
                           L.dX + have * kLmacIn, L.dR + have, &kept, &band);
        if (rc) break;
        expect_band = (double)std::max<long long>(band, 1);
        band_total += band;
        have += kept;
    }
    ctx->opts.mac = saved_mac;
    if (rc) return rc;
    if (have < 1024) return fail(ctx, NGRAV_ERR_INVALID_ARG, "too few band pairs to train on");
    const auto t1 = std::chrono::steady_clock::now();
    // ---- split, standardisation, initialisation ----
    const long long nval = std::max<long long>(have / 20, 256);
    const long long ntrain = have - nval;
    const float* Xtr = L.dX;
    const float* Rtr = L.dR;
    const float* Xva = L.dX + ntrain * kLmacIn;
    const float* Rva = L.dR + ntrain;
    const int nb = o->batch;
    NG_TRY(ensure_batch(ctx, std::max(nb, 65536)));
    {
        LmacNorm id{};
        for (int i = 0; i < kLmacIn; ++i) id.isd[i] = 1.f;
        const int ns = 65536;
        launch_lmac_make_batch(Xtr, Rtr, ntrain, id, ns, (uint32_t)(o->seed ^ 0xA5A5A5A5u), (float)o->u_range, false,
                               L.dXb, L.dyb, L.dwb, ctx->stream);
        std::vector<float> hx((size_t)ns * kLmacIn), hw(ns);
        NG_CUDA(cudaMemcpyAsync(hx.data(), L.dXb, sizeof(float) * hx.size(), cudaMemcpyDeviceToHost, ctx->stream));
        NG_CUDA(cudaMemcpyAsync(hw.data(), L.dwb, sizeof(float) * ns, cudaMemcpyDeviceToHost, ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        for (int i = 0; i < kLmacIn; ++i) {
            double s1 = 0.0, s2 = 0.0, c = 0.0;
            for (int k = 0; k < ns; ++k) {
                if (hw[k] <= 0.f) continue;
                const double v = hx[(size_t)k * kLmacIn + i];
                s1 += v;
                s2 += v * v;
                c += 1.0;
            }
            const double mu = c > 0 ? s1 / c : 0.0;
            const double var = c > 0 ? std::max(s2 / c - mu * mu, 0.0) : 1.0;
            L.norm.mu[i] = (float)mu;
            L.norm.isd[i] = (float)(1.0 / std::sqrt(std::max(var, 1e-12)));
        }
    }
    {
        std::mt19937 rng((uint32_t)o->seed);
        std::normal_distribution<float> g(0.f, 1.f);
        for (int i = 0; i < kLmacParams; ++i) L.hP[i] = 0.f;
        const float s1 = std::sqrt(2.f / kLmacIn), s2 = std::sqrt(2.f / kLmacHidden), s3 = std::sqrt(1.f / kLmacHidden);
        for (int i = 0; i < kLmacHidden * kLmacIn; ++i) L.hP[kLmacW1 + i] = s1 * g(rng);
        for (int i = 0; i < kLmacHidden * kLmacHidden; ++i) L.hP[kLmacW2 + i] = s2 * g(rng);
        for (int i = 0; i < kLmacHidden; ++i) L.hP[kLmacW3 + i] = s3 * g(rng);
        NG_CUDA(cudaMemcpyAsync(L.dP, L.hP, sizeof(L.hP), cudaMemcpyHostToDevice, ctx->stream));
        NG_CUDA(cudaMemsetAsync(L.dM, 0, sizeof(float) * kLmacParams, ctx->stream));
        NG_CUDA(cudaMemsetAsync(L.dV, 0, sizeof(float) * kLmacParams, ctx->stream));
    }
    // ---- Adam over mini-batches drawn with replacement ----
    const long long steps = std::max<long long>(1, (long long)o->epochs * ntrain / nb);
    double loss_first = -1.0, loss_last = 0.0, acc_last = 0.0;
    for (long long t = 1; t <= steps; ++t) {
        launch_lmac_make_batch(Xtr, Rtr, ntrain, L.norm, nb, (uint32_t)(o->seed * 1000003u + (uint32_t)t),
                               (float)o->u_range, true, L.dXb, L.dyb, L.dwb, ctx->stream);
        ctx->launches += 1;
        // cosine decay of the step size to 5 % of lr
        const double frac = (double)(t - 1) / (double)steps;
        const float lr = (float)(o->lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(3.141592653589793 * frac))));
        const bool report = t == 1 || t == steps;
        double ls = 0.0, cs = 0.0;
        NG_TRY(grad_pass(ctx, L.dP, nb, 1.f / (float)nb, true, lr, (int)t, report ? &ls : nullptr,
                         report ? &cs : nullptr));
        if (t == 1) loss_first = ls / nb;
        if (t == steps) {
            loss_last = ls / nb;
            acc_last = cs / nb;
        }
    }
    // ---- held-out pairs ----
    double vloss = 0.0, vacc = 0.0;
    {
        const int nv = 65536;
        NG_TRY(ensure_batch(ctx, nv));
        launch_lmac_make_batch(Xva, Rva, nval, L.norm, nv, (uint32_t)(o->seed ^ 0x3C6EF372u), (float)o->u_range,
                               true, L.dXb, L.dyb, L.dwb, ctx->stream);
        double ls = 0.0, cs = 0.0;
        NG_TRY(grad_pass(ctx, L.dP, nv, 0.f, false, 0.f, 1, &ls, &cs));
        vloss = ls / nv;
        vacc = cs / nv;
    }
    NG_CUDA(cudaMemcpyAsync(L.hP, L.dP, sizeof(L.hP), cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    NG_TRY(upload_model(ctx));
    L.reverted = false;
    L.evals_since_check = 0;
    const auto t2 = std::chrono::steady_clock::now();
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->pairs = have;
        out->band_pairs = band_total;
        out->loss_first = loss_first;
        out->loss_last = loss_last;
        out->acc_last = acc_last;
        out->val_loss = vloss;
        out->val_acc = vacc;
        out->ms_data = std::chrono::duration<double, std::milli>(t1 - t0).count();
        out->ms_train = std::chrono::duration<double, std::milli>(t2 - t1).count();
    }
    return NGRAV_OK;
}

int ngrav_gpu_lmac_get_model(ngrav_gpu_ctx* ctx, float* params, float* norm) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->lm || !ctx->lm->have_model) return fail(ctx, NGRAV_ERR_INVALID_ARG, "no learned model installed");
    if (params) std::memcpy(params, ctx->lm->hP, sizeof(ctx->lm->hP));
    if (norm) {
        std::memcpy(norm, ctx->lm->norm.mu, sizeof(float) * kLmacIn);
        std::memcpy(norm + kLmacIn, ctx->lm->norm.isd, sizeof(float) * kLmacIn);
    }
    return NGRAV_OK;
}

int ngrav_gpu_lmac_set_model(ngrav_gpu_ctx* ctx, const float* params, const float* norm) {
    if (!ctx || !params || !norm) return NGRAV_ERR_INVALID_ARG;
    for (int i = 0; i < kLmacParams; ++i)
        if (!std::isfinite(params[i])) return fail(ctx, NGRAV_ERR_INVALID_ARG, "non-finite model parameter");
    for (int i = 0; i < 2 * kLmacIn; ++i)
        if (!std::isfinite(norm[i])) return fail(ctx, NGRAV_ERR_INVALID_ARG, "non-finite standardisation");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    NG_TRY(ensure_state(ctx));
    std::memcpy(ctx->lm->hP, params, sizeof(ctx->lm->hP));
    std::memcpy(ctx->lm->norm.mu, norm, sizeof(float) * kLmacIn);
    std::memcpy(ctx->lm->norm.isd, norm + kLmacIn, sizeof(float) * kLmacIn);
    NG_TRY(upload_model(ctx));
    ctx->lm->reverted = false;
    ctx->lm->evals_since_check = 0;
    return NGRAV_OK;
}

int ngrav_gpu_lmac_reset(ngrav_gpu_ctx* ctx) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (ctx->lm) {
        ctx->lm->reverted = false;
        ctx->lm->evals_since_check = 0;
    }
    return NGRAV_OK;
}

int ngrav_gpu_lmac_collect(ngrav_gpu_ctx* ctx, double theta_record, double rho_lo, double rho_hi, double keep,
                           uint64_t seed, int cap, int* npairs, long long* nband, int* group_leaf, int* node,
                           float* features, float* r) {
    if (!ctx || !npairs || cap < 0) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have || !ctx->acc_valid) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no force evaluation to inspect");
    if (!(theta_record > 0.0) || !(rho_hi > rho_lo)) return fail(ctx, NGRAV_ERR_INVALID_ARG, "bad band");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    NG_TRY(ensure_state(ctx));
    LmacState& L = *ctx->lm;
    NG_TRY(ensure_data(ctx, std::max(cap, 1)));
    int kept = 0;
    long long band = 0;
    NG_TRY(collect_pairs(ctx, (float)theta_record, (float)rho_lo, (float)rho_hi, keep, (uint32_t)seed, cap, L.dX,
                         L.dR, &kept, &band));
    *npairs = kept;
    if (nband) *nband = band;
    if (kept > 0) {
        std::vector<int2> pr(kept);
        NG_CUDA(cudaMemcpy(pr.data(), L.dPairs, sizeof(int2) * kept, cudaMemcpyDeviceToHost));
        for (int i = 0; i < kept; ++i) {
            if (group_leaf) group_leaf[i] = pr[i].x;
            if (node) node[i] = pr[i].y;
        }
        if (features) NG_CUDA(cudaMemcpy(features, L.dX, sizeof(float) * kLmacIn * kept, cudaMemcpyDeviceToHost));
        if (r) NG_CUDA(cudaMemcpy(r, L.dR, sizeof(float) * kept, cudaMemcpyDeviceToHost));
    }
    return NGRAV_OK;
}

int ngrav_gpu_lmac_forward(ngrav_gpu_ctx* ctx, const float* x_std, int n, float* z) {
    if (!ctx || n < 0 || (n > 0 && (!x_std || !z))) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->lm || !ctx->lm->have_model) return fail(ctx, NGRAV_ERR_INVALID_ARG, "no learned model installed");
    if (n == 0) return NGRAV_OK;
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    LmacState& L = *ctx->lm;
    NG_TRY(ensure_batch(ctx, n));
    NG_TRY(ensure_z(ctx, n));
    NG_CUDA(cudaMemcpyAsync(L.dXb, x_std, sizeof(float) * kLmacIn * n, cudaMemcpyHostToDevice, ctx->stream));
    launch_lmac_forward(L.dXb, n, L.dP, L.dZ, ctx->stream);
    NG_CUDA(cudaMemcpyAsync(z, L.dZ, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    NG_CUDA(cudaGetLastError());
    return NGRAV_OK;
}

int ngrav_gpu_lmac_forward_tc(ngrav_gpu_ctx* ctx, const float* x_raw, int n, float* z) {
    if (!ctx || n < 0 || (n > 0 && (!x_raw || !z))) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->lm || !ctx->lm->have_model) return fail(ctx, NGRAV_ERR_INVALID_ARG, "no learned model installed");
    if (n == 0) return NGRAV_OK;
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    LmacState& L = *ctx->lm;
    NG_TRY(ensure_batch(ctx, n));
    NG_TRY(ensure_z(ctx, n));
    NG_CUDA(cudaMemcpyAsync(L.dXb, x_raw, sizeof(float) * kLmacIn * n, cudaMemcpyHostToDevice, ctx->stream));
    NG_CUDA(cudaMemsetAsync(L.dStatus, 0, sizeof(unsigned), ctx->stream));
    launch_lmac_tc_forward(L.dModel, L.dXb, n, L.dZ, L.dStatus, ctx->sm_count, ctx->stream);
    unsigned st = 0;
    NG_CUDA(cudaMemcpyAsync(z, L.dZ, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaMemcpyAsync(&st, L.dStatus, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    NG_CUDA(cudaGetLastError());
    if (st & kStTimeout) return fail(ctx, NGRAV_ERR_TIMEOUT, "tensor-core wait ran out");
    return NGRAV_OK;
}

int ngrav_gpu_lmac_grad(ngrav_gpu_ctx* ctx, const float* x_std, const float* y, const float* w, int n,
                        const float* params, double scale, float* grad, double* loss) {
    if (!ctx || n <= 0 || !x_std || !y || !grad) return NGRAV_ERR_INVALID_ARG;
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    NG_TRY(ensure_state(ctx));
    LmacState& L = *ctx->lm;
    if (!params && !L.have_model) return fail(ctx, NGRAV_ERR_INVALID_ARG, "no parameters given or installed");
    NG_TRY(ensure_batch(ctx, n));
    NG_CUDA(cudaMemcpyAsync(L.dXb, x_std, sizeof(float) * kLmacIn * n, cudaMemcpyHostToDevice, ctx->stream));
    NG_CUDA(cudaMemcpyAsync(L.dyb, y, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    if (w) {
        NG_CUDA(cudaMemcpyAsync(L.dwb, w, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    } else {
        std::vector<float> ones(n, 1.f);
        NG_CUDA(cudaMemcpyAsync(L.dwb, ones.data(), sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    // Outside training the first Adam moment buffer holds the caller's parameters.
    const float* P = L.dP;
    if (params) {
        NG_CUDA(cudaMemcpyAsync(L.dM, params, sizeof(float) * kLmacParams, cudaMemcpyHostToDevice, ctx->stream));
        P = L.dM;
    }
    double ls = 0.0;
    NG_TRY(grad_pass(ctx, P, n, (float)scale, false, 0.f, 1, &ls, nullptr));
    NG_CUDA(cudaMemcpyAsync(grad, L.dGrad, sizeof(float) * kLmacParams, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    NG_CUDA(cudaGetLastError());
    if (loss) *loss = ls;
    return NGRAV_OK;
}

}  // extern "C"
