// tune.cu -- the autotuner of include/ngrav_gpu.h: leaf capacity (the target
// group size), P2P batch tile and walk stack depth, picked by timing force
// evaluations of the caller's own state with the device events of the
// evaluation, under an error constraint checked against the direct sum.
#include "ctx_internal.cuh"
#include "ctx_kernels.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

using namespace ngrav_ctx;

namespace {

struct Trial {
    int ncrit, tile, stack;
    double ms, rms;
};

// Mean device time of `reps` evaluations (after one untimed), and the rms
// error of the last when `check`.
int measure(ngrav_gpu_ctx* ctx, int reps, bool check, int targets, Trial& t) {
    NG_TRY(evaluate(ctx, false, false, 0.f));  // warm: sizes buffers for this shape
    double ms = 0.0;
    for (int r = 0; r < reps; ++r) {
        NG_TRY(evaluate(ctx, false, false, 0.f));
        for (int i = 0; i < 6; ++i) ms += ctx->phase_ms[i];
    }
    t.ms = ms / std::max(reps, 1);
    t.rms = -1.0;
    if (check) {
        ngrav_gpu_ferr fe;
        NG_TRY(ngrav_gpu_force_error(ctx, (int)std::min<long long>(targets, ctx->n), 0x7u, 0, &fe));
        t.rms = fe.rms;
    }
    return NGRAV_OK;
}

}  // namespace

extern "C" {

int ngrav_gpu_default_tune_opts(ngrav_gpu_tune_opts* o) {
    if (!o) return NGRAV_ERR_INVALID_ARG;
    std::memset(o, 0, sizeof(*o));
    o->reps = 2;
    o->check_targets = 2048;
    o->rms_tolerance = 1.1;
    const int def[6] = {8, 12, 16, 24, 32, 48};
    for (int i = 0; i < 6; ++i) o->leaf_capacities[i] = def[i];
    return NGRAV_OK;
}

int ngrav_gpu_set_tuning(ngrav_gpu_ctx* ctx, int p2p_tile, int walk_stack) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (!(p2p_tile == 0 || p2p_tile == 64 || p2p_tile == 128 || p2p_tile == 256))
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "p2p_tile must be 0, 64, 128 or 256");
    if (!(walk_stack == 1024 || walk_stack == 2048 || walk_stack == 4096))
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "walk_stack must be 1024, 2048 or 4096");
    ctx->p2p_tile = p2p_tile;
    ctx->walk_stack = walk_stack;
    return NGRAV_OK;
}

int ngrav_gpu_autotune(ngrav_gpu_ctx* ctx, const ngrav_gpu_tune_opts* o, ngrav_gpu_tune_report* out) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    ngrav_gpu_tune_opts d;
    ngrav_gpu_default_tune_opts(&d);
    if (!o) o = &d;
    if (o->reps < 1 || o->check_targets < 1 || !(o->rms_tolerance >= 1.0))
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "tuning options out of range");
    std::vector<int> caps;
    for (int i = 0; i < 8 && o->leaf_capacities[i] > 0; ++i) caps.push_back(o->leaf_capacities[i]);
    if (caps.empty()) caps.assign(d.leaf_capacities, d.leaf_capacities + 6);
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const bool events0 = ctx->events;
    ctx->events = true;
    const ngrav_gpu_opts opts0 = ctx->opts;
    std::vector<Trial> tried;
    auto run = [&](int ncrit, int tile, int stack, bool check, Trial& t) -> int {
        ctx->opts.leaf_capacity = ncrit;
        ctx->p2p_tile = tile;
        ctx->walk_stack = stack;
        t = {ncrit, tile, stack, 0.0, -1.0};
        const int rc = measure(ctx, o->reps, check, o->check_targets, t);
        if (rc == NGRAV_OK) tried.push_back(t);
        return rc;
    };
    int rc = NGRAV_OK;
    Trial base{}, best{};
    // 1. the starting configuration sets the error bar
    rc = run(opts0.leaf_capacity, ctx->p2p_tile, ctx->walk_stack, true, base);
    best = base;
    const double rms_cap = base.rms * o->rms_tolerance;
    // 2. leaf capacity (target-group size), at the starting tile and stack
    for (size_t i = 0; rc == NGRAV_OK && i < caps.size(); ++i) {
        if (caps[i] == opts0.leaf_capacity) continue;
        Trial t;
        rc = run(caps[i], base.tile, base.stack, true, t);
        if (rc == NGRAV_OK && t.rms <= rms_cap && t.ms < best.ms) best = t;
    }
    // 3. P2P tile and 4. walk stack at the chosen capacity (same interactions)
    const int tiles[3] = {64, 128, 256}, stacks[3] = {1024, 2048, 4096};
    for (int i = 0; rc == NGRAV_OK && i < 3; ++i) {
        if (tiles[i] == (best.tile ? best.tile : 256)) continue;
        Trial t;
        rc = run(best.ncrit, tiles[i], best.stack, false, t);
        if (rc == NGRAV_OK && t.ms < best.ms) best = {best.ncrit, tiles[i], best.stack, t.ms, best.rms};
    }
    for (int i = 0; rc == NGRAV_OK && i < 3; ++i) {
        if (stacks[i] == best.stack) continue;
        Trial t;
        rc = run(best.ncrit, best.tile, stacks[i], false, t);
        if (rc == NGRAV_OK && t.ms < best.ms) best = {best.ncrit, best.tile, stacks[i], t.ms, best.rms};
    }
    // install the choice (or restore the start on failure)
    ctx->opts.leaf_capacity = rc == NGRAV_OK ? best.ncrit : opts0.leaf_capacity;
    ctx->p2p_tile = rc == NGRAV_OK ? best.tile : base.tile;
    ctx->walk_stack = rc == NGRAV_OK ? best.stack : base.stack;
    ctx->events = events0;
    ctx->primed = false;
    if (rc) return rc;
    Trial fin;
    ctx->events = true;
    rc = measure(ctx, o->reps, true, o->check_targets, fin);
    ctx->events = events0;
    if (rc) return rc;
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->leaf_capacity = best.ncrit;
        out->p2p_tile = best.tile ? best.tile : 256;
        out->walk_stack = best.stack;
        out->ms_before = base.ms;
        out->ms_after = fin.ms;
        out->rms_before = base.rms;
        out->rms_after = fin.rms;
        out->ntried = (int)std::min<size_t>(tried.size(), 32);
        for (int i = 0; i < out->ntried; ++i) {
            const Trial& t = tried[i];
            out->tried[i][0] = t.ncrit;
            out->tried[i][1] = t.tile ? t.tile : 256;
            out->tried[i][2] = t.stack;
            out->tried[i][3] = t.ms;
            out->tried[i][4] = t.rms;
        }
    }
    return NGRAV_OK;
}

}  // extern "C"
