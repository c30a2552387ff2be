// ctx.cu -- the C-ABI (include/ngrav_gpu.h): context, buffers, and the
// host-side orchestration of one force evaluation / KDK step.
//
// One force evaluation enqueues, on the context's stream:
//   reset counters -> bounding box + root cube -> 63-bit keys -> radix sort
//   (7 passes of 9-bit digits) -> gather the state into key order -> tree
//   levels 0..20 -> leaf list -> upward moments -> grouped walk (+ closing
//   kick)
// then synchronises once and reads the device status word.  A node-pool or
// walk-stack overflow is reported by the kernels (never silently dropped, as
// the reference's GL path does at GpuBarnesHut.cpp:259-260 and :428), the
// walk refuses to run on a truncated tree, and the host grows the pool and
// re-runs the evaluation.
#include "ngrav_gpu.h"

#include "ctx_internal.cuh"
#include "ctx_kernels.cuh"
#include "engine.cuh"
#include "softening.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <unordered_set>
#include <vector>

using namespace ngrav;
namespace ngrav_ctx {

int fail(ngrav_gpu_ctx* ctx, int code, const std::string& msg) {
    ctx->err = msg;
    return code;
}

int check_opts(ngrav_gpu_ctx* ctx, const ngrav_gpu_opts* o) {
    if (!o) return fail(ctx, NGRAV_ERR_INVALID_ARG, "opts is NULL");
    if (o->abi_version != NGRAV_GPU_ABI_VERSION) return fail(ctx, NGRAV_ERR_INVALID_ARG, "abi_version mismatch");
    if (o->leaf_capacity < 1 || o->leaf_capacity > (1 << 20))
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "leaf_capacity out of range");
    if (o->max_depth < 0) return fail(ctx, NGRAV_ERR_INVALID_ARG, "max_depth < 0");
    if (!(o->theta >= 0.0) || !(o->eps >= 0.0) || !std::isfinite(o->G))
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "theta/eps/G invalid");
    if (o->precision != NGRAV_PRECISION_PLAIN && o->precision != NGRAV_PRECISION_SPLIT)
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "unknown precision");
    if (o->mac != NGRAV_MAC_GEOMETRIC && o->mac != NGRAV_MAC_LEARNED && o->mac != NGRAV_MAC_RELATIVE)
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "unknown mac");
    return NGRAV_OK;
}

bool split_of(const ngrav_gpu_ctx* ctx) { return ctx->opts.precision == NGRAV_PRECISION_SPLIT; }

void free_particles(ngrav_gpu_ctx* ctx) {
    Particles& P = ctx->P;
    dfree(P.pos); dfree(P.plo); dfree(P.vel); dfree(P.vlo); dfree(P.acc); dfree(P.src); dfree(P.id);
    dfree(P.pos2); dfree(P.plo2); dfree(P.vel2); dfree(P.vlo2); dfree(P.acc2); dfree(P.id2);
    P.cap = 0;
    SortBuffers& S = ctx->SB;
    dfree(S.keys); dfree(S.keys_alt); dfree(S.vals); dfree(S.vals_alt); dfree(S.hist); dfree(S.scan_tmp);
    dfree(S.ktab);
    S.cap = 0;
    dfree(ctx->leaf_at); dfree(ctx->flags); dfree(ctx->scanbuf); dfree(ctx->leaf_list);
    dfree(ctx->stage); dfree(ctx->inv);
    ctx->cap_n = 0;
}

void free_nodes(ngrav_gpu_ctx* ctx) {
    NodeArrays& T = ctx->T;
    dfree(T.start); dfree(T.count); dfree(T.first_child); dfree(T.parent); dfree(T.visit);
    dfree(T.nchild); dfree(T.level); dfree(T.cx); dfree(T.cy); dfree(T.cz); dfree(T.half); dfree(T.sysroot);
    dfree(T.mass); dfree(T.comx); dfree(T.comy); dfree(T.comz); dfree(T.maxr); dfree(T.quad); dfree(T.amin);
    dfree(T.wA); dfree(T.wB); dfree(T.wC); dfree(T.wD); dfree(T.chi); dfree(T.clo);
    T.cap = 0;
}

int alloc_particles(ngrav_gpu_ctx* ctx, long long n) {
    if (n <= ctx->cap_n) return NGRAV_OK;
    free_particles(ctx);
    const long long c = n;
    Particles& P = ctx->P;
    NG_CUDA(dalloc(P.pos, c)); NG_CUDA(dalloc(P.plo, c)); NG_CUDA(dalloc(P.vel, c)); NG_CUDA(dalloc(P.acc, c));
    NG_CUDA(dalloc(P.vlo, c)); NG_CUDA(dalloc(P.vlo2, c));
    NG_CUDA(dalloc(P.src, c)); NG_CUDA(dalloc(P.id, c));
    NG_CUDA(dalloc(P.pos2, c)); NG_CUDA(dalloc(P.plo2, c)); NG_CUDA(dalloc(P.vel2, c)); NG_CUDA(dalloc(P.acc2, c));
    NG_CUDA(dalloc(P.id2, c));
    P.cap = c;
    SortBuffers& S = ctx->SB;
    NG_CUDA(dalloc(S.keys, c)); NG_CUDA(dalloc(S.keys_alt, c)); NG_CUDA(dalloc(S.vals, c));
    NG_CUDA(dalloc(S.vals_alt, c));
    S.hist_cap = radix_hist_size(c);
    NG_CUDA(dalloc(S.hist, S.hist_cap));
    S.scan_tmp_cap = scan_tmp_size(std::max(S.hist_cap, c)) + 16;
    NG_CUDA(dalloc(S.scan_tmp, S.scan_tmp_cap));
    NG_CUDA(dalloc(S.ktab, key_table_entries()));
    S.cap = c;
    NG_CUDA(dalloc(ctx->leaf_at, c)); NG_CUDA(dalloc(ctx->flags, c)); NG_CUDA(dalloc(ctx->scanbuf, c));
    NG_CUDA(dalloc(ctx->leaf_list, c)); NG_CUDA(dalloc(ctx->inv, c));
    NG_CUDA(dalloc(ctx->stage, 7 * c));
    ctx->cap_n = c;
    return NGRAV_OK;
}

int alloc_nodes(ngrav_gpu_ctx* ctx, int cap) {
    free_nodes(ctx);
    NodeArrays& T = ctx->T;
    NG_CUDA(dalloc(T.start, cap)); NG_CUDA(dalloc(T.count, cap)); NG_CUDA(dalloc(T.first_child, cap));
    NG_CUDA(dalloc(T.parent, cap)); NG_CUDA(dalloc(T.visit, cap)); NG_CUDA(dalloc(T.nchild, cap));
    NG_CUDA(dalloc(T.level, cap)); NG_CUDA(dalloc(T.cx, cap)); NG_CUDA(dalloc(T.cy, cap)); NG_CUDA(dalloc(T.cz, cap));
    NG_CUDA(dalloc(T.half, cap)); NG_CUDA(dalloc(T.sysroot, cap));
    NG_CUDA(dalloc(T.mass, cap)); NG_CUDA(dalloc(T.comx, cap)); NG_CUDA(dalloc(T.comy, cap));
    NG_CUDA(dalloc(T.comz, cap)); NG_CUDA(dalloc(T.maxr, cap)); NG_CUDA(dalloc(T.quad, 5LL * cap));
    NG_CUDA(dalloc(T.amin, cap));
    NG_CUDA(dalloc(T.wA, cap)); NG_CUDA(dalloc(T.wB, cap)); NG_CUDA(dalloc(T.wC, cap)); NG_CUDA(dalloc(T.wD, cap));
    NG_CUDA(dalloc(T.chi, cap)); NG_CUDA(dalloc(T.clo, cap));
    T.cap = cap;
    return NGRAV_OK;
}

int initial_node_cap(long long n, int leaf_cap) {
    long long c = 5 * n / std::max(1, leaf_cap) + 1024;
    c = std::min<long long>(c, 4 * n + 1024);
    return (int)std::min<long long>(c, 0x7FFFFFF0LL);
}

int alloc_stack(ngrav_gpu_ctx* ctx, int stack_cap) {
    dfree(ctx->LB.stack);
    NG_CUDA(dalloc(ctx->LB.stack, (long long)ctx->LB.nwarps * stack_cap));
    ctx->LB.stack_cap = stack_cap;
    return NGRAV_OK;
}

// Grow the chunk pools of the interaction lists (chunks of kListChunk ids).
int alloc_lists(ngrav_gpu_ctx* ctx, long long far_chunks, long long near_chunks) {
    ListBuffers& L = ctx->LB;
    far_chunks = std::min<long long>(far_chunks, 0x7FFFFFF0LL);
    near_chunks = std::min<long long>(near_chunks, 0x7FFFFFF0LL);
    if (far_chunks > L.far_chunk_cap) {
        dfree(L.far);
        dfree(L.far_next);
        NG_CUDA(dalloc(L.far, far_chunks * kListChunk));
        NG_CUDA(dalloc(L.far_next, far_chunks));
        L.far_chunk_cap = (int)far_chunks;
    }
    if (near_chunks > L.near_chunk_cap) {
        dfree(L.near);
        dfree(L.near_next);
        NG_CUDA(dalloc(L.near, near_chunks * kListChunk));
        NG_CUDA(dalloc(L.near_next, near_chunks));
        L.near_chunk_cap = (int)near_chunks;
    }
    return NGRAV_OK;
}

int alloc_group_info(ngrav_gpu_ctx* ctx, long long n) {
    dfree(ctx->LB.ginfo);
    NG_CUDA(dalloc(ctx->LB.ginfo, std::max<long long>(n, 1)));
    return NGRAV_OK;
}

WalkParams walk_params(const ngrav_gpu_ctx* ctx, bool kick, float hdt) {
    WalkParams wp{};
    const ngrav_gpu_opts& o = ctx->opts;
    wp.eps2 = (float)(o.eps * o.eps);
    wp.eps2_d = o.eps * o.eps;
    wp.theta = (float)o.theta;
    wp.theta2 = (float)(o.theta * o.theta);
    wp.theta2_d = o.theta * o.theta;
    wp.G = (float)o.G;
    wp.quadrupole = o.quadrupole ? 1 : 0;
    wp.split = split_of(ctx) ? 1 : 0;
    wp.retest = o.fp64_mac_retest ? 1 : 0;
    wp.kick = kick ? 1 : 0;
    wp.hdt = hdt;
    wp.stack_cap = ctx->LB.stack_cap;
    wp.node_limit = ctx->T.cap + 32;
    wp.global_stack = ctx->walk_global_stack ? 1 : 0;
    wp.smem_stack = ctx->walk_stack;
    wp.soft = ctx->soft;
    wp.ih = ctx->opts.eps > 0.0 ? (float)(1.0 / ctx->opts.eps) : 0.f;
    wp.p2p_tile = ctx->p2p_tile;
    return wp;
}

void rec(ngrav_gpu_ctx* ctx, int i) {
    if (!ctx->events) return;
    if (ctx->capturing)  // a timing node of the captured graph
        cudaEventRecordWithFlags(ctx->ev[i], ctx->stream, cudaEventRecordExternal);
    else
        cudaEventRecord(ctx->ev[i], ctx->stream);
}

// Enqueue one force evaluation. bbox_ready: the counters were reset and the
// bounding box accumulated by the preceding kick-drift.
void enqueue_eval(ngrav_gpu_ctx* ctx, bool bbox_ready, bool kick, float hdt) {
    cudaStream_t s = ctx->stream;
    const long long n = ctx->n;
    const bool split = split_of(ctx);
    Particles& P = ctx->P;
    rec(ctx, 0);
    if (!bbox_ready) {
        launch_reset_counters(ctx->C, s);
        launch_bbox(P.pos, split ? P.plo : nullptr, n, ctx->C, s);
        ctx->launches += 2;
    }
    launch_root(ctx->C, n, s);
    if (ctx->F.nsys > 1) {  // ensemble: every system's own root cube
        launch_forest_bbox(P.pos, split ? P.plo : nullptr, n, ctx->F, ctx->C, s);
        launch_forest_root(ctx->F, s);
        ctx->launches += 2;
    }
    ctx->launches += launch_keys(P.pos, split ? P.plo : nullptr, n, ctx->C, ctx->F, ctx->SB.ktab, ctx->SB.keys,
                                 ctx->SB.vals, s) - 1;
    rec(ctx, 1);
    // The keys are sorted on their top `levels` digits only (whole 9-bit
    // passes, so at least that many levels), as deep as the tree went at the
    // last evaluation plus a level; a node at the deepest sorted level that
    // would still split stops the build (kStSortDepth) and the evaluation
    // is redone on the full key.
    const int levels = ctx->F.nsys > 1 ? kKeyLevels : ctx->sort_levels;
    const int passes = std::min(kRsPasses, (3 * levels + kRsDigitBits - 1) / kRsDigitBits);
    radix_sort_pairs(ctx->SB, n, passes, 3 * kKeyLevels - kRsDigitBits * passes, s);
    ctx->sort_passes = passes;
    launch_permute(P, ctx->SB.vals, n, split, s);
    // root, keys, 3 per sort pass (histogram, digit scans, scatter), permute,
    // tree init, the levels, leaf list (mark, 3 scan kernels, compact), leaf
    // moments, the internal-moment levels, walk
    ctx->launches += 2 + (n > 1 ? 3 * passes : 0) + 1 + 1 + levels + 5 + 1 + levels + 1;
    std::swap(P.pos, P.pos2);
    std::swap(P.plo, P.plo2);
    std::swap(P.vel, P.vel2);
    std::swap(P.vlo, P.vlo2);
    std::swap(P.acc, P.acc2);
    std::swap(P.id, P.id2);
    rec(ctx, 2);
    launch_tree_init(ctx->T, ctx->C, n, ctx->opts.leaf_capacity, ctx->opts.max_depth, s);
    launch_tree_levels(ctx->T, ctx->C, ctx->SB.keys, n, ctx->opts.leaf_capacity, ctx->opts.max_depth, ctx->F, levels,
                       s);
    launch_leaf_list(ctx->T, ctx->C, n, ctx->leaf_at, ctx->flags, ctx->scanbuf, ctx->leaf_list, ctx->SB, s);
    rec(ctx, 3);
    launch_moments(ctx->T, ctx->C, P, ctx->leaf_list, n, (int)std::min<long long>(n, ctx->T.cap), split,
                   ctx->opts.quadrupole != 0, levels, s);
    rec(ctx, 4);
    WalkParams wp = walk_params(ctx, kick, hdt);
    const void* model = nullptr;
    if (ctx->block_on || ctx->opts.mac == NGRAV_MAC_RELATIVE) {
        // per-particle walk: decisions, sums and the closing kick in one
        // kernel; block timesteps take the geometric test on their targets
        // (ComputeAccelBarnesHutTargets, Solvers.cpp:384-405)
        rec(ctx, 5);
        launch_walk_pp(ctx->T, ctx->C, P, ctx->leaf_list, wp, ctx->block_on ? 0 : 1, ctx->alpha, nullptr,
                       ctx->block_on ? ctx->block_args : nullptr, ctx->block_base, ctx->LB.nwarps, s);
        rec(ctx, 6);
        ctx->launches += 1;
        return;
    }
    if (lmac_walk_setup(ctx, wp, &model))
        lmac_launch_walk(ctx, wp, model);
    else
        launch_walk(ctx->T, ctx->C, ctx->leaf_list, wp, ctx->LB, s);
    rec(ctx, 5);
    launch_eval(ctx->T, ctx->C, P, ctx->leaf_list, wp, ctx->LB, ctx->eval_nwarps, s);
    rec(ctx, 6);
    ctx->launches += 1;  // the evaluation kernel
}

int finish_eval(ngrav_gpu_ctx* ctx, bool& retry) {
    retry = false;
    NG_CUDA(cudaMemcpyAsync(&ctx->hc, ctx->C, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    NG_CUDA(cudaGetLastError());
    const unsigned st = ctx->hc.status;
    if (st & kStNonFinite) return fail(ctx, NGRAV_ERR_NONFINITE, "non-finite position or mass");
    if (st & kStTimeout) return fail(ctx, NGRAV_ERR_TIMEOUT, "a bounded device wait ran out");
    if (st & kStNodeOverflow) {
        const long long want = std::min<long long>((long long)ctx->T.cap * 2, 0x7FFFFFF0LL);
        if (want <= ctx->T.cap) return fail(ctx, NGRAV_ERR_CAPACITY, "node pool exhausted");
        NG_TRY(alloc_nodes(ctx, (int)want));
        retry = true;
        return NGRAV_OK;
    }
    if (st & kStSortDepth) {
        ctx->sort_levels = kKeyLevels;  // the tree went deeper than the sorted digits
        retry = true;
        return NGRAV_OK;
    }
    if (st & kStCorrupt) return fail(ctx, NGRAV_ERR_CAPACITY, "walk visit limit breached (inconsistent tree)");
    if (st & kStPendOverflow) {
        NG_TRY(lmac_grow_pools(ctx));
        retry = true;
        return NGRAV_OK;
    }
    if (st & kStStackOverflow) {
        if (!ctx->walk_global_stack) {
            ctx->walk_global_stack = true;  // the shared-memory stack was too small for this tree
        } else {
            if (ctx->LB.stack_cap >= (1 << 22)) return fail(ctx, NGRAV_ERR_CAPACITY, "walk stack exhausted");
            NG_TRY(alloc_stack(ctx, ctx->LB.stack_cap * 2));
        }
        retry = true;
        return NGRAV_OK;
    }
    if (st & kStListOverflow) {
        // The walk kept counting chunks past the pool: size the pools to that
        // (plus headroom) and run again.
        const long long fc = (long long)(unsigned)ctx->hc.far_chunks, nc = (long long)(unsigned)ctx->hc.near_chunks;
        if (fc >= 0x7FFFFFF0LL || nc >= 0x7FFFFFF0LL) return fail(ctx, NGRAV_ERR_CAPACITY, "list pool exhausted");
        NG_TRY(alloc_lists(ctx, fc + fc / 4 + 1024, nc + nc / 4 + 1024));
        retry = true;
        return NGRAV_OK;
    }
    // Keep headroom in the list pools for the next evaluation.
    {
        const long long fc = ctx->hc.far_chunks, nc = ctx->hc.near_chunks;
        if (fc > ctx->LB.far_chunk_cap - ctx->LB.far_chunk_cap / 8 ||
            nc > ctx->LB.near_chunk_cap - ctx->LB.near_chunk_cap / 8)
            NG_TRY(alloc_lists(ctx, std::max<long long>(ctx->LB.far_chunk_cap, fc + fc / 4),
                               std::max<long long>(ctx->LB.near_chunk_cap, nc + nc / 4)));
    }
    if (ctx->opts.strict_depth && ctx->hc.depth_limited > 0)
        return fail(ctx, NGRAV_ERR_DEPTH, "a leaf needs more than 21 key levels");
    if (ctx->events) {
        float ms;
        for (int i = 0; i < 6; ++i) {
            cudaEventElapsedTime(&ms, ctx->ev[i], ctx->ev[i + 1]);
            ctx->phase_ms[i] = ms;
        }
        ctx->cum_ms_walk += ctx->phase_ms[4];
        ctx->cum_ms_force += ctx->phase_ms[5];
        ctx->cum_ms_eval += ctx->phase_ms[0] + ctx->phase_ms[1] + ctx->phase_ms[2] + ctx->phase_ms[3] +
                            ctx->phase_ms[4] + ctx->phase_ms[5];
    }
    {
        // sort and build one level deeper than this tree next time; shrink only
        // when the tree is two levels shallower, so a depth that wavers by one
        // level does not re-capture the step graph
        const int want = std::min(kKeyLevels, std::max(1, ctx->hc.levels_used + 1));
        if (want > ctx->sort_levels || want + 1 < ctx->sort_levels) ctx->sort_levels = want + (want < ctx->sort_levels);
    }
    ctx->force_evals += 1;
    ctx->cum_particle_evals += ctx->block_on ? (long long)ctx->hc.targets : ctx->n;
    ctx->acc_valid = true;
    ctx->cum_evals += 1;
    ctx->cum_pairs += (long long)ctx->hc.p2p_pairs;
    ctx->cum_p2c += (long long)ctx->hc.p2c_terms;
    return NGRAV_OK;
}

int evaluate(ngrav_gpu_ctx* ctx, bool bbox_ready, bool kick, float hdt) {
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    for (int attempt = 0; attempt < 8; ++attempt) {
        lmac_prepare(ctx);
        enqueue_eval(ctx, bbox_ready, kick, hdt);
        bool retry = false;
        NG_TRY(finish_eval(ctx, retry));
        if (!retry) return lmac_after_eval(ctx);
        bbox_ready = false;
    }
    return fail(ctx, NGRAV_ERR_CAPACITY, "capacity growth did not converge");
}

int ensure_samp(ngrav_gpu_ctx* ctx, int ns) {
    if (ns <= ctx->samp_cap) return NGRAV_OK;
    dfree(ctx->dtargets);
    dfree(ctx->dslots);
    dfree(ctx->dsamp);
    NG_CUDA(dalloc(ctx->dtargets, ns));
    NG_CUDA(dalloc(ctx->dslots, ns));
    NG_CUDA(dalloc(ctx->dsamp, 3LL * ns));
    ctx->samp_cap = ns;
    return NGRAV_OK;
}

int ensure_partial(ngrav_gpu_ctx* ctx, long long count) {
    if (count <= ctx->dpartial_cap) return NGRAV_OK;
    dfree(ctx->dpartial);
    NG_CUDA(dalloc(ctx->dpartial, count));
    ctx->dpartial_cap = count;
    return NGRAV_OK;
}

template <typename T>
int set_particles_impl(ngrav_gpu_ctx* ctx, int64_t n, const T* x, const T* y, const T* z, const T* vx, const T* vy,
                       const T* vz, const T* m, bool f64) {
    if (n < 0 || n > 0x7FFFFFF0LL) return fail(ctx, NGRAV_ERR_INVALID_ARG, "n out of range");
    if (n > 0 && (!x || !y || !z || !m)) return fail(ctx, NGRAV_ERR_INVALID_ARG, "NULL position/mass array");
    ctx->sort_levels = kKeyLevels;  // a new particle set: sort and build on the full key once
    const bool have_v = vx && vy && vz;
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    NG_TRY(alloc_particles(ctx, std::max<int64_t>(n, 1)));
    if (ctx->T.cap < initial_node_cap(n, ctx->opts.leaf_capacity))
        NG_TRY(alloc_nodes(ctx, initial_node_cap(n, ctx->opts.leaf_capacity)));
    if (ctx->cap_n > 0 && (ctx->LB.ginfo == nullptr || n > ctx->gi_cap)) {
        NG_TRY(alloc_group_info(ctx, ctx->cap_n));
        ctx->gi_cap = ctx->cap_n;
    }
    // Initial pools: a few chunks per leaf group; the first evaluation sizes them.
    {
        const long long groups = std::max<long long>(n, 1) / std::max(1, ctx->opts.leaf_capacity / 2) + 1;
        NG_TRY(alloc_lists(ctx, 4 * groups + 1024, 2 * groups + 1024));
    }
    ctx->n = n;
    if (n > 0) {
        T* st = reinterpret_cast<T*>(ctx->stage);
        const size_t b = sizeof(T) * (size_t)n;
        const T* srcs[7] = {x, y, z, vx, vy, vz, m};
        for (int k = 0; k < 7; ++k) {
            if (!srcs[k]) continue;
            NG_CUDA(cudaMemcpyAsync(st + (size_t)k * n, srcs[k], b, cudaMemcpyHostToDevice, ctx->stream));
        }
        const T* dv[3] = {have_v ? st + 3 * (size_t)n : nullptr, have_v ? st + 4 * (size_t)n : nullptr,
                          have_v ? st + 5 * (size_t)n : nullptr};
        if (f64)
            launch_upload_f64(n, (const double*)st, (const double*)(st + n), (const double*)(st + 2 * n),
                              (const double*)dv[0], (const double*)dv[1], (const double*)dv[2],
                              (const double*)(st + 6 * n), ctx->P, split_of(ctx), ctx->stream);
        else
            launch_upload_f32(n, (const float*)st, (const float*)(st + n), (const float*)(st + 2 * n),
                              (const float*)dv[0], (const float*)dv[1], (const float*)dv[2],
                              (const float*)(st + 6 * n), ctx->P, split_of(ctx), ctx->stream);
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        NG_CUDA(cudaGetLastError());
    }
    ctx->have = n > 0;
    ctx->primed = false;
    ctx->acc_valid = false;
    free_forest(ctx);  // a new particle set is one system until set_ensemble
    return NGRAV_OK;
}

// Everything the launches of one KDK step bake in: buffers, sizes,
// parameters, the walk variant.  Equal keys replay the same graph.
std::vector<unsigned char> step_key(const ngrav_gpu_ctx* ctx, float hdt, float fdt) {
    std::vector<unsigned char> k;
    k.reserve(1024);
    auto put = [&](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        k.insert(k.end(), b, b + n);
    };
    put(&ctx->P, sizeof(ctx->P));
    put(&ctx->T, sizeof(ctx->T));
    put(&ctx->SB, sizeof(ctx->SB));
    put(&ctx->LB, sizeof(ctx->LB));
    put(&ctx->C, sizeof(ctx->C));
    put(&ctx->leaf_at, sizeof(ctx->leaf_at));
    put(&ctx->flags, sizeof(ctx->flags));
    put(&ctx->scanbuf, sizeof(ctx->scanbuf));
    put(&ctx->leaf_list, sizeof(ctx->leaf_list));
    put(&ctx->n, sizeof(ctx->n));
    put(&ctx->opts, sizeof(ctx->opts));
    put(&ctx->walk_global_stack, sizeof(ctx->walk_global_stack));
    put(&ctx->eval_nwarps, sizeof(ctx->eval_nwarps));
    put(&ctx->F, sizeof(ctx->F));
    put(&ctx->walk_stack, sizeof(ctx->walk_stack));
    put(&ctx->soft, sizeof(ctx->soft));
    put(&ctx->alpha, sizeof(ctx->alpha));
    put(&ctx->p2p_tile, sizeof(ctx->p2p_tile));
    put(&ctx->sort_levels, sizeof(ctx->sort_levels));
    put(&ctx->events, sizeof(ctx->events));
    put(&hdt, sizeof(hdt));
    put(&fdt, sizeof(fdt));
    lmac_key(ctx, k);
    return k;
}

void drop_graphs(ngrav_gpu_ctx* ctx) {
    for (auto& g : ctx->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        g.key.clear();
    }
}

// Enqueue one KDK step (kick-drift + evaluation with the closing kick) as a
// graph launch: replayed when a graph with the same key exists, else
// captured first.  Returns false (nothing enqueued) if capture failed; the
// caller then launches directly.
bool enqueue_step_graph(ngrav_gpu_ctx* ctx, float hdt, float fdt) {
    lmac_prepare(ctx);
    std::vector<unsigned char> key = step_key(ctx, hdt, fdt);
    for (auto& g : ctx->graphs) {
        if (g.exec && g.key == key) {
            if (cudaGraphLaunch(g.exec, ctx->stream) != cudaSuccess) return false;
            // the host side of the step the graph replays
            const void* model = nullptr;
            WalkParams wp = walk_params(ctx, true, hdt);
            lmac_walk_setup(ctx, wp, &model);
            std::swap(ctx->P.pos, ctx->P.pos2);
            std::swap(ctx->P.plo, ctx->P.plo2);
            std::swap(ctx->P.vel, ctx->P.vel2);
            std::swap(ctx->P.vlo, ctx->P.vlo2);
            std::swap(ctx->P.acc, ctx->P.acc2);
            std::swap(ctx->P.id, ctx->P.id2);
            ctx->launches += g.launches;
            ctx->graph_replays += 1;
            return true;
        }
    }
    Particles saved = ctx->P;
    const long long launches0 = ctx->launches;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
    ctx->capturing = true;
    launch_reset_counters(ctx->C, ctx->stream);
    launch_kick_drift(ctx->P, ctx->n, hdt, fdt, split_of(ctx), ctx->C, ctx->stream);
    ctx->launches += 2;
    enqueue_eval(ctx, true, true, hdt);
    ctx->capturing = false;
    const cudaError_t e1 = cudaStreamEndCapture(ctx->stream, &graph);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t e2 = (e1 == cudaSuccess) ? cudaGraphInstantiate(&exec, graph, 0) : e1;
    if (graph) cudaGraphDestroy(graph);
    if (e2 != cudaSuccess || cudaGraphLaunch(exec, ctx->stream) != cudaSuccess) {
        if (exec) cudaGraphExecDestroy(exec);
        cudaGetLastError();
        ctx->P = saved;  // nothing ran: undo the host side of the captured step
        ctx->launches = launches0;
        ctx->use_graphs = false;
        return false;
    }
    auto& slot = ctx->graphs[ctx->graph_next];
    ctx->graph_next ^= 1;
    if (slot.exec) cudaGraphExecDestroy(slot.exec);
    slot.exec = exec;
    slot.key = std::move(key);
    slot.launches = ctx->launches - launches0;
    ctx->graph_captures += 1;
    return true;
}

template <typename T>
int set_state_impl(ngrav_gpu_ctx* ctx, const T* x, const T* y, const T* z, const T* vx, const T* vy, const T* vz,
                   bool f64) {
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    if (!x || !y || !z) return fail(ctx, NGRAV_ERR_INVALID_ARG, "NULL position array");
    const bool have_v = vx && vy && vz;
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const long long n = ctx->n;
    T* st = reinterpret_cast<T*>(ctx->stage);
    const size_t b = sizeof(T) * (size_t)n;
    const T* srcs[6] = {x, y, z, vx, vy, vz};
    for (int k = 0; k < (have_v ? 6 : 3); ++k)
        NG_CUDA(cudaMemcpyAsync(st + (size_t)k * n, srcs[k], b, cudaMemcpyHostToDevice, ctx->stream));
    const T* v[3] = {have_v ? st + 3 * (size_t)n : nullptr, have_v ? st + 4 * (size_t)n : nullptr,
                     have_v ? st + 5 * (size_t)n : nullptr};
    if (f64)
        launch_state_f64(n, (const double*)st, (const double*)(st + n), (const double*)(st + 2 * n),
                         (const double*)v[0], (const double*)v[1], (const double*)v[2], ctx->P, split_of(ctx),
                         ctx->stream);
    else
        launch_state_f32(n, (const float*)st, (const float*)(st + n), (const float*)(st + 2 * n), (const float*)v[0],
                         (const float*)v[1], (const float*)v[2], ctx->P, split_of(ctx), ctx->stream);
    ctx->launches += 1;
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    NG_CUDA(cudaGetLastError());
    return NGRAV_OK;
}

}  // namespace ngrav_ctx

using namespace ngrav_ctx;

extern "C" {

int ngrav_gpu_default_opts(ngrav_gpu_opts* o) {
    if (!o) return NGRAV_ERR_INVALID_ARG;
    std::memset(o, 0, sizeof(*o));
    o->abi_version = NGRAV_GPU_ABI_VERSION;
    o->device = 0;
    o->leaf_capacity = 8;
    o->max_depth = 40;
    o->quadrupole = 1;
    o->mac = NGRAV_MAC_GEOMETRIC;
    o->precision = NGRAV_PRECISION_SPLIT;
    o->fp64_mac_retest = 1;
    o->strict_depth = 0;
    o->timing = 0;
    o->G = 1.0;
    o->eps = 0.05;
    o->theta = 0.5;
    return NGRAV_OK;
}

int ngrav_gpu_create(ngrav_gpu_ctx** out, const ngrav_gpu_opts* opts) {
    if (!out) return NGRAV_ERR_INVALID_ARG;
    *out = nullptr;
    ngrav_gpu_ctx* ctx = new (std::nothrow) ngrav_gpu_ctx();
    if (!ctx) return NGRAV_ERR_OOM;
    int rc = check_opts(ctx, opts);
    if (rc) {
        delete ctx;
        return rc;
    }
    ctx->opts = *opts;
    auto init = [&]() -> int {
        NG_CUDA(cudaSetDevice(ctx->opts.device));
        NG_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->opts.device));
        NG_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        NG_CUDA(cudaMalloc((void**)&ctx->C, sizeof(Counters)));
        eval_set_attributes();
        lmac_set_attributes();
        NG_CUDA(cudaGetLastError());
        // Walk: up to 32 resident warps per SM (latency-bound traversal);
        // evaluation: every warp the occupancy calculator allows.
        ctx->LB.nwarps = ctx->sm_count * std::min(walk_blocks_per_sm(), 32 / walk_warps_per_block()) *
                         walk_warps_per_block();
        ctx->eval_nwarps = ctx->sm_count * eval_blocks_per_sm() * eval_warps_per_block();
        NG_TRY(alloc_stack(ctx, 4096));
        for (int i = 0; i < 8; ++i) NG_CUDA(cudaEventCreate(&ctx->ev[i]));
        for (int i = 0; i < 2; ++i) NG_CUDA(cudaEventCreate(&ctx->sev[i]));
        ctx->events = ctx->opts.timing != 0;
        return NGRAV_OK;
    };
    rc = init();
    if (rc) {
        // keep the message reachable only through the return code
        ngrav_gpu_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return NGRAV_OK;
}

void ngrav_gpu_destroy(ngrav_gpu_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->opts.device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    drop_graphs(ctx);
    lmac_destroy(ctx);
    free_forest(ctx);
    free_particles(ctx);
    free_nodes(ctx);
    dfree(ctx->C);
    dfree(ctx->LB.stack);
    dfree(ctx->LB.far);
    dfree(ctx->LB.near);
    dfree(ctx->LB.far_next);
    dfree(ctx->LB.near_next);
    dfree(ctx->LB.ginfo);
    dfree(ctx->dpartial);
    dfree(ctx->dtargets);
    dfree(ctx->dslots);
    dfree(ctx->dsamp);
    for (int i = 0; i < 8; ++i)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    for (int i = 0; i < 2; ++i)
        if (ctx->sev[i]) cudaEventDestroy(ctx->sev[i]);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* ngrav_gpu_last_error(const ngrav_gpu_ctx* ctx) {
    if (!ctx) return "NULL context";
    return ctx->err.c_str();
}

int ngrav_gpu_set_opts(ngrav_gpu_ctx* ctx, const ngrav_gpu_opts* opts) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    NG_TRY(check_opts(ctx, opts));
    if (opts->device != ctx->opts.device) return fail(ctx, NGRAV_ERR_INVALID_ARG, "device cannot change");
    const bool prec_change = opts->precision != ctx->opts.precision;
    if (prec_change && ctx->have) {
        // PLAIN -> SPLIT starts with lo = 0; SPLIT -> PLAIN rounds hi + lo to FP32.
        NG_CUDA(cudaSetDevice(ctx->opts.device));
        if (opts->precision == NGRAV_PRECISION_SPLIT) {
            NG_CUDA(cudaMemsetAsync(ctx->P.plo, 0, sizeof(float4) * ctx->n, ctx->stream));
            NG_CUDA(cudaMemsetAsync(ctx->P.vlo, 0, sizeof(float4) * ctx->n, ctx->stream));
        } else {
            launch_collapse_split(ctx->P.pos, ctx->P.plo, ctx->n, ctx->stream);
            launch_collapse_split(ctx->P.vel, ctx->P.vlo, ctx->n, ctx->stream);  // keeps vel.w (the rung)
        }
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    if (opts->leaf_capacity != ctx->opts.leaf_capacity || opts->max_depth != ctx->opts.max_depth)
        ctx->sort_levels = kKeyLevels;  // another tree: sort and build on the full key once
    ctx->opts = *opts;
    ctx->events = ctx->opts.timing != 0;
    ctx->primed = false;
    return NGRAV_OK;
}

int ngrav_gpu_set_particles(ngrav_gpu_ctx* ctx, int64_t n, const double* x, const double* y, const double* z,
                            const double* vx, const double* vy, const double* vz, const double* m) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    return set_particles_impl<double>(ctx, n, x, y, z, vx, vy, vz, m, true);
}

int ngrav_gpu_set_particles_f32(ngrav_gpu_ctx* ctx, int64_t n, const float* x, const float* y, const float* z,
                                const float* vx, const float* vy, const float* vz, const float* m) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    return set_particles_impl<float>(ctx, n, x, y, z, vx, vy, vz, m, false);
}


int ngrav_gpu_adaptive_dt(ngrav_gpu_ctx* ctx, double eta, double dt_max, double* dt) {
    if (!ctx || !dt) return NGRAV_ERR_INVALID_ARG;
    if (!(dt_max > 0.0) || !(eta > 0.0)) return fail(ctx, NGRAV_ERR_INVALID_ARG, "bad eta / dt_max");
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    if (!ctx->primed) NG_TRY(ngrav_gpu_prime(ctx));
    *dt = dt_max;
    const double eps = ctx->opts.eps;
    if (ctx->n == 0 || !(eps > 0.0)) return NGRAV_OK;
    NG_TRY(ensure_partial(ctx, 1));
    unsigned long long* d = reinterpret_cast<unsigned long long*>(ctx->dpartial);
    NG_CUDA(cudaMemsetAsync(d, 0, sizeof(*d), ctx->stream));
    launch_amax(ctx->n, ctx->P.acc, d, ctx->stream);
    ctx->launches += 1;
    unsigned long long bits = 0;
    NG_CUDA(cudaMemcpyAsync(&bits, d, sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    double amax;
    std::memcpy(&amax, &bits, sizeof(amax));
    if (!(amax > 0.0)) return NGRAV_OK;
    const double t = eta * std::sqrt(eps / amax);
    *dt = std::min(std::max(t, dt_max / 4096.0), dt_max);
    return NGRAV_OK;
}

int ngrav_gpu_block_step(ngrav_gpu_ctx* ctx, double dt, double eta, int max_rung, int* rung_max) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (!(dt > 0.0) || !(eta > 0.0) || max_rung < 0 || max_rung > 20)
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "bad dt / eta / max_rung");
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    if (!ctx->primed) NG_TRY(ngrav_gpu_prime(ctx));
    NG_TRY(ensure_partial(ctx, 2));
    int* drmax = reinterpret_cast<int*>(ctx->dpartial);
    NG_CUDA(cudaMemsetAsync(drmax, 0, sizeof(int), ctx->stream));
    launch_rungs(ctx->n, ctx->P, dt, eta, ctx->opts.eps, max_rung, drmax, ctx->stream);
    int rmax = 0;
    NG_CUDA(cudaMemcpyAsync(&rmax, drmax, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->launches += 1;
    const int nsub = 1 << rmax;
    const float dtmin = (float)(dt / nsub);
    NG_CUDA(cudaEventRecord(ctx->sev[0], ctx->stream));
    int rc = NGRAV_OK;
    for (int sub = 0; sub < nsub && rc == NGRAV_OK; ++sub) {
        launch_block_kick_drift(ctx->n, ctx->P, split_of(ctx), dt, sub, rmax, dtmin, ctx->stream);
        ctx->launches += 1;
        ctx->block_on = true;
        ctx->block_args[0] = sub;
        ctx->block_args[1] = rmax;
        ctx->block_base = dt;
        rc = evaluate(ctx, false, true, 0.f);
        ctx->block_on = false;
    }
    NG_TRY(rc);
    NG_CUDA(cudaEventRecord(ctx->sev[1], ctx->stream));
    NG_CUDA(cudaEventSynchronize(ctx->sev[1]));
    float ms = 0.f;
    NG_CUDA(cudaEventElapsedTime(&ms, ctx->sev[0], ctx->sev[1]));
    ctx->cum_ms_step += ms;
    if (rung_max) *rung_max = rmax;
    return NGRAV_OK;
}

int ngrav_gpu_set_mac_alpha(ngrav_gpu_ctx* ctx, double alpha) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (!(alpha > 0.0) || !std::isfinite(alpha)) return fail(ctx, NGRAV_ERR_INVALID_ARG, "alpha must be positive");
    ctx->alpha = alpha;
    return NGRAV_OK;
}

int ngrav_gpu_set_softening(ngrav_gpu_ctx* ctx, int kind) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (kind != NGRAV_SOFTENING_PLUMMER && kind != NGRAV_SOFTENING_SPLINE)
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "unknown softening kind");
    if (kind == NGRAV_SOFTENING_SPLINE && !(ctx->opts.eps > 0.0))
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "spline softening needs eps > 0");
    ctx->soft = kind == NGRAV_SOFTENING_SPLINE ? kSoftSpline : kSoftPlummer;
    ctx->primed = false;
    return NGRAV_OK;
}

int ngrav_gpu_set_state(ngrav_gpu_ctx* ctx, const double* x, const double* y, const double* z, const double* vx,
                        const double* vy, const double* vz) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    return set_state_impl<double>(ctx, x, y, z, vx, vy, vz, true);
}

int ngrav_gpu_set_state_f32(ngrav_gpu_ctx* ctx, const float* x, const float* y, const float* z, const float* vx,
                            const float* vy, const float* vz) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    return set_state_impl<float>(ctx, x, y, z, vx, vy, vz, false);
}

int ngrav_gpu_compute_accel(ngrav_gpu_ctx* ctx, double* ax, double* ay, double* az) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (!ax || !ay || !az) return fail(ctx, NGRAV_ERR_INVALID_ARG, "NULL output array");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    NG_TRY(evaluate(ctx, false, false, 0.f));
    ctx->primed = true;
    const long long n = ctx->n;
    double* st = ctx->stage;
    launch_download(n, ctx->P.id, ctx->P.acc, nullptr, st, st + n, st + 2 * n, ctx->stream);
    NG_CUDA(cudaMemcpyAsync(ax, st, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaMemcpyAsync(ay, st + n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaMemcpyAsync(az, st + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    return NGRAV_OK;
}

int ngrav_gpu_prime(ngrav_gpu_ctx* ctx) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    NG_TRY(evaluate(ctx, false, false, 0.f));
    ctx->primed = true;
    return NGRAV_OK;
}

int ngrav_gpu_step(ngrav_gpu_ctx* ctx, int nsteps, double dt) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (nsteps < 0 || !std::isfinite(dt)) return fail(ctx, NGRAV_ERR_INVALID_ARG, "bad nsteps/dt");
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    if (!ctx->primed) NG_TRY(ngrav_gpu_prime(ctx));
    const float hdt = (float)(0.5 * dt), fdt = (float)dt;
    NG_CUDA(cudaEventRecord(ctx->sev[0], ctx->stream));
    for (int k = 0; k < nsteps; ++k) {
        if (ctx->use_graphs && enqueue_step_graph(ctx, hdt, fdt)) {
            bool retry = false;
            NG_TRY(finish_eval(ctx, retry));
            if (retry) {
                // capacities grew: redo this step's evaluation directly (the
                // kick-drift has run; the evaluation starts from its state)
                NG_TRY(evaluate(ctx, false, true, hdt));
            } else {
                NG_TRY(lmac_after_eval(ctx));
            }
            continue;
        }
        launch_reset_counters(ctx->C, ctx->stream);
        launch_kick_drift(ctx->P, ctx->n, hdt, fdt, split_of(ctx), ctx->C, ctx->stream);
        ctx->launches += 2;
        NG_TRY(evaluate(ctx, true, true, hdt));
    }
    NG_CUDA(cudaEventRecord(ctx->sev[1], ctx->stream));
    NG_CUDA(cudaEventSynchronize(ctx->sev[1]));
    float ms = 0.f;
    NG_CUDA(cudaEventElapsedTime(&ms, ctx->sev[0], ctx->sev[1]));
    ctx->cum_ms_step += ms;
    return NGRAV_OK;
}

int ngrav_gpu_get_state(ngrav_gpu_ctx* ctx, double* x, double* y, double* z, double* vx, double* vy, double* vz) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const long long n = ctx->n;
    double* st = ctx->stage;
    launch_download(n, ctx->P.id, ctx->P.pos, split_of(ctx) ? ctx->P.plo : nullptr, st, st + n, st + 2 * n,
                    ctx->stream);
    launch_download(n, ctx->P.id, ctx->P.vel, split_of(ctx) ? ctx->P.vlo : nullptr, st + 3 * n, st + 4 * n, st + 5 * n,
                    ctx->stream);
    double* outs[6] = {x, y, z, vx, vy, vz};
    for (int k = 0; k < 6; ++k)
        if (outs[k])
            NG_CUDA(cudaMemcpyAsync(outs[k], st + k * n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    return NGRAV_OK;
}

int ngrav_gpu_get_frame_f32(ngrav_gpu_ctx* ctx, float* pos, float* vel) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const long long n = ctx->n;
    float* st = reinterpret_cast<float*>(ctx->stage);  // 7n doubles hold the 6n floats
    launch_frame_download(n, ctx->P.id, ctx->P.pos, split_of(ctx) ? ctx->P.plo : nullptr, ctx->P.vel,
                          split_of(ctx) ? ctx->P.vlo : nullptr,
                          pos ? st : nullptr, vel ? st + 3 * n : nullptr, ctx->stream);
    if (pos) NG_CUDA(cudaMemcpyAsync(pos, st, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (vel) NG_CUDA(cudaMemcpyAsync(vel, st + 3 * n, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    return NGRAV_OK;
}

int ngrav_gpu_get_rungs(ngrav_gpu_ctx* ctx, int* rung) {
    if (!ctx || !rung) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const long long n = ctx->n;
    int* st = reinterpret_cast<int*>(ctx->stage);
    launch_rung_download(n, ctx->P.id, ctx->P.vel, st, ctx->stream);
    NG_CUDA(cudaMemcpyAsync(rung, st, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    return NGRAV_OK;
}

int ngrav_gpu_get_accel(ngrav_gpu_ctx* ctx, double* ax, double* ay, double* az) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const long long n = ctx->n;
    double* st = ctx->stage;
    launch_download(n, ctx->P.id, ctx->P.acc, nullptr, st, st + n, st + 2 * n, ctx->stream);
    double* outs[3] = {ax, ay, az};
    for (int k = 0; k < 3; ++k)
        if (outs[k])
            NG_CUDA(cudaMemcpyAsync(outs[k], st + k * n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    return NGRAV_OK;
}

int ngrav_gpu_diagnostics(ngrav_gpu_ctx* ctx, int exact_potential, ngrav_gpu_diag* out) {
    if (!ctx || !out) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const long long n = ctx->n;
    const bool split = split_of(ctx);
    const int nb = diag_blocks(n);
    const int npb = potential_blocks(n);
    NG_TRY(ensure_partial(ctx, std::max<long long>(8LL * nb, npb) + 8));
    std::vector<double> h(std::max<long long>(8LL * nb, npb));
    launch_diag_pass1(n, ctx->P, split, ctx->dpartial, ctx->stream);
    NG_CUDA(cudaMemcpyAsync(h.data(), ctx->dpartial, sizeof(double) * 8 * nb, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    double s1[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < 8; ++k) s1[k] += h[8 * b + k];
    const double M = s1[0];
    double com[3] = {s1[1], s1[2], s1[3]};
    if (M > 0.0)
        for (double& c : com) c /= M;
    launch_diag_pass2(n, ctx->P, split, com[0], com[1], com[2], ctx->dpartial, ctx->stream);
    NG_CUDA(cudaMemcpyAsync(h.data(), ctx->dpartial, sizeof(double) * 3 * nb, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    double L[3] = {0, 0, 0};
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < 3; ++k) L[k] += h[3 * b + k];
    out->kinetic = s1[4];
    for (int k = 0; k < 3; ++k) {
        out->com[k] = com[k];
        out->L[k] = L[k];
        out->P[k] = s1[5 + k];
    }
    if (exact_potential < 0 || exact_potential > 2)
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "exact_potential must be 0, 1 or 2");
    // mode 2: the exact pair set with FP32 pair terms (Plummer; a spline run
    // takes the FP64 path)
    const bool pairs32 = exact_potential == 2 && ctx->soft != kSoftSpline;
    const bool exact = exact_potential != 0 || n <= 262144;
    out->potential_exact = pairs32 ? 2 : (exact ? 1 : 0);
    if (pairs32) {
        const int pb = potential_f32_blocks(n, ctx->sm_count);
        NG_TRY(ensure_partial(ctx, pb));
        std::vector<double> hp(pb);
        launch_potential_f32(n, ctx->P, split, ctx->opts.eps * ctx->opts.eps, pb, ctx->dpartial, ctx->stream);
        NG_CUDA(cudaMemcpyAsync(hp.data(), ctx->dpartial, sizeof(double) * pb, cudaMemcpyDeviceToHost, ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        double pot = 0.0;
        for (int b = 0; b < pb; ++b) pot += hp[b];
        out->potential = ctx->opts.G * pot;
    } else if (exact) {
        launch_potential(n, ctx->P, split, ctx->opts.eps * ctx->opts.eps, spline_h(ctx), ctx->dpartial, ctx->stream);
        NG_CUDA(cudaMemcpyAsync(h.data(), ctx->dpartial, sizeof(double) * npb, cudaMemcpyDeviceToHost,
                                ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        double pot = 0.0;
        for (int b = 0; b < npb; ++b) pot += h[b];
        out->potential = ctx->opts.G * pot;
    } else {
        out->potential = std::nan("");
    }
    out->energy = out->kinetic + out->potential;
    return NGRAV_OK;
}

int ngrav_gpu_force_error(ngrav_gpu_ctx* ctx, int nsample, uint64_t seed, int fp64_pairs, ngrav_gpu_ferr* out) {
    if (!ctx || !out) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    const long long n = ctx->n;
    if (nsample <= 0 || nsample > n) return fail(ctx, NGRAV_ERR_INVALID_ARG, "nsample out of range");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    // Floyd's sampling without replacement, splitmix64 stream.
    uint64_t st = seed;
    auto next = [&st]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    std::unordered_set<long long> chosen;
    std::vector<int> targets;
    targets.reserve(nsample);
    for (long long j = n - nsample; j < n; ++j) {
        const long long t = (long long)(next() % (uint64_t)(j + 1));
        const long long pick = chosen.count(t) ? j : t;
        chosen.insert(pick);
        targets.push_back((int)pick);
    }
    std::sort(targets.begin(), targets.end());
    NG_TRY(ensure_samp(ctx, nsample));
    NG_CUDA(cudaMemcpyAsync(ctx->dtargets, targets.data(), sizeof(int) * nsample, cudaMemcpyHostToDevice,
                            ctx->stream));
    launch_inverse_id(n, ctx->P.id, ctx->inv, ctx->stream);
    launch_gather_slots(ctx->inv, ctx->dtargets, nsample, ctx->dslots, ctx->stream);
    if (ctx->F.nsys > 1) {  // ensemble: each target against its own system only
        launch_forest_sampler(ctx->P, split_of(ctx), ctx->dslots, nsample, ctx->F, ctx->opts.eps * ctx->opts.eps,
                              spline_h(ctx), ctx->dsamp, ctx->stream);
    } else {
        const int shares = sampler_shares(n, nsample, ctx->sm_count);
        NG_TRY(ensure_partial(ctx, 3LL * shares * nsample));
        launch_sampler(n, ctx->P, split_of(ctx), ctx->dslots, nsample, ctx->opts.eps * ctx->opts.eps, spline_h(ctx),
                       fp64_pairs != 0, ctx->dsamp, ctx->dpartial, shares, ctx->stream);
    }
    std::vector<double> ref(3 * (size_t)nsample);
    std::vector<int> slots(nsample);
    NG_CUDA(cudaMemcpyAsync(ref.data(), ctx->dsamp, sizeof(double) * 3 * nsample, cudaMemcpyDeviceToHost,
                            ctx->stream));
    NG_CUDA(cudaMemcpyAsync(slots.data(), ctx->dslots, sizeof(int) * nsample, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    NG_CUDA(cudaGetLastError());
    std::vector<float4> acc(nsample);
    NG_TRY(ensure_partial(ctx, std::max<long long>(ctx->dpartial_cap, 2LL * nsample)));
    launch_gather_float4(ctx->P.acc, ctx->dslots, nsample, reinterpret_cast<float4*>(ctx->dpartial), ctx->stream);
    NG_CUDA(cudaMemcpyAsync(acc.data(), ctx->dpartial, sizeof(float4) * nsample, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<double> rel(nsample);
    double s2 = 0.0, mx = 0.0;
    for (int k = 0; k < nsample; ++k) {
        const double G = ctx->opts.G;
        const double rx = G * ref[3 * k], ry = G * ref[3 * k + 1], rz = G * ref[3 * k + 2];
        const double ex = acc[k].x - rx, ey = acc[k].y - ry, ez = acc[k].z - rz;
        const double r = std::sqrt(ex * ex + ey * ey + ez * ez) /
                         std::max(std::sqrt(rx * rx + ry * ry + rz * rz), 1e-30);
        rel[k] = r;
        s2 += r * r;
        mx = std::max(mx, r);
    }
    std::sort(rel.begin(), rel.end());
    out->rms = std::sqrt(s2 / nsample);
    out->max = mx;
    out->median = (nsample & 1) ? rel[nsample / 2] : 0.5 * (rel[nsample / 2 - 1] + rel[nsample / 2]);
    double sum = 0.0;
    for (double r : rel) sum += r;
    out->mean = sum / nsample;
    out->nsample = nsample;
    return NGRAV_OK;
}

int ngrav_gpu_get_stats(ngrav_gpu_ctx* ctx, ngrav_gpu_stats* out) {
    if (!ctx || !out) return NGRAV_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    const Counters& c = ctx->hc;
    out->ms_bbox_keys = ctx->phase_ms[0];
    out->ms_sort = ctx->phase_ms[1];
    out->ms_build = ctx->phase_ms[2];
    out->ms_moments = ctx->phase_ms[3];
    out->cum_particle_evals = ctx->cum_particle_evals;
    out->sort_passes = ctx->sort_passes;
    out->ms_walk = ctx->phase_ms[4];
    out->ms_force = ctx->phase_ms[5];
    out->ms_total = ctx->phase_ms[0] + ctx->phase_ms[1] + ctx->phase_ms[2] + ctx->phase_ms[3] + ctx->phase_ms[4] +
                    ctx->phase_ms[5];
    out->p2p_pairs = (long long)c.p2p_pairs;
    out->p2c_terms = (long long)c.p2c_terms;
    out->mac_tests = (long long)c.mac_tests;
    out->mac_retests = (long long)c.mac_retests;
    out->groups = (long long)c.groups;
    out->nodes = std::min(c.next_free, ctx->T.cap);
    out->leaves = c.nleaves;
    out->levels = c.levels_used;
    out->max_leaf_count = c.max_leaf_count;
    out->depth_limited_leaves = c.depth_limited;
    out->walk_stack_max = c.stack_max;
    out->status_bits = c.status;
    out->force_evals = ctx->force_evals;
    out->n = ctx->n;
    out->cum_evals = ctx->cum_evals;
    out->cum_p2p_pairs = ctx->cum_pairs;
    out->cum_p2c_terms = ctx->cum_p2c;
    out->cum_ms_walk = ctx->cum_ms_walk;
    out->cum_ms_force = ctx->cum_ms_force;
    out->far_entries = (long long)c.far_chunks * kListChunk;
    out->near_entries = (long long)c.near_chunks * kListChunk;
    out->list_max = c.list_max;
    out->cum_ms_eval = ctx->cum_ms_eval;
    out->cum_ms_step = ctx->cum_ms_step;
    out->cum_launches = ctx->launches;
    out->graph_captures = ctx->graph_captures;
    out->graph_replays = ctx->graph_replays;
    lmac_fill_stats(ctx, out);
    return NGRAV_OK;
}

int ngrav_gpu_reset_cumulative(ngrav_gpu_ctx* ctx) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    ctx->launches = 0;
    ctx->cum_evals = ctx->cum_pairs = ctx->cum_p2c = 0;
    ctx->cum_ms_walk = ctx->cum_ms_force = ctx->cum_ms_eval = ctx->cum_ms_step = 0.0;
    ctx->cum_particle_evals = 0;
    return NGRAV_OK;
}

int ngrav_gpu_probe_fp32_peak(int device, double* tflops) {
    if (!tflops) return NGRAV_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return NGRAV_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return NGRAV_ERR_CUDA;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return NGRAV_ERR_CUDA;
    *tflops = run_fma_probe(sms, s);
    cudaStreamDestroy(s);
    return *tflops > 0.0 ? NGRAV_OK : NGRAV_ERR_CUDA;
}

int ngrav_gpu_debug_shrink_pools(ngrav_gpu_ctx* ctx, int node_cap, int far_chunks, int near_chunks,
                                 int pend_chunks) {
    if (!ctx) return NGRAV_ERR_INVALID_ARG;
    if (node_cap < 0 || far_chunks < 0 || near_chunks < 0 || pend_chunks < 0)
        return fail(ctx, NGRAV_ERR_INVALID_ARG, "negative pool size");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (node_cap > 0) NG_TRY(alloc_nodes(ctx, std::max(node_cap, 1)));
    if (far_chunks > 0 || near_chunks > 0) {
        ListBuffers& L = ctx->LB;
        const long long fc = far_chunks > 0 ? far_chunks : L.far_chunk_cap;
        const long long nc = near_chunks > 0 ? near_chunks : L.near_chunk_cap;
        dfree(L.far);
        dfree(L.far_next);
        dfree(L.near);
        dfree(L.near_next);
        L.far_chunk_cap = L.near_chunk_cap = 0;
        NG_TRY(alloc_lists(ctx, fc, nc));
    }
    if (pend_chunks > 0) NG_TRY(lmac_debug_shrink(ctx, pend_chunks));
    return NGRAV_OK;
}

int ngrav_gpu_debug_tree(ngrav_gpu_ctx* ctx, int* nnodes, uint64_t* keys, int* order, int* level, uint64_t* prefix,
                         int* count, int* is_leaf, double* center, double* half, double* com, double* mass,
                         double* max_radius, double* quad) {
    if (!ctx || !nnodes) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have || ctx->force_evals == 0) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no tree built yet");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const int nn = std::min(ctx->hc.next_free, ctx->T.cap);
    *nnodes = nn;
    if (!keys && !order && !level) return NGRAV_OK;
    const long long n = ctx->n;
    std::vector<unsigned long long> hk(n);
    std::vector<int> id(n);
    NG_CUDA(cudaMemcpy(hk.data(), ctx->SB.keys, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost));
    NG_CUDA(cudaMemcpy(id.data(), ctx->P.id, sizeof(int) * n, cudaMemcpyDeviceToHost));
    if (keys)
        for (long long k = 0; k < n; ++k) keys[id[k]] = hk[k];
    std::vector<int> st(nn), ct(nn), fc(nn);
    std::vector<unsigned char> lv(nn);
    NG_CUDA(cudaMemcpy(st.data(), ctx->T.start, sizeof(int) * nn, cudaMemcpyDeviceToHost));
    NG_CUDA(cudaMemcpy(ct.data(), ctx->T.count, sizeof(int) * nn, cudaMemcpyDeviceToHost));
    NG_CUDA(cudaMemcpy(fc.data(), ctx->T.first_child, sizeof(int) * nn, cudaMemcpyDeviceToHost));
    NG_CUDA(cudaMemcpy(lv.data(), ctx->T.level, nn, cudaMemcpyDeviceToHost));
    if (order) {
        // Leaves partition [0, n) in key order; within a leaf the reference
        // lists members in ascending original index (Tree.cpp:130-133, :169).
        for (long long k = 0; k < n; ++k) order[k] = id[k];
        for (int v = 0; v < nn; ++v)
            if (fc[v] == -1) std::sort(order + st[v], order + st[v] + ct[v]);
    }
    std::vector<double> tmp(nn);
    for (int v = 0; v < nn; ++v) {
        if (level) level[v] = lv[v];
        if (prefix) prefix[v] = lv[v] == 0 ? 0ull : (hk[st[v]] >> (3 * (kKeyLevels - lv[v])));
        if (count) count[v] = ct[v];
        if (is_leaf) is_leaf[v] = fc[v] == -1;
    }
    if (half) NG_CUDA(cudaMemcpy(half, ctx->T.half, sizeof(double) * nn, cudaMemcpyDeviceToHost));
    auto get3 = [&](double* dst, const double* a, const double* b, const double* c) -> int {
        if (!dst) return NGRAV_OK;
        const double* src[3] = {a, b, c};
        for (int k = 0; k < 3; ++k) {
            NG_CUDA(cudaMemcpy(tmp.data(), src[k], sizeof(double) * nn, cudaMemcpyDeviceToHost));
            for (int v = 0; v < nn; ++v) dst[3 * v + k] = tmp[v];
        }
        return NGRAV_OK;
    };
    NG_TRY(get3(center, ctx->T.cx, ctx->T.cy, ctx->T.cz));
    NG_TRY(get3(com, ctx->T.comx, ctx->T.comy, ctx->T.comz));
    if (mass) NG_CUDA(cudaMemcpy(mass, ctx->T.mass, sizeof(double) * nn, cudaMemcpyDeviceToHost));
    if (max_radius) {
        // Leaves carry maxRadius from the device; internal nodes take the
        // reference's upsweep, max over children of maxR_c + |com_c - com|
        // (Tree.cpp:193-201), here on the host from the exported arrays.
        NG_CUDA(cudaMemcpy(max_radius, ctx->T.maxr, sizeof(double) * nn, cudaMemcpyDeviceToHost));
        std::vector<double> cm(3 * (size_t)nn);
        NG_TRY(get3(cm.data(), ctx->T.comx, ctx->T.comy, ctx->T.comz));
        std::vector<unsigned char> nch(nn);
        NG_CUDA(cudaMemcpy(nch.data(), ctx->T.nchild, nn, cudaMemcpyDeviceToHost));
        std::vector<int> by_level(nn);
        for (int v = 0; v < nn; ++v) by_level[v] = v;
        std::stable_sort(by_level.begin(), by_level.end(), [&](int a, int b) { return lv[a] > lv[b]; });
        for (int v : by_level) {
            if (fc[v] == -1) continue;
            double r = 0.0;
            for (int c = fc[v]; c < fc[v] + nch[v]; ++c) {
                const double dx = cm[3 * c] - cm[3 * v], dy = cm[3 * c + 1] - cm[3 * v + 1],
                             dz = cm[3 * c + 2] - cm[3 * v + 2];
                r = std::max(r, max_radius[c] + std::sqrt(dx * dx + dy * dy + dz * dz));
            }
            max_radius[v] = r;
        }
    }
    if (quad) NG_CUDA(cudaMemcpy(quad, ctx->T.quad, sizeof(double) * 5 * nn, cudaMemcpyDeviceToHost));
    return NGRAV_OK;
}

}  // extern "C"
