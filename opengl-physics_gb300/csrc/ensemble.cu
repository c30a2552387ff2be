// ensemble.cu -- independent systems of uneven N advanced together: the C-ABI
// of the ensemble (ngrav_gpu_set_ensemble and its per-system error and
// diagnostics) and the per-system kernels behind it.
//
// The systems share one particle set and one launch per phase: system s holds
// slots [off[s], off[s+1]), its id is the top digits of every key, each system
// has its own root cube (the reference's BuildRoot over its particles,
// Tree.cpp:54-88) and its own tree, and every walk starts at its group's
// system root (the Forest of engine.cuh).  The KDK step, the graph capture and
// the learned opening test need nothing else.
#include "ctx_internal.cuh"
#include "ctx_kernels.cuh"
#include "softening.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_set>
#include <vector>

namespace ngrav {

// Direct sum of each target's own system, FP32 pairs, FP64 totals; one block
// per target.
template <int SOFT>
__global__ void __launch_bounds__(256) forest_sampler_kernel(const float4* __restrict__ pos,
                                                             const float4* __restrict__ plo,
                                                             const int* __restrict__ slots, Forest F, float eps2,
                                                             float ih, double* __restrict__ out) {
    __shared__ double red[3][8];
    const int ti = slots[blockIdx.x];
    const int sys = forest_system(F, ti);
    const long long j0 = F.off[sys], j1 = F.off[sys + 1];
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 tp = pos[ti];
    const float4 tl = plo ? plo[ti] : zero;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (long long base = j0; base < j1; base += 64 * 256) {
        float px = 0.f, py = 0.f, pz = 0.f;
        const long long end = base + 64 * 256 < j1 ? base + 64 * 256 : j1;
        for (long long j = base + threadIdx.x; j < end; j += 256) {
            if (j == ti) continue;
            const float4 p = pos[j];
            const float4 l = plo ? plo[j] : zero;
            const float dx = (p.x - tp.x) + (l.x - tl.x);
            const float dy = (p.y - tp.y) + (l.y - tl.y);
            const float dz = (p.z - tp.z) + (l.z - tl.z);
            const float f = pair_factor<SOFT>(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), p.w, eps2, ih);
            px = fmaf(f, dx, px);
            py = fmaf(f, dy, py);
            pz = fmaf(f, dz, pz);
        }
        ax += px;
        ay += py;
        az += pz;
    }
    double v[3] = {ax, ay, az};
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = 0; c < 3; ++c) {
        for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
        if (lane == 0) red[c][w] = v[c];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int k = 0; k < 8; ++k) t += red[threadIdx.x][k];
        out[3 * blockIdx.x + threadIdx.x] = t;
    }
}

__global__ void gather_float4_kernel(const float4* __restrict__ a, const int* __restrict__ slots, int ns,
                                     float4* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ns) out[k] = a[slots[k]];
}

// Per-system FP64 sums, one block per system: mass, m x (3), kinetic, m v (3)
// into part[8 s ..], then the angular momentum about the system's COM into
// part[8 nsys + 3 s ..].
__global__ void __launch_bounds__(256) forest_diag_kernel(const float4* __restrict__ pos,
                                                          const float4* __restrict__ plo,
                                                          const float4* __restrict__ vel,
                                                          const float4* __restrict__ vlo, Forest F,
                                                          double* __restrict__ part) {
    __shared__ double red[8][8];
    __shared__ double com[3];
    const int sys = blockIdx.x;
    const long long j0 = F.off[sys], j1 = F.off[sys + 1];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long j = j0 + threadIdx.x; j < j1; j += 256) {
        const float4 p = pos[j];
        const float4 l = plo ? plo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 v = vel[j];
        const float4 vl = vlo ? vlo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        const double vx = (double)v.x + vl.x, vy = (double)v.y + vl.y, vz = (double)v.z + vl.z;
        const double m = p.w, x = (double)p.x + l.x, y = (double)p.y + l.y, z = (double)p.z + l.z;
        a[0] += m;
        a[1] += m * x;
        a[2] += m * y;
        a[3] += m * z;
        a[4] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        a[5] += m * vx;
        a[6] += m * vy;
        a[7] += m * vz;
    }
    for (int c = 0; c < 8; ++c) {
        for (int o = 16; o > 0; o >>= 1) a[c] += __shfl_xor_sync(0xffffffffu, a[c], o);
        if (lane == 0) red[c][w] = a[c];
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double t = 0.0;
        for (int k = 0; k < 8; ++k) t += red[threadIdx.x][k];
        part[8 * sys + threadIdx.x] = t;
        if (threadIdx.x >= 1 && threadIdx.x <= 3) com[threadIdx.x - 1] = t;
    }
    __syncthreads();
    const double M = part[8 * sys];
    const double cx = M > 0.0 ? com[0] / M : 0.0, cy = M > 0.0 ? com[1] / M : 0.0, cz = M > 0.0 ? com[2] / M : 0.0;
    double L[3] = {0, 0, 0};
    for (long long j = j0 + threadIdx.x; j < j1; j += 256) {
        const float4 p = pos[j];
        const float4 l = plo ? plo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 v = vel[j];
        const float4 vl = vlo ? vlo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        const double vx = (double)v.x + vl.x, vy = (double)v.y + vl.y, vz = (double)v.z + vl.z;
        const double m = p.w;
        const double dx = (double)p.x + l.x - cx, dy = (double)p.y + l.y - cy, dz = (double)p.z + l.z - cz;
        L[0] += m * (dy * vz - dz * vy);
        L[1] += m * (dz * vx - dx * vz);
        L[2] += m * (dx * vy - dy * vx);
    }
    __syncthreads();
    for (int c = 0; c < 3; ++c) {
        for (int o = 16; o > 0; o >>= 1) L[c] += __shfl_xor_sync(0xffffffffu, L[c], o);
        if (lane == 0) red[c][w] = L[c];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int k = 0; k < 8; ++k) t += red[threadIdx.x][k];
        part[8 * F.nsys + 3 * sys + threadIdx.x] = t;
    }
}

// Exact pair potential of each system in FP64: block (s, chunk) sums the
// pairs (i < j) whose first member lies in its chunk of system s.
__global__ void __launch_bounds__(256) forest_potential_kernel(const float4* __restrict__ pos,
                                                               const float4* __restrict__ plo, Forest F, double eps2,
                                                               int chunks, double* __restrict__ part) {
    __shared__ double red[8];
    const int sys = blockIdx.x / chunks, ck = blockIdx.x % chunks;
    const long long j0 = F.off[sys], j1 = F.off[sys + 1], ns = j1 - j0;
    const long long per = (ns + chunks - 1) / chunks;
    const long long i0 = j0 + ck * per, i1 = i0 + per < j1 ? i0 + per : j1;
    double pot = 0.0;
    for (long long i = i0; i < i1; ++i) {
        const float4 pi = pos[i];
        const float4 li = plo ? plo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const double xi = (double)pi.x + li.x, yi = (double)pi.y + li.y, zi = (double)pi.z + li.z;
        for (long long j = i + 1 + threadIdx.x; j < j1; j += 256) {
            const float4 pj = pos[j];
            const float4 lj = plo ? plo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            const double dx = (double)pj.x + lj.x - xi, dy = (double)pj.y + lj.y - yi, dz = (double)pj.z + lj.z - zi;
            pot -= (double)pi.w * pj.w / sqrt(dx * dx + dy * dy + dz * dz + eps2);
        }
    }
    for (int o = 16; o > 0; o >>= 1) pot += __shfl_xor_sync(0xffffffffu, pot, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = pot;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < 8; ++k) t += red[k];
        part[blockIdx.x] = t;
    }
}

void launch_forest_sampler(const Particles& P, bool split, const int* slots, int nslots, const Forest& F,
                           double eps2, double spline_h, double* out, cudaStream_t s) {
    if (nslots <= 0) return;
    if (spline_h > 0.0)
        forest_sampler_kernel<kSoftSpline><<<nslots, 256, 0, s>>>(P.pos, split ? P.plo : nullptr, slots, F, 0.f,
                                                                 (float)(1.0 / spline_h), out);
    else
        forest_sampler_kernel<kSoftPlummer><<<nslots, 256, 0, s>>>(P.pos, split ? P.plo : nullptr, slots, F,
                                                                  (float)eps2, 0.f, out);
}

void launch_forest_diag(const Particles& P, bool split, const Forest& F, double* part, cudaStream_t s) {
    forest_diag_kernel<<<F.nsys, 256, 0, s>>>(P.pos, split ? P.plo : nullptr, P.vel, split ? P.vlo : nullptr, F,
                                              part);
}

void launch_forest_potential(const Particles& P, bool split, const Forest& F, double eps2, int chunks, double* part,
                             cudaStream_t s) {
    forest_potential_kernel<<<F.nsys * chunks, 256, 0, s>>>(P.pos, split ? P.plo : nullptr, F, eps2, chunks, part);
}

void launch_gather_float4(const float4* a, const int* slots, int ns, float4* out, cudaStream_t s) {
    if (ns <= 0) return;
    gather_float4_kernel<<<(ns + 255) / 256, 256, 0, s>>>(a, slots, ns, out);
}

}  // namespace ngrav

namespace ngrav_ctx {

void free_forest(ngrav_gpu_ctx* ctx) {
    dfree(ctx->f_off);
    dfree(ctx->f_root);
    dfree(ctx->f_bbox);
    ctx->F = Forest{};
    ctx->h_off.clear();
}

}  // namespace ngrav_ctx

using namespace ngrav_ctx;

extern "C" {

int ngrav_gpu_set_ensemble(ngrav_gpu_ctx* ctx, int nsys, const int64_t* offsets) {
    if (!ctx || nsys < 1 || !offsets) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    if (offsets[0] != 0 || offsets[nsys] != ctx->n) return fail(ctx, NGRAV_ERR_INVALID_ARG, "offsets must span [0, n]");
    for (int s = 0; s < nsys; ++s)
        if (offsets[s + 1] < offsets[s]) return fail(ctx, NGRAV_ERR_INVALID_ARG, "offsets must not decrease");
    int levels = 0;
    for (long long cap = 1; cap < nsys; cap *= 8) ++levels;
    if (levels > 6) return fail(ctx, NGRAV_ERR_INVALID_ARG, "at most 8^6 systems");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    free_forest(ctx);
    ctx->sort_levels = kKeyLevels;  // another tree: sort and build on the full key once
    if (nsys == 1) return NGRAV_OK;  // one system: the plain tree
    NG_CUDA(dalloc(ctx->f_off, nsys + 1));
    NG_CUDA(dalloc(ctx->f_root, 4LL * nsys));
    NG_CUDA(dalloc(ctx->f_bbox, 6LL * nsys));
    std::vector<long long> off(offsets, offsets + nsys + 1);
    std::vector<unsigned long long> box(6LL * nsys);
    for (int s = 0; s < nsys; ++s)
        for (int a = 0; a < 3; ++a) {
            box[6 * s + a] = ~0ull;
            box[6 * s + 3 + a] = 0ull;
        }
    NG_CUDA(cudaMemcpy(ctx->f_off, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice));
    NG_CUDA(cudaMemcpy(ctx->f_bbox, box.data(), sizeof(unsigned long long) * box.size(), cudaMemcpyHostToDevice));
    ctx->h_off = off;
    ctx->F.nsys = nsys;
    ctx->F.sys_levels = levels;
    ctx->F.off = ctx->f_off;
    ctx->F.root = ctx->f_root;
    ctx->F.bbox = ctx->f_bbox;
    ctx->primed = false;
    ctx->acc_valid = false;
    return NGRAV_OK;
}

int ngrav_gpu_ensemble_force_error(ngrav_gpu_ctx* ctx, int targets_per_system, uint64_t seed, double* rms,
                                   double* max) {
    if (!ctx || targets_per_system < 1 || !rms) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have || !ctx->acc_valid) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no force evaluation to check");
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const int nsys = ctx->F.nsys;
    std::vector<long long> off = nsys > 1 ? ctx->h_off : std::vector<long long>{0, ctx->n};
    // Floyd sampling per system (splitmix64 stream), original particle ids
    std::vector<int> targets, owner;
    for (int s = 0; s < nsys; ++s) {
        const long long ns = off[s + 1] - off[s];
        const long long k = std::min<long long>(targets_per_system, ns);
        uint64_t st = seed * 0x9E3779B97F4A7C15ull + (uint64_t)s;
        auto next = [&st]() {
            uint64_t z = (st += 0x9E3779B97F4A7C15ull);
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            return z ^ (z >> 31);
        };
        std::unordered_set<long long> chosen;
        for (long long j = ns - k; j < ns; ++j) {
            const long long t = (long long)(next() % (uint64_t)(j + 1));
            const long long pick = chosen.count(t) ? j : t;
            chosen.insert(pick);
            targets.push_back((int)(off[s] + pick));
            owner.push_back(s);
        }
    }
    const int nt = (int)targets.size();
    NG_TRY(ensure_samp(ctx, nt));
    NG_TRY(ensure_partial(ctx, 2LL * nt));
    NG_CUDA(cudaMemcpyAsync(ctx->dtargets, targets.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, ctx->stream));
    launch_inverse_id(ctx->n, ctx->P.id, ctx->inv, ctx->stream);
    launch_gather_slots(ctx->inv, ctx->dtargets, nt, ctx->dslots, ctx->stream);
    Forest F = ctx->F;
    long long one_off[2] = {0, ctx->n};
    long long* d_one = nullptr;
    if (nsys == 1) {
        NG_CUDA(dalloc(d_one, 2));
        NG_CUDA(cudaMemcpy(d_one, one_off, sizeof(one_off), cudaMemcpyHostToDevice));
        F.off = d_one;
    }
    launch_forest_sampler(ctx->P, split_of(ctx), ctx->dslots, nt, F, ctx->opts.eps * ctx->opts.eps, spline_h(ctx),
                          ctx->dsamp, ctx->stream);
    launch_gather_float4(ctx->P.acc, ctx->dslots, nt, reinterpret_cast<float4*>(ctx->dpartial), ctx->stream);
    std::vector<double> ref(3 * (size_t)nt);
    std::vector<float4> acc(nt);
    NG_CUDA(cudaMemcpyAsync(ref.data(), ctx->dsamp, sizeof(double) * 3 * nt, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaMemcpyAsync(acc.data(), ctx->dpartial, sizeof(float4) * nt, cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (d_one) dfree(d_one);
    std::vector<double> s2(nsys, 0.0), mx(nsys, 0.0), cnt(nsys, 0.0);
    for (int k = 0; k < nt; ++k) {
        const double G = ctx->opts.G;
        const double rx = G * ref[3 * k], ry = G * ref[3 * k + 1], rz = G * ref[3 * k + 2];
        const double ex = acc[k].x - rx, ey = acc[k].y - ry, ez = acc[k].z - rz;
        const double r = std::sqrt(ex * ex + ey * ey + ez * ez) / std::max(std::sqrt(rx * rx + ry * ry + rz * rz), 1e-30);
        s2[owner[k]] += r * r;
        mx[owner[k]] = std::max(mx[owner[k]], r);
        cnt[owner[k]] += 1.0;
    }
    for (int s = 0; s < nsys; ++s) {
        rms[s] = cnt[s] > 0 ? std::sqrt(s2[s] / cnt[s]) : 0.0;
        if (max) max[s] = mx[s];
    }
    return NGRAV_OK;
}

int ngrav_gpu_ensemble_diagnostics(ngrav_gpu_ctx* ctx, int exact_potential, ngrav_gpu_diag* out) {
    if (!ctx || !out) return NGRAV_ERR_INVALID_ARG;
    if (!ctx->have) return fail(ctx, NGRAV_ERR_NO_PARTICLES, "no particles set");
    if (ctx->F.nsys == 1) return ngrav_gpu_diagnostics(ctx, exact_potential, out);
    NG_CUDA(cudaSetDevice(ctx->opts.device));
    const int nsys = ctx->F.nsys;
    const bool split = split_of(ctx);
    const int chunks = 16;
    NG_TRY(ensure_partial(ctx, std::max<long long>(11LL * nsys, (long long)chunks * nsys)));
    launch_forest_diag(ctx->P, split, ctx->F, ctx->dpartial, ctx->stream);
    std::vector<double> h(11LL * nsys);
    NG_CUDA(cudaMemcpyAsync(h.data(), ctx->dpartial, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream));
    NG_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<double> pot(nsys, std::nan(""));
    if (exact_potential) {
        launch_forest_potential(ctx->P, split, ctx->F, ctx->opts.eps * ctx->opts.eps, chunks, ctx->dpartial,
                                ctx->stream);
        std::vector<double> hp((size_t)chunks * nsys);
        NG_CUDA(cudaMemcpyAsync(hp.data(), ctx->dpartial, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost,
                                ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        for (int s = 0; s < nsys; ++s) {
            double t = 0.0;
            for (int c = 0; c < chunks; ++c) t += hp[(size_t)s * chunks + c];
            pot[s] = ctx->opts.G * t;
        }
    }
    for (int s = 0; s < nsys; ++s) {
        const double* a = &h[8 * (size_t)s];
        ngrav_gpu_diag& d = out[s];
        std::memset(&d, 0, sizeof(d));
        const double M = a[0];
        for (int k = 0; k < 3; ++k) {
            d.com[k] = M > 0.0 ? a[1 + k] / M : 0.0;
            d.P[k] = a[5 + k];
            d.L[k] = h[8 * (size_t)nsys + 3 * s + k];
        }
        d.kinetic = a[4];
        d.potential = pot[s];
        d.energy = d.kinetic + d.potential;
        d.potential_exact = exact_potential ? 1 : 0;
    }
    return NGRAV_OK;
}

}  // extern "C"
