// kdk.cu -- state upload/download, the fused opening kick + drift, FP64
// conservation diagnostics and the direct-sum force-error sampler.
//
// KDK (restating projects/nbody_core/src/Integrator.cpp:9-39):
//   v += dt/2 a;  x += dt v;  a = F(x);  v += dt/2 a.
// The first two updates are one streaming kernel here (kick_drift_kernel);
// the closing kick is fused into the walk's epilogue.  In SPLIT precision the
// drift adds dt*v to a double-float (hi, lo) position with an error-free
// two-sum, so the state keeps ~48 significant bits.
//
// Diagnostics (restating include/ngrav/System.hpp:119-193 and
// src/DeckSim.cpp:147-153): kinetic energy, centre of mass, angular momentum
// about the COM and linear momentum are FP64 block reductions combined in a
// fixed order (deterministic); the potential is the exact FP64 pair sum
// sum_{i<j} -G m_i m_j / sqrt(r^2 + eps^2).
#include "engine.cuh"

#include <algorithm>
#include "softening.cuh"
#include "ctx_kernels.cuh"

namespace ngrav {

__device__ __forceinline__ unsigned long long enc_f64_k(double d) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

// ---------------------------------------------------------------------------
// Upload / download
// ---------------------------------------------------------------------------

template <typename T>
__global__ void upload_kernel(long long n, const T* __restrict__ x, const T* __restrict__ y,
                              const T* __restrict__ z, const T* __restrict__ vx, const T* __restrict__ vy,
                              const T* __restrict__ vz, const T* __restrict__ m, Particles P, int split) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double dx = (double)x[i], dy = (double)y[i], dz = (double)z[i];
        const float hx = (float)dx, hy = (float)dy, hz = (float)dz;
        P.pos[i] = make_float4(hx, hy, hz, (float)m[i]);
        if (split) P.plo[i] = make_float4((float)(dx - (double)hx), (float)(dy - (double)hy), (float)(dz - (double)hz), 0.f);
        const double ux = vx ? (double)vx[i] : 0.0, uy = vx ? (double)vy[i] : 0.0, uz = vx ? (double)vz[i] : 0.0;
        const float gx = (float)ux, gy = (float)uy, gz = (float)uz;
        P.vel[i] = make_float4(gx, gy, gz, 0.f);
        P.vlo[i] = split ? make_float4((float)(ux - (double)gx), (float)(uy - (double)gy), (float)(uz - (double)gz), 0.f)
                         : make_float4(0.f, 0.f, 0.f, 0.f);
        P.acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        P.id[i] = (int)i;
    }
}

// New positions / velocities for the current particles, in the caller's
// order: slot k takes particle id[k]'s values; masses, order and the carried
// accelerations stay.
template <typename T>
__global__ void state_kernel(long long n, const T* __restrict__ x, const T* __restrict__ y,
                             const T* __restrict__ z, const T* __restrict__ vx, const T* __restrict__ vy,
                             const T* __restrict__ vz, Particles P, int split) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int i = P.id[k];
        const double dx = (double)x[i], dy = (double)y[i], dz = (double)z[i];
        const float hx = (float)dx, hy = (float)dy, hz = (float)dz;
        P.pos[k] = make_float4(hx, hy, hz, P.pos[k].w);
        if (split) P.plo[k] = make_float4((float)(dx - (double)hx), (float)(dy - (double)hy), (float)(dz - (double)hz), 0.f);
        if (vx) {
            const double ux = (double)vx[i], uy = (double)vy[i], uz = (double)vz[i];
            const float gx = (float)ux, gy = (float)uy, gz = (float)uz;
            P.vel[k] = make_float4(gx, gy, gz, 0.f);
            P.vlo[k] = split ? make_float4((float)(ux - (double)gx), (float)(uy - (double)gy),
                                           (float)(uz - (double)gz), 0.f)
                             : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

static unsigned grid_for(long long n, int threads, int max_blocks) {
    long long b = (n + threads - 1) / threads;
    if (b > max_blocks) b = max_blocks;
    if (b < 1) b = 1;
    return (unsigned)b;
}

void launch_upload_f64(long long n, const double* x, const double* y, const double* z, const double* vx,
                       const double* vy, const double* vz, const double* m, const Particles& P, bool split,
                       cudaStream_t s) {
    upload_kernel<double><<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, x, y, z, vx, vy, vz, m, P, split ? 1 : 0);
}

void launch_upload_f32(long long n, const float* x, const float* y, const float* z, const float* vx,
                       const float* vy, const float* vz, const float* m, const Particles& P, bool split,
                       cudaStream_t s) {
    upload_kernel<float><<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, x, y, z, vx, vy, vz, m, P, split ? 1 : 0);
}

void launch_state_f64(long long n, const double* x, const double* y, const double* z, const double* vx,
                      const double* vy, const double* vz, const Particles& P, bool split, cudaStream_t s) {
    state_kernel<double><<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, x, y, z, vx, vy, vz, P, split ? 1 : 0);
}

void launch_state_f32(long long n, const float* x, const float* y, const float* z, const float* vx,
                      const float* vy, const float* vz, const Particles& P, bool split, cudaStream_t s) {
    state_kernel<float><<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, x, y, z, vx, vy, vz, P, split ? 1 : 0);
}

// out[id[k]] = value of slot k, as FP64, for positions (hi + lo), velocities
// or accelerations.
__global__ void download_kernel(long long n, const int* __restrict__ id, const float4* __restrict__ a,
                                const float4* __restrict__ alo, double* __restrict__ ox, double* __restrict__ oy,
                                double* __restrict__ oz) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const float4 v = a[k];
        double x = v.x, y = v.y, z = v.z;
        if (alo) {
            const float4 l = alo[k];
            x += (double)l.x;
            y += (double)l.y;
            z += (double)l.z;
        }
        const int i = id[k];
        ox[i] = x;
        oy[i] = y;
        oz[i] = z;
    }
}

void launch_download(long long n, const int* id, const float4* a, const float4* alo, double* ox, double* oy,
                     double* oz, cudaStream_t s) {
    download_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, id, a, alo, ox, oy, oz);
}

// Frame fields in input order as N x 3 FP32 rows, each component the FP64
// state value rounded once (the static_cast<float> of DeckSim::Snapshot).
__global__ void frame_download_kernel(long long n, const int* __restrict__ id, const float4* __restrict__ pos,
                                      const float4* __restrict__ plo, const float4* __restrict__ vel,
                                      const float4* __restrict__ vlo, float* __restrict__ opos,
                                      float* __restrict__ ovel) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long i = 3LL * id[k];
        if (opos) {
            const float4 p = pos[k];
            if (plo) {
                const float4 l = plo[k];
                opos[i + 0] = (float)((double)p.x + (double)l.x);
                opos[i + 1] = (float)((double)p.y + (double)l.y);
                opos[i + 2] = (float)((double)p.z + (double)l.z);
            } else {
                opos[i + 0] = p.x;
                opos[i + 1] = p.y;
                opos[i + 2] = p.z;
            }
        }
        if (ovel) {
            const float4 v = vel[k];
            if (vlo) {
                const float4 l = vlo[k];
                ovel[i + 0] = (float)((double)v.x + (double)l.x);
                ovel[i + 1] = (float)((double)v.y + (double)l.y);
                ovel[i + 2] = (float)((double)v.z + (double)l.z);
            } else {
                ovel[i + 0] = v.x;
                ovel[i + 1] = v.y;
                ovel[i + 2] = v.z;
            }
        }
    }
}

void launch_frame_download(long long n, const int* id, const float4* pos, const float4* plo, const float4* vel,
                           const float4* vlo, float* opos, float* ovel, cudaStream_t s) {
    frame_download_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, id, pos, plo, vel, vlo, opos, ovel);
}

__global__ void rung_download_kernel(long long n, const int* __restrict__ id, const float4* __restrict__ vel,
                                     int* __restrict__ out) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        out[id[k]] = (int)vel[k].w;
}

void launch_rung_download(long long n, const int* id, const float4* vel, int* out, cudaStream_t s) {
    rung_download_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, id, vel, out);
}

__global__ void inverse_id_kernel(long long n, const int* __restrict__ id, int* __restrict__ inv) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        inv[id[k]] = (int)k;
}

void launch_inverse_id(long long n, const int* id, int* inv, cudaStream_t s) {
    inverse_id_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, id, inv);
}

__global__ void gather_slots_kernel(const int* __restrict__ inv, const int* __restrict__ targets, int nt,
                                    int* __restrict__ slots) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nt) slots[k] = inv[targets[k]];
}

void launch_gather_slots(const int* inv, const int* targets, int nt, int* slots, cudaStream_t s) {
    if (nt > 0) gather_slots_kernel<<<(nt + 255) / 256, 256, 0, s>>>(inv, targets, nt, slots);
}

// ---------------------------------------------------------------------------
// Opening kick + drift (+ the bounding box of the drifted positions)
// ---------------------------------------------------------------------------

template <bool SPLIT>
__global__ void __launch_bounds__(256) kick_drift_kernel(long long n, float4* __restrict__ pos,
                                                         float4* __restrict__ plo, float4* __restrict__ vel,
                                                         float4* __restrict__ vlo, const float4* __restrict__ acc,
                                                         float hdt, float dt, Counters* C) {
    double lo[3] = {1.0 / 0.0, 1.0 / 0.0, 1.0 / 0.0};
    double hi[3] = {-1.0 / 0.0, -1.0 / 0.0, -1.0 / 0.0};
    bool bad = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 v = vel[i];
        float4 vl = SPLIT ? vlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 a = acc[i];
        kick_v(v, SPLIT ? &vl : nullptr, hdt, a);
        vel[i] = v;
        if (SPLIT) vlo[i] = vl;
        float4 p = pos[i];
        double q[3];
        if (SPLIT) {
            float4 l = plo[i];
            float* ph = &p.x;
            float* pl = &l.x;
            const float dv[3] = {fmaf(dt, v.x, dt * vl.x), fmaf(dt, v.y, dt * vl.y), fmaf(dt, v.z, dt * vl.z)};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                // two-sum of hi + d, error folded into lo, then renormalised
                const float s = ph[k] + dv[k];
                const float bb = s - ph[k];
                const float e = (ph[k] - (s - bb)) + (dv[k] - bb);
                const float lo2 = pl[k] + e;
                const float h2 = s + lo2;
                pl[k] = lo2 - (h2 - s);
                ph[k] = h2;
                q[k] = (double)ph[k] + (double)pl[k];
            }
            plo[i] = l;
        } else {
            p.x = fmaf(dt, v.x, p.x);
            p.y = fmaf(dt, v.y, p.y);
            p.z = fmaf(dt, v.z, p.z);
            q[0] = p.x;
            q[1] = p.y;
            q[2] = p.z;
        }
        pos[i] = p;
        bad |= !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z));
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = fmin(lo[k], q[k]);
            hi[k] = fmax(hi[k], q[k]);
        }
    }
    __shared__ double slo[3][8], shi[3][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double l = lo[k], h = hi[k];
        for (int o = 16; o > 0; o >>= 1) {
            l = fmin(l, __shfl_xor_sync(0xffffffffu, l, o));
            h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
        }
        if (lane == 0) {
            slo[k][w] = l;
            shi[k][w] = h;
        }
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        double l = slo[k][0], h = shi[k][0];
        for (int j = 1; j < 8; ++j) {
            l = fmin(l, slo[k][j]);
            h = fmax(h, shi[k][j]);
        }
        atomicMin(&C->bbox_min[k], enc_f64_k(l));
        atomicMax(&C->bbox_max[k], enc_f64_k(h));
    }
    if (threadIdx.x == 0 && bad) atomicOr(&C->status, kStNonFinite);
}

void launch_kick_drift(const Particles& P, long long n, float hdt, float dt, bool split, Counters* C,
                       cudaStream_t s) {
    const unsigned b = grid_for(n, 256, 152 * 8);
    if (split)
        kick_drift_kernel<true><<<b, 256, 0, s>>>(n, P.pos, P.plo, P.vel, P.vlo, P.acc, hdt, dt, C);
    else
        kick_drift_kernel<false><<<b, 256, 0, s>>>(n, P.pos, nullptr, P.vel, nullptr, P.acc, hdt, dt, C);
}

// ---------------------------------------------------------------------------
// FP64 diagnostics
// ---------------------------------------------------------------------------

constexpr int kDiagThreads = 256;

__device__ __forceinline__ double block_sum_d(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    return t;
}

__device__ __forceinline__ void load_state_d(long long i, const float4* pos, const float4* plo, const float4* vel,
                                             const float4* vlo, double& x, double& y, double& z, double& vx,
                                             double& vy, double& vz, double& m) {
    const float4 p = pos[i];
    x = p.x;
    y = p.y;
    z = p.z;
    if (plo) {
        const float4 l = plo[i];
        x += (double)l.x;
        y += (double)l.y;
        z += (double)l.z;
    }
    m = p.w;
    const float4 v = vel[i];
    vx = v.x;
    vy = v.y;
    vz = v.z;
    if (vlo) {
        const float4 l = vlo[i];
        vx += (double)l.x;
        vy += (double)l.y;
        vz += (double)l.z;
    }
}

// Pass 1: per block {M, Mx, My, Mz, KE, Px, Py, Pz}.
__global__ void __launch_bounds__(kDiagThreads) diag_pass1_kernel(long long n, const float4* __restrict__ pos,
                                                                  const float4* __restrict__ plo,
                                                                  const float4* __restrict__ vel,
                                                                  const float4* __restrict__ vlo,
                                                                  double* __restrict__ partial) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double x, y, z, vx, vy, vz, m;
        load_state_d(i, pos, plo, vel, vlo, x, y, z, vx, vy, vz, m);
        acc[0] += m;
        acc[1] += m * x;
        acc[2] += m * y;
        acc[3] += m * z;
        acc[4] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        acc[5] += m * vx;
        acc[6] += m * vy;
        acc[7] += m * vz;
    }
    __shared__ double sh[32];
    for (int k = 0; k < 8; ++k) {
        const double t = block_sum_d(acc[k], sh);
        if (threadIdx.x == 0) partial[blockIdx.x * 8 + k] = t;
    }
}

// Pass 2: per block {Lx, Ly, Lz} about the given COM.
__global__ void __launch_bounds__(kDiagThreads) diag_pass2_kernel(long long n, const float4* __restrict__ pos,
                                                                  const float4* __restrict__ plo,
                                                                  const float4* __restrict__ vel,
                                                                  const float4* __restrict__ vlo, double cx,
                                                                  double cy, double cz, double* __restrict__ partial) {
    double L[3] = {0, 0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double x, y, z, vx, vy, vz, m;
        load_state_d(i, pos, plo, vel, vlo, x, y, z, vx, vy, vz, m);
        const double rx = x - cx, ry = y - cy, rz = z - cz;
        L[0] += m * (ry * vz - vy * rz);
        L[1] += m * (rz * vx - vz * rx);
        L[2] += m * (rx * vy - vx * ry);
    }
    __shared__ double sh[32];
    for (int k = 0; k < 3; ++k) {
        const double t = block_sum_d(L[k], sh);
        if (threadIdx.x == 0) partial[blockIdx.x * 3 + k] = t;
    }
}

int diag_blocks(long long n) { return (int)grid_for(n, kDiagThreads, 152 * 2); }

void launch_diag_pass1(long long n, const Particles& P, bool split, double* partial, cudaStream_t s) {
    diag_pass1_kernel<<<diag_blocks(n), kDiagThreads, 0, s>>>(n, P.pos, split ? P.plo : nullptr, P.vel,
                                                               split ? P.vlo : nullptr, partial);
}

void launch_diag_pass2(long long n, const Particles& P, bool split, double cx, double cy, double cz, double* partial,
                       cudaStream_t s) {
    diag_pass2_kernel<<<diag_blocks(n), kDiagThreads, 0, s>>>(n, P.pos, split ? P.plo : nullptr, P.vel,
                                                               split ? P.vlo : nullptr, cx, cy, cz,
                                                              partial);
}

// Exact pair potential: thread i sums j > i over shared-memory tiles, in FP64.
constexpr int kPotThreads = 256;

// spline_h > 0: the spline pair potential of smoothing length spline_h
// (softening.cuh); else Plummer with eps2.
__global__ void __launch_bounds__(kPotThreads) potential_kernel(long long n, const float4* __restrict__ pos,
                                                                const float4* __restrict__ plo, double eps2,
                                                                double spline_h, double* __restrict__ partial) {
    __shared__ double sx[kPotThreads], sy[kPotThreads], sz[kPotThreads], sm[kPotThreads];
    __shared__ double red[32];
    const long long i = blockIdx.x * (long long)kPotThreads + threadIdx.x;
    double xi = 0, yi = 0, zi = 0, mi = 0;
    if (i < n) {
        const float4 p = pos[i];
        xi = p.x;
        yi = p.y;
        zi = p.z;
        mi = p.w;
        if (plo) {
            const float4 l = plo[i];
            xi += (double)l.x;
            yi += (double)l.y;
            zi += (double)l.z;
        }
    }
    double local = 0.0;
    const long long first_tile = blockIdx.x * (long long)kPotThreads;
    for (long long t = first_tile; t < n; t += kPotThreads) {
        const long long j = t + threadIdx.x;
        __syncthreads();
        if (j < n) {
            const float4 p = pos[j];
            double x = p.x, y = p.y, z = p.z;
            if (plo) {
                const float4 l = plo[j];
                x += (double)l.x;
                y += (double)l.y;
                z += (double)l.z;
            }
            sx[threadIdx.x] = x;
            sy[threadIdx.x] = y;
            sz[threadIdx.x] = z;
            sm[threadIdx.x] = p.w;
        }
        __syncthreads();
        if (i < n) {
            const int kmax = (int)min((long long)kPotThreads, n - t);
            for (int k = 0; k < kmax; ++k) {
                if (t + k <= i) continue;
                const double dx = sx[k] - xi, dy = sy[k] - yi, dz = sz[k] - zi;
                if (spline_h > 0.0) {
                    const double r = sqrt(dx * dx + dy * dy + dz * dz);
                    local += sm[k] * spline_phi_d(r / spline_h) / spline_h;
                } else {
                    const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                    local -= sm[k] * rsqrt(r2);
                }
            }
        }
    }
    local *= mi;
    const double t = block_sum_d(local, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

int potential_blocks(long long n) { return (int)((n + kPotThreads - 1) / kPotThreads); }

// The same pair set (every i < j, Plummer) with FP32 pair terms and FP64
// sums, for sizes where the FP64 pipe is too slow (n = 4M: 8.8e12 pairs).
// Thread = target i; sources staged through shared memory as double-float
// positions, each offset formed as (hi_j - hi_i) + (lo_j - lo_i) in FP32 (an
// error of order 2^-24 of the separation, not of |x|); a tile's FP32
// partial joins the thread's FP64 sum per tile.  Block b of B takes target
// tiles b, 2B-1-b, 2B+b, 4B-1-b, ...: a long and a short row of the
// triangle in turn, so the blocks finish together.
constexpr int kPot32Threads = 256;

__device__ double pot32_tile(long long n, long long t0, const float4* __restrict__ pos,
                             const float4* __restrict__ plo, float eps2, float4* sh, float4* sl) {
    const long long i = t0 + threadIdx.x;
    float4 th = make_float4(0.f, 0.f, 0.f, 0.f), tl = th;
    if (i < n) {
        th = pos[i];
        if (plo) tl = plo[i];
    }
    double sum = 0.0;
    for (long long s0 = t0; s0 < n; s0 += kPot32Threads) {
        const long long j = s0 + threadIdx.x;
        __syncthreads();
        sh[threadIdx.x] = j < n ? pos[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        sl[threadIdx.x] = (j < n && plo) ? plo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        if (i >= n) continue;
        const int kmax = (int)min((long long)kPot32Threads, n - s0);
        const int k0 = s0 == t0 ? (int)threadIdx.x + 1 : 0;  // j > i
        float part = 0.f;
        for (int k = k0; k < kmax; ++k) {
            const float4 h = sh[k], l = sl[k];
            const float dx = (h.x - th.x) + (l.x - tl.x);
            const float dy = (h.y - th.y) + (l.y - tl.y);
            const float dz = (h.z - th.z) + (l.z - tl.z);
            part = fmaf(h.w, rsqrtf(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)))), part);
        }
        sum += (double)part;
    }
    return -(double)th.w * sum;
}

__global__ void __launch_bounds__(kPot32Threads) potential_f32_kernel(long long n, const float4* __restrict__ pos,
                                                                      const float4* __restrict__ plo, float eps2,
                                                                      double* __restrict__ partial) {
    __shared__ float4 sh[kPot32Threads], sl[kPot32Threads];
    __shared__ double red[32];
    const long long ntiles = (n + kPot32Threads - 1) / kPot32Threads;
    const long long B = gridDim.x, b = blockIdx.x;
    double local = 0.0;
    for (long long base = 0; base < ntiles; base += 2 * B) {
        const long long ta = base + b, tb = base + 2 * B - 1 - b;
        if (ta < ntiles) local += pot32_tile(n, ta * kPot32Threads, pos, plo, eps2, sh, sl);
        if (tb < ntiles) local += pot32_tile(n, tb * kPot32Threads, pos, plo, eps2, sh, sl);
    }
    const double t = block_sum_d(local, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

int potential_f32_blocks(long long n, int sm_count) {
    const long long ntiles = (n + kPot32Threads - 1) / kPot32Threads;
    const long long want = 8LL * std::max(sm_count, 1);
    return (int)std::max<long long>(1, std::min(ntiles, want));
}

void launch_potential_f32(long long n, const Particles& P, bool split, double eps2, int blocks, double* partial,
                          cudaStream_t s) {
    potential_f32_kernel<<<blocks, kPot32Threads, 0, s>>>(n, P.pos, split ? P.plo : nullptr, (float)eps2, partial);
}

void launch_potential(long long n, const Particles& P, bool split, double eps2, double spline_h, double* partial,
                      cudaStream_t s) {
    potential_kernel<<<potential_blocks(n), kPotThreads, 0, s>>>(n, P.pos, split ? P.plo : nullptr, eps2, spline_h,
                                                                 partial);
}

// ---------------------------------------------------------------------------
// Block (power-of-two rung) timesteps, System::BlockStep (System.hpp:239-294):
// rung_k = min(max_rung, ceil(log2(dt / tau))) with tau = eta sqrt(eps / |a|)
// (0 when tau >= dt or |a| = 0), stored in vel.w so it travels with the
// particle through every re-sort; per finest substep the particles whose rung
// step starts there take their opening half-kick, then everyone drifts.
// ---------------------------------------------------------------------------

__global__ void rung_kernel(long long n, float4* __restrict__ vel, const float4* __restrict__ acc, double base,
                            double eta, double eps, int max_rung, int* __restrict__ rmax) {
    int local = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 a = acc[i];
        const double amag = sqrt((double)a.x * a.x + (double)a.y * a.y + (double)a.z * a.z);
        int k = 0;
        if (amag > 0.0 && eps > 0.0) {
            const double tau = eta * sqrt(eps / amag);
            if (tau < base) {
                const double r = ceil(log2(base / tau));
                k = r < (double)max_rung ? (int)r : max_rung;
            }
        }
        float4 v = vel[i];
        v.w = (float)k;
        vel[i] = v;
        local = max(local, k);
    }
    for (int o = 16; o > 0; o >>= 1) local = max(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0) atomicMax(rmax, local);
}

// max_i |a_i| as the bit pattern of a non-negative double (which orders
// like the unsigned integer), for the adaptive step rule.
__global__ void amax_kernel(long long n, const float4* __restrict__ acc, unsigned long long* __restrict__ out) {
    double local = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 a = acc[i];
        local = fmax(local, sqrt((double)a.x * a.x + (double)a.y * a.y + (double)a.z * a.z));
    }
    for (int o = 16; o > 0; o >>= 1) local = fmax(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(local));
}

void launch_amax(long long n, const float4* acc, unsigned long long* out, cudaStream_t s) {
    amax_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, s>>>(n, acc, out);
}

template <bool SPLIT>
__global__ void __launch_bounds__(256) block_kick_drift_kernel(long long n, float4* __restrict__ pos,
                                                               float4* __restrict__ plo, float4* __restrict__ vel,
                                                               float4* __restrict__ vlo,
                                                               const float4* __restrict__ acc, double base, int sub,
                                                               int rmax, float dtmin) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 v = vel[i];
        float4 vl = SPLIT ? vlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const int rung = (int)v.w;
        const int units = 1 << (rmax - rung);
        if (sub % units == 0) {
            const float h = (float)(0.5 * base / (double)(1 << rung));
            kick_v(v, SPLIT ? &vl : nullptr, h, acc[i]);
            vel[i] = v;
            if (SPLIT) vlo[i] = vl;
        }
        float4 p = pos[i];
        if (SPLIT) {
            float4 l = plo[i];
            float* ph = &p.x;
            float* pl = &l.x;
            const float dv[3] = {fmaf(dtmin, v.x, dtmin * vl.x), fmaf(dtmin, v.y, dtmin * vl.y),
                                 fmaf(dtmin, v.z, dtmin * vl.z)};
#pragma unroll
            for (int k = 0; k < 3; ++k) {  // (hi, lo) += d with an error-free two-sum
                const float s = ph[k] + dv[k];
                const float bb = s - ph[k];
                const float err = (ph[k] - (s - bb)) + (dv[k] - bb);
                const float lo = pl[k] + err;
                const float hi2 = s + lo;
                pl[k] = lo - (hi2 - s);
                ph[k] = hi2;
            }
            plo[i] = l;
        } else {
            p.x = fmaf(dtmin, v.x, p.x);
            p.y = fmaf(dtmin, v.y, p.y);
            p.z = fmaf(dtmin, v.z, p.z);
        }
        pos[i] = p;
    }
}

void launch_rungs(long long n, const Particles& P, double base, double eta, double eps, int max_rung, int* rmax,
                  cudaStream_t s) {
    rung_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, P.vel, P.acc, base, eta, eps, max_rung, rmax);
}

void launch_block_kick_drift(long long n, const Particles& P, bool split, double base, int sub, int rmax, float dtmin,
                             cudaStream_t s) {
    if (split)
        block_kick_drift_kernel<true><<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, P.pos, P.plo, P.vel, P.vlo,
                                                                                 P.acc, base, sub, rmax, dtmin);
    else
        block_kick_drift_kernel<false><<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, P.pos, nullptr, P.vel, nullptr,
                                                                                  P.acc, base, sub, rmax, dtmin);
}

// ---------------------------------------------------------------------------
// Direct-sum force-error sampler.  FP64 pairs: one block per target slot.
// ---------------------------------------------------------------------------

constexpr int kSampThreads = 256;

__global__ void __launch_bounds__(kSampThreads) sampler_kernel(long long n, const float4* __restrict__ pos,
                                                               const float4* __restrict__ plo,
                                                               const int* __restrict__ slots, double eps2,
                                                               double spline_h, double* __restrict__ out) {
    __shared__ double red[32];
    const int ti = slots[blockIdx.x];
    const float4 tp = pos[ti];
    const float4 tl = plo ? plo[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
    double ax = 0.0, ay = 0.0, az = 0.0;
    const double xi = (double)tp.x + (double)tl.x, yi = (double)tp.y + (double)tl.y, zi = (double)tp.z + (double)tl.z;
    for (long long j = threadIdx.x; j < n; j += kSampThreads) {
        if (j == ti) continue;
        const float4 p = pos[j];
        double x = p.x, y = p.y, z = p.z;
        if (plo) {
            const float4 l = plo[j];
            x += (double)l.x;
            y += (double)l.y;
            z += (double)l.z;
        }
        const double dx = x - xi, dy = y - yi, dz = z - zi;
        double s;
        if (spline_h > 0.0) {
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double r = sqrt(r2);
            s = r2 > 0.0 ? (double)p.w * spline_chi_d(r / spline_h) / (r2 * r) : 0.0;
        } else {
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double inv = rsqrt(r2);
            s = (double)p.w * inv * inv * inv;
        }
        ax += s * dx;
        ay += s * dy;
        az += s * dz;
    }
    const double sx = block_sum_d(ax, red);
    const double sy = block_sum_d(ay, red);
    const double sz = block_sum_d(az, red);
    if (threadIdx.x == 0) {
        out[3 * blockIdx.x + 0] = sx;
        out[3 * blockIdx.x + 1] = sy;
        out[3 * blockIdx.x + 2] = sz;
    }
}

// ---------------------------------------------------------------------------
// FP32 FMA throughput probe: 8 independent register-resident FMA chains per
// thread, no memory traffic inside the loop.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) fma_probe_kernel(float* __restrict__ out, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f, x4 = x0 + 4.f, x5 = x0 + 5.f,
          x6 = x0 + 6.f, x7 = x0 + 7.f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            x0 = fmaf(x0, a, b);
            x1 = fmaf(x1, a, b);
            x2 = fmaf(x2, a, b);
            x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b);
            x5 = fmaf(x5, a, b);
            x6 = fmaf(x6, a, b);
            x7 = fmaf(x7, a, b);
        }
    }
    const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains live
}

// Returns TFLOP/s (2 flops per FMA) of one timed launch after a warm-up.
double run_fma_probe(int sm_count, cudaStream_t s) {
    const int blocks = sm_count * 8, threads = 256, iters = 1024;
    float* out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * blocks) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_probe_kernel<<<blocks, threads, 0, s>>>(out, iters, 0.9999999f, 1e-7f);
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0, s);
        fma_probe_kernel<<<blocks, threads, 0, s>>>(out, iters, 0.9999999f, 1e-7f);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double fmas = (double)blocks * threads * iters * 64.0;
    return 2.0 * fmas / (best * 1e-3) / 1e12;
}

// FP32 pairs, tiled: a block holds 512 targets (two per thread, sharing each
// source read from shared memory) and streams one contiguous share of the
// sources through shared memory; each source tile is summed in FP32 and added
// to the thread's FP64 totals.  Partial sums per (share, target) are reduced
// in share order by sampler_reduce_kernel.  The self pair needs no test: its
// separation is exactly zero, so it adds zero (with eps > 0, and for the
// spline, whose factor is 0 at r = 0); only the unsoftened Plummer form
// (MASK0) masks r = 0.
constexpr int kSampTile = 256;
constexpr int kSampBlockTargets = 2 * kSampTile;

template <int SOFT, bool SPLIT, bool MASK0>
__device__ __forceinline__ void samp_pair(const float4& p, const float4& l, const float4& t, const float4& tl,
                                          float eps2, float ih, float& px, float& py, float& pz) {
    float dx = p.x - t.x, dy = p.y - t.y, dz = p.z - t.z;
    if (SPLIT) {
        dx += l.x - tl.x;
        dy += l.y - tl.y;
        dz += l.z - tl.z;
    }
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float f = pair_factor<SOFT>(r2, p.w, eps2, ih);
    if (MASK0) f = r2 > 0.f ? f : 0.f;
    px = fmaf(f, dx, px);
    py = fmaf(f, dy, py);
    pz = fmaf(f, dz, pz);
}

template <int SOFT, bool SPLIT, bool MASK0>
__global__ void __launch_bounds__(kSampTile) sampler_tiled_kernel(long long n, const float4* __restrict__ pos,
                                                                 const float4* __restrict__ plo,
                                                                 const int* __restrict__ slots, int nslots,
                                                                 float eps2, float ih, long long share,
                                                                 double* __restrict__ partial) {
    __shared__ float4 sp[kSampTile];
    __shared__ float4 sl[SPLIT ? kSampTile : 1];
    const int t0 = blockIdx.x * kSampBlockTargets + threadIdx.x, t1 = t0 + kSampTile;
    const bool v0 = t0 < nslots, v1 = t1 < nslots;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 ta = v0 ? pos[slots[t0]] : zero, tb = v1 ? pos[slots[t1]] : zero;
    const float4 tla = (v0 && SPLIT) ? plo[slots[t0]] : zero, tlb = (v1 && SPLIT) ? plo[slots[t1]] : zero;
    const long long j0 = (long long)blockIdx.y * share;
    const long long j1 = j0 + share < n ? j0 + share : n;
    double ax = 0.0, ay = 0.0, az = 0.0, bx = 0.0, by = 0.0, bz = 0.0;
    for (long long base = j0; base < j1; base += kSampTile) {
        const long long j = base + threadIdx.x;
        sp[threadIdx.x] = j < j1 ? pos[j] : zero;
        if (SPLIT) sl[threadIdx.x] = j < j1 ? plo[j] : zero;
        __syncthreads();
        const int cnt = (int)(j1 - base < kSampTile ? j1 - base : kSampTile);
        float pax = 0.f, pay = 0.f, paz = 0.f, pbx = 0.f, pby = 0.f, pbz = 0.f;
        for (int k = 0; k < cnt; ++k) {
            const float4 p = sp[k];
            const float4 l = SPLIT ? sl[k] : zero;
            samp_pair<SOFT, SPLIT, MASK0>(p, l, ta, tla, eps2, ih, pax, pay, paz);
            samp_pair<SOFT, SPLIT, MASK0>(p, l, tb, tlb, eps2, ih, pbx, pby, pbz);
        }
        ax += pax;
        ay += pay;
        az += paz;
        bx += pbx;
        by += pby;
        bz += pbz;
        __syncthreads();
    }
    if (v0) {
        double* o = partial + ((long long)blockIdx.y * nslots + t0) * 3;
        o[0] = ax;
        o[1] = ay;
        o[2] = az;
    }
    if (v1) {
        double* o = partial + ((long long)blockIdx.y * nslots + t1) * 3;
        o[0] = bx;
        o[1] = by;
        o[2] = bz;
    }
}

__global__ void sampler_reduce_kernel(const double* __restrict__ partial, int nslots, int shares,
                                      double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * nslots) return;
    double s = 0.0;
    for (int k = 0; k < shares; ++k) s += partial[(long long)k * 3 * nslots + i];
    out[i] = s;
}

int sampler_shares(long long n, int nslots, int sm_count) {
    const int tb = (nslots + kSampBlockTargets - 1) / kSampBlockTargets;
    long long sh = ((long long)sm_count * 4 + tb - 1) / tb;
    const long long max_sh = (n + kSampTile - 1) / kSampTile;
    if (sh > max_sh) sh = max_sh;
    return (int)(sh < 1 ? 1 : sh);
}

void launch_sampler(long long n, const Particles& P, bool split, const int* slots, int nslots, double eps2,
                    double spline_h, bool fp64_pairs, double* out, double* partial, int shares, cudaStream_t s) {
    if (nslots <= 0) return;
    if (fp64_pairs) {
        sampler_kernel<<<nslots, kSampThreads, 0, s>>>(n, P.pos, split ? P.plo : nullptr, slots, eps2, spline_h, out);
        return;
    }
    long long share = (n + shares - 1) / shares;
    share = (share + kSampTile - 1) / kSampTile * kSampTile;
    const dim3 grid((nslots + kSampBlockTargets - 1) / kSampBlockTargets, shares);
    const float ih = spline_h > 0.0 ? (float)(1.0 / spline_h) : 0.f;
    const float4* lo = split ? P.plo : nullptr;
#define NGRAV_SAMP(SOFT, SP, M0) \
    sampler_tiled_kernel<SOFT, SP, M0><<<grid, kSampTile, 0, s>>>(n, P.pos, lo, slots, nslots, (float)eps2, ih, share, partial)
    if (spline_h > 0.0) {
        if (split) NGRAV_SAMP(kSoftSpline, true, false);
        else NGRAV_SAMP(kSoftSpline, false, false);
    } else if (eps2 > 0.0) {
        if (split) NGRAV_SAMP(kSoftPlummer, true, false);
        else NGRAV_SAMP(kSoftPlummer, false, false);
    } else {
        if (split) NGRAV_SAMP(kSoftPlummer, true, true);
        else NGRAV_SAMP(kSoftPlummer, false, true);
    }
#undef NGRAV_SAMP
    sampler_reduce_kernel<<<(3 * nslots + 255) / 256, 256, 0, s>>>(partial, nslots, shares, out);
}

}  // namespace ngrav
