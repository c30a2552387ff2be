// noalloc.cu -- FP64 conservation diagnostics over caller-owned device arrays
// with no device allocation at all.
//
// Some callers cannot allocate device memory: a simulation loop that runs
// under a framework's caching allocator which owns (and may have reserved)
// all of the device's memory; an application that has to keep
// cudaMalloc/cudaFree out of its frame loop because cudaFree synchronises
// the whole device and stalls its other streams; a host program with a fixed
// device-memory budget.  ngrav_gpu_diagnostics_noalloc serves them: the
// caller passes the particle arrays (already on the device) and a host
// result struct, and the block partial sums the reductions need live in the
// file-scope array below instead of in memory allocated per call.
//
// The scratch array is a static __device__ symbol: every GPU that loads this
// library holds its 256 KiB until the process exits.  In host code the name
// g_noalloc_scratch is only a host-side stand-in for the symbol, not a
// device address, so the host never passes it to a kernel; instead, on the
// first call on each device (with that device current) the address is looked
// up once with cudaGetSymbolAddress and cached.  Because that set-up happens
// on a device's first call, make the first call before any stream capture.
// Every call on a device shares the same scratch: two calls whose work
// overlaps on the GPU (different host threads or streams) race and must be
// serialised by the caller.  Each call overwrites every partial it reads, so
// nothing needs clearing between calls.
//
// The potential is the exact O(N^2) FP64 sum of the Plummer pair potential
// -G m_i m_j / sqrt(r^2 + eps^2) (System::TotalEnergy,
// include/ngrav/System.hpp:119-164, with Plummer softening only).  It runs
// as its own kernel: targets in tiles of 256 (one per thread), sources j > i
// staged through shared memory, every block taking a light and a heavy
// target tile of the triangle in turn so the blocks finish together.  Its
// cost is n^2 / 2 FP64 pair terms: about 1 s at n = 262,144 on one GB300
// (FP64 on the CUDA cores), and about 4,000 times that, above an hour, at
// the 16,777,216-particle maximum -- ask for it only at sizes where that
// fits.
#include "ngrav_gpu.h"

#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

namespace {

constexpr int kThreads = 256;
constexpr long long kPerBlock = 4096;                   // particles per block of passes 1 and 2
constexpr int kMaxBlocks = NGRAV_NOALLOC_MAX_N / 4096;  // 4096 blocks
constexpr int kSlots = 8;                               // doubles per block partial
constexpr int kPotTile = kThreads;                      // potential: targets and sources per tile

// kMaxBlocks rows of block partials + 2 rows of pass totals: 262,160 bytes.
static __device__ __align__(256) double g_noalloc_scratch[(kMaxBlocks + 2) * kSlots];

constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_setup_mutex;

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < kThreads / 32; ++k) t += sh[k];
    return t;
}

// Pass 1, block b covers particles [b*4096, (b+1)*4096): {M, Mx, My, Mz, KE, Px, Py, Pz}.
__global__ void __launch_bounds__(kThreads) na_pass1(long long n, const float* __restrict__ x,
                                                     const float* __restrict__ y, const float* __restrict__ z,
                                                     const float* __restrict__ vx, const float* __restrict__ vy,
                                                     const float* __restrict__ vz, const float* __restrict__ m,
                                                     double* __restrict__ scratch) {
    __shared__ double sh[kThreads / 32];
    double a[kSlots] = {0, 0, 0, 0, 0, 0, 0, 0};
    const long long lo = blockIdx.x * kPerBlock, hi = min(n, lo + kPerBlock);
    for (long long i = lo + threadIdx.x; i < hi; i += kThreads) {
        const double mi = m[i], xi = x[i], yi = y[i], zi = z[i], u = vx[i], v = vy[i], w = vz[i];
        a[0] += mi;
        a[1] += mi * xi;
        a[2] += mi * yi;
        a[3] += mi * zi;
        a[4] += 0.5 * mi * (u * u + v * v + w * w);
        a[5] += mi * u;
        a[6] += mi * v;
        a[7] += mi * w;
    }
    for (int k = 0; k < kSlots; ++k) {
        const double t = block_sum(a[k], sh);
        if (threadIdx.x == 0) scratch[blockIdx.x * kSlots + k] = t;
    }
}

// Pass 2: {Lx, Ly, Lz} about the COM; slot 3 is zeroed for the potential pass.
__global__ void __launch_bounds__(kThreads) na_pass2(long long n, const float* __restrict__ x,
                                                     const float* __restrict__ y, const float* __restrict__ z,
                                                     const float* __restrict__ vx, const float* __restrict__ vy,
                                                     const float* __restrict__ vz, const float* __restrict__ m,
                                                     const double* __restrict__ com, double* __restrict__ scratch) {
    __shared__ double sh[kThreads / 32];
    const double cx = com[0], cy = com[1], cz = com[2];
    double L[3] = {0, 0, 0};
    const long long lo = blockIdx.x * kPerBlock, hi = min(n, lo + kPerBlock);
    for (long long i = lo + threadIdx.x; i < hi; i += kThreads) {
        const double mi = m[i], rx = x[i] - cx, ry = y[i] - cy, rz = z[i] - cz;
        const double u = vx[i], v = vy[i], w = vz[i];
        L[0] += mi * (ry * w - v * rz);
        L[1] += mi * (rz * u - w * rx);
        L[2] += mi * (rx * v - u * ry);
    }
    const double t0 = block_sum(L[0], sh), t1 = block_sum(L[1], sh), t2 = block_sum(L[2], sh);
    if (threadIdx.x == 0) {
        scratch[blockIdx.x * kSlots + 0] = t0;
        scratch[blockIdx.x * kSlots + 1] = t1;
        scratch[blockIdx.x * kSlots + 2] = t2;
        scratch[blockIdx.x * kSlots + 3] = 0.0;
    }
}

// Sum over j > i of -m_i m_j / sqrt(r^2 + eps^2) for the targets of one
// tile (thread = target), the sources staged kPotTile at a time.
__device__ double pot_tile(long long n, long long t0, const float* __restrict__ x, const float* __restrict__ y,
                           const float* __restrict__ z, const float* __restrict__ m, double eps2, double* sx,
                           double* sy, double* sz, double* sm) {
    const long long i = t0 + threadIdx.x;
    double xi = 0.0, yi = 0.0, zi = 0.0, mi = 0.0;
    if (i < n) {
        xi = x[i];
        yi = y[i];
        zi = z[i];
        mi = m[i];
    }
    double local = 0.0;
    for (long long s0 = t0; s0 < n; s0 += kPotTile) {  // source tiles from the target tile on
        const long long j = s0 + threadIdx.x;
        __syncthreads();
        if (j < n) {
            sx[threadIdx.x] = x[j];
            sy[threadIdx.x] = y[j];
            sz[threadIdx.x] = z[j];
            sm[threadIdx.x] = m[j];
        }
        __syncthreads();
        if (i < n) {
            const int kmax = (int)min((long long)kPotTile, n - s0);
            for (int k = 0; k < kmax; ++k) {
                if (s0 + k <= i) continue;
                const double dx = sx[k] - xi, dy = sy[k] - yi, dz = sz[k] - zi;
                local -= sm[k] * rsqrt(dx * dx + dy * dy + dz * dz + eps2);
            }
        }
    }
    return mi * local;
}

// Exact pair potential.  Block b takes target tiles b, 2B-1-b, 2B+b,
// 4B-1-b, ... of the ntiles: a tile near the start of the triangle (long)
// with one near its end (short), so the B blocks carry about equal work.
// Each block writes its sum to slot 3 of its own partial row; rows at or
// past nb_l (which pass 2 did not write) get zero angular momentum.
__global__ void __launch_bounds__(kThreads) na_potential(long long n, const float* __restrict__ x,
                                                         const float* __restrict__ y, const float* __restrict__ z,
                                                         const float* __restrict__ m, double eps2, int nb_l,
                                                         double* __restrict__ scratch) {
    __shared__ double sx[kPotTile], sy[kPotTile], sz[kPotTile], sm[kPotTile];
    __shared__ double sh[kThreads / 32];
    const long long ntiles = (n + kPotTile - 1) / kPotTile;
    const long long B = gridDim.x, b = blockIdx.x;
    double pot = 0.0;
    for (long long base = 0; base < ntiles; base += 2 * B) {
        const long long ta = base + b, tb = base + 2 * B - 1 - b;
        if (ta < ntiles) pot += pot_tile(n, ta * kPotTile, x, y, z, m, eps2, sx, sy, sz, sm);
        if (tb < ntiles) pot += pot_tile(n, tb * kPotTile, x, y, z, m, eps2, sx, sy, sz, sm);
    }
    const double t = block_sum(pot, sh);
    if (threadIdx.x == 0) {
        double* row = scratch + (size_t)blockIdx.x * kSlots;
        if ((int)blockIdx.x >= nb_l) row[0] = row[1] = row[2] = 0.0;
        row[3] = t;
    }
}

// Sums `nb` block partials slot-wise (fixed order: deterministic) into
// out[0..kSlots) of the same scratch region past the partials.
__global__ void na_reduce(int nb, double* __restrict__ scratch, double* __restrict__ out) {
    const int k = threadIdx.x;
    if (k < kSlots) {
        double s = 0.0;
        for (int b = 0; b < nb; ++b) s += scratch[b * kSlots + k];
        out[k] = s;
    }
}

// COM from the pass-1 totals, written to the scratch slot pass 2 reads.
__global__ void na_com(const double* __restrict__ tot, double* __restrict__ com) {
    const double M = tot[0];
    com[0] = M > 0.0 ? tot[1] / M : tot[1];
    com[1] = M > 0.0 ? tot[2] / M : tot[2];
    com[2] = M > 0.0 ? tot[3] / M : tot[3];
}

int scratch_for_current_device(int device, double** out) {
    if (device < 0 || device >= kMaxDevices) return NGRAV_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return NGRAV_ERR_CUDA;
        g_scratch_ptr[device] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[device];
    return NGRAV_OK;
}

// The work of one call with `device` current.
int run_diagnostics(int device, int64_t n, const float* x, const float* y, const float* z, const float* vx,
                    const float* vy, const float* vz, const float* m, double G, double eps, int with_potential,
                    ngrav_gpu_diag* out) {
    double* scratch = nullptr;
    const int rc = scratch_for_current_device(device, &scratch);
    if (rc) return rc;
    const int nb = (int)((n + kPerBlock - 1) / kPerBlock);
    // Layout: rows [0, nb) block partials (nb <= kMaxBlocks); row kMaxBlocks
    // the pass-1 totals; row kMaxBlocks + 1 the COM, then the pass-2 totals.
    double* tot1 = scratch + (size_t)kMaxBlocks * kSlots;
    double* tot2 = scratch + (size_t)(kMaxBlocks + 1) * kSlots;
    cudaStream_t s = 0;  // legacy default stream: ordered with the caller's default-stream work
    na_pass1<<<nb, kThreads, 0, s>>>(n, x, y, z, vx, vy, vz, m, scratch);
    na_reduce<<<1, 32, 0, s>>>(nb, scratch, tot1);
    na_com<<<1, 1, 0, s>>>(tot1, tot2);
    na_pass2<<<nb, kThreads, 0, s>>>(n, x, y, z, vx, vy, vz, m, tot2, scratch);
    int rows = nb;
    if (with_potential) {
        // one block per target tile up to the kMaxBlocks partial rows
        // (ntiles >= nb, so every row pass 2 wrote gets its potential)
        const long long ntiles = (n + kPotTile - 1) / kPotTile;
        rows = (int)(ntiles < kMaxBlocks ? ntiles : kMaxBlocks);
        na_potential<<<rows, kThreads, 0, s>>>(n, x, y, z, m, eps * eps, nb, scratch);
    }
    double h1[kSlots];
    if (cudaMemcpy(h1, tot1, sizeof(h1), cudaMemcpyDeviceToHost) != cudaSuccess) return NGRAV_ERR_CUDA;
    na_reduce<<<1, 32, 0, s>>>(rows, scratch, tot2);
    double h2[kSlots];
    if (cudaMemcpy(h2, tot2, sizeof(h2), cudaMemcpyDeviceToHost) != cudaSuccess) return NGRAV_ERR_CUDA;
    if (cudaGetLastError() != cudaSuccess) return NGRAV_ERR_CUDA;
    const double M = h1[0];
    out->kinetic = h1[4];
    for (int k = 0; k < 3; ++k) {
        out->com[k] = M > 0.0 ? h1[1 + k] / M : h1[1 + k];
        out->P[k] = h1[5 + k];
        out->L[k] = h2[k];
    }
    // Without the potential, potential and energy are NaN, as in
    // ngrav_gpu_diagnostics, so a drift computed from them cannot pass for
    // an energy drift.
    out->potential_exact = with_potential ? 1 : 0;
    out->potential = with_potential ? G * h2[3] : std::nan("");
    out->energy = out->kinetic + out->potential;
    return NGRAV_OK;
}

}  // namespace

extern "C" int ngrav_gpu_diagnostics_noalloc(int device, int64_t n, const float* x, const float* y, const float* z,
                                             const float* vx, const float* vy, const float* vz, const float* m,
                                             double G, double eps, int with_potential, ngrav_gpu_diag* out) {
    if (!out || n <= 0 || !x || !y || !z || !vx || !vy || !vz || !m) return NGRAV_ERR_INVALID_ARG;
    if (n > (int64_t)NGRAV_NOALLOC_MAX_N) return NGRAV_ERR_INVALID_ARG;  // beyond the static scratch
    // The caller's current device is put back before returning.
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return NGRAV_ERR_CUDA;
    if (device != prev && cudaSetDevice(device) != cudaSuccess) return NGRAV_ERR_CUDA;
    const int rc = run_diagnostics(device, n, x, y, z, vx, vy, vz, m, G, eps, with_potential, out);
    if (device != prev && cudaSetDevice(prev) != cudaSuccess) return rc ? rc : NGRAV_ERR_CUDA;
    return rc;
}
