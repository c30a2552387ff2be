// lmac_train.cu -- training of the learned opening test's network on the GPU:
// mini-batch assembly, forward + backward (binary cross-entropy on the logit),
// Adam.  All FP32; results are deterministic for a given seed (fixed sample
// order inside each block, fixed block order in the reduction).
//
// Samples: (x, r) with x the unit-budget features of a (group, node) pair and
// r its measured worst relative multipole error.  A batch draws pairs with
// replacement and places the budget at b = r * 2^u, u ~ U(-U, U), per draw:
//     f3 <- f3 - log2 b,     y = [r <= b] = [u >= 0],
// so the network learns P(r <= b | geometry, b) over the whole budget range.
#include "lmac.cuh"
#include "lmac_internal.cuh"

namespace ngrav {

__device__ __forceinline__ uint32_t train_hash(uint32_t a, uint32_t b) {
    uint32_t h = a * 0x9E3779B1u + b * 0x85EBCA77u + 0x165667B1u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}

// Xb[k] = standardised features, yb[k] = label, wb[k] = 1 (0 for samples
// whose label is unavailable).
__global__ void lmac_make_batch_kernel(const float* __restrict__ X, const float* __restrict__ r, long long n,
                                       LmacNorm norm, int nb, uint32_t seed, float u_range, int standardise,
                                       float* __restrict__ Xb, float* __restrict__ yb, float* __restrict__ wb) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += gridDim.x * blockDim.x) {
        const uint32_t h1 = train_hash(seed, (uint32_t)k);
        const uint32_t h2 = train_hash(h1, 0x5bd1e995u);
        const long long i = (long long)(((unsigned long long)h1 * (unsigned long long)n) >> 32);
        const float ri = r[i];
        const float u = ((float)(h2 >> 8) * (1.f / 16777216.f) * 2.f - 1.f) * u_range;
        const float log2r = ri > 0.f ? fmaxf(__log2f(ri), -40.f) : -40.f;
        float f[kLmacIn];
#pragma unroll
        for (int j = 0; j < kLmacIn; ++j) f[j] = X[i * kLmacIn + j];
        f[3] -= log2r + u;
#pragma unroll
        for (int j = 0; j < kLmacIn; ++j)
            Xb[(long long)k * kLmacIn + j] = standardise ? (f[j] - norm.mu[j]) * norm.isd[j] : f[j];
        yb[k] = u >= 0.f ? 1.f : 0.f;
        wb[k] = ri >= 0.f ? 1.f : 0.f;
    }
}

constexpr int kTrainThreads = 128;
constexpr int kHP = kLmacHidden + 1;  // padded row

// One sample per thread; per block the gradient of
//   sum_k w_k * BCE(z_k, y_k) * scale
// is written to partial[blockIdx.x][*], the loss sum and the number of
// correctly classified samples to stats[blockIdx.x][0..1].
__global__ void __launch_bounds__(kTrainThreads) lmac_grad_kernel(const float* __restrict__ Xb,
                                                                  const float* __restrict__ yb,
                                                                  const float* __restrict__ wb, int nb,
                                                                  const float* __restrict__ P, float scale,
                                                                  float* __restrict__ partial,
                                                                  float* __restrict__ stats) {
    extern __shared__ float sm[];
    float* sP = sm;                                   // kLmacParams
    float* xs = sP + ((kLmacParams + 3) & ~3);        // [128][9]
    float* h1s = xs + kTrainThreads * 9;              // [128][33]
    float* h2s = h1s + kTrainThreads * kHP;           // [128][33]
    float* d1s = h2s + kTrainThreads * kHP;           // [128][33]
    float* d2s = d1s + kTrainThreads * kHP;           // [128][33]
    float* dzs = d2s + kTrainThreads * kHP;           // [128]
    float* red = dzs + kTrainThreads;                 // [2][128]
    const int t = threadIdx.x;
    for (int i = t; i < kLmacParams; i += kTrainThreads) sP[i] = P[i];
    __syncthreads();
    const int k = blockIdx.x * kTrainThreads + t;
    const bool valid = k < nb;
    float x[kLmacIn];
#pragma unroll
    for (int i = 0; i < kLmacIn; ++i) {
        x[i] = valid ? Xb[(long long)k * kLmacIn + i] : 0.f;
        xs[t * 9 + i] = x[i];
    }
    const float y = valid ? yb[k] : 0.f;
    const float w = valid ? wb[k] : 0.f;
    // forward
    float h1[kLmacHidden];
#pragma unroll
    for (int j = 0; j < kLmacHidden; ++j) {
        float a = sP[kLmacB1 + j];
#pragma unroll
        for (int i = 0; i < kLmacIn; ++i) a = fmaf(sP[kLmacW1 + j * kLmacIn + i], x[i], a);
        h1[j] = fmaxf(a, 0.f);
        h1s[t * kHP + j] = h1[j];
    }
    float z = sP[kLmacB3];
    for (int j = 0; j < kLmacHidden; ++j) {
        float a = sP[kLmacB2 + j];
#pragma unroll
        for (int i = 0; i < kLmacHidden; ++i) a = fmaf(sP[kLmacW2 + j * kLmacHidden + i], h1[i], a);
        const float h2 = fmaxf(a, 0.f);
        h2s[t * kHP + j] = h2;
        z = fmaf(sP[kLmacW3 + j], h2, z);
    }
    // loss and dL/dz
    const float p = 1.f / (1.f + __expf(-z));
    const float loss = fmaxf(z, 0.f) - y * z + log1pf(__expf(-fabsf(z)));
    const float dz = w * scale * (p - y);
    dzs[t] = dz;
    red[t] = w * loss;
    red[kTrainThreads + t] = (w > 0.f && ((z > 0.f) == (y > 0.5f))) ? 1.f : 0.f;
    // backward through layer 2: d2 = dz * w3 * [h2 > 0]
    float d2[kLmacHidden];
#pragma unroll
    for (int j = 0; j < kLmacHidden; ++j) {
        d2[j] = h2s[t * kHP + j] > 0.f ? dz * sP[kLmacW3 + j] : 0.f;
        d2s[t * kHP + j] = d2[j];
    }
    // d1 = (W2^T d2) * [h1 > 0]
#pragma unroll 4
    for (int i = 0; i < kLmacHidden; ++i) {
        float a = 0.f;
#pragma unroll
        for (int j = 0; j < kLmacHidden; ++j) a = fmaf(sP[kLmacW2 + j * kLmacHidden + i], d2[j], a);
        d1s[t * kHP + i] = h1[i] > 0.f ? a : 0.f;
    }
    __syncthreads();
    // parameter gradients: sums over the block's samples in a fixed order
    float* out = partial + (long long)blockIdx.x * kLmacParams;
    for (int q = t; q < kLmacParams; q += kTrainThreads) {
        float g = 0.f;
        if (q < kLmacB1) {
            const int j = q / kLmacIn, i = q % kLmacIn;
            for (int s = 0; s < kTrainThreads; ++s) g = fmaf(d1s[s * kHP + j], xs[s * 9 + i], g);
        } else if (q < kLmacW2) {
            const int j = q - kLmacB1;
            for (int s = 0; s < kTrainThreads; ++s) g += d1s[s * kHP + j];
        } else if (q < kLmacB2) {
            const int j = (q - kLmacW2) / kLmacHidden, i = (q - kLmacW2) % kLmacHidden;
            for (int s = 0; s < kTrainThreads; ++s) g = fmaf(d2s[s * kHP + j], h1s[s * kHP + i], g);
        } else if (q < kLmacW3) {
            const int j = q - kLmacB2;
            for (int s = 0; s < kTrainThreads; ++s) g += d2s[s * kHP + j];
        } else if (q < kLmacB3) {
            const int j = q - kLmacW3;
            for (int s = 0; s < kTrainThreads; ++s) g = fmaf(dzs[s], h2s[s * kHP + j], g);
        } else {
            for (int s = 0; s < kTrainThreads; ++s) g += dzs[s];
        }
        out[q] = g;
    }
    if (t == 0) {
        float ls = 0.f, cs = 0.f;
        for (int s = 0; s < kTrainThreads; ++s) {
            ls += red[s];
            cs += red[kTrainThreads + s];
        }
        stats[2 * blockIdx.x] = ls;
        stats[2 * blockIdx.x + 1] = cs;
    }
}

// Sum of the per-block partial gradients (fixed order) -> grad; optional
// Adam step on P with moments m, v.  bc1 = 1 - beta1^t, bc2 = 1 - beta2^t.
__global__ void lmac_adam_kernel(const float* __restrict__ partial, int nblocks, float* __restrict__ grad,
                                 float* __restrict__ P, float* __restrict__ m, float* __restrict__ v, int do_step,
                                 float lr, float beta1, float beta2, float bc1, float bc2, float adam_eps) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kLmacParams) return;
    float g = 0.f;
    for (int b = 0; b < nblocks; ++b) g += partial[(long long)b * kLmacParams + q];
    grad[q] = g;
    if (!do_step) return;
    const float mq = beta1 * m[q] + (1.f - beta1) * g;
    const float vq = beta2 * v[q] + (1.f - beta2) * g * g;
    m[q] = mq;
    v[q] = vq;
    P[q] -= lr * (mq / bc1) / (sqrtf(vq / bc2) + adam_eps);
}

__global__ void lmac_forward_kernel(const float* __restrict__ X, int n, const float* __restrict__ P,
                                    float* __restrict__ z) {
    __shared__ float sP[kLmacParams];
    for (int i = threadIdx.x; i < kLmacParams; i += blockDim.x) sP[i] = P[i];
    __syncthreads();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        float x[kLmacIn];
#pragma unroll
        for (int i = 0; i < kLmacIn; ++i) x[i] = X[(long long)k * kLmacIn + i];
        z[k] = lmac_forward_f32(sP, x);
    }
}

size_t lmac_grad_smem_bytes() {
    return sizeof(float) * (((kLmacParams + 3) & ~3) + kTrainThreads * 9 + 4 * kTrainThreads * kHP +
                            kTrainThreads + 2 * kTrainThreads);
}

int lmac_grad_blocks(int nb) { return (nb + kTrainThreads - 1) / kTrainThreads; }

void launch_lmac_make_batch(const float* X, const float* r, long long n, const LmacNorm& norm, int nb,
                            uint32_t seed, float u_range, bool standardise, float* Xb, float* yb, float* wb,
                            cudaStream_t s) {
    const int b = (nb + 255) / 256;
    lmac_make_batch_kernel<<<b, 256, 0, s>>>(X, r, n, norm, nb, seed, u_range, standardise ? 1 : 0, Xb, yb, wb);
}

void launch_lmac_grad(const float* Xb, const float* yb, const float* wb, int nb, const float* P, float scale,
                      float* partial, float* stats, cudaStream_t s) {
    static bool attr = false;
    const size_t smem = lmac_grad_smem_bytes();
    if (!attr) {
        cudaFuncSetAttribute(lmac_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    lmac_grad_kernel<<<lmac_grad_blocks(nb), kTrainThreads, smem, s>>>(Xb, yb, wb, nb, P, scale, partial, stats);
}

void launch_lmac_adam(const float* partial, int nblocks, float* grad, float* P, float* m, float* v, bool step,
                      float lr, float beta1, float beta2, float bc1, float bc2, float adam_eps, cudaStream_t s) {
    lmac_adam_kernel<<<(kLmacParams + 255) / 256, 256, 0, s>>>(partial, nblocks, grad, P, m, v, step ? 1 : 0, lr,
                                                               beta1, beta2, bc1, bc2, adam_eps);
}

void launch_lmac_forward(const float* X, int n, const float* P, float* z, cudaStream_t s) {
    if (n <= 0) return;
    int b = (n + 255) / 256;
    if (b > 152 * 8) b = 152 * 8;
    lmac_forward_kernel<<<b, 256, 0, s>>>(X, n, P, z);
}

}  // namespace ngrav
