// lmac.cuh -- the learned opening test ("learned MAC") of the grouped walk:
// its input features, its network layout and the decision rule.
//
// The geometric test of the reference (Mac.hpp:25-29, Solvers.cpp:261-271)
// accepts a node N for a target group G iff
//     worst = |com_N - com_G| - maxR_G > 0  and  2h_N < theta * worst.
// The learned test asks instead whether using N's multipole (softened
// monopole + quadrupole, Solvers.cpp:147-179) keeps every target t of G
// within a per-target error budget:
//     max_t |a_exact,N(t) - a_multipole,N(t)| / |a(t)|  <=  b.
// A small network, 8 features -> 32 -> 32 -> 1 (ReLU, logit out), predicts
// the probability of that event.  Features are scale-free ratios of the pair's
// geometry and moments, so one network serves every node level:
//   f0 = log2(2h_N / worst)                 the geometric opening ratio
//   f1 = log2(maxR_N / worst)               the node's actual extent
//   f2 = log2(maxR_G / worst)               the target group's extent
//   f3 = log2(G M_N / (worst^2 amin_G)) - log2(b)
//                                           the node's pull on the weakest-pulled
//                                           member, in units of the budget
//   f4 = |Q_N|_F / (M_N maxR_N^2)           quadrupole strength
//   f5 = (d^.Q_N.d^) / (M_N maxR_N^2)       quadrupole along the line of sight
//   f6 = eps / worst                        softening at the nearest member
//   f7 = log2(count_N)                      particles behind the multipole
// amin_G = min over the group's members of |a| from the previous force
// evaluation.  Log-ratios are clamped to [-30, 30].  Before the network the
// features are standardised with the training set's mean and deviation.
//
// Decision: pairs far outside the network's band are settled geometrically
// (rho = 2h/worst <= rho_lo: accept; rho >= rho_hi or worst <= 0: open); in
// the band the logit z decides when |z| >= z_gate (accept iff z > 0) and the
// geometric test with the run's theta decides otherwise (the low-confidence
// fallback).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ngrav {

constexpr int kLmacIn = 8;
constexpr int kLmacHidden = 32;
// Parameter vector layout (FP32 master copy): W1[32][8], b1[32], W2[32][32],
// b2[32], w3[32], b3.
constexpr int kLmacW1 = 0;
constexpr int kLmacB1 = kLmacW1 + kLmacHidden * kLmacIn;
constexpr int kLmacW2 = kLmacB1 + kLmacHidden;
constexpr int kLmacB2 = kLmacW2 + kLmacHidden * kLmacHidden;
constexpr int kLmacW3 = kLmacB2 + kLmacHidden;
constexpr int kLmacB3 = kLmacW3 + kLmacHidden;
constexpr int kLmacParams = kLmacB3 + 1;  // 1377

struct LmacNorm {
    float mu[kLmacIn];
    float isd[kLmacIn];
};

// The model as the walk evaluates it: standardisation, FP32 biases and output
// weights, and the two hidden layers as BF16 tensor-core B operands.  Both are
// block-diagonal over two pairs per accumulator row (pair 0 in columns 0-31,
// pair 1 in columns 32-63), stored K-major in 8x16-byte core matrices:
//   w1t: N = 64 x K = 16 (LBO 128 B, SBO 256 B)
//   w2t: N = 64 x K = 64 (LBO 128 B, SBO 1024 B)
struct LmacDev {
    float mu[kLmacIn], isd[kLmacIn];
    float b1[kLmacHidden], b2[kLmacHidden], w3[kLmacHidden];
    float b3, pad[3];
    uint16_t w1t[64 * 16];
    uint16_t w2t[64 * 64];
};
constexpr uint32_t kW1Lbo = 128, kW1Sbo = 256, kW2Lbo = 128, kW2Sbo = 1024;

__device__ __forceinline__ float lmac_log2c(float v) {
    return fminf(30.f, fmaxf(-30.f, __log2f(fmaxf(v, 1e-30f))));
}

// Features of one (group, node) pair from the FP32 walk records.  gA/gD: the
// group leaf's com_hi+mass / com_lo; gR its maxRadius; amin its acceleration
// scale.  A/B/Cw/D: the node's records; count its particle count.
// log2b: log2 of the per-target error budget.  Returns worst (the caller
// settles worst <= 0 itself).
__device__ __forceinline__ float lmac_features(const float4 gA, const float4 gD, float gR, float amin,
                                               const float4 A, const float4 B, const float4 Cw, const float4 D,
                                               int count, float G, float eps, float log2b, float f[kLmacIn]) {
    const float dx = (A.x - gA.x) + (D.x - gD.x);
    const float dy = (A.y - gA.y) + (D.y - gD.y);
    const float dz = (A.z - gA.z) + (D.z - gD.z);
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float d = sqrtf(d2);
    const float worst = d - gR;
    const float iw = 1.f / fmaxf(worst, 1e-30f);
    const float M = A.w, maxr = Cw.x, size = Cw.y;
    f[0] = lmac_log2c(size * iw);
    f[1] = lmac_log2c(maxr * iw);
    f[2] = lmac_log2c(gR * iw);
    f[3] = lmac_log2c(G * M * iw * iw / fmaxf(amin, 1e-30f)) - log2b;
    const float qxx = B.x, qyy = B.y, qxy = B.z, qxz = B.w, qyz = D.w, qzz = -qxx - qyy;
    const float s2 = fmaxf(M * maxr * maxr, 1e-30f);
    const float qn = sqrtf(qxx * qxx + qyy * qyy + qzz * qzz + 2.f * (qxy * qxy + qxz * qxz + qyz * qyz));
    const float dqd = qxx * dx * dx + qyy * dy * dy + qzz * dz * dz + 2.f * (qxy * dx * dy + qxz * dx * dz + qyz * dy * dz);
    f[4] = qn / s2;
    f[5] = dqd / (s2 * fmaxf(d2, 1e-30f));
    f[6] = fminf(eps * iw, 16.f);
    f[7] = __log2f((float)max(count, 1));
    return worst;
}

// FP32 forward pass of the network on standardised features (training and
// reference evaluation; the walk evaluates the BF16 copy on tensor cores).
__device__ __forceinline__ float lmac_forward_f32(const float* __restrict__ P, const float x[kLmacIn]) {
    float h1[kLmacHidden];
#pragma unroll
    for (int j = 0; j < kLmacHidden; ++j) {
        float a = P[kLmacB1 + j];
#pragma unroll
        for (int i = 0; i < kLmacIn; ++i) a = fmaf(P[kLmacW1 + j * kLmacIn + i], x[i], a);
        h1[j] = fmaxf(a, 0.f);
    }
    float z = P[kLmacB3];
#pragma unroll 4
    for (int j = 0; j < kLmacHidden; ++j) {
        float a = P[kLmacB2 + j];
#pragma unroll
        for (int i = 0; i < kLmacHidden; ++i) a = fmaf(P[kLmacW2 + j * kLmacHidden + i], h1[i], a);
        z = fmaf(P[kLmacW3 + j], fmaxf(a, 0.f), z);
    }
    return z;
}

}  // namespace ngrav
