// softening.cuh -- the two softened pair forces of the reference
// (include/ngrav/Softening.hpp, src/Solvers.cpp:19-63).
//
// Plummer: a = G m d / (|d|^2 + eps^2)^(3/2).
// Spline (Hernquist & Katz 1989): the point mass convolved with the cubic
// B-spline kernel of smoothing length h = eps (support 2h):
//   a = G m chi(q) d / |d|^3,  q = |d| / h, with the enclosed-mass fraction
//   chi(q) = q^3 (4/3 - 6/5 q^2 + 1/2 q^3)                  q < 1
//          = 1 - 4 (t^4/4 - t^5/5 + t^6/24),  t = 2 - q     1 <= q < 2
//          = 1                                              q >= 2
// (exactly Newtonian outside 2h), and the pair potential G m_i m_j phi(q) / h
//   phi(q) = -(7/5 - 2/3 q^2 + 3/10 q^4 - 1/10 q^5)          q < 1
//          = -((1 - 4F)/q + t^4/2 - t^5/5),  F = t^4/4 - t^5/5 + t^6/24
//          = -1/q                                            q >= 2.
#pragma once

#include <cuda_runtime.h>

namespace ngrav {

enum : int { kSoftPlummer = 0, kSoftSpline = 1 };

__host__ __device__ __forceinline__ float spline_chi(float q) {
    if (q >= 2.f) return 1.f;
    if (q < 1.f) {
        const float q2 = q * q;
        return q2 * q * (4.f / 3.f - 1.2f * q2 + 0.5f * q2 * q);
    }
    const float t = 2.f - q, t2 = t * t, t4 = t2 * t2;
    return 1.f - 4.f * (0.25f * t4 - 0.2f * t4 * t + t4 * t2 * (1.f / 24.f));
}

__host__ __device__ __forceinline__ double spline_chi_d(double q) {
    if (q >= 2.0) return 1.0;
    if (q < 1.0) return q * q * q * (4.0 / 3.0 - 1.2 * q * q + 0.5 * q * q * q);
    const double t = 2.0 - q, t2 = t * t, t4 = t2 * t2;
    return 1.0 - 4.0 * (t4 / 4.0 - t4 * t / 5.0 + t4 * t2 / 24.0);
}

__host__ __device__ __forceinline__ double spline_phi_d(double q) {
    if (q >= 2.0) return -1.0 / q;
    if (q < 1.0) return -(1.4 - (2.0 / 3.0) * q * q + 0.3 * q * q * q * q - 0.1 * q * q * q * q * q);
    const double t = 2.0 - q, t2 = t * t, t4 = t2 * t2;
    const double F = t4 / 4.0 - t4 * t / 5.0 + t4 * t2 / 24.0;
    return -((1.0 - 4.0 * F) / q + t4 / 2.0 - t4 * t / 5.0);
}

// Force factor f (a += f * d) of one FP32 pair: r2 = |d|^2, m the source mass.
// Plummer adds eps^2; spline uses ih = 1/h.  Coincident points give 0.
template <int SOFT>
__device__ __forceinline__ float pair_factor(float r2, float m, float eps2, float ih) {
    if (SOFT == kSoftSpline) {
        const float ir = rsqrtf(r2);
        const float q = r2 * ir * ih;
        return r2 > 0.f ? m * spline_chi(q) * (ir * ir * ir) : 0.f;
    } else {
        const float ir = rsqrtf(r2 + eps2);
        return m * (ir * ir * ir);
    }
}

}  // namespace ngrav
