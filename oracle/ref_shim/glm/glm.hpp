// Minimal glm-compatible vector header, written for this project so that the
// reference's GL-free CPU sources (projects/nbody_core/src/{Tree,Solvers,
// Integrator,MutualFmm}.cpp) compile without the real glm, which is absent
// from this image. It provides only what those files use: vec<2|3, T, Q>
// with .x/.y/.z, componentwise + - * /, scalar broadcast, unary minus, the
// compound assignments, dot, length, cross, min and max. Every operation is a
// plain componentwise IEEE operation, the same arithmetic glm performs.
//
// Test infrastructure only: used by the oracle/_ref build recipe, never by
// the product library.
#pragma once

#include <cmath>
#include <cstddef>

namespace glm {

enum qualifier { packed_highp, defaultp = packed_highp };

template <int L, typename T, qualifier Q = defaultp>
struct vec;

template <typename T, qualifier Q>
struct vec<2, T, Q> {
    T x, y;
    vec() : x(T(0)), y(T(0)) {}
    explicit vec(T s) : x(s), y(s) {}
    vec(T a, T b) : x(a), y(b) {}
    T& operator[](std::size_t i) { return i == 0 ? x : y; }
    const T& operator[](std::size_t i) const { return i == 0 ? x : y; }
};

template <typename T, qualifier Q>
struct vec<3, T, Q> {
    T x, y, z;
    vec() : x(T(0)), y(T(0)), z(T(0)) {}
    explicit vec(T s) : x(s), y(s), z(s) {}
    vec(T a, T b, T c) : x(a), y(b), z(c) {}
    T& operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <typename T, qualifier Q>
struct vec<4, T, Q> {
    T x, y, z, w;
    vec() : x(T(0)), y(T(0)), z(T(0)), w(T(0)) {}
    explicit vec(T s) : x(s), y(s), z(s), w(s) {}
    vec(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    vec(const vec<3, T, Q>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
};

using dvec2 = vec<2, double>;
using dvec3 = vec<3, double>;
using vec2 = vec<2, float>;
using vec3 = vec<3, float>;
using vec4 = vec<4, float>;

// Componentwise application helpers (L = 2 or 3).
#define NGRAV_GLM_BINOP(OP)                                                                    \
    template <int L, typename T, qualifier Q>                                                  \
    inline vec<L, T, Q> operator OP(const vec<L, T, Q>& a, const vec<L, T, Q>& b) {            \
        vec<L, T, Q> r;                                                                        \
        for (int i = 0; i < L; ++i) r[static_cast<std::size_t>(i)] = a[i] OP b[i];             \
        return r;                                                                              \
    }                                                                                          \
    template <int L, typename T, qualifier Q>                                                  \
    inline vec<L, T, Q> operator OP(const vec<L, T, Q>& a, T s) {                              \
        vec<L, T, Q> r;                                                                        \
        for (int i = 0; i < L; ++i) r[static_cast<std::size_t>(i)] = a[i] OP s;                \
        return r;                                                                              \
    }                                                                                          \
    template <int L, typename T, qualifier Q>                                                  \
    inline vec<L, T, Q> operator OP(T s, const vec<L, T, Q>& a) {                              \
        vec<L, T, Q> r;                                                                        \
        for (int i = 0; i < L; ++i) r[static_cast<std::size_t>(i)] = s OP a[i];                \
        return r;                                                                              \
    }                                                                                          \
    template <int L, typename T, qualifier Q>                                                  \
    inline vec<L, T, Q>& operator OP##=(vec<L, T, Q>& a, const vec<L, T, Q>& b) {              \
        for (int i = 0; i < L; ++i) a[static_cast<std::size_t>(i)] = a[i] OP b[i];             \
        return a;                                                                              \
    }                                                                                          \
    template <int L, typename T, qualifier Q>                                                  \
    inline vec<L, T, Q>& operator OP##=(vec<L, T, Q>& a, T s) {                                \
        for (int i = 0; i < L; ++i) a[static_cast<std::size_t>(i)] = a[i] OP s;                \
        return a;                                                                              \
    }

NGRAV_GLM_BINOP(+)
NGRAV_GLM_BINOP(-)
NGRAV_GLM_BINOP(*)
NGRAV_GLM_BINOP(/)
#undef NGRAV_GLM_BINOP

template <int L, typename T, qualifier Q>
inline vec<L, T, Q> operator-(const vec<L, T, Q>& a) {
    vec<L, T, Q> r;
    for (int i = 0; i < L; ++i) r[static_cast<std::size_t>(i)] = -a[i];
    return r;
}

template <int L, typename T, qualifier Q>
inline T dot(const vec<L, T, Q>& a, const vec<L, T, Q>& b) {
    T s = a[0] * b[0];
    for (int i = 1; i < L; ++i) s = s + a[i] * b[i];
    return s;
}

template <int L, typename T, qualifier Q>
inline T length(const vec<L, T, Q>& a) {
    return std::sqrt(dot(a, a));
}

template <typename T, qualifier Q>
inline vec<3, T, Q> cross(const vec<3, T, Q>& a, const vec<3, T, Q>& b) {
    return vec<3, T, Q>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

template <int L, typename T, qualifier Q>
inline vec<L, T, Q> min(const vec<L, T, Q>& a, const vec<L, T, Q>& b) {
    vec<L, T, Q> r;
    for (int i = 0; i < L; ++i) r[static_cast<std::size_t>(i)] = (b[i] < a[i]) ? b[i] : a[i];
    return r;
}

template <int L, typename T, qualifier Q>
inline vec<L, T, Q> max(const vec<L, T, Q>& a, const vec<L, T, Q>& b) {
    vec<L, T, Q> r;
    for (int i = 0; i < L; ++i) r[static_cast<std::size_t>(i)] = (a[i] < b[i]) ? b[i] : a[i];
    return r;
}

template <typename T>
inline T mix(T a, T b, float t) {
    return a * (1.0f - t) + b * t;
}

} // namespace glm
