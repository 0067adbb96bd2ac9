// Stand-in for the subset of glm 0.9.9 that the reference's src/base math
// uses.  It fixes glm's scalar (non-SIMD) operation order: vec ops are
// component-wise, dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, length = sqrt(dot),
// distance(a,b) = length(b - a), mat4*vec4 = (m0*x + m1*y) + (m2*z + m3*w).
// Only used by oracle/build_ref.sh to compile reference sources for the oracle's pin.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstddef>
#include <limits>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <utility>

namespace glm {
typedef int length_t;
template <length_t L, typename T> struct vec;

template <typename T> struct vec<2, T> {
    T x, y;
    vec() : x(0), y(0) {}
    explicit vec(T s) : x(s), y(s) {}
    vec(T a, T b) : x(a), y(b) {}
    template <typename U> explicit vec(const vec<3, U>& v) : x(T(v.x)), y(T(v.y)) {}
    template <typename U> explicit vec(const vec<4, U>& v) : x(T(v.x)), y(T(v.y)) {}
    T& operator[](length_t i) { return (&x)[i]; }
    const T& operator[](length_t i) const { return (&x)[i]; }
};
template <typename T> struct vec<3, T> {
    T x, y, z;
    vec() : x(0), y(0), z(0) {}
    explicit vec(T s) : x(s), y(s), z(s) {}
    vec(T a, T b, T c) : x(a), y(b), z(c) {}
    template <typename U> explicit vec(const vec<4, U>& v) : x(T(v.x)), y(T(v.y)), z(T(v.z)) {}
    T& operator[](length_t i) { return (&x)[i]; }
    const T& operator[](length_t i) const { return (&x)[i]; }
    vec& operator+=(const vec& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec& operator-=(const vec& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
};
template <typename T> struct vec<4, T> {
    T x, y, z, w;
    vec() : x(0), y(0), z(0), w(0) {}
    explicit vec(T s) : x(s), y(s), z(s), w(s) {}
    vec(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    vec(const vec<3, T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    T& operator[](length_t i) { return (&x)[i]; }
    const T& operator[](length_t i) const { return (&x)[i]; }
};

#define GLM_SHIM_BINOP(OP)                                                                 \
    template <typename T> vec<2, T> operator OP(const vec<2, T>& a, const vec<2, T>& b) {  \
        return vec<2, T>(a.x OP b.x, a.y OP b.y); }                                        \
    template <typename T> vec<3, T> operator OP(const vec<3, T>& a, const vec<3, T>& b) {  \
        return vec<3, T>(a.x OP b.x, a.y OP b.y, a.z OP b.z); }                            \
    template <typename T> vec<4, T> operator OP(const vec<4, T>& a, const vec<4, T>& b) {  \
        return vec<4, T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); }                \
    template <typename T> vec<2, T> operator OP(const vec<2, T>& a, T s) {                 \
        return vec<2, T>(a.x OP s, a.y OP s); }                                            \
    template <typename T> vec<3, T> operator OP(const vec<3, T>& a, T s) {                 \
        return vec<3, T>(a.x OP s, a.y OP s, a.z OP s); }                                  \
    template <typename T> vec<4, T> operator OP(const vec<4, T>& a, T s) {                 \
        return vec<4, T>(a.x OP s, a.y OP s, a.z OP s, a.w OP s); }                        \
    template <typename T> vec<2, T> operator OP(T s, const vec<2, T>& a) {                 \
        return vec<2, T>(s OP a.x, s OP a.y); }                                            \
    template <typename T> vec<3, T> operator OP(T s, const vec<3, T>& a) {                 \
        return vec<3, T>(s OP a.x, s OP a.y, s OP a.z); }                                  \
    template <typename T> vec<4, T> operator OP(T s, const vec<4, T>& a) {                 \
        return vec<4, T>(s OP a.x, s OP a.y, s OP a.z, s OP a.w); }
GLM_SHIM_BINOP(+)
GLM_SHIM_BINOP(-)
GLM_SHIM_BINOP(*)
GLM_SHIM_BINOP(/)
#undef GLM_SHIM_BINOP

template <typename T> T dot(const vec<2, T>& a, const vec<2, T>& b) { vec<2, T> t = a * b; return t.x + t.y; }
template <typename T> T dot(const vec<3, T>& a, const vec<3, T>& b) { vec<3, T> t = a * b; return t.x + t.y + t.z; }
template <length_t L, typename T> T length(const vec<L, T>& v) { return std::sqrt(dot(v, v)); }
template <length_t L, typename T> T distance(const vec<L, T>& a, const vec<L, T>& b) { return length(b - a); }
template <typename T> vec<3, T> normalize(const vec<3, T>& v) { return v * (T(1) / std::sqrt(dot(v, v))); }
template <typename T> vec<3, T> cross(const vec<3, T>& a, const vec<3, T>& b) {
    return vec<3, T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

template <length_t C, length_t R, typename T> struct mat {
    vec<R, T> m[C];
    mat() {}
    explicit mat(T s) {
        for (length_t c = 0; c < C; ++c)
            for (length_t r = 0; r < R; ++r) m[c][r] = (c == r) ? s : T(0);
    }
    template <length_t C2, length_t R2> explicit mat(const mat<C2, R2, T>& o) {
        for (length_t c = 0; c < C; ++c)
            for (length_t r = 0; r < R; ++r) m[c][r] = (c < C2 && r < R2) ? o.m[c][r] : T(c == r);
    }
    vec<R, T>& operator[](length_t c) { return m[c]; }
    const vec<R, T>& operator[](length_t c) const { return m[c]; }
};

template <typename T> vec<4, T> operator*(const mat<4, 4, T>& m, const vec<4, T>& v) {
    vec<4, T> Mul0 = m[0] * v.x, Mul1 = m[1] * v.y, Mul2 = m[2] * v.z, Mul3 = m[3] * v.w;
    return (Mul0 + Mul1) + (Mul2 + Mul3);
}
template <typename T> vec<3, T> operator*(const mat<4, 3, T>& m, const vec<4, T>& v) {
    return vec<3, T>(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z + m[3][0] * v.w,
                     m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z + m[3][1] * v.w,
                     m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z + m[3][2] * v.w);
}

template <typename T> mat<4, 4, T> scale(const mat<4, 4, T>& m, const vec<3, T>& v) {
    mat<4, 4, T> r;
    r[0] = m[0] * v.x; r[1] = m[1] * v.y; r[2] = m[2] * v.z; r[3] = m[3];
    return r;
}
template <typename T> mat<4, 4, T> perspective(T fovy, T aspect, T zNear, T zFar) {
    T const tanHalfFovy = std::tan(fovy / static_cast<T>(2));
    mat<4, 4, T> r(static_cast<T>(0));
    r[0][0] = static_cast<T>(1) / (aspect * tanHalfFovy);
    r[1][1] = static_cast<T>(1) / (tanHalfFovy);
    r[2][2] = -(zFar + zNear) / (zFar - zNear);
    r[2][3] = -static_cast<T>(1);
    r[3][2] = -(static_cast<T>(2) * zFar * zNear) / (zFar - zNear);
    return r;
}

struct quat { float w, x, y, z; };

typedef vec<2, float> vec2; typedef vec<3, float> vec3; typedef vec<4, float> vec4;
typedef vec<2, int> ivec2; typedef vec<3, int> ivec3; typedef vec<4, int> ivec4;
typedef vec<2, unsigned> uvec2; typedef vec<3, unsigned> uvec3; typedef vec<4, unsigned> uvec4;
typedef mat<2, 2, float> mat2; typedef mat<3, 3, float> mat3; typedef mat<4, 4, float> mat4;
typedef mat<4, 3, float> mat4x3;
}  // namespace glm
