// OpenCL C built-ins and vector types for compiling the reference's kernels
// (kernels/*.cl, rewritten by rewrite.py) as C++ on the CPU: TEST
// INFRASTRUCTURE ONLY.  Vectors are unions of their components and read-only
// swizzle views (v.xyz converts to a float3), component-wise operators,
// comparisons giving -1 / 0 masks, and the work-item functions of the
// fiber runtime in ref_kernels.cpp.
//
// The reference builds its kernels with -cl-fast-relaxed-math
// -cl-mad-enable, which leave the rounding of contractions, divisions,
// float-to-int conversions and native_sin open.  The shim fixes them as the
// oracle does: contraction is the compiler's (a*b + c*d fuses the first
// product, as gcc and LLVM contract), a float division x / y is
// x * RN(1 / y) (the vector operators here; rewrite.py routes the scalar ones
// through cl_fdiv), (int) of a float truncates and saturates with NaN -> 0
// (cl_f2i), and native_sin is the oracle's sine (or_sinf).
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>

namespace clshim {

// x / y: x * RN(1 / y) for floats, integer division for ints
inline float div(float x, float y) { return x * (1.0f / y); }
inline int div(int x, int y) { return x / y; }

// N: the components of the vector the view lies in (its size must not grow).
template <class E, class R, int N, int... I>
struct Swz {
    E s[N];
    operator R() const { return R(s[I]...); }
};

}  // namespace clshim

#define CLSHIM_VEC_OPS(T, E, N)                                                                  \
    inline T operator+(T a, T b) { T r; for (int i = 0; i < N; ++i) r.s[i] = a.s[i] + b.s[i]; return r; } \
    inline T operator-(T a, T b) { T r; for (int i = 0; i < N; ++i) r.s[i] = a.s[i] - b.s[i]; return r; } \
    inline T operator*(T a, T b) { T r; for (int i = 0; i < N; ++i) r.s[i] = a.s[i] * b.s[i]; return r; } \
    inline T operator/(T a, T b) { T r; for (int i = 0; i < N; ++i) r.s[i] = clshim::div(a.s[i], b.s[i]); return r; } \
    inline T operator+(T a, E b) { return a + T(b); }                                           \
    inline T operator-(T a, E b) { return a - T(b); }                                           \
    inline T operator*(T a, E b) { return a * T(b); }                                           \
    inline T operator/(T a, E b) { return a / T(b); }                                           \
    inline T operator+(E a, T b) { return T(a) + b; }                                           \
    inline T operator-(E a, T b) { return T(a) - b; }                                           \
    inline T operator*(E a, T b) { return T(a) * b; }                                           \
    inline T operator/(E a, T b) { return T(a) / b; }                                           \
    inline T operator-(T a) { T r; for (int i = 0; i < N; ++i) r.s[i] = -a.s[i]; return r; }    \
    inline T& operator+=(T& a, T b) { a = a + b; return a; }                                    \
    inline T& operator-=(T& a, T b) { a = a - b; return a; }                                    \
    inline T& operator*=(T& a, T b) { a = a * b; return a; }

typedef unsigned char uchar;

struct float2;
struct float3;
struct float4;
struct int2;
struct int3;
struct int4;

struct float2 {
    union {
        float s[2];
        struct { float x, y; };
    };
    float2() : s{0, 0} {}
    explicit float2(float a) : s{a, a} {}
    float2(float a, float b) : s{a, b} {}
};
struct int2 {
    union {
        int s[2];
        struct { int x, y; };
        clshim::Swz<int, int3, 2, 0, 0, 0> xxx;
        clshim::Swz<int, int3, 2, 1, 1, 1> yyy;
    };
    int2() : s{0, 0} {}
    int2(int a) : s{a, a} {}
    int2(int a, int b) : s{a, b} {}
};
struct float3 {
    union {
        float s[4];
        struct { float x, y, z; };
        clshim::Swz<float, float3, 4, 1, 2, 0> yzx;
    };
    float3() : s{0, 0, 0, 0} {}
    explicit float3(float a) : s{a, a, a, 0} {}
    float3(float a, float b, float c) : s{a, b, c, 0} {}
};
struct int3 {
    union {
        int s[4];
        struct { int x, y, z; };
        clshim::Swz<int, int3, 4, 1, 2, 0> yzx;
    };
    int3() : s{0, 0, 0, 0} {}
    int3(int a) : s{a, a, a, 0} {}
    int3(int a, int b, int c) : s{a, b, c, 0} {}
};
struct float4 {
    union {
        float s[4];
        struct { float x, y, z, w; };
        clshim::Swz<float, float3, 4, 0, 1, 2> xyz;
        clshim::Swz<float, float3, 4, 0, 1, 3> xyw;
        clshim::Swz<float, float3, 4, 0, 3, 2> xwz;
        clshim::Swz<float, float2, 4, 0, 1> xy;
    };
    float4() : s{0, 0, 0, 0} {}
    explicit float4(float a) : s{a, a, a, a} {}
    float4(float a, float b, float c, float d) : s{a, b, c, d} {}
};
struct int4 {
    union {
        int s[4];
        struct { int x, y, z, w; };
        clshim::Swz<int, int3, 4, 0, 1, 3> xyw;
        clshim::Swz<int, int3, 4, 0, 3, 2> xwz;
        clshim::Swz<int, int2, 4, 0, 1> xy;
        clshim::Swz<int, int2, 4, 2, 3> zw;
        clshim::Swz<int, int2, 4, 2, 0> zx;
    };
    int4() : s{0, 0, 0, 0} {}
    int4(int a) : s{a, a, a, a} {}
    int4(int a, int b, int c, int d) : s{a, b, c, d} {}
};
struct float16 {
    union {
        float s[16];
        clshim::Swz<float, float4, 16, 0, 4, 8, 12> s048C;
        clshim::Swz<float, float4, 16, 1, 5, 9, 13> s159D;
        clshim::Swz<float, float4, 16, 2, 6, 10, 14> s26AE;
        clshim::Swz<float, float4, 16, 3, 7, 11, 15> s37BF;
    };
    float16() : s{} {}
};

static_assert(sizeof(float2) == 8 && sizeof(int2) == 8 && sizeof(float3) == 16 && sizeof(int3) == 16 &&
                  sizeof(float4) == 16 && sizeof(int4) == 16 && sizeof(float16) == 64,
              "OpenCL vector sizes");

CLSHIM_VEC_OPS(float2, float, 2)
CLSHIM_VEC_OPS(float3, float, 3)
CLSHIM_VEC_OPS(float4, float, 4)
CLSHIM_VEC_OPS(int2, int, 2)
CLSHIM_VEC_OPS(int3, int, 3)
CLSHIM_VEC_OPS(int4, int, 4)

// integer shifts
inline int2 operator<<(int2 a, int b) { return int2(a.x << b, a.y << b); }
inline int2 operator>>(int2 a, int b) { return int2(a.x >> b, a.y >> b); }

// comparisons and logic on vectors: -1 (true) / 0 per component
#define CLSHIM_CMP(T, M, N, OP)                                                                 \
    inline M operator OP(T a, T b) { M r; for (int i = 0; i < N; ++i) r.s[i] = a.s[i] OP b.s[i] ? -1 : 0; return r; }
CLSHIM_CMP(int2, int2, 2, ==)
CLSHIM_CMP(int3, int3, 3, >)
CLSHIM_CMP(int3, int3, 3, ==)
inline int2 operator==(int2 a, int b) { return a == int2(b); }
inline int3 operator>(int3 a, int b) { return a > int3(b); }
inline int3 operator==(int3 a, int b) { return a == int3(b); }
inline int3 operator||(int3 a, int3 b) { int3 r; for (int i = 0; i < 3; ++i) r.s[i] = (a.s[i] || b.s[i]) ? -1 : 0; return r; }
inline int3 operator&&(int3 a, int3 b) { int3 r; for (int i = 0; i < 3; ++i) r.s[i] = (a.s[i] && b.s[i]) ? -1 : 0; return r; }
// OpenCL's component-wise a ? b : c on a vector condition (rewrite.py maps
// the reference's one use onto it)
inline int3 vselect3(int3 m, int3 a, int3 b) { int3 r; for (int i = 0; i < 3; ++i) r.s[i] = m.s[i] < 0 ? a.s[i] : b.s[i]; return r; }

inline int all(int2 m) { return m.x < 0 && m.y < 0; }
inline int all(int3 m) { return m.x < 0 && m.y < 0 && m.z < 0; }

// math
inline float2 mix(float2 a, float2 b, float2 t) { return a + (b - a) * t; }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float3 cross(float3 a, float3 b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float3 normalize(float3 v) { return v / std::sqrt(dot(v, v)); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline float3 min(float3 a, float3 b) { return float3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline float3 max(float3 a, float3 b) { return float3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
inline float distance(float2 a, float2 b) { return std::sqrt(dot(a - b, a - b)); }
inline int2 max(int2 a, int2 b) { return int2(max(a.x, b.x), max(a.y, b.y)); }
inline int2 min(int2 a, int2 b) { return int2(min(a.x, b.x), min(a.y, b.y)); }
inline float clamp(float x, float a, float b) { return std::fmin(std::fmax(x, a), b); }
inline int2 clamp(int2 v, int a, int b) { return int2(min(max(v.x, a), b), min(max(v.y, a), b)); }
extern "C" float or_sinf(float x);
inline float native_sin(float x) { return or_sinf(x); }
inline float cl_fdiv(float x, float y) { return clshim::div(x, y); }
inline int cl_f2i(float x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int)x;
}
inline int4 isnan(float4 v) {
    return int4(std::isnan(v.x) ? -1 : 0, std::isnan(v.y) ? -1 : 0, std::isnan(v.z) ? -1 : 0, std::isnan(v.w) ? -1 : 0);
}
inline float4 select(float4 a, float4 b, int4 m) {
    return float4(m.x < 0 ? b.x : a.x, m.y < 0 ? b.y : a.y, m.z < 0 ? b.z : a.z, m.w < 0 ? b.w : a.w);
}
inline float3 convert_float3(int3 v) { return float3((float)v.x, (float)v.y, (float)v.z); }
inline int4 vload4(size_t o, const int* p) { return int4(p[4 * o], p[4 * o + 1], p[4 * o + 2], p[4 * o + 3]); }
inline float4 vload4(size_t o, const float* p) { return float4(p[4 * o], p[4 * o + 1], p[4 * o + 2], p[4 * o + 3]); }

// atomics (work-group local memory and global buffers)
inline int atomic_min(volatile int* p, int v) {
    int old = __atomic_load_n((int*)p, __ATOMIC_SEQ_CST);
    while (v < old && !__atomic_compare_exchange_n((int*)p, &old, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
    }
    return old;
}
inline int atomic_max(volatile int* p, int v) {
    int old = __atomic_load_n((int*)p, __ATOMIC_SEQ_CST);
    while (v > old && !__atomic_compare_exchange_n((int*)p, &old, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
    }
    return old;
}
inline int atomic_xchg(volatile int* p, int v) { return __atomic_exchange_n((int*)p, v, __ATOMIC_SEQ_CST); }

// work-item functions and barriers of the fiber runtime (ref_kernels.cpp)
size_t get_global_id(int d);
size_t get_local_id(int d);
size_t get_group_id(int d);
void barrier(int flags);
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

// address spaces and kernel qualifiers
#define __kernel
#define kernel
#define __global
#define global
#define constant
#define private
#define local
