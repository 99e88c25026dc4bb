/*
 * opencl_c.hpp -- the OpenCL C 1.2 kernel language, as far as the reference's
 * rs.cl uses it, for a C++17 compiler: vector types with swizzles, vector
 * literals, the built-in functions, images read through the linear
 * clamp-to-edge sampler, work-item indices and work-group barriers.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/ref/Makefile compiles the reference's own
 * rs.cl, preceded by its rs_enum.h as rs.c does when it builds the program
 * (rs.c:1083-1110), through this header into oracle/_ref/, so that the tests
 * can run the reference's kernel source itself on the CPU and compare the
 * oracle's restatement (oracle/rsoracle.c) with it.  clc_to_cpp.py rewrites
 * on the way the two spellings C++ cannot parse: vector literals and vector
 * casts "(float4)(a, b)" / "(float4)r" become calls "float4_make(a, b)" /
 * "float4_make(r)", and swizzles ".xyz" / ".s012" / ".hi" become member calls
 * ".xyz()".  Nothing else of the source changes, line for line.
 *
 * What the OpenCL specification leaves to the device is fixed here the way
 * the oracle fixes it: every operation rounds to single precision on its own
 * (the unit is compiled with -ffp-contract=off), division and sqrt are
 * correctly rounded, the elementary functions (sin, cos, sincos, acos, atan2,
 * log, log1p, exp, pow) are those of rsmath.h, length is the square root of
 * the dot product summed from the first lane, normalize divides every lane by
 * the length, and read_imagef evaluates the specification's linear-filter
 * formula (OpenCL 1.2 section 8.2) in single precision.  Functions the
 * specification defines by a formula (clamp, mix, fract, sign, radians,
 * degrees, fma) follow that formula.  Everything rs.cl writes itself -- its
 * operation order, constants, branches and lane arithmetic -- is compiled as
 * written.
 */
#ifndef SIMRADAR_OPENCL_C_HPP
#define SIMRADAR_OPENCL_C_HPP

#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <ucontext.h>

#include <utility>
#include <vector>

#include "rsmath.h"
#include "rsoracle.h"

/* address-space and access qualifiers, kernel attribute */
#define __kernel
#define __global
#define __local
#define __constant
#define __private
#define __read_only
#define __write_only
#define __read_write

namespace rscl {

typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned long ulong;

/* ---- vector types ---- */

template <class T, int N> struct vec;
template <class T, int M> struct vref;
template <int... I> constexpr int lane_count = (int)sizeof...(I);

/* The swizzle names rs.cl uses, with their lanes (x y z w = s0 s1 s2 s3). */
#define RSCL_SINGLES(X)                                                                                        \
    X(x, 0) X(y, 1) X(z, 2) X(w, 3) X(s0, 0) X(s1, 1) X(s2, 2) X(s3, 3) X(s4, 4) X(s5, 5) X(s6, 6) X(s7, 7)     \
    X(s8, 8) X(s9, 9) X(sa, 10) X(sb, 11) X(sc, 12) X(sd, 13) X(se, 14) X(sf, 15) X(sA, 10) X(sB, 11)          \
    X(sC, 12) X(sD, 13) X(sE, 14) X(sF, 15)
#define RSCL_MULTIS(X)                                                                                         \
    X(xy, 0, 1) X(xyz, 0, 1, 2) X(xyzw, 0, 1, 2, 3) X(s01, 0, 1) X(s012, 0, 1, 2) X(s0123, 0, 1, 2, 3)       \
    X(s23, 2, 3) X(s02, 0, 2) X(s13, 1, 3) X(s45, 4, 5) X(s456, 4, 5, 6) X(s4567, 4, 5, 6, 7) X(s89, 8, 9)   \
    X(s89ab, 8, 9, 10, 11) X(scde, 12, 13, 14)

/* Member functions shared by vec and vref: each swizzle name returns a
 * reference to its lanes (a scalar reference for one lane, a vref for
 * several); lo and hi are the two halves of an even-sized vector. */
#define RSCL_SINGLE_FN(name, i) \
    T &name() { return lane<i>(); }
#define RSCL_MULTI_FN(name, ...) \
    vref<T, lane_count<__VA_ARGS__>> name() { return ref<__VA_ARGS__>(); }
#define RSCL_SWIZZLE_MEMBERS                                                        \
    RSCL_SINGLES(RSCL_SINGLE_FN)                                                    \
    RSCL_MULTIS(RSCL_MULTI_FN)                                                      \
    vref<T, N / 2> lo() { return half<0>(std::make_integer_sequence<int, N / 2>()); } \
    vref<T, N / 2> hi() { return half<1>(std::make_integer_sequence<int, N / 2>()); }

/* the same names on a const vector, returning values */
#define RSCL_CSINGLE_FN(name, i) \
    const T &name() const { return clane<i>(); }
#define RSCL_CMULTI_FN(name, ...) \
    vec<T, lane_count<__VA_ARGS__>> name() const { return get<__VA_ARGS__>(); }

template <class T, int N> struct vec {
    static_assert(N == 2 || N == 3 || N == 4 || N == 8 || N == 16, "OpenCL vector size");
    static constexpr int kN = N;
    T s[N == 3 ? 4 : N];   /* a 3-vector occupies four lanes, as in OpenCL */

    template <int I> T &lane() {
        static_assert(I < N, "swizzle lane beyond the vector");
        return s[I];
    }
    template <int I> const T &clane() const {
        static_assert(I < N, "swizzle lane beyond the vector");
        return s[I];
    }
    template <int... I> vref<T, sizeof...(I)> ref() {
        static_assert(((I < N) && ...), "swizzle lane beyond the vector");
        return vref<T, sizeof...(I)>{{&s[I]...}};
    }
    template <int... I> vec<T, sizeof...(I)> get() const {
        static_assert(((I < N) && ...), "swizzle lane beyond the vector");
        return vec<T, sizeof...(I)>{{s[I]...}};
    }
    template <int H, int... K> vref<T, N / 2> half(std::integer_sequence<int, K...>) {
        static_assert(N % 2 == 0, "lo / hi of an odd vector");
        return vref<T, N / 2>{{&s[H * (N / 2) + K]...}};
    }
    template <int H, int... K> vec<T, N / 2> chalf(std::integer_sequence<int, K...>) const {
        static_assert(N % 2 == 0, "lo / hi of an odd vector");
        return vec<T, N / 2>{{s[H * (N / 2) + K]...}};
    }

    RSCL_SWIZZLE_MEMBERS
    RSCL_SINGLES(RSCL_CSINGLE_FN)
    RSCL_MULTIS(RSCL_CMULTI_FN)
    vec<T, N / 2> lo() const { return chalf<0>(std::make_integer_sequence<int, N / 2>()); }
    vec<T, N / 2> hi() const { return chalf<1>(std::make_integer_sequence<int, N / 2>()); }

    vec &operator+=(const vec &o) { for (int k = 0; k < N; k++) s[k] = s[k] + o.s[k]; return *this; }
    vec &operator-=(const vec &o) { for (int k = 0; k < N; k++) s[k] = s[k] - o.s[k]; return *this; }
    vec &operator*=(const vec &o) { for (int k = 0; k < N; k++) s[k] = s[k] * o.s[k]; return *this; }
    vec &operator/=(const vec &o) { for (int k = 0; k < N; k++) s[k] = s[k] / o.s[k]; return *this; }
    vec &operator+=(T o) { for (int k = 0; k < N; k++) s[k] = s[k] + o; return *this; }
    vec &operator-=(T o) { for (int k = 0; k < N; k++) s[k] = s[k] - o; return *this; }
    vec &operator*=(T o) { for (int k = 0; k < N; k++) s[k] = s[k] * o; return *this; }
    vec &operator/=(T o) { for (int k = 0; k < N; k++) s[k] = s[k] / o; return *this; }
};

/* A reference to M lanes of a vector (a swizzle): reads convert to a vector,
 * writes store into the lanes. */
template <class T, int M> struct vref {
    static constexpr int N = M;
    T *p[M];

    operator vec<T, M>() const {
        vec<T, M> r{};
        for (int k = 0; k < M; k++) r.s[k] = *p[k];
        return r;
    }
    vec<T, M> val() const { return *this; }
    vref &operator=(const vec<T, M> &v) {
        const vec<T, M> t = v;   /* the value first: a swizzle may read lanes it writes */
        for (int k = 0; k < M; k++) *p[k] = t.s[k];
        return *this;
    }
    vref &operator=(const vref &o) { return *this = o.val(); }

    template <int I> T &lane() {
        static_assert(I < M, "swizzle lane beyond the vector");
        return *p[I];
    }
    template <int... I> vref<T, sizeof...(I)> ref() {
        static_assert(((I < M) && ...), "swizzle lane beyond the vector");
        return vref<T, sizeof...(I)>{{p[I]...}};
    }
    template <int H, int... K> vref<T, M / 2> half(std::integer_sequence<int, K...>) {
        static_assert(M % 2 == 0, "lo / hi of an odd vector");
        return vref<T, M / 2>{{p[H * (M / 2) + K]...}};
    }
    RSCL_SWIZZLE_MEMBERS
};

/* operators and built-ins are written for each concrete vector type (not as
 * templates), so that a swizzle (vref) converts to its vector type where one
 * is passed */
#define RSCL_ARITH(V, T, N)                                                                        \
    inline V operator+(const V &a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] + b.s[k]; return r; } \
    inline V operator-(const V &a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] - b.s[k]; return r; } \
    inline V operator*(const V &a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] * b.s[k]; return r; } \
    inline V operator/(const V &a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] / b.s[k]; return r; } \
    inline V operator+(const V &a, T b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] + b; return r; }             \
    inline V operator-(const V &a, T b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] - b; return r; }             \
    inline V operator*(const V &a, T b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] * b; return r; }             \
    inline V operator/(const V &a, T b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] / b; return r; }             \
    inline V operator+(T a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a + b.s[k]; return r; }             \
    inline V operator-(T a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a - b.s[k]; return r; }             \
    inline V operator*(T a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a * b.s[k]; return r; }             \
    inline V operator/(T a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a / b.s[k]; return r; }             \
    inline V operator-(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = -a.s[k]; return r; }                     \
    inline V operator+(const V &a) { return a; }                                                                           \
    inline vref<T, N> &operator+=(vref<T, N> &&a, const V &b) { return a = a.val() + b; }                                  \
    inline vref<T, N> &operator-=(vref<T, N> &&a, const V &b) { return a = a.val() - b; }                                  \
    inline vref<T, N> &operator*=(vref<T, N> &&a, const V &b) { return a = a.val() * b; }                                  \
    inline vref<T, N> &operator/=(vref<T, N> &&a, const V &b) { return a = a.val() / b; }                                  \
    inline vref<T, N> &operator*=(vref<T, N> &&a, T b) { return a = a.val() * b; }

#define RSCL_BITS(V, N)                                                                                             \
    inline V operator&(const V &a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] & b.s[k]; return r; } \
    inline V operator|(const V &a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] | b.s[k]; return r; } \
    inline V operator^(const V &a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] ^ b.s[k]; return r; }

typedef vec<float, 2> float2;
typedef vec<float, 3> float3;
typedef vec<float, 4> float4;
typedef vec<float, 8> float8;
typedef vec<float, 16> float16;
typedef vec<int, 2> int2;
typedef vec<int, 3> int3;
typedef vec<int, 4> int4;
typedef vec<uint, 2> uint2;
typedef vec<uint, 3> uint3;
typedef vec<uint, 4> uint4;

RSCL_ARITH(float2, float, 2)
RSCL_ARITH(float3, float, 3)
RSCL_ARITH(float4, float, 4)
RSCL_ARITH(float8, float, 8)
RSCL_ARITH(float16, float, 16)
RSCL_ARITH(int2, int, 2)
RSCL_ARITH(int3, int, 3)
RSCL_ARITH(int4, int, 4)
RSCL_ARITH(uint2, uint, 2)
RSCL_ARITH(uint3, uint, 3)
RSCL_ARITH(uint4, uint, 4)
RSCL_BITS(int2, 2)
RSCL_BITS(int3, 3)
RSCL_BITS(int4, 4)
RSCL_BITS(uint2, 2)
RSCL_BITS(uint3, 3)
RSCL_BITS(uint4, 4)

/* vector literals "(floatN)(a, b, ...)" and casts "(floatN)s": the lanes of
 * the arguments in order, or one scalar repeated */
template <class T> struct lanes {
    T v[16];
    int n = 0;
    void add(T x) {
        if (n >= 16) abort();
        v[n++] = x;
    }
    template <int M> void add(const vec<T, M> &x) {
        for (int k = 0; k < M; k++) add(x.s[k]);
    }
    template <int M> void add(const vref<T, M> &x) { add(x.val()); }
};
template <class T, int N, class... A> inline vec<T, N> vmake(const A &...a) {
    lanes<T> l;
    (l.add(a), ...);
    vec<T, N> r{};
    if (l.n == 1) {
        for (int k = 0; k < N; k++) r.s[k] = l.v[0];
    } else {
        if (l.n != N) abort();   /* a literal must give every lane */
        for (int k = 0; k < N; k++) r.s[k] = l.v[k];
    }
    return r;
}
#define RSCL_MAKE(V, T, N) \
    template <class... A> inline V V##_make(const A &...a) { return vmake<T, N>(a...); }
RSCL_MAKE(float2, float, 2)
RSCL_MAKE(float3, float, 3)
RSCL_MAKE(float4, float, 4)
RSCL_MAKE(float8, float, 8)
RSCL_MAKE(float16, float, 16)
RSCL_MAKE(int2, int, 2)
RSCL_MAKE(int3, int, 3)
RSCL_MAKE(int4, int, 4)
RSCL_MAKE(uint2, uint, 2)
RSCL_MAKE(uint3, uint, 3)
RSCL_MAKE(uint4, uint, 4)

/* ---- constants (OpenCL 1.2 section 6.12.2: the float nearest each value) ---- */
constexpr float M_PI_F = 3.14159274f;
constexpr float M_PI_2_F = 1.57079637f;
constexpr float M_PI_4_F = 0.785398185f;
constexpr float M_1_PI_F = 0.318309873f;
constexpr float M_SQRT1_2_F = 0.707106769f;
constexpr float M_SQRT2_F = 1.41421354f;

/* ---- scalar built-ins ---- */
inline float fma(float a, float b, float c) { return fmaf(a, b, c); }
inline float sqrt(float x) { return sqrtf(x); }
inline float fabs(float x) { return fabsf(x); }
inline float floor(float x) { return floorf(x); }
inline float copysign(float a, float b) { return copysignf(a, b); }
inline float fmax(float a, float b) { return fmaxf(a, b); }
inline float fmin(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }
inline float min(float a, float b) { return fminf(a, b); }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline float clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
inline float mix(float a, float b, float t) { return a + (b - a) * t; }
inline float fract(float x, float *ip) {
    const float fl = floorf(x);
    *ip = fl;
    return fminf(x - fl, 0x1.fffffep-1f);
}
inline float sign(float x) {
    if (x > 0.0f) return 1.0f;
    if (x < 0.0f) return -1.0f;
    if (x == 0.0f) return x;   /* +0 or -0 */
    return 0.0f;               /* NaN */
}
inline float radians(float d) { return (float)(3.14159265358979323846 / 180.0) * d; }
inline float degrees(float r) { return (float)(180.0 / 3.14159265358979323846) * r; }
inline float sin(float x) { return rsm_sinf(x); }
inline float cos(float x) { return rsm_cosf(x); }
inline float sincos(float x, float *c) {
    float s;
    rsm_sincosf(x, &s, c);
    return s;
}
inline float acos(float x) { return rsm_acosf(x); }
inline float atan2(float y, float x) { return rsm_atan2f(y, x); }
inline float atan(float x) { return rsm_atan2f(x, 1.0f); }
inline float atan2pi(float y, float x) { return rsm_atan2f(y, x) * M_1_PI_F; }
inline float log(float x) { return rsm_logf(x); }
inline float log1p(float x) { return rsm_log1pf(x); }
inline float log10(float x) { return rsm_logf(x) * 0.434294482f; }
inline float native_log10(float x) { return log10(x); }
inline float exp(float x) { return rsm_expf(x); }
inline float pow(float b, float e) { return rsm_powf(b, e); }
inline float pown(float x, int n) {
    /* x^|n| by repeated multiplication from the left, its reciprocal for n < 0 */
    float p = 1.0f;
    const int m = n < 0 ? -n : n;
    for (int k = 0; k < m; k++) p = k == 0 ? x : p * x;
    return n < 0 ? 1.0f / p : p;
}
inline float length(float x) { return fabsf(x); }

/* float -> uint, rounding toward zero (the default of convert_uint); the
 * kernels only convert clamped, non-negative indices */
inline uint f2u_rtz(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xffffffffu;
    return (uint)f;
}

/* relational functions: scalar forms return 1 / 0, vector forms -1 / 0 */
inline int islessequal(float a, float b) { return a <= b; }
inline int isgreaterequal(float a, float b) { return a >= b; }

/* ---- vector built-ins ---- */
#define RSCL_FLOAT_FNS(V, N, IV, UV)                                                                     \
    inline V fma(const V &a, const V &b, const V &c) { V r{}; for (int k = 0; k < N; k++) r.s[k] = fmaf(a.s[k], b.s[k], c.s[k]); return r; } \
    inline V sqrt(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = sqrtf(a.s[k]); return r; }               \
    inline V fabs(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = fabsf(a.s[k]); return r; }               \
    inline V floor(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = floorf(a.s[k]); return r; }             \
    inline V copysign(const V &a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = copysignf(a.s[k], b.s[k]); return r; } \
    inline V clamp(const V &x, float lo, float hi) { V r{}; for (int k = 0; k < N; k++) r.s[k] = clamp(x.s[k], lo, hi); return r; } \
    inline V clamp(const V &x, const V &lo, const V &hi) { V r{}; for (int k = 0; k < N; k++) r.s[k] = clamp(x.s[k], lo.s[k], hi.s[k]); return r; } \
    inline V mix(const V &a, const V &b, const V &t) { V r{}; for (int k = 0; k < N; k++) r.s[k] = mix(a.s[k], b.s[k], t.s[k]); return r; } \
    inline V mix(const V &a, const V &b, float t) { V r{}; for (int k = 0; k < N; k++) r.s[k] = mix(a.s[k], b.s[k], t); return r; } \
    inline V fract(const V &x, V *ip) { V r{}; for (int k = 0; k < N; k++) r.s[k] = fract(x.s[k], &ip->s[k]); return r; } \
    inline V radians(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = radians(a.s[k]); return r; }         \
    inline V degrees(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = degrees(a.s[k]); return r; }         \
    inline V sin(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = sin(a.s[k]); return r; }                 \
    inline V cos(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = cos(a.s[k]); return r; }                 \
    inline V sincos(const V &a, V *c) { V r{}; for (int k = 0; k < N; k++) r.s[k] = sincos(a.s[k], &c->s[k]); return r; } \
    inline V acos(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = acos(a.s[k]); return r; }               \
    inline V log(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = log(a.s[k]); return r; }                 \
    inline V log1p(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = log1p(a.s[k]); return r; }             \
    inline V exp(const V &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = exp(a.s[k]); return r; }                 \
    inline V pow(const V &a, const V &b) { V r{}; for (int k = 0; k < N; k++) r.s[k] = pow(a.s[k], b.s[k]); return r; } \
    inline V pown(const V &a, const IV &n) { V r{}; for (int k = 0; k < N; k++) r.s[k] = pown(a.s[k], n.s[k]); return r; } \
    inline float dot(const V &a, const V &b) {                                                                         \
        float d = a.s[0] * b.s[0];                                                                                     \
        for (int k = 1; k < N; k++) d = d + a.s[k] * b.s[k];                                                           \
        return d;                                                                                                      \
    }                                                                                                                  \
    inline float length(const V &a) { return sqrtf(dot(a, a)); }                                                      \
    inline V normalize(const V &a) { const float l = length(a); V r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] / l; return r; } \
    inline IV islessequal(const V &a, const V &b) { IV r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] <= b.s[k] ? -1 : 0; return r; } \
    inline IV isgreaterequal(const V &a, const V &b) { IV r{}; for (int k = 0; k < N; k++) r.s[k] = a.s[k] >= b.s[k] ? -1 : 0; return r; } \
    inline UV convert_uint##N(const V &a) { UV r{}; for (int k = 0; k < N; k++) r.s[k] = f2u_rtz(a.s[k]); return r; } \
    inline V convert_float##N(const UV &a) { V r{}; for (int k = 0; k < N; k++) r.s[k] = (float)a.s[k]; return r; }

RSCL_FLOAT_FNS(float2, 2, int2, uint2)
RSCL_FLOAT_FNS(float3, 3, int3, uint3)
RSCL_FLOAT_FNS(float4, 4, int4, uint4)

/* fma with scalar arguments widened to the vector type (rs.cl:822-824 passes
 * scalars beside vectors, which OpenCL compilers widen) */
#define RSCL_FMA_WIDEN(V)                                                                                    \
    inline V fma(float a, const V &b, float c) { return fma(vmake<float, V::kN>(a), b, vmake<float, V::kN>(c)); } \
    inline V fma(float a, const V &b, const V &c) { return fma(vmake<float, V::kN>(a), b, c); }                  \
    inline V fma(const V &a, float b, float c) { return fma(a, vmake<float, V::kN>(b), vmake<float, V::kN>(c)); } \
    inline V fma(const V &a, float b, const V &c) { return fma(a, vmake<float, V::kN>(b), c); }                  \
    inline V fma(const V &a, const V &b, float c) { return fma(a, b, vmake<float, V::kN>(c)); }                  \
    inline V fma(float a, float b, const V &c) { return fma(vmake<float, V::kN>(a), vmake<float, V::kN>(b), c); }
RSCL_FMA_WIDEN(float2)
RSCL_FMA_WIDEN(float3)
RSCL_FMA_WIDEN(float4)

/* any: 1 when the sign bit of some lane is set */
inline int any(const int2 &a) { return (a.s[0] | a.s[1]) < 0; }
inline int any(const int3 &a) { return (a.s[0] | a.s[1] | a.s[2]) < 0; }
inline int any(const int4 &a) { return (a.s[0] | a.s[1] | a.s[2] | a.s[3]) < 0; }

inline float4 shuffle(const float4 &x, const uint4 &m) {
    float4 r{};
    for (int k = 0; k < 4; k++) r.s[k] = x.s[m.s[k] & 3u];
    return r;
}

/* ---- images: CL_RGBA / CL_FLOAT, x fastest, read through the one sampler
 * rs.cl declares (unnormalised coordinates, clamp to edge, linear filter) ---- */
struct image2d_t {
    or_image im;
};
struct image3d_t {
    or_image im;
};
typedef int sampler_t;
enum { CLK_NORMALIZED_COORDS_FALSE = 0, CLK_ADDRESS_CLAMP_TO_EDGE = 2, CLK_FILTER_LINEAR = 0x20 };
enum { CLK_LOCAL_MEM_FENCE = 1, CLK_GLOBAL_MEM_FENCE = 2 };

/* one axis of the linear filter: u - 0.5 split into floor and fraction, the
 * two neighbouring texels clamped to [0, n - 1] */
struct texel_axis {
    int i0, i1;
    float a;
};
inline texel_axis tex_coord(float u, int n) {
    const float t = u - 0.5f;
    const float fl = floorf(t);
    texel_axis r;
    r.a = t - fl;
    const int i = (int)fminf(fmaxf(fl, -1.0f), (float)n);   /* NaN -> -1 */
    r.i0 = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
    r.i1 = i + 1 < 0 ? 0 : (i + 1 > n - 1 ? n - 1 : i + 1);
    return r;
}
inline float4 texel(const or_image &im, int i, int j, int k) {
    const of4 t = im.data[(size_t)i + (size_t)im.nx * ((size_t)j + (size_t)im.ny * (size_t)k)];
    return float4{{t.x, t.y, t.z, t.w}};
}
/* OpenCL 1.2 section 8.2: T = (1-a)(1-b)(1-c) T000 + a(1-b)(1-c) T100 +
 * (1-a)b(1-c) T010 + ab(1-c) T110 + (1-a)(1-b)c T001 + a(1-b)c T101 +
 * (1-a)bc T011 + abc T111, each weight formed first, the terms added in
 * that order */
inline float4 read_imagef(const image3d_t &img, sampler_t, const float4 &coord) {
    const texel_axis X = tex_coord(coord.s[0], img.im.nx), Y = tex_coord(coord.s[1], img.im.ny),
                     Z = tex_coord(coord.s[2], img.im.nz);
    const float a = X.a, b = Y.a, c = Z.a;
    const float w[8] = {(1.0f - a) * (1.0f - b) * (1.0f - c), a * (1.0f - b) * (1.0f - c),
                        (1.0f - a) * b * (1.0f - c),          a * b * (1.0f - c),
                        (1.0f - a) * (1.0f - b) * c,          a * (1.0f - b) * c,
                        (1.0f - a) * b * c,                   a * b * c};
    const float4 t[8] = {texel(img.im, X.i0, Y.i0, Z.i0), texel(img.im, X.i1, Y.i0, Z.i0),
                         texel(img.im, X.i0, Y.i1, Z.i0), texel(img.im, X.i1, Y.i1, Z.i0),
                         texel(img.im, X.i0, Y.i0, Z.i1), texel(img.im, X.i1, Y.i0, Z.i1),
                         texel(img.im, X.i0, Y.i1, Z.i1), texel(img.im, X.i1, Y.i1, Z.i1)};
    float4 r = w[0] * t[0];
    for (int q = 1; q < 8; q++) r = r + w[q] * t[q];
    return r;
}
/* the two-dimensional form: (1-a)(1-b) T00 + a(1-b) T10 + (1-a)b T01 + ab T11 */
inline float4 read_imagef(const image2d_t &img, sampler_t, const float2 &coord) {
    const texel_axis X = tex_coord(coord.s[0], img.im.nx), Y = tex_coord(coord.s[1], img.im.ny);
    const float a = X.a, b = Y.a;
    const float w[4] = {(1.0f - a) * (1.0f - b), a * (1.0f - b), (1.0f - a) * b, a * b};
    const float4 t[4] = {texel(img.im, X.i0, Y.i0, 0), texel(img.im, X.i1, Y.i0, 0), texel(img.im, X.i0, Y.i1, 0),
                         texel(img.im, X.i1, Y.i1, 0)};
    float4 r = w[0] * t[0];
    for (int q = 1; q < 4; q++) r = r + w[q] * t[q];
    return r;
}

/* ---- work items and work groups ----
 * A launch without barriers runs its work items as a loop (threads across
 * items).  A work group whose kernel calls barrier runs its items as
 * user-level contexts on one thread: each runs until its next barrier (or
 * its end), then the next item runs, so every item has reached a barrier
 * before any passes it. */
struct work_item {
    size_t gid, lid, group, lsize, gsize, ngroups;
};
inline thread_local work_item wi;

inline size_t get_global_id(uint d) { return d == 0 ? wi.gid : 0; }
inline size_t get_local_id(uint d) { return d == 0 ? wi.lid : 0; }
inline size_t get_local_size(uint d) { return d == 0 ? wi.lsize : 1; }
inline size_t get_group_id(uint d) { return d == 0 ? wi.group : 0; }
inline size_t get_global_size(uint d) { return d == 0 ? wi.gsize : 1; }
inline size_t get_num_groups(uint d) { return d == 0 ? wi.ngroups : 1; }

struct group_run {
    ucontext_t sched;
    std::vector<ucontext_t> ctx;
    std::vector<unsigned char> done;
    size_t cur = 0;
    void (*body)(void *) = nullptr;
    void *arg = nullptr;
};
inline thread_local group_run *g_group = nullptr;
inline thread_local std::vector<char> g_stacks;
constexpr size_t kItemStack = 64 * 1024;

inline void barrier(int) {
    group_run *g = g_group;
    if (g == nullptr) abort();   /* a barrier in a launch run as a plain loop */
    swapcontext(&g->ctx[g->cur], &g->sched);
}

inline void item_main() {
    group_run *g = g_group;
    g->body(g->arg);
    g->done[g->cur] = 1;   /* returning resumes the scheduler (uc_link) */
}

/* run work group `group` of a launch of ngroups x lsize items */
inline void run_group(size_t group, size_t lsize, size_t ngroups, void (*body)(void *), void *arg) {
    group_run g;
    g.ctx.resize(lsize);
    g.done.assign(lsize, 0);
    g.body = body;
    g.arg = arg;
    if (g_stacks.size() < lsize * kItemStack) g_stacks.resize(lsize * kItemStack);
    for (size_t l = 0; l < lsize; l++) {
        getcontext(&g.ctx[l]);
        g.ctx[l].uc_stack.ss_sp = g_stacks.data() + l * kItemStack;
        g.ctx[l].uc_stack.ss_size = kItemStack;
        g.ctx[l].uc_link = &g.sched;
        makecontext(&g.ctx[l], item_main, 0);
    }
    group_run *prev = g_group;
    g_group = &g;
    for (bool pending = true; pending;) {
        pending = false;
        /* volatile: swapcontext returns twice, like setjmp */
        for (volatile size_t l = 0; l < lsize; l++) {
            if (g.done[l]) continue;
            g.cur = l;
            wi = work_item{group * lsize + l, l, group, lsize, ngroups * lsize, ngroups};
            swapcontext(&g.sched, &g.ctx[l]);
            if (!g.done[l]) pending = true;
        }
    }
    g_group = prev;
}

}  // namespace rscl

#endif
