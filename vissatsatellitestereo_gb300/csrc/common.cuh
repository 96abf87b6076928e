// Shared helpers of the sm_103a geometry kernels: status handling, launch geometry,
// double-float (compensated FP32) arithmetic and order-preserving integer keys.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vissat_gb300.h"

namespace vs {

// ---- host-side error reporting ------------------------------------------------------
void set_error(const char *fmt, ...);
int check_launch(const char *what);          // VS_OK or VS_ERR_CUDA after a launch

#define VS_REQUIRE(cond, ...)            \
    do {                                 \
        if (!(cond)) {                   \
            ::vs::set_error(__VA_ARGS__); \
            return VS_ERR_ARG;           \
        }                                \
    } while (0)

#define VS_LAUNCH_CHECK(what)                         \
    do {                                              \
        int _st = ::vs::check_launch(what);           \
        if (_st != VS_OK) return _st;                 \
    } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (152 on GB300), cached per process.
int sm_count();

// Carves aligned sub-buffers out of a caller workspace.
struct Carver {
    char *base;
    size_t used = 0;
    explicit Carver(void *p) : base(static_cast<char *>(p)) {}
    template <typename T>
    T *take(size_t count) {
        used = (used + 255) & ~size_t(255);
        T *p = reinterpret_cast<T *>(base ? base + used : nullptr);
        used += count * sizeof(T);
        return p;
    }
};

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---- rare-path FP64 operations --------------------------------------------------------
// GB300 runs FP64 arithmetic and the float<->double conversions on a narrow pipe.  The
// per-element kernels keep them off the common path, but the compiler would if-convert a
// cheap-looking fallback (hoist it out of its branch and execute it for every element);
// volatile asm has side effects as far as the compiler knows, so these stay in their
// branch.
__device__ __forceinline__ double rare_dsub(double a, double b) {
    double r;
    asm volatile("sub.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}
__device__ __forceinline__ double rare_dadd(double a, double b) {
    double r;
    asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}
__device__ __forceinline__ double rare_dmul(double a, double b) {
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}
__device__ __forceinline__ double rare_ddiv(double a, double b) {
    double r;
    asm volatile("div.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}
__device__ __forceinline__ float rare_d2f(double a) {
    float r;
    asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(r) : "d"(a));
    return r;
}
__device__ __forceinline__ double rare_f2d(float a) {
    double r;
    asm volatile("cvt.f64.f32 %0, %1;" : "=d"(r) : "f"(a));
    return r;
}

// ---- double-float arithmetic ---------------------------------------------------------
// A value hi + lo with |lo| <= ulp(hi)/2 carried in two floats (about 48 significant
// bits).  Error-free transformations after Knuth (TwoSum) and Dekker (TwoProduct with
// an FMA); the file is compiled without fast-math so the compiler keeps their order.
struct df {
    float hi, lo;
};

__device__ __forceinline__ df two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
    float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ df two_prod(float a, float b) {
    float p = a * b;
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    df t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_add_f(df a, float b) {
    df s = two_sum(a.hi, b);
    s.lo += a.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul(df a, df b) {
    df p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
    df p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
// Double-float sum whose error is ~2^-48 of the operands' magnitudes (not of the result):
// one TwoSum of the high parts, the low parts added plainly.  For sums whose accuracy
// budget is absolute in the operands' scale (cancellation harmless).
__device__ __forceinline__ df df_add_ops(df a, df b) {
    const df s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

// ---- packed double-float pairs --------------------------------------------------------
// Two independent double-float values per operation with Blackwell's FP32x2 instructions
// (FADD2 / FMUL2 / FFMA2: IEEE round-to-nearest in each lane), so each lane computes
// exactly what the scalar helpers above compute.  A difference y - x is fma(x, -1, y)
// (one rounding, like the subtraction); a negated product -fl(a b) is fl((-a) b).
struct df2 {
    float2 hi, lo;
};
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 sub2(float2 y, float2 x) { return __ffma2_rn(x, f2s(-1.0f), y); }
__device__ __forceinline__ df2 two_sum2(float2 a, float2 b) {
    const float2 s = __fadd2_rn(a, b);
    const float2 bb = sub2(s, a);
    return {s, __fadd2_rn(sub2(a, sub2(s, bb)), sub2(b, bb))};
}
__device__ __forceinline__ df2 fast_two_sum2(float2 a, float2 b) {  // |a| >= |b| per lane
    const float2 s = __fadd2_rn(a, b);
    return {s, sub2(b, sub2(s, a))};
}
// two_prod per lane given nb = -b: the error term fma(a, b, -fl(a b)), -fl(a b) = fl(a (-b))
__device__ __forceinline__ df2 two_prod2(float2 a, float2 b, float2 nb) {
    return {__fmul2_rn(a, b), __ffma2_rn(a, b, __fmul2_rn(a, nb))};
}
// df_mul per lane given nb_hi = -b.hi
__device__ __forceinline__ df2 df_mul2(df2 a, df2 b, float2 nb_hi) {
    df2 p = two_prod2(a.hi, b.hi, nb_hi);
    p.lo = __ffma2_rn(a.hi, b.lo, __ffma2_rn(a.lo, b.hi, p.lo));
    return fast_two_sum2(p.hi, p.lo);
}
// df_add per lane
__device__ __forceinline__ df2 df_add2(df2 a, df2 b) {
    df2 s = two_sum2(a.hi, b.hi);
    const df2 t = two_sum2(a.lo, b.lo);
    s.lo = __fadd2_rn(s.lo, t.hi);
    s = fast_two_sum2(s.hi, s.lo);
    s.lo = __fadd2_rn(s.lo, t.lo);
    return fast_two_sum2(s.hi, s.lo);
}
// df_add_ops per lane
__device__ __forceinline__ df2 df_add_ops2(df2 a, df2 b) {
    const df2 s = two_sum2(a.hi, b.hi);
    return fast_two_sum2(s.hi, __fadd2_rn(s.lo, __fadd2_rn(a.lo, b.lo)));
}
// df_recip per lane: 1 - p.hi is exact (p.hi = w.hi q is within 2^-21 of 1), so -p.hi is
// recovered exactly as (1 - p.hi) - 1 for the error term of the product.
__device__ __forceinline__ df2 df_recip2(df2 w) {
    const float2 q = f2(__fdividef(1.0f, w.hi.x), __fdividef(1.0f, w.hi.y));
    const float2 phi = __fmul2_rn(w.hi, q);
    const float2 t = sub2(f2s(1.0f), phi);                               // 1 - p.hi
    const float2 plo = __ffma2_rn(w.hi, q, __fadd2_rn(t, f2s(-1.0f)));   // fma(w.hi, q, -p.hi)
    const float2 e = sub2(sub2(t, plo), __fmul2_rn(w.lo, q));
    return fast_two_sum2(q, __fmul2_rn(q, e));
}

// 1 / w in double-float: an approximate reciprocal refined by one Newton step whose residual
// 1 - w q is formed exactly (two_prod; 1 - p.hi is exact for p.hi near 1): relative error
// about the square of the first estimate's, below 2^-43.
__device__ __forceinline__ df df_recip(df w) {
    const float q = __fdividef(1.0f, w.hi);
    const df p = two_prod(w.hi, q);
    const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p.hi), p.lo), __fmul_rn(w.lo, q));
    return fast_two_sum(q, __fmul_rn(q, e));
}

__host__ __device__ inline df df_from_double(double v) {
    float hi = static_cast<float>(v);
    return {hi, static_cast<float>(v - static_cast<double>(hi))};
}
// float -> double by bit manipulation, exact (the conversion instruction shares GB300's
// narrow FP64 pipe, and even a never-taken branch holding one slows the kernel).
__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned long long sign = static_cast<unsigned long long>(u & 0x80000000u) << 32;
    unsigned e = (u >> 23) & 0xffu;
    unsigned m = u & 0x7fffffu;
    unsigned long long b;
    if (e == 0xffu) {                 // inf / NaN
        b = sign | 0x7ff0000000000000ull | (static_cast<unsigned long long>(m) << 29) | (m ? (1ull << 51) : 0ull);
    } else if (e == 0) {              // zero / subnormal: normalise the mantissa
        if (m == 0) {
            b = sign;
        } else {
            const int lz = __clz(m) - 8;          // m < 2^23: shift until bit 23 is set
            m = (m << lz) & 0x7fffffu;
            b = sign | (static_cast<unsigned long long>(1023 - 126 - lz) << 52) | (static_cast<unsigned long long>(m) << 29);
        }
    } else {
        b = sign | (static_cast<unsigned long long>(e + 1023u - 127u) << 52) | (static_cast<unsigned long long>(m) << 29);
    }
    return __longlong_as_double(static_cast<long long>(b));
}

// Round-to-nearest-even double -> float (astype(np.float32)) with 32/64-bit integer
// operations only.  f64_to_f32_slow covers every input; f64_to_f32 runs the straight-line
// normal-range path and branches to it only for inf/NaN, overflow and the float-subnormal
// range.
static __device__ __noinline__ float f64_to_f32_slow(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    const unsigned hi = static_cast<unsigned>(b >> 32), lo = static_cast<unsigned>(b);
    const unsigned sign = hi & 0x80000000u;
    const int e = static_cast<int>((hi >> 20) & 0x7ffu);
    const unsigned mhi = hi & 0xfffffu;
    if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | ((mhi | lo) ? 0x400000u : 0u));   // inf / NaN
    const int e32 = e - 1023 + 127;
    if (e32 >= 255) return __uint_as_float(sign | 0x7f800000u);                                     // overflow
    if (e32 <= 0) {                   // float subnormal range (or zero): units of 2^-149
        const int shift = 926 - e;    // value = M * 2^(e - 1075), M = 2^52 + mantissa
        if (e == 0 || shift >= 64) return __uint_as_float(sign);                                     // rounds to 0
        const unsigned long long M = (1ull << 52) | (b & 0xfffffffffffffull);
        const unsigned long long q = M >> shift, rem = M & ((1ull << shift) - 1), half = 1ull << (shift - 1);
        const unsigned up = (rem > half) || (rem == half && (q & 1ull));
        return __uint_as_float(sign | static_cast<unsigned>(q + up));   // may round up to the least normal
    }
    const unsigned m23 = (mhi << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    const unsigned up = (rem > 0x10000000u) || (rem == 0x10000000u && (m23 & 1u));
    return __uint_as_float(sign | ((static_cast<unsigned>(e32) << 23) + m23 + up));
}

__device__ __forceinline__ float f64_to_f32(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    const unsigned hi = static_cast<unsigned>(b >> 32), lo = static_cast<unsigned>(b);
    const unsigned ebits = (hi >> 20) & 0x7ffu;
    // normal float range: 897 <= e <= 1150 (e32 = e - 896 in 1..254)
    if (ebits - 897u > 253u) return f64_to_f32_slow(v);
    const unsigned m23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    const unsigned up = (rem > 0x10000000u) | ((rem == 0x10000000u) & m23);
    // the carry of a round-up may step into the next binade or to inf: both are correct
    return __uint_as_float((hi & 0x80000000u) | (((ebits - 896u) << 23) + m23 + (up & 1u)));
}

__device__ __forceinline__ double df_to_double(df a) { return __dadd_rn(f32_to_f64(a.hi), f32_to_f64(a.lo)); }

// ---- order-preserving keys --------------------------------------------------------------
// Unsigned keys whose integer order is the numeric order of the float value; key 0 is
// reserved for "no value" (it would decode to a NaN).
__device__ __forceinline__ unsigned long long key_from_double(double v) {
    unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double double_from_key(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double(static_cast<long long>(b));
}
__device__ __forceinline__ unsigned key_from_float(float v) {
    unsigned b = __float_as_uint(v);
    return (b >> 31) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float float_from_key(unsigned k) {
    unsigned b = (k >> 31) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(b);
}

}  // namespace vs
