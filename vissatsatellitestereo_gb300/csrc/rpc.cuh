// Device-side RPC camera evaluation shared by the projection and camera-approximation
// kernels.  Two arithmetics:
//
//  * exact: FP64 in the reference's operation order (lib/rpc_model.py:52-62,160-168),
//    explicit round-to-nearest intrinsics so nothing is contracted into an FMA -- the
//    result is bit-identical to the numpy code;
//  * fast: GB300 runs FP64 at ~1/64 of the FP32 rate, so the fast form splits each FP64
//    input into a double-float (hi + lo floats) with integer operations, normalises and
//    evaluates the dominant constant+linear terms in double-float, the sixteen small
//    higher-order terms in plain FP32 (their magnitude bounds their rounding), and takes
//    the num/den ratio and the denormalisation in double-float.  |error| < 1e-4 px for
//    images up to 8192 px with WorldView-like coefficient magnitudes.
#pragma once

#include "common.cuh"

namespace vs {

// Per-camera constants of the fast form, prepared once per call.  The four polynomials
// travel as two (col, row) pairs through packed FP32x2 arithmetic: pair 0 = (colNum,
// rowNum), pair 1 = (colDen, rowDen).
struct RpcFast {
    df lat_off, lon_off, alt_off;       // offsets (double-float)
    df inv_lat, inv_lon, inv_alt;       // 1 / scale (double-float)
    float2 lin_hi[2][4], lin_lo[2][4];  // [pair][0..3] constant + linear coefficients
    float2 lin_nhi[2][4];               // -lin_hi (error terms of the products)
    float2 hot[2][16];                  // [pair][k-4] higher-order coefficients (FP32)
    float2 scale_hi, scale_lo, scale_nhi, off_hi, off_lo;   // (col, row) denormalisation
    float width, height;
};

// ---- exact FP64 (reference order) ------------------------------------------------------
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ double poly_exact(const double *c, double x, double y, double z) {
    double out = da(0.0, c[0]);
    out = da(out, da(da(dm(c[1], y), dm(c[2], x)), dm(c[3], z)));
    out = da(out, da(da(dm(dm(c[4], y), x), dm(dm(c[5], y), z)), dm(dm(c[6], x), z)));
    out = da(out, da(da(dm(dm(c[7], y), y), dm(dm(c[8], x), x)), dm(dm(c[9], z), z)));
    out = da(out, dm(dm(dm(c[10], x), y), z));
    out = da(out, dm(dm(dm(c[11], y), y), y));
    out = da(out, da(da(dm(dm(dm(c[12], y), x), x), dm(dm(dm(c[13], y), z), z)), dm(dm(dm(c[14], y), y), x)));
    out = da(out, dm(dm(dm(c[15], x), x), x));
    out = da(out, da(da(dm(dm(dm(c[16], x), z), z), dm(dm(dm(c[17], y), y), z)), dm(dm(dm(c[18], x), x), z)));
    out = da(out, dm(dm(dm(c[19], z), z), z));
    return out;
}

__device__ __forceinline__ void project_exact(const VsRpcCamera &cam, double lat, double lon, double alt,
                                              double &col, double &row) {
    const double c_lon = __ddiv_rn(__dsub_rn(lon, cam.lon_off), cam.lon_scale);
    const double c_lat = __ddiv_rn(__dsub_rn(lat, cam.lat_off), cam.lat_scale);
    const double c_alt = __ddiv_rn(__dsub_rn(alt, cam.alt_off), cam.alt_scale);
    const double c_col = __ddiv_rn(poly_exact(cam.col_num, c_lat, c_lon, c_alt),
                                   poly_exact(cam.col_den, c_lat, c_lon, c_alt));
    const double c_row = __ddiv_rn(poly_exact(cam.row_num, c_lat, c_lon, c_alt),
                                   poly_exact(cam.row_den, c_lat, c_lon, c_alt));
    col = da(dm(c_col, cam.col_scale), cam.col_off);
    row = da(dm(c_row, cam.row_scale), cam.row_off);
}

// ---- fast (double-float) ------------------------------------------------------------------
// Splits an FP64 value into hi + lo floats without FP64 arithmetic: hi keeps the top 24
// significant bits (truncated from the bit pattern, so the remainder is exact), lo is the
// remaining 29 bits converted to a float (one rounding) and scaled by their power of two.
// Magnitudes outside 2^+-100 (zero, tiny, huge, inf, NaN) become the nearest float with
// lo = 0.  The integer conversion is one instruction (measured faster here than the
// two-halves float trick it replaced, the fit 2.69 -> 2.64 ms).
__device__ __forceinline__ df split_double(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    const int e = static_cast<int>((b >> 52) & 0x7ff);
    if (e < 1023 - 100 || e > 1023 + 100) return {f64_to_f32(v), 0.0f};
    const unsigned sign = static_cast<unsigned>(b >> 32) & 0x80000000u;
    const unsigned mant_hi = static_cast<unsigned>((b >> 29) & 0x7fffffu);   // top 23 fraction bits
    const float hi = __uint_as_float(sign | (static_cast<unsigned>(e - 1023 + 127) << 23) | mant_hi);
    const unsigned rest = static_cast<unsigned>(b & 0x1fffffffu);            // low 29 fraction bits
    // value of the low bits: rest * 2^(e - 1075); 2^(e-1075) = 2^(e-1023) * 2^-52
    const float scale = __uint_as_float(static_cast<unsigned>(e - 1023 - 52 + 127) << 23);
    float lo = __uint2float_rn(rest) * scale;
    lo = sign ? -lo : lo;
    return {hi, lo};
}

// constant + three linear terms in double-float, plus the FP32 higher-order sum, for the
// two polynomials of a pair at once (same operations per lane as the scalar form: exact
// products of the high parts with their cross terms in the low word, the TwoSum chain of
// constant, linear terms and higher-order sum)
__device__ __forceinline__ df2 poly_fast2(const float2 (&hi)[4], const float2 (&lo)[4], const float2 (&nhi)[4],
                                          const float2 (&hot)[16], df x, df y, df z, const float (&m)[16]) {
    const float2 Y = f2s(y.hi), X = f2s(x.hi), Z = f2s(z.hi);
    // two_prod(c, v): -fl(c v) = fl((-c) v) from the negated coefficients
    const df2 p1 = {__fmul2_rn(hi[1], Y), __ffma2_rn(hi[1], Y, __fmul2_rn(nhi[1], Y))};
    const df2 p2 = {__fmul2_rn(hi[2], X), __ffma2_rn(hi[2], X, __fmul2_rn(nhi[2], X))};
    const df2 p3 = {__fmul2_rn(hi[3], Z), __ffma2_rn(hi[3], Z, __fmul2_rn(nhi[3], Z))};
    float2 low = __fadd2_rn(__fadd2_rn(__fadd2_rn(lo[0], p1.lo), p2.lo), p3.lo);
    low = __ffma2_rn(hi[1], f2s(y.lo), __ffma2_rn(lo[1], Y, low));
    low = __ffma2_rn(hi[2], f2s(x.lo), __ffma2_rn(lo[2], X, low));
    low = __ffma2_rn(hi[3], f2s(z.lo), __ffma2_rn(lo[3], Z, low));
    float2 h = f2s(0.0f);
#pragma unroll
    for (int k = 0; k < 16; ++k) h = __ffma2_rn(hot[k], f2s(m[k]), h);
    df2 s = two_sum2(hi[0], p1.hi);
    low = __fadd2_rn(low, s.lo);
    s = two_sum2(s.hi, p2.hi);
    low = __fadd2_rn(low, s.lo);
    s = two_sum2(s.hi, p3.hi);
    low = __fadd2_rn(low, s.lo);
    s = two_sum2(s.hi, h);
    low = __fadd2_rn(low, s.lo);
    return fast_two_sum2(s.hi, low);
}

// monomials 4..19 of the RPC order from the high parts of the normalised coordinates
__device__ __forceinline__ void monomials(float x, float y, float z, float (&m)[16]) {
    const float yx = y * x, yz = y * z, xz = x * z, yy = y * y, xx = x * x, zz = z * z;
    m[0] = yx; m[1] = yz; m[2] = xz; m[3] = yy; m[4] = xx; m[5] = zz;
    m[6] = yx * z;       // xyz
    m[7] = yy * y;       // y^3
    m[8] = y * xx;       // y x^2
    m[9] = y * zz;       // y z^2
    m[10] = yy * x;      // y^2 x
    m[11] = xx * x;      // x^3
    m[12] = x * zz;      // x z^2
    m[13] = yy * z;      // y^2 z
    m[14] = xx * z;      // x^2 z
    m[15] = zz * z;      // z^3
}

// (v - off) * inv: the difference's error is ~2^-48 of |v| (a few 1e-13 degrees), far below
// what the 1e-4 px bound allows after the scale.
__device__ __forceinline__ df normalise(df v, df off, df inv) {
    return df_mul(df_add_ops(v, {-off.hi, -off.lo}), inv);
}

// (col, row) as double-floats for one point given as split lat/lon/alt: the numerator
// pair and the denominator pair, then both quotients and denormalisations as one pair.
__device__ __forceinline__ void project_fast(const RpcFast &c, df lat, df lon, df alt, df &col, df &row) {
    const df x = normalise(lat, c.lat_off, c.inv_lat);
    const df y = normalise(lon, c.lon_off, c.inv_lon);
    const df z = normalise(alt, c.alt_off, c.inv_alt);
    float m[16];
    monomials(x.hi, y.hi, z.hi, m);
    const df2 num = poly_fast2(c.lin_hi[0], c.lin_lo[0], c.lin_nhi[0], c.hot[0], x, y, z, m);
    const df2 den = poly_fast2(c.lin_hi[1], c.lin_lo[1], c.lin_nhi[1], c.hot[1], x, y, z, m);
    // quotients through a Newton-refined reciprocal (relative error < 2^-43)
    const df2 r = df_recip2(den);
    const df2 q = df_mul2(num, r, sub2(f2s(0.0f), r.hi));
    const df2 v = df_add_ops2(df_mul2(q, {c.scale_hi, c.scale_lo}, c.scale_nhi), {c.off_hi, c.off_lo});
    col = {v.hi.x, v.lo.x};
    row = {v.hi.y, v.lo.y};
}

// df < float bound, for the in-image mask (col >= 0, col < width)
__device__ __forceinline__ bool df_lt(df a, float b) { return a.hi < b || (a.hi == b && a.lo < 0.0f); }
__device__ __forceinline__ bool df_ge0(df a) { return a.hi > 0.0f || (a.hi == 0.0f && a.lo >= 0.0f); }

// Fills an RpcFast from a camera (device code, one thread per camera).
__device__ __forceinline__ void prepare_fast(const VsRpcCamera &cam, RpcFast &f) {
    f.lat_off = df_from_double(cam.lat_off);
    f.lon_off = df_from_double(cam.lon_off);
    f.alt_off = df_from_double(cam.alt_off);
    f.inv_lat = df_from_double(1.0 / cam.lat_scale);
    f.inv_lon = df_from_double(1.0 / cam.lon_scale);
    f.inv_alt = df_from_double(1.0 / cam.alt_scale);
    const double *polys[2][2] = {{cam.col_num, cam.row_num}, {cam.col_den, cam.row_den}};
    for (int p = 0; p < 2; ++p) {
        for (int k = 0; k < 4; ++k) {
            const df a = df_from_double(polys[p][0][k]), b = df_from_double(polys[p][1][k]);
            f.lin_hi[p][k] = make_float2(a.hi, b.hi);
            f.lin_lo[p][k] = make_float2(a.lo, b.lo);
            f.lin_nhi[p][k] = make_float2(-a.hi, -b.hi);
        }
        for (int k = 4; k < 20; ++k)
            f.hot[p][k - 4] = make_float2(static_cast<float>(polys[p][0][k]), static_cast<float>(polys[p][1][k]));
    }
    const df cs = df_from_double(cam.col_scale), co = df_from_double(cam.col_off);
    const df rs = df_from_double(cam.row_scale), ro = df_from_double(cam.row_off);
    f.scale_hi = make_float2(cs.hi, rs.hi);
    f.scale_lo = make_float2(cs.lo, rs.lo);
    f.scale_nhi = make_float2(-cs.hi, -rs.hi);
    f.off_hi = make_float2(co.hi, ro.hi);
    f.off_lo = make_float2(co.lo, ro.lo);
    f.width = static_cast<float>(cam.width);
    f.height = static_cast<float>(cam.height);
}

}  // namespace vs
