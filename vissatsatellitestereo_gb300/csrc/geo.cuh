// Depth map -> UTM points on the device (aggregate_2p5d_util.py:75-98): a pixel (col, row)
// with depth d goes through the view's 4x4 inverse projection and a homogeneous divide to
// ENU (east, north, up) about the AOI origin, then ENU -> geodetic (coordinate_system.py:41-50,
// pymap3d.enu2geodetic) and geodetic -> UTM (lib/latlon_utm_converter.py:38-52, pyproj).
//
// Two arithmetics, shared by every kernel of the chain (points, fused rasterisation, plan):
//
//  * exact: FP64 restatements of the published algorithms -- ENU -> ECEF rotation, You
//    (2000) "Transformation of Cartesian to Geodetic Coordinates without Iterations",
//    Krueger's transverse Mercator series to n^6 -- with every operation explicitly rounded
//    (no contraction) so each kernel computes the same bits.
//
//  * fast: GB300 runs FP64 at ~1/64 of the FP32 rate, and this chain needs ~1000 FP64
//    operations per point.  Over an AOI box the map ENU -> (easting, northing, altitude) is
//    smooth at the Earth-radius scale, so a plan fits it once with a total-degree-4
//    polynomial in box-normalised coordinates (Chebyshev interpolation at 5^3 exact nodes,
//    truncated and converted to monomials) and validates it against the exact chain.  Per
//    pixel: the projective stage in double-float, the constant + linear terms in
//    double-float, the 31 terms of degree 2..4 in FP32 (their magnitude bounds their
//    rounding), and the FP64 result assembled in 2^-30 m fixed point and turned into FP64
//    bit patterns with integer operations.  No FP64 instruction on this path.
#pragma once

#include <math.h>

#include "common.cuh"

namespace vs {

// ---- constants of one frame (ENU origin + UTM zone), FP64 ---------------------------------
struct GeoFrame {
    double x0, y0, z0;              // ECEF of the ENU origin
    double sphi, cphi, slam, clam;  // sine / cosine of the origin's latitude and longitude
    double a, b, a2, b2;            // WGS-84 semi-axes and their squares
    double esq;                     // a^2 - b^2 (You's E^2)
    double E;                       // sqrt(a^2 - b^2)
    double ecc;                     // first eccentricity
    double a_over_b;
    double lam0;                    // central meridian (radians)
    double k0A;                     // k0 * rectifying radius
    double fe, fn;                  // false easting / northing
    double alpha[6];                // Krueger series coefficients
};

constexpr int kGeoFxBits = 30;      // fixed point of the fast path: units of 2^-30 m
constexpr int kGeoNl = 31;          // monomials of degree 2..4 in three variables (6 + 10 + 15)

// Fast-path plan: box-normalised coordinates s = (enu - cen) / half (half a power of two).
struct GeoFast {
    float cen[3];                   // box centre, ENU metres (floats)
    float half[3];                  // half-widths, powers of two
    float inv_half[3];
    int enabled;                    // validated: the fast path may be used
    long long c0[3];                // constant terms of easting, northing, altitude (2^-30 m)
    df lin[3][3];                   // [output][axis] linear coefficients (metres per unit of s)
    float nl[3][kGeoNl];            // [output][monomial] degree 2..4 coefficients (metres)
};

// Exponents (a, b, c) of monomial j of degree 2..4, the order of GeoFast::nl.
__host__ __device__ __forceinline__ void geo_monomial(int j, int &a, int &b, int &c) {
    int k = 0;
    for (int deg = 2; deg <= 4; ++deg)
        for (int x = deg; x >= 0; --x)
            for (int y = deg - x; y >= 0; --y) {
                if (k == j) {
                    a = x;
                    b = y;
                    c = deg - x - y;
                    return;
                }
                ++k;
            }
    a = b = c = 0;
}

// ---- exact chain (FP64, explicitly rounded) ------------------------------------------------
__device__ __forceinline__ double gm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ga(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double gs(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double gd(double a, double b) { return __ddiv_rn(a, b); }

// pymap3d enu2ecef: (e, n, u) rotated into ECEF axes plus the origin.
__device__ __forceinline__ void enu_to_ecef(const GeoFrame &g, double e, double n, double u, double &x,
                                            double &y, double &z) {
    const double t = gs(gm(g.cphi, u), gm(g.sphi, n));
    const double w = ga(gm(g.sphi, u), gm(g.cphi, n));
    x = ga(g.x0, gs(gm(g.clam, t), gm(g.slam, e)));
    y = ga(g.y0, ga(gm(g.slam, t), gm(g.clam, e)));
    z = ga(g.z0, w);
}

// You (2000): ECEF -> latitude, longitude (radians), height.
__device__ __forceinline__ void ecef_to_geodetic(const GeoFrame &g, double x, double y, double z, double &lat,
                                                 double &lon, double &alt) {
    const double r2 = ga(ga(gm(x, x), gm(y, y)), gm(z, z));
    const double d = gs(r2, g.esq);
    const double u = sqrt(ga(gm(0.5, d), gm(0.5, sqrt(ga(gm(d, d), gm(gm(4.0, g.esq), gm(z, z)))))));
    const double Q = hypot(x, y);
    const double huE = hypot(u, g.E);
    double beta = atan(gd(gm(gd(huE, u), z), Q));
    double sb, cb;
    sincos(beta, &sb, &cb);
    const double eps = gd(gm(ga(gs(gm(g.b, u), gm(g.a, huE)), g.esq), sb), gs(gd(gm(g.a, huE), cb), gm(g.esq, cb)));
    beta = ga(beta, eps);
    lat = atan(gm(g.a_over_b, tan(beta)));
    lon = atan2(y, x);
    sincos(beta, &sb, &cb);
    alt = hypot(gs(z, gm(g.b, sb)), gs(Q, gm(g.a, cb)));
    const double inside = ga(ga(gd(gm(x, x), g.a2), gd(gm(y, y), g.a2)), gd(gm(z, z), g.b2));
    if (inside < 1.0) alt = -alt;
}

// Krueger series transverse Mercator: latitude, longitude (radians) -> easting, northing.
__device__ __forceinline__ void geodetic_to_tm(const GeoFrame &g, double lat, double lon, double &east,
                                               double &north) {
    const double kPi = 3.141592653589793;
    double dlam = gs(lon, g.lam0);
    if (dlam > kPi) dlam = gs(dlam, 2.0 * kPi);
    if (dlam < -kPi) dlam = ga(dlam, 2.0 * kPi);
    const double tau = tan(lat);
    const double s1 = sqrt(ga(1.0, gm(tau, tau)));
    const double sig = sinh(gm(g.ecc, atanh(gd(gm(g.ecc, tau), s1))));
    const double taup = gs(gm(tau, sqrt(ga(1.0, gm(sig, sig)))), gm(sig, s1));
    double sl, cl;
    sincos(dlam, &sl, &cl);
    const double xip = atan2(taup, cl);
    const double etap = asinh(gd(sl, sqrt(ga(gm(taup, taup), gm(cl, cl)))));
    double xi = xip, eta = etap;
#pragma unroll 1
    for (int j = 1; j <= 6; ++j) {
        const double k = 2.0 * j;
        double s2, c2;
        sincos(gm(k, xip), &s2, &c2);
        xi = ga(xi, gm(gm(g.alpha[j - 1], s2), cosh(gm(k, etap))));
        eta = ga(eta, gm(gm(g.alpha[j - 1], c2), sinh(gm(k, etap))));
    }
    east = ga(g.fe, gm(g.k0A, eta));
    north = ga(g.fn, gm(g.k0A, xi));
}

// ENU -> (easting, northing, altitude), plus latitude (radians) for the hemisphere check.
static __device__ __noinline__ void geo_exact(const GeoFrame *__restrict__ gp, double e, double n, double u, double &east,
                                       double &north, double &alt, double &lat) {
    const GeoFrame &g = *gp;
    double x, y, z, lon;
    enu_to_ecef(g, e, n, u, x, y, z);
    ecef_to_geodetic(g, x, y, z, lat, lon, alt);
    geodetic_to_tm(g, lat, lon, east, north);
}

// ---- fast path --------------------------------------------------------------------------
// round(x * 2^30) of a float with integer operations (|x| < 2^32).
__device__ __forceinline__ long long fx30(float x) {
    const unsigned u = __float_as_uint(x);
    const int e = static_cast<int>((u >> 23) & 0xffu);
    const long long m = static_cast<long long>((u & 0x7fffffu) | 0x800000u);
    const int sh = e - 120;                   // x = m * 2^(e - 150) = m * 2^(sh - 30)
    long long v;
    if (e == 0) v = 0;                        // zero (and subnormals, < 2^-126 m)
    else if (sh >= 0) v = m << sh;
    else if (sh > -25) v = (m + (1ll << (-sh - 1))) >> (-sh);
    else v = 0;
    return (u >> 31) ? -v : v;
}

// FP64 bit pattern of S * 2^-30 with integer operations: the leading bit sets the exponent,
// the next 52 bits the mantissa, the dropped bits round half away from zero.
__device__ __forceinline__ unsigned long long fx30_to_bits(long long S) {
    if (S == 0) return 0ull;
    const unsigned long long sign = S < 0 ? 0x8000000000000000ull : 0ull;
    const unsigned long long m = S < 0 ? (0ull - static_cast<unsigned long long>(S)) : static_cast<unsigned long long>(S);
    const int p = 63 - __clzll(static_cast<long long>(m));
    unsigned long long mant;
    if (p > 52) {
        const int sh = p - 52;
        mant = (m + (1ull << (sh - 1))) >> sh;     // 2^52 <= mant <= 2^53 (a carry bumps the exponent)
    } else {
        mant = m << (52 - p);
    }
    return sign | ((static_cast<unsigned long long>(p - kGeoFxBits + 1022) << 52) + mant);
}

// Sum of three double-float products.
__device__ __forceinline__ df df_dot3(const df (&c)[3], const df (&s)[3]) {
    df acc = df_mul(c[0], s[0]);
    acc = df_add_ops(acc, df_mul(c[1], s[1]));
    return df_add_ops(acc, df_mul(c[2], s[2]));
}

// (easting, northing, altitude) FP64 bits of an ENU point given in double-float.  Returns
// false (nothing written) when the point lies outside the plan's box.
__device__ __forceinline__ bool geo_fast(const GeoFast &f, const df (&enu)[3], unsigned long long (&bits)[3]) {
    df s[3];
    bool inside = true;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const df d = df_add_f(enu[i], -f.cen[i]);
        inside &= fabsf(d.hi) <= f.half[i];
        s[i] = {__fmul_rn(d.hi, f.inv_half[i]), __fmul_rn(d.lo, f.inv_half[i])};   // exact: power of two
    }
    if (!inside) return false;
    float p[3][5];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        p[i][0] = 1.0f;
        p[i][1] = s[i].hi;
        p[i][2] = __fmul_rn(s[i].hi, s[i].hi);
        p[i][3] = __fmul_rn(p[i][2], s[i].hi);
        p[i][4] = __fmul_rn(p[i][2], p[i][2]);
    }
    // monomials of degree 2..4 in the order of geo_monomial (compile-time exponents)
    float m[kGeoNl];
    int j = 0;
#pragma unroll
    for (int deg = 2; deg <= 4; ++deg)
#pragma unroll
        for (int x = deg; x >= 0; --x)
#pragma unroll
            for (int y = deg - x; y >= 0; --y) m[j++] = __fmul_rn(__fmul_rn(p[0][x], p[1][y]), p[2][deg - x - y]);
#pragma unroll
    for (int o = 0; o < 3; ++o) {
        float nl = 0.0f;
#pragma unroll
        for (int j = kGeoNl - 1; j >= 0; --j) nl = __fmaf_rn(f.nl[o][j], m[j], nl);   // small terms first
        const df v = df_add_f(df_dot3(f.lin[o], s), nl);
        bits[o] = fx30_to_bits(f.c0[o] + fx30(v.hi) + fx30(v.lo));
    }
    return true;
}

// ---- projective stage ---------------------------------------------------------------------
// Per-view inverse projection (row-major 4x4) in double-float and FP64.
struct DepthView {
    df m[4][4];
    double md[4][4];
};

// Row i of M [col, row, 1, d] in double-float; col and row are exact floats.  The terms
// reach ~1e6 (a camera centre hundreds of km away cancelling along the ray), so the sums'
// operand-relative error of ~2^-48 is ~1e-9 m absolute.
__device__ __forceinline__ df proj_row(const DepthView &v, int i, float col, float row, float d) {
    df acc = df_mul_f(v.m[i][0], col);
    acc = df_add_ops(acc, df_mul_f(v.m[i][1], row));
    acc = df_add_ops(acc, v.m[i][2]);
    return df_add_ops(acc, df_mul_f(v.m[i][3], d));
}

// Pixel classes: 0 no point (depth <= 0 or NaN); 1 fast candidate (finite positive depth,
// non-zero homogeneous w: z is finite, the pixel has a point); 2 decided by FP64 (infinite
// depth or zero w).  w: the homogeneous w in double-float.
__device__ __forceinline__ int pixel_class(const DepthView &v, float col, float row, float d, df &w) {
    w = {0.0f, 0.0f};
    if (!(d > 0.0f)) return 0;
    if (d == __int_as_float(0x7f800000)) return 2;
    w = proj_row(v, 3, col, row, d);
    return w.hi != 0.0f ? 1 : 2;
}
__device__ __forceinline__ int pixel_class(const DepthView &v, float col, float row, float d) {
    df w;
    return pixel_class(v, col, row, d, w);
}

// FP64 ENU of a pixel from the row-major matrix md; false when its homogeneous z is NaN
// (the reference drops it).
__device__ __forceinline__ double proj_row_exact(const double *md, int i, double col, double row, double d) {
    return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(md[4 * i], col), __dmul_rn(md[4 * i + 1], row)), md[4 * i + 2]),
                     __dmul_rn(md[4 * i + 3], d));
}

__device__ __forceinline__ bool pixel_enu_exact(const double *md, float col, float row, float d, double (&enu)[3]) {
    const double c = static_cast<double>(col), r = static_cast<double>(row), dd = static_cast<double>(d);
    const double w = proj_row_exact(md, 3, c, r, dd);
    const double z = __ddiv_rn(proj_row_exact(md, 2, c, r, dd), w);
    if (z != z) return false;
    enu[0] = __ddiv_rn(proj_row_exact(md, 0, c, r, dd), w);
    enu[1] = __ddiv_rn(proj_row_exact(md, 1, c, r, dd), w);
    enu[2] = z;
    return true;
}

// The FP64 path of one pixel (rare: outside the fast box, exact mode, class 2), kept out of
// line so the fast path keeps its registers.  md: the view's FP64 matrix (shared memory).
struct PixelBits {
    unsigned long long e, n, a;
    int ok;
};
static __device__ __noinline__ PixelBits pixel_point_exact(const double *md, const GeoFrame *g, float col, float row,
                                                          float d, int cls, int south, int *flags) {
    PixelBits out{0x7ff8000000000000ull, 0x7ff8000000000000ull, 0x7ff8000000000000ull, 1};
    double enu[3];
    if (!pixel_enu_exact(md, col, row, d, enu)) {
        out.ok = cls == 2 ? 0 : 1;           // a class-1 pixel keeps its point (NaN coordinates)
        return out;
    }
    double east, north, alt, lat;
    geo_exact(g, enu[0], enu[1], enu[2], east, north, alt, lat);
    if (flags && ((lat < 0.0) != (south != 0))) atomicOr(flags, VS_GEO_FLAG_HEMISPHERE);
    out.e = static_cast<unsigned long long>(__double_as_longlong(east));
    out.n = static_cast<unsigned long long>(__double_as_longlong(north));
    out.a = static_cast<unsigned long long>(__double_as_longlong(alt));
    return out;
}

// FP64 validity of a class-2 pixel.
static __device__ __noinline__ bool pixel_valid_exact(const double *md, float col, float row, float d) {
    double enu[3];
    return pixel_enu_exact(md, col, row, d, enu);
}

// ---- per-pixel drivers shared by the points and the fused rasterisation kernels ------------
constexpr int kDepthPix = 8;                 // consecutive pixels per thread

__device__ __forceinline__ void load_depths(const float *__restrict__ depth, long long p, long long total,
                                            float (&d)[kDepthPix]) {
    const float *src = depth + p;
    if (p + kDepthPix <= total && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
        const float4 a = __ldcs(reinterpret_cast<const float4 *>(src));
        const float4 b = __ldcs(reinterpret_cast<const float4 *>(src) + 1);
        d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w;
        d[4] = b.x; d[5] = b.y; d[6] = b.z; d[7] = b.w;
    } else {
#pragma unroll
        for (int k = 0; k < kDepthPix; ++k) d[k] = p + k < total ? __ldcs(src + k) : -1.0f;
    }
}

// (easting, northing, altitude) bits of a pixel of class cls (1 or 2) with homogeneous w:
// the fast path when the mode and plan allow it and the point lies in the plan's box, else
// the FP64 chain.  Returns false when the pixel has no point (class 2 with a NaN
// homogeneous z).  A class-1 pixel always has one (NaN coordinates in the degenerate case of
// a zero FP64 w).
__device__ __forceinline__ bool pixel_point(const DepthView &v, const double *md, const GeoFast &f,
                                            const GeoFrame *g, int mode, int cls, df w, float col, float row,
                                            float d, int south, unsigned long long (&bits)[3], int *flags) {
    if (cls == 1 && mode == VS_GEO_FAST && f.enabled) {
        const df rw = df_recip(w);
        df enu[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) enu[i] = df_mul(proj_row(v, i, col, row, d), rw);
        if (geo_fast(f, enu, bits)) return true;
    }
    const PixelBits pb = pixel_point_exact(md, g, col, row, d, cls, south, flags);
    bits[0] = pb.e;
    bits[1] = pb.n;
    bits[2] = pb.a;
    return pb.ok != 0;
}

// The view's FP64 matrix in shared memory for the out-of-line FP64 path.
__device__ __forceinline__ void stage_matrix(const DepthView &v, double *smd) {
    if (threadIdx.x < 16) smd[threadIdx.x] = v.md[threadIdx.x >> 2][threadIdx.x & 3];
    __syncthreads();
}

// Host side (geo.cu): frame constants, per-view matrices, plan accessors.
void build_geo_frame(const VsGeoFrame &in, GeoFrame &g);
bool make_depth_view(const double *m, DepthView &v);
const GeoFast &geo_plan_fast(const VsGeoPlan *p);
const GeoFrame *geo_plan_frame(const VsGeoPlan *p);
int geo_plan_south(const VsGeoPlan *p);

}  // namespace vs
