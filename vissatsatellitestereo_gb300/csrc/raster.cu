// (c) Max-height rasterisation onto the DSM grid: proj_to_grid (lib/proj_to_grid.py:41-81)
// and the float32 3x3 median blur that produce_dsm applies to it (produce_dsm.py:58).
//
// Exactness without FP64 on the per-point path
// ---------------------------------------------
// The reference bins with FP64:  row = floor(fl(fl(yoff - y) / xres)),
// col = floor(fl(fl(x - xoff) / yres)).  GB300's FP64 rate is ~1/64 of FP32, so doing
// that per point would make the kernel FP64-bound.  Instead, when y has the same sign and
// binary exponent as yoff, fl(yoff - y) is exact (Sterbenz) and equals d * ulp(yoff) with
// the integer d = bits(yoff) - bits(y).  fl(d*ulp / res) is monotone in d, so each row r
// starts at an integer threshold T[r] (smallest d landing in row >= r).  The thresholds are
// computed once per grid with the reference's FP64 expression, and a point's row is found
// from an FP32 estimate corrected against T: integer and FP32 work only, same result.
// Points outside the fast path's precondition (other exponent, non-finite) take the
// literal FP64 expression.
//
// Per-cell nanmax: heights become order-preserving 64-bit keys and meet in atomicMax.
// numpy_groupies (numba flavour, the reference's pinned environment) keeps the first of
// two equal values, which only shows for +0/-0: zeros share one key and, when a cell's
// maximum is zero, a second pass finds the first zero of that cell in input order.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>

#include "common.cuh"

namespace vs {
namespace {

constexpr unsigned long long kEmptyKey = 0ull;
constexpr unsigned long long kZeroKey = 0x8000000000000000ull;   // key of +0.0
constexpr unsigned long long kNoIndex = ~0ull;

// One axis of the DSM grid.  dir = +1: a = v - off (columns), dir = -1: a = off - v (rows).
struct Axis {
    double off, res;
    long long n;                 // cells along the axis
    const long long *thr;        // n + 1 integer thresholds (ulps of off), fast path only
    unsigned long long top12;    // sign + exponent of off
    unsigned long long mul;      // floor(2^64 * ulp(off) / res): row estimate = mulhi(d, mul)
    int neg;                     // off < 0
    int dir;
    int fast;                    // fast path usable
};

struct Tables {
    Axis row, col;
};

__device__ __forceinline__ long long axis_exact(const Axis &ax, double v) {
    double a = ax.dir > 0 ? __dsub_rn(v, ax.off) : __dsub_rn(ax.off, v);
    double q = __ddiv_rn(a, ax.res);
    if (!(q >= 0.0 && q < static_cast<double>(ax.n))) return -1;
    return static_cast<long long>(q);   // q >= 0: truncation is floor
}

// Cell index along one axis, or -1 when the point falls outside the grid.
__device__ __forceinline__ long long axis_index(const Axis &ax, double v) {
    unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    if (ax.fast && (b >> 52) == ax.top12) {
        long long bo = static_cast<long long>(__double_as_longlong(ax.off));
        long long bv = static_cast<long long>(b);
        long long d = ((ax.dir > 0) != (ax.neg != 0)) ? (bv - bo) : (bo - bv);
        if (d < 0 || d >= __ldg(ax.thr + ax.n)) return -1;
        // integer estimate (no conversion instructions: on GB300 they share the FP64 pipe)
        long long r = static_cast<long long>(__umul64hi(static_cast<unsigned long long>(d), ax.mul));
        r = r >= ax.n ? ax.n - 1 : r;
#pragma unroll 1
        for (int it = 0; it < 8 && __ldg(ax.thr + r) > d; ++it) --r;
#pragma unroll 1
        for (int it = 0; it < 8 && __ldg(ax.thr + r + 1) <= d; ++it) ++r;
        return r;
    }
    return axis_exact(ax, v);
}

// T[r] = smallest d >= 0 with floor(fl(d*ulp / res)) >= r, for r = 0..n.  d*ulp is exact,
// so this is the reference's expression evaluated at the representable differences.
__global__ void axis_thresholds_kernel(long long *thr, long long n, double ulp, double res) {
    long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (r > n) return;
    if (r == 0) {
        thr[0] = 0;
        return;
    }
    const double rd = static_cast<double>(r);
    long long d = static_cast<long long>(ceil(rd * res / ulp));
    if (d < 0) d = 0;
    // walk to the exact boundary (a handful of steps; bounded)
    for (int it = 0; it < 64 && d > 0 && floor(__ddiv_rn(static_cast<double>(d - 1) * ulp, res)) >= rd; ++it) --d;
    for (int it = 0; it < 64 && floor(__ddiv_rn(static_cast<double>(d) * ulp, res)) < rd; ++it) ++d;
    thr[r] = d;
}

__device__ __forceinline__ bool is_nan_bits(unsigned long long b) {
    return (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}

// Zero heights are collected in a side list during binning: (cell, point index) pairs.
struct ZeroList {
    unsigned long long *entries;   // [2 * kZeroCap]: cell, index
    int *count;                    // number of zero points seen (may exceed kZeroCap)
};
constexpr int kZeroCap = 1 << 16;

// Pass 1: bin every point of one view and atomicMax its height key into the cell.
// View v owns points [offsets[v], offsets[v+1]); vk is its key grid.
__global__ void __launch_bounds__(256) bin_max_kernel(const double *__restrict__ pts,
                                                      const long long *__restrict__ offsets, int v,
                                                      long long single_n, Tables tb,
                                                      unsigned long long *__restrict__ vk, ZeroList zl) {
    const long long begin = offsets ? offsets[v] : 0;
    const long long end = offsets ? offsets[v + 1] : single_n;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x * 2;
    for (long long i = begin + (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) * 2;
         i < end; i += stride) {
        double p[6];
        const double *src = pts + 3 * i;
        if (i + 1 < end && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
            const double2 *s2 = reinterpret_cast<const double2 *>(src);
            double2 a = __ldcs(s2), b = __ldcs(s2 + 1), c = __ldcs(s2 + 2);
            p[0] = a.x; p[1] = a.y; p[2] = b.x; p[3] = b.y; p[4] = c.x; p[5] = c.y;
        } else {
            p[0] = __ldcs(src); p[1] = __ldcs(src + 1); p[2] = __ldcs(src + 2);
            if (i + 1 < end) { p[3] = __ldcs(src + 3); p[4] = __ldcs(src + 4); p[5] = __ldcs(src + 5); }
            else { p[3] = 0.0; p[4] = 0.0; p[5] = __longlong_as_double(0x7ff8000000000000ll); }
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const double x = p[3 * k], y = p[3 * k + 1], z = p[3 * k + 2];
            unsigned long long zb = static_cast<unsigned long long>(__double_as_longlong(z));
            if (is_nan_bits(zb)) continue;
            long long r = axis_index(tb.row, y);
            if (r < 0) continue;
            long long c = axis_index(tb.col, x);
            if (c < 0) continue;
            const long long cell = r * tb.col.n + c;
            unsigned long long key;
            if ((zb << 1) == 0) {            // +-0: one shared key, sign resolved afterwards
                key = kZeroKey;
                const int slot = atomicAdd(zl.count, 1);
                if (slot < kZeroCap) {
                    zl.entries[2 * slot] = static_cast<unsigned long long>(cell);
                    zl.entries[2 * slot + 1] = static_cast<unsigned long long>(i + k);
                }
            } else {
                key = key_from_double(z);
            }
            atomicMax(vk + cell, key);
        }
    }
}

// Zero-sign resolution: first[cell] = smallest index of a zero point of a cell whose
// maximum is zero.  Normally from the side list; a full pass if the list overflowed.
__global__ void zero_list_init_kernel(const unsigned long long *__restrict__ keys,
                                      unsigned long long *__restrict__ first, ZeroList zl) {
    const int n = min(*zl.count, kZeroCap);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const unsigned long long cell = zl.entries[2 * e];
        if (keys[cell] == kZeroKey) first[cell] = kNoIndex;
    }
}

__global__ void zero_list_min_kernel(const unsigned long long *__restrict__ keys,
                                     unsigned long long *__restrict__ first, ZeroList zl) {
    const int n = min(*zl.count, kZeroCap);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const unsigned long long cell = zl.entries[2 * e];
        if (keys[cell] == kZeroKey) atomicMin(first + cell, zl.entries[2 * e + 1]);
    }
}

__global__ void zero_init_kernel(const unsigned long long *__restrict__ keys,
                                 unsigned long long *__restrict__ first, long long total, ZeroList zl) {
    if (*zl.count <= kZeroCap) return;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x)
        if (keys[c] == kZeroKey) first[c] = kNoIndex;
}

__global__ void zero_first_kernel(const double *__restrict__ pts, const long long *__restrict__ offsets, int v,
                                  long long single_n, Tables tb,
                                  const unsigned long long *__restrict__ keys,
                                  unsigned long long *__restrict__ first, ZeroList zl) {
    if (*zl.count <= kZeroCap) return;
    const long long begin = offsets ? offsets[v] : 0;
    const long long end = offsets ? offsets[v + 1] : single_n;
    for (long long i = begin + blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < end;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        unsigned long long zb = static_cast<unsigned long long>(__double_as_longlong(pts[3 * i + 2]));
        if ((zb << 1) != 0) continue;
        long long r = axis_index(tb.row, pts[3 * i + 1]);
        if (r < 0) continue;
        long long c = axis_index(tb.col, pts[3 * i]);
        if (c < 0) continue;
        long long cell = r * tb.col.n + c;
        if (keys[cell] == kZeroKey) atomicMin(first + cell, static_cast<unsigned long long>(i));
    }
}

// Key of a cell's nanmax with the zero sign resolved (0 = empty cell).
__device__ __forceinline__ unsigned long long cell_key(unsigned long long k, long long cell,
                                                       const unsigned long long *first, const double *pts,
                                                       int has_zero) {
    if (k == kZeroKey && has_zero) return key_from_double(pts[3 * first[cell] + 2]);
    return k;
}

__device__ __forceinline__ double key_value(unsigned long long k) {
    return k == kEmptyKey ? __longlong_as_double(0x7ff8000000000000ll) : double_from_key(k);
}

// nanmax grid (FP64) from the keys.
__global__ void decode_kernel(const unsigned long long *__restrict__ keys,
                              const unsigned long long *__restrict__ first,
                              const double *__restrict__ pts, ZeroList zl,
                              double *__restrict__ out, long long total) {
    const int hz = *zl.count > 0;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x)
        out[c] = key_value(cell_key(keys[c], c, first, pts, hz));
}

// numpy's median of the n <= 8 non-NaN neighbour values, given as order-preserving keys:
// sorted s, odd n -> (0 + s[n/2]) / 1, even n -> ((0 + s[n/2-1]) + s[n/2]) / 2 (the sum
// reduction starts from its identity 0, which also turns -0 into +0).
__device__ __forceinline__ double median_keys(unsigned long long *s, int n) {
    for (int i = 1; i < n; ++i) {          // insertion sort
        const unsigned long long v = s[i];
        int j = i - 1;
        while (j >= 0 && s[j] > v) {
            s[j + 1] = s[j];
            --j;
        }
        s[j + 1] = v;
    }
    if (n & 1) {
        unsigned long long k = s[n >> 1];
        if (k == 0x7fffffffffffffffull) k = kZeroKey;   // -0 + 0 = +0
        return double_from_key(k);
    }
    return __dmul_rn(__dadd_rn(__dadd_rn(0.0, double_from_key(s[(n >> 1) - 1])), double_from_key(s[n >> 1])), 0.5);
}

__device__ __forceinline__ bool nan_double(double v) {
    return is_nan_bits(static_cast<unsigned long long>(__double_as_longlong(v)));
}

// Non-propagating hole fill (lib/proj_to_grid.py:64-79) on an FP64 grid.
__global__ void hole_fill_kernel(const double *__restrict__ in, double *__restrict__ out, long long H,
                                 long long W, long long total) {
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long plane = c / (H * W);
        const long long rc = c - plane * H * W;
        const long long r = rc / W, col = rc - r * W;
        const double *img = in + plane * H * W;
        double v = img[rc];
        if (!nan_double(v)) {
            out[c] = v;
            continue;
        }
        unsigned long long s[8];
        int n = 0;
        for (int dj = -1; dj <= 1; ++dj)
            for (int dk = -1; dk <= 1; ++dk) {
                long long j = r + dj, k = col + dk;
                if (j < 0 || j >= H || k < 0 || k >= W) continue;
                double u = img[j * W + k];
                if (!nan_double(u)) s[n++] = key_from_double(u);
            }
        out[c] = n ? median_keys(s, n) : v;
    }
}

// Round-to-nearest FP64 -> FP32 (astype(np.float32)) with integer operations; the
// conversion instruction runs on GB300's narrow FP64 pipe, so it is kept for the
// float-subnormal range only.
__device__ __forceinline__ float f64_to_f32(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    const unsigned sign = static_cast<unsigned>(b >> 32) & 0x80000000u;
    const int e = static_cast<int>((b >> 52) & 0x7ff);
    const unsigned long long m = b & 0xfffffffffffffull;
    if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));   // inf / NaN
    const int e32 = e - 1023 + 127;
    if (e32 >= 255) return __uint_as_float(sign | 0x7f800000u);                          // overflow
    if (e == 0 && m == 0) return __uint_as_float(sign);                                   // signed zero
    if (e32 <= 0) return __double2float_rn(v);                                           // float-subnormal range
    const unsigned m23 = static_cast<unsigned>(m >> 29);
    const unsigned rem = static_cast<unsigned>(m & 0x1fffffffu);
    const unsigned up = (rem > 0x10000000u) || (rem == 0x10000000u && (m23 & 1u));
    return __uint_as_float(sign | ((static_cast<unsigned>(e32) << 23) + m23 + up));       // carry may round to inf
}

// ---- 3x3 median blur (float32, replicate border, NaN after every number) -----------------
__device__ __forceinline__ unsigned blur_key(float v) {
    const unsigned b = __float_as_uint(v);
    return (b & 0x7fffffffu) > 0x7f800000u ? 0xffffffffu : key_from_float(v);
}
__device__ __forceinline__ void sort3(unsigned &a, unsigned &b, unsigned &c) {
    unsigned lo = min(a, b), hi = max(a, b);
    a = lo; b = hi;
    lo = min(b, c); hi = max(b, c);
    b = lo; c = hi;
    lo = min(a, b); hi = max(a, b);
    a = lo; b = hi;
}
__device__ __forceinline__ unsigned med3(unsigned a, unsigned b, unsigned c) {
    return max(min(a, b), min(max(a, b), c));
}
// Median of 9 from three sorted columns: med3(max of lows, med3 of mids, min of highs).
__device__ __forceinline__ float median9(unsigned a0, unsigned a1, unsigned a2, unsigned b0,
                                         unsigned b1, unsigned b2, unsigned c0, unsigned c1,
                                         unsigned c2) {
    sort3(a0, a1, a2);
    sort3(b0, b1, b2);
    sort3(c0, c1, c2);
    unsigned k = med3(max(max(a0, b0), c0), med3(a1, b1, c1), min(min(a2, b2), c2));
    return k == 0xffffffffu ? __uint_as_float(0x7fffffffu) : float_from_key(k);
}

template <typename T>
__device__ __forceinline__ float as_f32(T v) { return static_cast<float>(v); }
template <>
__device__ __forceinline__ float as_f32<double>(double v) { return f64_to_f32(v); }

template <typename T>
__global__ void median_blur3x3_kernel(const T *__restrict__ in, float *__restrict__ out, long long H,
                                      long long W, long long total) {
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long plane = c / (H * W);
        const long long rc = c - plane * H * W;
        const long long r = rc / W, col = rc - r * W;
        const T *img = in + plane * H * W;
        const long long rm = r > 0 ? r - 1 : 0, rp = r + 1 < H ? r + 1 : H - 1;
        const long long cm = col > 0 ? col - 1 : 0, cp = col + 1 < W ? col + 1 : W - 1;
        unsigned k[9];
        const long long rows[3] = {rm, r, rp}, cols[3] = {cm, col, cp};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) k[3 * b + a] = blur_key(as_f32(img[rows[a] * W + cols[b]]));
        out[c] = median9(k[0], k[1], k[2], k[3], k[4], k[5], k[6], k[7], k[8]);
    }
}

// ---- fused produce_dsm epilogue: keys -> nanmax -> hole fill -> float32 -> blur ---------
// One 32x8 output tile per CTA; the key tile carries a 2-cell halo (hole fill needs the
// 3x3 neighbourhood of each blurred cell's 3x3 neighbourhood).
constexpr int TX = 32, TY = 8;

__global__ void __launch_bounds__(TX *TY) dsm_epilogue_kernel(
    const unsigned long long *__restrict__ vk, const unsigned long long *__restrict__ first,
    const double *__restrict__ pts, ZeroList zl, float *__restrict__ out, long long H, long long W) {
    __shared__ unsigned long long raw[TY + 4][TX + 4];   // 0: empty cell or outside the image
    __shared__ float filled[TY + 2][TX + 2];
    const long long r0 = static_cast<long long>(blockIdx.y) * TY, c0 = static_cast<long long>(blockIdx.x) * TX;
    const int hz = *zl.count > 0;
    const int tid = threadIdx.y * TX + threadIdx.x;
    for (int i = tid; i < (TY + 4) * (TX + 4); i += TX * TY) {
        int ly = i / (TX + 4), lx = i - ly * (TX + 4);
        long long r = r0 + ly - 2, c = c0 + lx - 2;
        unsigned long long k = kEmptyKey;
        if (r >= 0 && r < H && c >= 0 && c < W) {
            long long cell = r * W + c;
            k = cell_key(vk[cell], cell, first, pts, hz);
        }
        raw[ly][lx] = k;
    }
    __syncthreads();
    for (int i = tid; i < (TY + 2) * (TX + 2); i += TX * TY) {
        int ly = i / (TX + 2), lx = i - ly * (TX + 2);
        const unsigned long long k = raw[ly + 1][lx + 1];
        float f;
        if (k != kEmptyKey) {
            f = f64_to_f32(double_from_key(k));
        } else {
            unsigned long long s[8];
            int n = 0;
            for (int dj = 0; dj < 3; ++dj)
                for (int dk = 0; dk < 3; ++dk) {
                    const unsigned long long u = raw[ly + dj][lx + dk];
                    if (u != kEmptyKey) s[n++] = u;
                }
            f = n ? f64_to_f32(median_keys(s, n)) : __uint_as_float(0x7fffffffu);
        }
        filled[ly][lx] = f;
    }
    __syncthreads();
    const long long r = r0 + threadIdx.y, c = c0 + threadIdx.x;
    if (r >= H || c >= W) return;
    // replicate border: clamp the neighbour coordinates into the image
    unsigned k[9];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        long long rr = r + a - 1;
        rr = rr < 0 ? 0 : (rr >= H ? H - 1 : rr);
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            long long cc = c + b - 1;
            cc = cc < 0 ? 0 : (cc >= W ? W - 1 : cc);
            k[3 * b + a] = blur_key(filled[rr - r0 + 1][cc - c0 + 1]);
        }
    }
    out[r * W + c] = median9(k[0], k[1], k[2], k[3], k[4], k[5], k[6], k[7], k[8]);
}

// ---- host side --------------------------------------------------------------------------
int make_axis(Axis &ax, double off, double res, long long n, int dir, long long *thr,
              cudaStream_t st) {
    ax.off = off;
    ax.res = res;
    ax.n = n;
    ax.thr = thr;
    ax.dir = dir;
    ax.neg = off < 0;
    unsigned long long b;
    memcpy(&b, &off, sizeof b);
    ax.top12 = b >> 52;
    const unsigned e = static_cast<unsigned>((b >> 52) & 0x7ff);
    ax.fast = 0;
    ax.mul = 0;
    if (!(e >= 1 && e <= 2046 && isfinite(res) && res >= 1e-9 && res <= 1e9)) return VS_OK;
    const double ulp = ldexp(1.0, static_cast<int>(e) - 1075);
    // thresholds below 2^52 ulps (same-exponent differences) and an estimate multiplier < 2^64
    if (static_cast<double>(n + 1) * res / ulp >= 4503599627370496.0 || ulp >= res) return VS_OK;
    ax.fast = 1;
    ax.mul = static_cast<unsigned long long>(ldexp(ulp / res, 64));
    const int threads = 256;
    axis_thresholds_kernel<<<static_cast<unsigned>(ceil_div(n + 1, threads)), threads, 0, st>>>(thr, n, ulp, res);
    return check_launch("axis_thresholds_kernel");
}

struct RasterWs {
    unsigned long long *keys, *first;   // one grid, reused view after view
    long long *row_thr, *col_thr;
    ZeroList zl;
    size_t bytes;
};

RasterWs carve_raster(void *ws, long long xsize, long long ysize) {
    Carver cv(ws);
    RasterWs r;
    const size_t cells = static_cast<size_t>(xsize) * ysize;
    r.keys = cv.take<unsigned long long>(cells);
    r.first = cv.take<unsigned long long>(cells);
    r.row_thr = cv.take<long long>(ysize + 1);
    r.col_thr = cv.take<long long>(xsize + 1);
    r.zl.entries = cv.take<unsigned long long>(2 * static_cast<size_t>(kZeroCap));
    r.zl.count = cv.take<int>(1);
    r.bytes = cv.used;
    return r;
}

int make_tables(double xoff, double yoff, double xres, double yres, long long xsize, long long ysize,
                RasterWs &w, Tables &tb, cudaStream_t st) {
    int s;
    // rows: a = yoff - y divided by xresolution; cols: a = x - xoff divided by yresolution
    if ((s = make_axis(tb.row, yoff, xres, ysize, -1, w.row_thr, st)) != VS_OK) return s;
    return make_axis(tb.col, xoff, yres, xsize, +1, w.col_thr, st);
}

// Bins one view's points into the (reset) key grid and resolves zero signs.  Views are
// processed in stream order so that the key grid being hit by the atomics stays in L2.
int bin_view(const double *points, const long long *offsets, int v, long long single_n, long long max_points,
             const Tables &tb, RasterWs &w, long long cells, cudaStream_t st) {
    if (cudaMemsetAsync(w.keys, 0, sizeof(unsigned long long) * cells, st) != cudaSuccess ||
        cudaMemsetAsync(w.zl.count, 0, sizeof(int), st) != cudaSuccess) {
        set_error("cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
    if (max_points <= 0) return VS_OK;
    const int threads = 256;
    long long want = ceil_div(ceil_div(max_points, 2), threads);
    long long cap = static_cast<long long>(sm_count()) * 8;
    unsigned gx = static_cast<unsigned>(std::max(1LL, std::min(want, cap)));
    bin_max_kernel<<<gx, threads, 0, st>>>(points, offsets, v, single_n, tb, w.keys, w.zl);
    VS_LAUNCH_CHECK("bin_max_kernel");
    const unsigned gl = static_cast<unsigned>(kZeroCap / threads);
    zero_list_init_kernel<<<gl, threads, 0, st>>>(w.keys, w.first, w.zl);
    VS_LAUNCH_CHECK("zero_list_init_kernel");
    zero_list_min_kernel<<<gl, threads, 0, st>>>(w.keys, w.first, w.zl);
    VS_LAUNCH_CHECK("zero_list_min_kernel");
    unsigned gz = static_cast<unsigned>(std::min<long long>(ceil_div(cells, threads), sm_count() * 8LL));
    zero_init_kernel<<<gz, threads, 0, st>>>(w.keys, w.first, cells, w.zl);
    VS_LAUNCH_CHECK("zero_init_kernel");
    zero_first_kernel<<<std::max<unsigned>(gx / 4, 1u), threads, 0, st>>>(points, offsets, v, single_n, tb, w.keys,
                                                                          w.first, w.zl);
    VS_LAUNCH_CHECK("zero_first_kernel");
    return VS_OK;
}

}  // namespace

int launch_blur_f32(const float *in, float *out, long long h, long long w, cudaStream_t st) {
    const long long total = h * w;
    const int threads = 256;
    unsigned g = static_cast<unsigned>(std::min<long long>(ceil_div(total, threads), sm_count() * 16LL));
    median_blur3x3_kernel<float><<<g, threads, 0, st>>>(in, out, h, w, total);
    return check_launch("median_blur3x3_kernel<float>");
}

}  // namespace vs

using namespace vs;

extern "C" size_t vs_proj_to_grid_workspace_size(int64_t xsize, int64_t ysize) {
    if (xsize <= 0 || ysize <= 0) return 0;
    return carve_raster(nullptr, xsize, ysize).bytes + sizeof(double) * xsize * ysize + 512;
}

extern "C" int vs_proj_to_grid(const double *points, int64_t n, double xoff, double yoff,
                               double xresolution, double yresolution, int64_t xsize, int64_t ysize,
                               double *dsm, void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n >= 0 && xsize > 0 && ysize > 0, "vs_proj_to_grid: bad sizes n=%lld grid=%lldx%lld",
               (long long)n, (long long)xsize, (long long)ysize);
    VS_REQUIRE(dsm && (points || n == 0) && workspace, "vs_proj_to_grid: null pointer");
    const size_t need = vs_proj_to_grid_workspace_size(xsize, ysize);
    if (workspace_bytes < need) {
        set_error("vs_proj_to_grid: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    RasterWs w = carve_raster(workspace, xsize, ysize);
    Carver cv(workspace);
    cv.used = w.bytes;
    double *nanmax = cv.take<double>(static_cast<size_t>(xsize) * ysize);
    Tables tb;
    const long long cells = xsize * ysize;
    int s = make_tables(xoff, yoff, xresolution, yresolution, xsize, ysize, w, tb, st);
    if (s == VS_OK) s = bin_view(points, nullptr, 0, n, n, tb, w, cells, st);
    if (s != VS_OK) return s;
    const int threads = 256;
    unsigned g = static_cast<unsigned>(std::min<long long>(ceil_div(cells, threads), sm_count() * 16LL));
    decode_kernel<<<g, threads, 0, st>>>(w.keys, w.first, points, w.zl, nanmax, cells);
    VS_LAUNCH_CHECK("decode_kernel");
    hole_fill_kernel<<<g, threads, 0, st>>>(nanmax, dsm, ysize, xsize, cells);
    VS_LAUNCH_CHECK("hole_fill_kernel");
    return VS_OK;
}

extern "C" size_t vs_dsm_from_points_workspace_size(int n_views, int64_t xsize, int64_t ysize) {
    if (n_views <= 0 || xsize <= 0 || ysize <= 0) return 0;
    return carve_raster(nullptr, xsize, ysize).bytes + 256;
}

extern "C" int vs_dsm_from_points(const double *points, const int64_t *offsets, int n_views, double xoff,
                                  double yoff, double xresolution, double yresolution, int64_t xsize,
                                  int64_t ysize, float *dsm, void *workspace, size_t workspace_bytes,
                                  void *stream) {
    VS_REQUIRE(n_views > 0 && xsize > 0 && ysize > 0, "vs_dsm_from_points: bad sizes views=%d grid=%lldx%lld",
               n_views, (long long)xsize, (long long)ysize);
    VS_REQUIRE(points && offsets && dsm && workspace, "vs_dsm_from_points: null pointer");
    const size_t need = vs_dsm_from_points_workspace_size(n_views, xsize, ysize);
    if (workspace_bytes < need) {
        set_error("vs_dsm_from_points: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    RasterWs w = carve_raster(workspace, xsize, ysize);
    Tables tb;
    const long long cells = xsize * ysize;
    int s = make_tables(xoff, yoff, xresolution, yresolution, xsize, ysize, w, tb, st);
    if (s != VS_OK) return s;
    // per-view counts live on the device: launch for a full GPU and let the grid stride
    const long long launch_points = static_cast<long long>(sm_count()) * 8 * 256 * 2;
    const dim3 egrid(static_cast<unsigned>(ceil_div(xsize, TX)), static_cast<unsigned>(ceil_div(ysize, TY)));
    for (int v = 0; v < n_views; ++v) {
        s = bin_view(points, reinterpret_cast<const long long *>(offsets), v, 0, launch_points, tb, w, cells, st);
        if (s != VS_OK) return s;
        dsm_epilogue_kernel<<<egrid, dim3(TX, TY), 0, st>>>(w.keys, w.first, points, w.zl, dsm + v * cells,
                                                            ysize, xsize);
        VS_LAUNCH_CHECK("dsm_epilogue_kernel");
    }
    return VS_OK;
}

extern "C" int vs_median_blur3x3_f32(const float *in, float *out, int64_t h, int64_t w, int64_t n_img,
                                     void *stream) {
    VS_REQUIRE(h > 0 && w > 0 && n_img > 0 && in && out && in != out, "vs_median_blur3x3_f32: bad arguments");
    const long long total = h * w * n_img;
    const int threads = 256;
    unsigned g = static_cast<unsigned>(std::min<long long>(ceil_div(total, threads), sm_count() * 16LL));
    median_blur3x3_kernel<float><<<g, threads, 0, as_stream(stream)>>>(in, out, h, w, total);
    VS_LAUNCH_CHECK("median_blur3x3_kernel<float>");
    return VS_OK;
}

extern "C" int vs_median_blur3x3_f64(const double *in, float *out, int64_t h, int64_t w, int64_t n_img,
                                     void *stream) {
    VS_REQUIRE(h > 0 && w > 0 && n_img > 0 && in && out, "vs_median_blur3x3_f64: bad arguments");
    const long long total = h * w * n_img;
    const int threads = 256;
    unsigned g = static_cast<unsigned>(std::min<long long>(ceil_div(total, threads), sm_count() * 16LL));
    median_blur3x3_kernel<double><<<g, threads, 0, as_stream(stream)>>>(in, out, h, w, total);
    VS_LAUNCH_CHECK("median_blur3x3_kernel<double>");
    return VS_OK;
}
