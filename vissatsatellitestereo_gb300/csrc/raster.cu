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
// two equal values, which only shows for +0/-0: zeros share one key, and every zero point
// also posts its index into a per-cell "first zero" word (atomicMax of a view epoch tag and
// the complemented index), from which the epilogue takes the sign when a cell's maximum is
// zero.  The epoch tag makes stale words of earlier views lose without any clearing.
//
// GB300 issues FP64 arithmetic, FP64 compares, 64-bit multiply-high and several
// conversions to a narrow pipe (measured: DADD 1.6, umul64hi 6.4, F2I 15 lane-ops per
// clock per SM, against ~100 for FFMA and ~136 for 32-bit IMAD), so the per-point and
// per-cell paths here use 32-bit integer and FP32 operations only.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cstdlib>
#include <vector>

#include "common.cuh"
#include "geo.cuh"

namespace vs {
namespace {

constexpr unsigned long long kEmptyKey = 0ull;
constexpr unsigned long long kZeroKey = 0x8000000000000000ull;   // key of +0.0

// One axis of the DSM grid.  dir = +1: a = v - off (columns), dir = -1: a = off - v (rows).
struct Axis {
    double off, res;
    long long n;                 // cells along the axis
    const long long *thr;        // n + 1 integer thresholds (ulps of off), fast path only
    long long tmax;              // thr[n]: first difference beyond the grid
    unsigned top12;              // sign + exponent of off
    int shift;                   // d >> shift < 2^32
    float scale;                 // 2^shift * ulp(off) / res, so that q ~ (d >> shift) * scale
    float err_abs, err_rel;      // bound of |q - d * ulp / res|: err_abs + err_rel * q
    // integer estimate: umulhi(d >> shift, mul) ~ q * 2^fbits; its fraction f (low fbits
    // bits) proves the row when 4 <= f <= 2^fbits - 5
    unsigned mul, fmask, fsure;
    int fbits;
    int neg;                     // off < 0
    int dir;
    int fast;                    // fast path usable
    int contained;               // grid range (+-2 cells) inside off's sign/exponent interval
};

struct Tables {
    Axis row, col;
};

__device__ __forceinline__ int axis_exact(const Axis &ax, double v) {
    const double a = ax.dir > 0 ? rare_dsub(v, ax.off) : rare_dsub(ax.off, v);
    const double q = rare_ddiv(a, ax.res);
    if (!(q >= 0.0 && q < static_cast<double>(ax.n))) return -1;
    return static_cast<int>(q);   // q >= 0: truncation is floor
}

// Cell index along one axis, or -1 when the point falls outside the grid.  The FP32
// estimate q carries a proven error bound; unless q lies within that bound of an integer,
// its floor is the reference's floor(fl(d*ulp/res)).  Near a boundary the integer
// threshold table decides (about 0.1% of points).  A point with another sign or exponent
// than the origin is off-grid when the grid lies inside the origin's exponent interval;
// otherwise (EXACT instantiation) it takes the literal FP64 expression.
template <bool EXACT>
__device__ __forceinline__ int axis_index(const Axis &ax, double v) {
    const long long bv = __double_as_longlong(v);
    const unsigned hi = static_cast<unsigned>(static_cast<unsigned long long>(bv) >> 32);
    if (ax.fast && (hi >> 20) == ax.top12) {
        const long long bo = __double_as_longlong(ax.off);
        const long long d = ((ax.dir > 0) != (ax.neg != 0)) ? (bv - bo) : (bo - bv);
        if (d < 0 || d >= ax.tmax) return -1;
        const unsigned u = static_cast<unsigned>(static_cast<unsigned long long>(d) >> ax.shift);
        const float q = __fmul_rn(__uint2float_rn(u), ax.scale);
        const float big = __fadd_rn(q, 12582912.0f);                  // 1.5 * 2^23: rounds q to an integer
        const float rn = __fsub_rn(big, 12582912.0f);
        const float fr = __fsub_rn(q, rn);                            // exact, in [-0.5, 0.5]
        int r = (__float_as_int(big) - 0x4b400000) - (fr < 0.0f ? 1 : 0);
        if (fabsf(fr) > __fmaf_rn(ax.err_rel, q, ax.err_abs)) return min(max(r, 0), static_cast<int>(ax.n - 1));
        r = min(max(r, 0), static_cast<int>(ax.n - 1));
#pragma unroll 1
        for (int it = 0; it < 8 && __ldg(ax.thr + r) > d; ++it) --r;
#pragma unroll 1
        for (int it = 0; it < 8 && __ldg(ax.thr + r + 1) <= d; ++it) ++r;
        return r;
    }
    if constexpr (EXACT) {
        return axis_exact(ax, v);
    } else {
        return -1;
    }
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

// "first zero" words: epoch tag in the top 24 bits, complemented point index below.
constexpr unsigned long long kIdxMask = (1ull << 40) - 1;
__host__ __device__ __forceinline__ unsigned long long epoch_tag(int view) {
    return static_cast<unsigned long long>(view + 1) << 40;
}

constexpr int kPts = 4;   // consecutive points per thread (runs in the same cell merge)

template <bool EXACT>
__device__ __forceinline__ void bin_point(const Tables &tb, double x, double y, double z, long long index,
                                          unsigned long long *vk, unsigned long long *first,
                                          unsigned long long tag, long long &run_cell,
                                          unsigned long long &run_key) {
    const unsigned long long zb = static_cast<unsigned long long>(__double_as_longlong(z));
    if (is_nan_bits(zb)) return;
    const int r = axis_index<EXACT>(tb.row, y);
    if (r < 0) return;
    const int c = axis_index<EXACT>(tb.col, x);
    if (c < 0) return;
    const long long cell = static_cast<long long>(static_cast<unsigned long long>(static_cast<unsigned>(r)) *
                                                  static_cast<unsigned>(tb.col.n)) + c;
    unsigned long long key;
    if ((zb << 1) == 0) {            // +-0: one shared key; the sign comes from the first zero
        key = kZeroKey;
        atomicMax(first + cell, tag | (kIdxMask - static_cast<unsigned long long>(index)));
    } else {
        key = key_from_double(z);
    }
    if (cell == run_cell) {
        run_key = max(run_key, key);
    } else {
        if (run_key) atomicMax(vk + run_cell, run_key);
        run_cell = cell;
        run_key = key;
    }
}

// Bins one view's points: atomicMax of the height keys into the view's key grid.
// View v owns points [offsets[v], offsets[v+1]).
template <bool EXACT>
__global__ void __launch_bounds__(256) bin_max_kernel(const double *__restrict__ pts,
                                                      const long long *__restrict__ offsets, int v,
                                                      long long single_n, Tables tb,
                                                      unsigned long long *__restrict__ vk,
                                                      unsigned long long *__restrict__ first) {
    const long long begin = offsets ? offsets[v] : 0;
    const long long end = offsets ? offsets[v + 1] : single_n;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x * kPts;
    const unsigned long long tag = epoch_tag(v);
    for (long long i = begin + (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) * kPts; i < end;
         i += stride) {
        double p[3 * kPts];
        const double *src = pts + 3 * i;
        if (i + kPts <= end && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
            const double2 *s2 = reinterpret_cast<const double2 *>(src);
#pragma unroll
            for (int k = 0; k < 3 * kPts / 2; ++k) {
                const double2 a = __ldcs(s2 + k);
                p[2 * k] = a.x;
                p[2 * k + 1] = a.y;
            }
        } else {
#pragma unroll
            for (int k = 0; k < kPts; ++k) {
                const bool in = i + k < end;
                p[3 * k] = in ? __ldcs(src + 3 * k) : 0.0;
                p[3 * k + 1] = in ? __ldcs(src + 3 * k + 1) : 0.0;
                p[3 * k + 2] = in ? __ldcs(src + 3 * k + 2) : __longlong_as_double(0x7ff8000000000000ll);
            }
        }
        long long run_cell = -1;
        unsigned long long run_key = 0;
#pragma unroll
        for (int k = 0; k < kPts; ++k)
            bin_point<EXACT>(tb, p[3 * k], p[3 * k + 1], p[3 * k + 2], i + k, vk, first, tag, run_cell, run_key);
        if (run_key) atomicMax(vk + run_cell, run_key);
    }
}

// ---- the common-case binning kernel -------------------------------------------------------
// Both axes on the fast path and the grid inside the origins' exponent intervals: every
// point is handled with integer and FP32 operations, the coordinates are carried as raw
// 64-bit patterns (double-typed values make the compiler emit FP64 moves), the axis
// constants live in registers, the row/column estimates are branch-free, and the four
// points of a thread are merged into runs before their atomics.
struct FastAxis {
    long long off_bits, tmax;
    const long long *thr;
    unsigned top12;
    int shift, nm1;
    float scale, err_abs, err_rel;
    unsigned mul, fmask, fsure;
    int fbits;
};

FastAxis fast_axis_of(const Axis &ax) {
    FastAxis fa;
    memcpy(&fa.off_bits, &ax.off, sizeof(long long));
    fa.tmax = ax.tmax;
    fa.thr = ax.thr;
    fa.top12 = ax.top12;
    fa.shift = ax.shift;
    fa.nm1 = static_cast<int>(ax.n - 1);
    fa.scale = ax.scale;
    fa.err_abs = ax.err_abs;
    fa.err_rel = ax.err_rel;
    fa.mul = ax.mul;
    fa.fmask = ax.fmask;
    fa.fsure = ax.fsure;
    fa.fbits = ax.fbits;
    return fa;
}

// Row from u = d >> shift by one 32-bit multiply-high: hi = floor(u * mul / 2^32) is the
// quotient q = d * ulp / res in units of 2^-fbits cells, within [-0.5, 1.5) units plus
// the reference's own FP64 rounding (2^-21 units); so when its fraction f = hi mod 2^fbits
// keeps 4 units from both cell boundaries, hi >> fbits is the reference's
// floor(fl(d * ulp / res)).  Integer multiply and logic only (no conversion, no FP32).
__device__ __forceinline__ void axis_estimate(const FastAxis &a, unsigned u, int &r, bool &sure) {
    const unsigned hi = __umulhi(u, a.mul);
    r = static_cast<int>(hi >> a.fbits);
    sure = ((hi & a.fmask) - 4u) < a.fsure;
}

template <bool FLIP>   // FLIP: d = off - v (rows of a positive origin, columns of a negative one)
__device__ __forceinline__ bool axis_fast(const FastAxis &a, long long bv, int &r, long long &d, bool &sure) {
    const unsigned hi = static_cast<unsigned>(static_cast<unsigned long long>(bv) >> 32);
    d = FLIP ? (a.off_bits - bv) : (bv - a.off_bits);
    const bool ok = ((hi >> 20) == a.top12) & (d >= 0) & (d < a.tmax);
    const unsigned u = static_cast<unsigned>(static_cast<unsigned long long>(d) >> a.shift);
    const float q = __fmul_rn(__uint2float_rn(u), a.scale);
    const float big = __fadd_rn(q, 12582912.0f);
    const float fr = __fsub_rn(q, __fsub_rn(big, 12582912.0f));
    const int rn = static_cast<int>(static_cast<unsigned>(__float_as_int(big)) - 0x4b400000u);
    r = min(max(rn - (fr < 0.0f ? 1 : 0), 0), a.nm1);
    sure = fabsf(fr) > __fmaf_rn(a.err_rel, q, a.err_abs);
    return ok;
}

__device__ __noinline__ int axis_correct(const long long *thr, int r, long long d) {
    for (int it = 0; it < 8 && __ldg(thr + r) > d; ++it) --r;
    for (int it = 0; it < 8 && __ldg(thr + r + 1) <= d; ++it) ++r;
    return r;
}

// Row/column of a contained axis from the coordinate's bit pattern.  d is the wrapped
// 64-bit difference of the bit patterns; one unsigned compare with tmax rejects every
// coordinate off the grid, including those of the other sign or another binade (their
// wrapped difference is at least the origin's bit pattern, far above tmax, because the
// grid +-2 cells lies inside the origin's binade) and NaN/inf.
template <bool FLIP>
__device__ __forceinline__ bool axis_contained(const FastAxis &a, long long bv, int &r, long long &d, bool &sure) {
    const unsigned long long ud = FLIP ? static_cast<unsigned long long>(a.off_bits) - static_cast<unsigned long long>(bv)
                                       : static_cast<unsigned long long>(bv) - static_cast<unsigned long long>(a.off_bits);
    d = static_cast<long long>(ud);
    const bool ok = ud < static_cast<unsigned long long>(a.tmax);
    axis_estimate(a, static_cast<unsigned>(ud >> a.shift), r, sure);   // r <= nm1 when ok && sure
    return ok;
}

// Points per thread of the fast binning kernel.  Measured on one 4096^2 view (16.8 M points,
// 2000^2 grid, 2 waves of CTAs of 256): 2 points per thread bin it in 0.0765 ms, 4 in
// 0.0814 ms, 8 in 0.098 ms; issuing the next points' loads before binning the current ones
// (register double buffering) is slower too -- the kernel is bound by the latency of its
// binning chain, so resident warps matter more than loads in flight per thread.  Grids
// of 1.33 or 2.67 waves were slower than whole waves.
constexpr int kFastPts = 2;

// The kFastPts points of one thread: raw 64-bit words (x, y, z per point).
struct PointBlock {
    long long w[3 * kFastPts];
};

__device__ __forceinline__ void load_block(const long long *__restrict__ bits, long long i, long long end,
                                           PointBlock &b) {
    const long long *src = bits + 3 * i;
    if (i + kFastPts <= end && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
        const longlong2 *s2 = reinterpret_cast<const longlong2 *>(src);
#pragma unroll
        for (int k = 0; k < 3 * kFastPts / 2; ++k) {
            const longlong2 a = __ldcs(s2 + k);
            b.w[2 * k] = a.x;
            b.w[2 * k + 1] = a.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kFastPts; ++k) {
            const bool in = i + k < end;
            b.w[3 * k] = in ? __ldcs(src + 3 * k) : 0ll;
            b.w[3 * k + 1] = in ? __ldcs(src + 3 * k + 1) : 0ll;
            b.w[3 * k + 2] = in ? __ldcs(src + 3 * k + 2) : 0x7ff8000000000000ll;
        }
    }
}

// The kFastPts consecutive points of one thread starting at index i: each point's cell from
// its coordinates' bit patterns (32-bit cell indices: the grid holds < 2^31 cells), runs of
// consecutive points in one cell merged before the 64-bit atomicMax of their keys.
template <bool FLIP_ROW, bool FLIP_COL>
__device__ __forceinline__ void bin_fast_block(const long long *__restrict__ bits, long long i, long long end,
                                               const FastAxis &R, const FastAxis &C, unsigned ncols,
                                               unsigned long long tag, unsigned long long *__restrict__ vk,
                                               unsigned long long *__restrict__ first) {
    PointBlock b;
    load_block(bits, i, end, b);
    unsigned cell[kFastPts];
    unsigned long long key[kFastPts];
    bool okk[kFastPts];
#pragma unroll
    for (int k = 0; k < kFastPts; ++k) {
        const unsigned long long zb = static_cast<unsigned long long>(b.w[3 * k + 2]);
        int r, c;
        long long dr, dc;
        bool sr, sc;
        bool ok = axis_contained<FLIP_ROW>(R, b.w[3 * k + 1], r, dr, sr);
        ok &= axis_contained<FLIP_COL>(C, b.w[3 * k], c, dc, sc);
        ok &= !is_nan_bits(zb);
        if (ok && !sr) r = axis_correct(R.thr, min(r, R.nm1), dr);
        if (ok && !sc) c = axis_correct(C.thr, min(c, C.nm1), dc);
        const unsigned cl = static_cast<unsigned>(r) * ncols + static_cast<unsigned>(c);
        const bool zero = (zb << 1) == 0;
        if (ok && zero) atomicMax(first + cl, tag | (kIdxMask - static_cast<unsigned long long>(i + k)));
        const unsigned long long kz = (zb >> 63) ? ~zb : (zb | 0x8000000000000000ull);
        key[k] = ok ? (zero ? kZeroKey : kz) : kEmptyKey;
        cell[k] = cl;
        okk[k] = ok;
    }
#pragma unroll
    for (int k = 1; k < kFastPts; ++k) {     // merge runs of consecutive points in one cell
        const bool same = okk[k] & okk[k - 1] & (cell[k] == cell[k - 1]);
        key[k] = same ? max(key[k], key[k - 1]) : key[k];
        key[k - 1] = same ? kEmptyKey : key[k - 1];
    }
#pragma unroll
    for (int k = 0; k < kFastPts; ++k)
        if (key[k] != kEmptyKey) atomicMax(vk + cell[k], key[k]);
}

// Grid-stride over blocks of kFastPts consecutive points.
template <bool FLIP_ROW, bool FLIP_COL>
__global__ void __launch_bounds__(256) bin_fast_kernel(const double *__restrict__ pts,
                                                       const long long *__restrict__ offsets, int v,
                                                       long long single_n, FastAxis ra, FastAxis ca,
                                                       unsigned long long *__restrict__ vk,
                                                       unsigned long long *__restrict__ first) {
    const long long begin = offsets ? offsets[v] : 0;
    const long long end = offsets ? offsets[v + 1] : single_n;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x * kFastPts;
    const unsigned long long tag = epoch_tag(v);
    const FastAxis R = ra, C = ca;
    const unsigned ncols = static_cast<unsigned>(C.nm1 + 1);
    const long long *bits = reinterpret_cast<const long long *>(pts);
    for (long long i = begin + (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) * kFastPts; i < end;
         i += stride)
        bin_fast_block<FLIP_ROW, FLIP_COL>(bits, i, end, R, C, ncols, tag, vk, first);
}

// Key of a cell's nanmax with the zero sign resolved (0 = empty cell).
__device__ __noinline__ unsigned long long zero_key(long long cell, const unsigned long long *first,
                                                    const double *pts) {
    const unsigned long long idx = kIdxMask - (first[cell] & kIdxMask);
    return key_from_double(pts[3 * idx + 2]);
}

__device__ __forceinline__ unsigned long long cell_key(unsigned long long k, long long cell,
                                                       const unsigned long long *first, const double *pts) {
    return k != kZeroKey ? k : zero_key(cell, first, pts);
}

__device__ __forceinline__ double key_value(unsigned long long k) {
    return k == kEmptyKey ? __longlong_as_double(0x7ff8000000000000ll) : double_from_key(k);
}

// nanmax grid (FP64) from the keys.
__global__ void decode_kernel(const unsigned long long *__restrict__ keys,
                              const unsigned long long *__restrict__ first,
                              const double *__restrict__ pts, double *__restrict__ out, long long total) {
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x)
        out[c] = key_value(cell_key(keys[c], c, first, pts));
}

// numpy's median of the non-empty keys among 8 (empty = 0), without local memory: the
// keys are sorted by an 8-input network with empty slots ordered last, and the middle
// one(s) selected by the count.
__device__ __forceinline__ void cswap(unsigned long long &a, unsigned long long &b) {
    const unsigned long long lo = a < b ? a : b, hi = a < b ? b : a;
    a = lo;
    b = hi;
}

// s[idx] through a select tree on the index bits (an indexed read would move s to local memory)
__device__ __forceinline__ unsigned long long select8(const unsigned long long (&s)[8], int idx) {
    const bool b0 = idx & 1, b1 = idx & 2, b2 = idx & 4;
    const unsigned long long a0 = b0 ? s[1] : s[0], a1 = b0 ? s[3] : s[2];
    const unsigned long long a2 = b0 ? s[5] : s[4], a3 = b0 ? s[7] : s[6];
    const unsigned long long c0 = b1 ? a1 : a0, c1 = b1 ? a3 : a2;
    return b2 ? c1 : c0;
}

// numpy's median from the middle keys of n sorted values (n odd: lo == hi's slot).
__device__ __forceinline__ double median_from_middle(unsigned long long lo, unsigned long long hi, int n) {
    if (n & 1) {
        if (hi == 0x7fffffffffffffffull) hi = kZeroKey;   // -0 + 0 = +0
        return double_from_key(hi);
    }
    return rare_dmul(rare_dadd(rare_dadd(0.0, double_from_key(lo)), double_from_key(hi)), 0.5);
}

__device__ __forceinline__ double median8_keys(unsigned long long (&s)[8]) {
    int n = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        n += s[i] != kEmptyKey;
        s[i] = s[i] == kEmptyKey ? ~0ull : s[i];      // empty sorts last
    }
    // Batcher's odd-even merge sort for 8 inputs (19 comparators)
    cswap(s[0], s[1]); cswap(s[2], s[3]); cswap(s[4], s[5]); cswap(s[6], s[7]);
    cswap(s[0], s[2]); cswap(s[1], s[3]); cswap(s[4], s[6]); cswap(s[5], s[7]);
    cswap(s[1], s[2]); cswap(s[5], s[6]);
    cswap(s[0], s[4]); cswap(s[1], s[5]); cswap(s[2], s[6]); cswap(s[3], s[7]);
    cswap(s[2], s[4]); cswap(s[3], s[5]);
    cswap(s[1], s[2]); cswap(s[3], s[4]); cswap(s[5], s[6]);
    return median_from_middle(select8(s, (n - 1) >> 1), select8(s, n >> 1), n);
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
        int m = 0;
        bool any = false;
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj)
#pragma unroll
            for (int dk = -1; dk <= 1; ++dk) {
                if (dj == 0 && dk == 0) continue;
                const long long j = r + dj, k = col + dk;
                unsigned long long key = kEmptyKey;
                if (j >= 0 && j < H && k >= 0 && k < W) {
                    const double u = img[j * W + k];
                    if (!nan_double(u)) key = key_from_double(u);
                }
                any |= key != kEmptyKey;
                s[m++] = key;
            }
        out[c] = any ? median8_keys(s) : v;
    }
}

// ---- 3x3 median blur: cv2.medianBlur(float32, ksize 3) ---------------------------------
// OpenCV 4.0's medianBlur_SortNet for ksize 3: Paeth's 9-input median network in
// Devillard's order (19 compare-exchanges, output p4), replicate border.  Its
// compare-exchange is `t = a; a = min(a, b); b = max(b, t)`, which decides what NaN does:
//   * scalar columns (MinMax32f, std::min/std::max): exchanged only when b < a;
//   * vector columns (MinMaxVec32f, SSE minps/maxps, which return the second operand
//     unless the comparison holds): kept only when a < b, so ties and NaN exchange.
// Per row OpenCV runs column 0 scalar, then 4 columns at a time from column 1 while
// j <= W - 5, then the remaining columns scalar.  A 1-high or 1-wide image is a median
// of 3 along the line with the scalar op.
template <bool VEC>
__device__ __forceinline__ void cv_exchange(float &a, float &b) {
    const bool x = VEC ? !(a < b) : (b < a);
    const float t = a;
    a = x ? b : a;
    b = x ? t : b;
}

template <bool VEC>
__device__ __forceinline__ float cv_median9(float p0, float p1, float p2, float p3, float p4, float p5, float p6,
                                            float p7, float p8) {
    cv_exchange<VEC>(p1, p2); cv_exchange<VEC>(p4, p5); cv_exchange<VEC>(p7, p8);
    cv_exchange<VEC>(p0, p1); cv_exchange<VEC>(p3, p4); cv_exchange<VEC>(p6, p7);
    cv_exchange<VEC>(p1, p2); cv_exchange<VEC>(p4, p5); cv_exchange<VEC>(p7, p8);
    cv_exchange<VEC>(p0, p3); cv_exchange<VEC>(p5, p8); cv_exchange<VEC>(p4, p7);
    cv_exchange<VEC>(p3, p6); cv_exchange<VEC>(p1, p4); cv_exchange<VEC>(p2, p5);
    cv_exchange<VEC>(p4, p7); cv_exchange<VEC>(p4, p2); cv_exchange<VEC>(p6, p4);
    cv_exchange<VEC>(p4, p2);
    return p4;
}

// p0..p8 = the window row by row; `vec` = the column is one of OpenCV's SSE columns.
__device__ __forceinline__ float cv_median9(bool vec, float p0, float p1, float p2, float p3, float p4, float p5,
                                            float p6, float p7, float p8) {
    return vec ? cv_median9<true>(p0, p1, p2, p3, p4, p5, p6, p7, p8)
               : cv_median9<false>(p0, p1, p2, p3, p4, p5, p6, p7, p8);
}

// The 1-D path (image 1 high or 1 wide): p0, p1, p2 consecutive along the line.
__device__ __forceinline__ float cv_median3_line(float p0, float p1, float p2) {
    cv_exchange<false>(p0, p1);
    cv_exchange<false>(p1, p2);
    cv_exchange<false>(p0, p1);
    return p1;
}

// Columns [1, 1 + 4 nv) of a W-wide image go through OpenCV's 4-lane loop.
__device__ __forceinline__ bool cv_vector_column(long long c, long long W) {
    const long long nv = W >= 6 ? (W - 6) / 4 + 1 : 0;
    return c >= 1 && c < 1 + 4 * nv;
}

// Sorted triple and median of three for NaN-free values (IEEE min/max).
__device__ __forceinline__ void sort3f(float a, float b, float c, float &lo, float &mid, float &hi) {
    const float l = fminf(a, b), h = fmaxf(a, b);
    lo = fminf(l, c);
    hi = fmaxf(h, c);
    mid = fmaxf(l, fminf(h, c));
}
__device__ __forceinline__ float med3f(float a, float b, float c) { return fmaxf(fminf(a, b), fminf(fmaxf(a, b), c)); }

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
        if (H == 1 || W == 1) {
            // the line runs along the dimension that is longer than 1 (both 1: the value)
            const long long a = H == 1 ? cm : rm * W, b = H == 1 ? col : r * W, d = H == 1 ? cp : rp * W;
            out[c] = cv_median3_line(as_f32(img[a]), as_f32(img[b]), as_f32(img[d]));
            continue;
        }
        float p[9];
        const long long rows[3] = {rm, r, rp}, cols[3] = {cm, col, cp};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) p[3 * a + b] = as_f32(img[rows[a] * W + cols[b]]);
        out[c] = cv_median9(cv_vector_column(col, W), p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8]);
    }
}

// ---- fused produce_dsm epilogue: keys -> nanmax -> hole fill -> float32 -> blur ---------
// One 32x32 output tile per CTA of 32x8 threads (4 outputs per thread, rows ty + 8j).  The
// key tile carries a 2-cell halo (hole fill needs the 3x3 neighbourhood of each blurred
// cell's 3x3 neighbourhood); the hole-filled float32 values are staged for the blur;
// 32-bit indexing (grid dimensions < 2^31).
constexpr int TX = 32, TY = 8, TILE_Y = 32;
constexpr int RAW_W = TX + 4, RAW_H = TILE_Y + 4, FK_W = TX + 2, FK_H = TILE_Y + 2;

// Shared-memory working set of one epilogue tile.
struct EpilogueSmem {
    unsigned long long raw[RAW_H * RAW_W];   // 0: empty cell or outside the image
    float fk[FK_H][FK_W];                    // hole-filled cells as float32 (the blur's input)
    unsigned short holes[FK_H * FK_W];
    int n_holes;
};

// One 32 x 32 output tile: keys (decoded by `dec(key, cell)`, which resolves zero keys to
// their signed value) -> nanmax values -> hole fill -> float32 -> 3x3 median blur.
// Threads are TX x TY; the caller synchronises before reusing `sm`.  With `next_keys` it
// also clears this tile of the idle key grid (the next view's), which nobody reads
// concurrently, so no per-view memset is needed.  Empty cells (a few percent) are
// collected in a shared list and filled by consecutive threads, so the hole-fill work does
// not diverge every warp that happens to hold one.
template <class Dec>
__device__ __forceinline__ void epilogue_tile(const unsigned long long *__restrict__ vk, const Dec &dec,
                                              float *__restrict__ out, unsigned long long *__restrict__ next_keys,
                                              int H, int W, int r0, int c0, EpilogueSmem &sm) {
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx, lane = tid & 31;
    bool special = false;          // this thread staged a NaN or a zero
    if (tid == 0) sm.n_holes = 0;
    __syncthreads();
    // one pass over the key block: stage the keys (the hole fill reads the neighbours) and,
    // for the blur input's cells, the float32 values and the list of empty cells
    for (int base = 0; base < RAW_H * RAW_W; base += TX * TY) {
        const int i = base + tid;
        const bool in = i < RAW_H * RAW_W;
        const int ly = i / RAW_W, lx = i - ly * RAW_W;
        const int r = r0 + ly - 2, c = c0 + lx - 2;
        unsigned long long k = kEmptyKey;
        if (in && static_cast<unsigned>(r) < static_cast<unsigned>(H) && static_cast<unsigned>(c) < static_cast<unsigned>(W)) {
            const long long cell = static_cast<long long>(r) * W + c;
            k = dec(vk[cell], cell);
        }
        if (in) sm.raw[i] = k;
        const bool inner = in && ly >= 1 && ly <= RAW_H - 2 && lx >= 1 && lx <= RAW_W - 2;
        if (inner && k != kEmptyKey) {
            // the conversion instruction (IEEE round-to-nearest, like f64_to_f32): one issue
            // slot on the narrow FP64 pipe instead of a dozen integer instructions -- here,
            // at ~1.3 conversions per cell, the issue slots are the scarcer resource
            const float f = __double2float_rn(double_from_key(k));
            sm.fk[ly - 1][lx - 1] = f;
            special |= isnan(f) || f == 0.0f;
        }
        // warp-aggregated append of the empty cells to the hole list
        const bool hole = inner && k == kEmptyKey;
        const unsigned empty = __ballot_sync(0xffffffffu, hole);
        if (empty) {
            int slot = 0;
            if (lane == __ffs(empty) - 1) slot = atomicAdd(&sm.n_holes, __popc(empty));
            slot = __shfl_sync(0xffffffffu, slot, __ffs(empty) - 1);
            if (hole)
                sm.holes[slot + __popc(empty & ((1u << lane) - 1u))] =
                    static_cast<unsigned short>((ly - 1) * FK_W + (lx - 1));
        }
    }
    __syncthreads();
    for (int h = tid; h < sm.n_holes; h += TX * TY) {
        const int i = sm.holes[h];
        const int ly = i / FK_W, lx = i - ly * FK_W;
        unsigned long long s8[8];
        int m = 0;
#pragma unroll
        for (int dj = 0; dj < 3; ++dj)
#pragma unroll
            for (int dk = 0; dk < 3; ++dk)
                if (dj != 1 || dk != 1) s8[m++] = sm.raw[(ly + dj) * RAW_W + lx + dk];
        bool any = false;
#pragma unroll
        for (int q = 0; q < 8; ++q) any |= s8[q] != kEmptyKey;
        const float f = any ? f64_to_f32(median8_keys(s8)) : __uint_as_float(0x7fffffffu);
        sm.fk[ly][lx] = f;
        special |= isnan(f) || f == 0.0f;
    }
    // A tile whose staged values hold no NaN and no zero takes the sorted-column median:
    // with no NaN and no -0/+0 pair every compare-exchange order yields the same value, so
    // OpenCV's network and the column form agree bit for bit.
    const bool exact_net = __syncthreads_or(special) != 0 || H == 1 || W == 1;
    const int c = c0 + tx;
    int xa = tx, xb = tx + 1, xc = tx + 2;
    if (c == 0) xa = xb;                 // replicate border: clamp the neighbours into the image
    if (c == W - 1) xc = xb;
    if (!exact_net) {
        // lane tx owns fk column tx + 1; lanes 0 and 31 also sort the halo columns 0 and 33
        const int xe = tx == 0 ? 0 : (tx == TX - 1 ? TX + 1 : tx + 1);
#pragma unroll
        for (int j = 0; j < TILE_Y / TY; ++j) {
            const int oy = ty + TY * j, r = r0 + oy;
            int ya = oy, yb = oy + 1, yc = oy + 2;
            if (r == 0) ya = yb;
            if (r == H - 1) yc = yb;
            float lo, mid, hi, elo, emid, ehi;
            sort3f(sm.fk[ya][tx + 1], sm.fk[yb][tx + 1], sm.fk[yc][tx + 1], lo, mid, hi);
            sort3f(sm.fk[ya][xe], sm.fk[yb][xe], sm.fk[yc][xe], elo, emid, ehi);
            float llo = __shfl_up_sync(0xffffffffu, lo, 1), lmid = __shfl_up_sync(0xffffffffu, mid, 1),
                  lhi = __shfl_up_sync(0xffffffffu, hi, 1);
            float rlo = __shfl_down_sync(0xffffffffu, lo, 1), rmid = __shfl_down_sync(0xffffffffu, mid, 1),
                  rhi = __shfl_down_sync(0xffffffffu, hi, 1);
            if (tx == 0) { llo = elo; lmid = emid; lhi = ehi; }
            if (tx == TX - 1) { rlo = elo; rmid = emid; rhi = ehi; }
            if (c == 0) { llo = lo; lmid = mid; lhi = hi; }           // replicate border
            if (c == W - 1) { rlo = lo; rmid = mid; rhi = hi; }
            if (c >= W || r >= H) continue;
            const long long cell = static_cast<long long>(r) * W + c;
            if (next_keys) next_keys[cell] = kEmptyKey;
            out[cell] = med3f(fmaxf(fmaxf(llo, lo), rlo), med3f(lmid, mid, rmid), fminf(fminf(lhi, hi), rhi));
        }
        return;
    }
    if (c >= W) return;
    const bool vec = cv_vector_column(c, W);
#pragma unroll
    for (int j = 0; j < TILE_Y / TY; ++j) {
        const int oy = ty + TY * j, r = r0 + oy;
        if (r >= H) break;
        int ya = oy, yb = oy + 1, yc = oy + 2;
        if (r == 0) ya = yb;
        if (r == H - 1) yc = yb;
        const long long cell = static_cast<long long>(r) * W + c;
        if (next_keys) next_keys[cell] = kEmptyKey;
        if (H == 1)
            out[cell] = cv_median3_line(sm.fk[yb][xa], sm.fk[yb][xb], sm.fk[yb][xc]);
        else if (W == 1)
            out[cell] = cv_median3_line(sm.fk[ya][xb], sm.fk[yb][xb], sm.fk[yc][xb]);
        else
            out[cell] = cv_median9(vec, sm.fk[ya][xa], sm.fk[ya][xb], sm.fk[ya][xc], sm.fk[yb][xa], sm.fk[yb][xb],
                                   sm.fk[yb][xc], sm.fk[yc][xa], sm.fk[yc][xb], sm.fk[yc][xc]);
    }
}

// Zero keys resolved through the per-cell "first zero" word and the point list.
struct PointsZeroDecoder {
    const unsigned long long *first;
    const double *pts;
    __device__ __forceinline__ unsigned long long operator()(unsigned long long k, long long cell) const {
        return cell_key(k, cell, first, pts);
    }
};

__global__ void __launch_bounds__(TX *TY) dsm_epilogue_kernel(
    const unsigned long long *__restrict__ vk, const unsigned long long *__restrict__ first,
    const double *__restrict__ pts, float *__restrict__ out, unsigned long long *__restrict__ next_keys, int H,
    int W) {
    __shared__ EpilogueSmem sm;
    epilogue_tile(vk, PointsZeroDecoder{first, pts}, out, next_keys, H, W, blockIdx.y * TILE_Y, blockIdx.x * TX, sm);
}

// ---- pipelined rasterisation: view v's binning and view v-1's epilogue in one launch -----
// The binning streams the points from HBM and waits on loads; the epilogue works on an
// L2-resident key grid and is issue-bound.  Launched one after the other they barely
// overlap (the binning's resident wave fills every SM until its tail), so one launch
// carries both: its work items -- chunks of view v's points and 32x32 tiles of view v-1's
// epilogue, interleaved evenly -- are handed out by a device counter, so every SM runs a
// mix of both kinds until the launch drains.  The epilogue's inputs (view v-1's key grid
// and first-zero words) were completed by the previous launch on the same stream; nothing
// waits on another CTA.
constexpr int kChunkIters = 8;                                   // blocks of kFastPts points per thread
constexpr long long kChunkPoints = 1LL * TX * TY * kFastPts * kChunkIters;

struct PipeBin {          // view v's binning (active = 0: none)
    const long long *offsets;
    int v, active;
    FastAxis row, col;
    unsigned long long *keys, *first;
};

struct PipeEpi {          // view v-1's epilogue (n_tiles = 0: none)
    const unsigned long long *keys, *first;
    float *out;
    unsigned long long *clear;   // the key grid of view v+1, cleared tile by tile
    int H, W, tiles_x;
    long long n_tiles;
};

// MINB: resident CTAs per SM the registers are budgeted for (6: 40 registers, 5: 48).
template <bool FLIP_ROW, bool FLIP_COL, int MINB>
__global__ void __launch_bounds__(TX *TY, MINB) raster_pipe_kernel(const double *__restrict__ pts, PipeBin bin,
                                                                    PipeEpi epi, unsigned *__restrict__ counter) {
    __shared__ EpilogueSmem sm;
    __shared__ long long item_sh[2];
    const int tid = threadIdx.y * TX + threadIdx.x;
    const long long *bits = reinterpret_cast<const long long *>(pts);
    long long begin = 0, end = 0;
    if (bin.active) {
        begin = bin.offsets[bin.v];
        end = bin.offsets[bin.v + 1];
    }
    const long long n_chunks = end > begin ? (end - begin + kChunkPoints - 1) / kChunkPoints : 0;
    const long long total = n_chunks + epi.n_tiles;
    const unsigned long long tag = epoch_tag(bin.v);
    const unsigned ncols = static_cast<unsigned>(bin.col.nm1 + 1);
    for (int it = 0;; ++it) {
        // thread 0 fetches the next item and classifies it: tiles sit at the items where
        // floor(item * n_tiles / total) steps, chunks in between (encoded as -1 - chunk)
        if (tid == 0) {
            const long long item = atomicAdd(counter, 1u);
            long long code = total;                       // done
            if (item < total) {
                const long long t0 = item * epi.n_tiles / total, t1 = (item + 1) * epi.n_tiles / total;
                code = t1 > t0 ? t0 : -1 - (item - t0);
            }
            item_sh[it & 1] = code;
        }
        __syncthreads();    // also ends the previous item's use of the shared tile
        const long long code = item_sh[it & 1];
        if (code >= total) break;
        if (code >= 0) {
            const int ty = static_cast<int>(code / epi.tiles_x), tx = static_cast<int>(code - static_cast<long long>(ty) * epi.tiles_x);
            epilogue_tile(epi.keys, PointsZeroDecoder{epi.first, pts}, epi.out, epi.clear, epi.H, epi.W, ty * TILE_Y,
                          tx * TX, sm);
        } else {
            const long long c0 = begin + (-1 - code) * kChunkPoints;
#pragma unroll 1
            for (int k = 0; k < kChunkIters; ++k) {
                const long long i = c0 + (static_cast<long long>(k) * (TX * TY) + tid) * kFastPts;
                if (i < end) bin_fast_block<FLIP_ROW, FLIP_COL>(bits, i, end, bin.row, bin.col, ncols, tag, bin.keys,
                                                                bin.first);
            }
        }
    }
}

// ---- host side --------------------------------------------------------------------------
// Host copy of the threshold search of axis_thresholds_kernel (same IEEE FP64 expression).
long long host_threshold(long long r, double ulp, double res) {
    const double rd = static_cast<double>(r);
    long long d = static_cast<long long>(ceil(rd * res / ulp));
    if (d < 0) d = 0;
    for (int it = 0; it < 64 && d > 0 && floor((static_cast<double>(d - 1) * ulp) / res) >= rd; ++it) --d;
    for (int it = 0; it < 64 && floor((static_cast<double>(d) * ulp) / res) < rd; ++it) ++d;
    return d;
}

int make_axis(Axis &ax, double off, double res, long long n, int dir, long long *thr, cudaStream_t st) {
    ax.off = off;
    ax.res = res;
    ax.n = n;
    ax.thr = thr;
    ax.dir = dir;
    ax.neg = off < 0;
    unsigned long long b;
    memcpy(&b, &off, sizeof b);
    ax.top12 = static_cast<unsigned>(b >> 52);
    const unsigned e = static_cast<unsigned>((b >> 52) & 0x7ff);
    ax.fast = 0;
    ax.contained = 0;
    ax.shift = 0;
    ax.scale = 0.f;
    ax.err_abs = ax.err_rel = 0.f;
    ax.tmax = 0;
    ax.mul = ax.fmask = ax.fsure = 0;
    ax.fbits = 0;
    // the FP32 estimate needs cell indices below 2^22 and sane resolutions
    if (!(e >= 1 && e <= 2046 && isfinite(res) && res >= 1e-9 && res <= 1e9 && n < (1LL << 22))) return VS_OK;
    const double ulp = ldexp(1.0, static_cast<int>(e) - 1075);
    const double dmax = static_cast<double>(n + 1) * res / ulp + 2.0;   // > thr[n]
    if (dmax >= 4503599627370496.0) return VS_OK;                       // differences below 2^52 ulps
    int bits = 0;
    frexp(dmax, &bits);                              // dmax < 2^bits
    ax.shift = bits > 32 ? bits - 32 : 0;            // d >> shift < 2^32
    const double scale = ldexp(ulp / res, ax.shift);
    ax.scale = static_cast<float>(scale);
    // |q - d*ulp/res| <= dropped low bits (< 2^shift ulps) + rounding of u, scale and the
    // product (3 x 2^-24 relative), plus the half-ulp of the reference's own FP64 quotient
    ax.err_abs = static_cast<float>(1.01 * scale + 1e-9);
    ax.err_rel = static_cast<float>(4.0 * ldexp(1.0, -24));
    ax.tmax = host_threshold(n, ulp, res);
    // integer estimate: mul = round(scale * 2^(32 + fbits)) in [2^31, 2^32]
    int ke = 0;
    frexp(scale, &ke);                               // scale = m * 2^ke, m in [0.5, 1)
    int fb = -ke;
    double m = nearbyint(ldexp(scale, 32 + fb));
    if (m >= 4294967296.0) {
        --fb;
        m = nearbyint(ldexp(scale, 32 + fb));
    }
    if (fb < 4 || fb > 31 || m < 2147483648.0 || m >= 4294967296.0) return VS_OK;   // (cannot happen for n < 2^22)
    ax.mul = static_cast<unsigned>(m);
    ax.fbits = fb;
    ax.fmask = (1u << fb) - 1u;
    ax.fsure = (1u << fb) - 8u;
    ax.fast = 1;
    // the grid spans off .. off -/+ (n + 2) * res; contained when both ends keep off's sign
    // and exponent, so that any point with another sign/exponent lies >= 2 cells outside
    const double far = dir > 0 ? off + (static_cast<double>(n) + 2.0) * res : off - (static_cast<double>(n) + 2.0) * res;
    const double near = dir > 0 ? off - 2.0 * res : off + 2.0 * res;
    unsigned long long bf, bn;
    memcpy(&bf, &far, sizeof bf);
    memcpy(&bn, &near, sizeof bn);
    ax.contained = (bf >> 52) == (b >> 52) && (bn >> 52) == (b >> 52);
    const int threads = 256;
    axis_thresholds_kernel<<<static_cast<unsigned>(ceil_div(n + 1, threads)), threads, 0, st>>>(thr, n, ulp, res);
    return check_launch("axis_thresholds_kernel");
}

struct RasterWs {
    unsigned long long *keys[2];   // key grids, alternating view by view
    unsigned long long *first;     // "first zero" words (epoch-tagged)
    long long *row_thr, *col_thr;
    size_t bytes;
};

RasterWs carve_raster(void *ws, long long xsize, long long ysize, bool two_grids) {
    Carver cv(ws);
    RasterWs r;
    const size_t cells = static_cast<size_t>(xsize) * ysize;
    r.keys[0] = cv.take<unsigned long long>(cells);
    r.keys[1] = two_grids ? cv.take<unsigned long long>(cells) : r.keys[0];
    r.first = cv.take<unsigned long long>(cells);
    r.row_thr = cv.take<long long>(ysize + 1);
    r.col_thr = cv.take<long long>(xsize + 1);
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

// CTAs per SM of the point-binning launches (0: as many as fit); set through
// vs_set_binning_ctas_per_sm.
int g_bin_ctas_per_sm = 0;

// Both axes on the contained fast path and 32-bit cell indices: bin_fast_kernel applies.
// L2 set-aside for the key grids (vs_set_l2_persisting): bytes reserved in this context for
// persisting accesses (0: off) and the device's largest access-policy window.
size_t g_l2_persist = 0, g_l2_window_max = 0;

// Launches `kernel` with an access-policy window that marks the key grid [base, base + bytes)
// persisting in L2 -- the streamed points (evict-first loads) then cannot push the grid the
// binning's atomics land in out of L2 -- when a set-aside is configured; otherwise a plain
// launch.  The window is a per-launch attribute: the caller's stream keeps its own.
template <typename... KArgs, typename... Args>
cudaError_t launch_with_key_window(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st,
                                   const void *base, size_t bytes, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    if (g_l2_persist > 0 && base && bytes > 0) {
        const size_t nb = std::min(bytes, g_l2_window_max);
        attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[0].val.accessPolicyWindow.base_ptr = const_cast<void *>(base);
        attr[0].val.accessPolicyWindow.num_bytes = nb;
        attr[0].val.accessPolicyWindow.hitRatio =
            nb <= g_l2_persist ? 1.0f : static_cast<float>(g_l2_persist) / static_cast<float>(nb);
        attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

bool fast_binning(const Tables &tb) {
    return tb.row.fast && tb.row.contained && tb.col.fast && tb.col.contained && tb.row.n * tb.col.n < (1LL << 31);
}

void fast_axes(const Tables &tb, FastAxis fa[2]) {
    fa[0] = fast_axis_of(tb.row);
    fa[1] = fast_axis_of(tb.col);
}

int bin_launch(const double *points, const long long *offsets, int v, long long single_n, long long max_points,
               const Tables &tb, unsigned long long *keys, unsigned long long *first, cudaStream_t st) {
    if (max_points <= 0) return VS_OK;
    const int threads = 256;
    long long want = ceil_div(ceil_div(max_points, kPts), threads);
    long long cap = static_cast<long long>(sm_count()) * 8;
    unsigned gx = static_cast<unsigned>(std::max(1LL, std::min(want, cap)));
    if (fast_binning(tb)) {
        FastAxis fa[2];
        fast_axes(tb, fa);
        // rows: a = off - v unless the origin is negative; columns: a = v - off unless negative
        const bool flip_row = !tb.row.neg, flip_col = tb.col.neg != 0;
        // one wave of resident CTAs (grid-stride): a partial second wave would leave most
        // SMs idle at the tail
        static int resident = 0;
        if (!resident) {
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bin_fast_kernel<true, false>, threads, 0) !=
                    cudaSuccess || per_sm <= 0)
                per_sm = 4;
            resident = per_sm;
        }
        const int per_sm = g_bin_ctas_per_sm > 0 ? std::min(g_bin_ctas_per_sm, resident) : resident;
        gx = static_cast<unsigned>(std::max<long long>(
            1LL, std::min<long long>(ceil_div(ceil_div(max_points, kFastPts), threads),
                                     static_cast<long long>(sm_count()) * per_sm)));
        const size_t key_bytes = sizeof(unsigned long long) * static_cast<size_t>(tb.row.n * tb.col.n);
        auto kern = flip_row ? (flip_col ? bin_fast_kernel<true, true> : bin_fast_kernel<true, false>)
                             : (flip_col ? bin_fast_kernel<false, true> : bin_fast_kernel<false, false>);
        if (launch_with_key_window(kern, dim3(gx), dim3(threads), st, keys, key_bytes, points, offsets, v, single_n,
                                   fa[0], fa[1], keys, first) != cudaSuccess)
            return check_launch("bin_fast_kernel");
    } else {
        bin_max_kernel<true><<<gx, threads, 0, st>>>(points, offsets, v, single_n, tb, keys, first);
    }
    return check_launch("bin_max_kernel");
}

// ---- batched form: per-view FP32 height maps, many AOIs -----------------------------------
// A view's points are its height-map pixels, placed by a fixed-point affine pixel -> UTM
// map (units of 2^-28 m).  Coordinates are exact doubles, and in the binade of the grid
// origin (contained grid) the double bit pattern of x = x_fx * 2^-28 is
//     bits(x) = ((E + 1023) << 52) - 2^52 + (x_fx << (24 - E)),   E = exponent of the origin,
// an integer expression that is monotone in x_fx; outside the binade it leaves the origin's
// exponent field, which the axis test rejects (off-grid, as the containment guarantees).
// So each pixel is binned with integer and FP32 operations only, reading 4 bytes.
constexpr unsigned long long kMapIdxLimit = 1ull << 28;   // pixels per view

// FP64 point list of one height map in pixel order (the plain per-view form's input):
// pixel (i, j) -> (easting, northing, height) with easting = (e0 + ej (2j+1-W) + ei (2i+1-H))
// 2^-28 m (exact doubles: the integers stay below 2^53).
__global__ void map_points_kernel(const float *__restrict__ map, long long stride, int W, int H, long long e0,
                                  long long n0, long long ej, long long ei, long long nj, long long ni,
                                  double *__restrict__ pts) {
    const long long total = static_cast<long long>(W) * H;
    for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < total;
         p += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long i = p / W, j = p - i * W;
        const long long dj = 2 * j + 1 - W, di = 2 * i + 1 - H;
        const double east = __ll2double_rn(e0 + ej * dj + ei * di) * 0x1p-28;
        const double north = __ll2double_rn(n0 + nj * dj + ni * di) * 0x1p-28;
        pts[3 * p] = east;
        pts[3 * p + 1] = north;
        pts[3 * p + 2] = static_cast<double>(map[i * stride + j]);
    }
}

struct MapViewDev {
    const float *map;
    long long stride;
    long long e0, n0;
    int ej, ei, nj, ni;
    int W, H;
    int aoi;
    int vec;                  // rows are 16-byte aligned: float4 loads
    long long off;            // cell offset of the view's DSM in the run's buffer
    float *out;               // the view's DSM, or null: the run's buffer at `off`
    // the axes' differences from the grid origin (in ulps of the origin's binade) are
    // affine in the pixel indices: d = d0 + d_di * (2i+1-H) + d_dj * (2j+1-W)
    long long dc0, dc_di, dc_dj;   // columns: bits(x) - bits(xoff)
    long long dr0, dr_di, dr_dj;   // rows:    bits(yoff) - bits(y)
    // pixel box of a cell region: pixel (i, j) as an affine function of the cell
    // coordinates (s_col, s_row) = (d_col, d_row) * ulp / res (cell r spans [r, r + 1))
    double bi0, bic, bir, bj0, bjc, bjr;
    double bmarg;             // pixels added on each side of a box (rounding of the map)
    int box_all;              // singular map: every tile reads the whole map
};

struct AoiDev {
    FastAxis row, col;
    long long bx, by;         // bit-pattern bases of the origins' binades
    int shx, shy;
    int xsize, ysize;
};

// Largest index i in [lo, hi] with starts[i] <= x (starts ascending, starts[lo] <= x).
__device__ __forceinline__ int find_range(const long long *starts, int lo, int hi, long long x) {
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(starts + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

constexpr int kMapThreads = 256;
constexpr unsigned kMapKeyZero = 0x80000000u;   // key of +0.0f; any zero while binning
constexpr int kMapUnitPx = 8;                   // consecutive pixels of a row per thread step

// Shared-memory tile of one work item: an OW x OH block of one view's DSM.  The key tile
// carries a 2-cell halo (the hole fill of the blur's 1-cell halo needs its neighbours);
// its keys are 32-bit order keys of the float32 heights (0: no point), enough for the
// nanmax because the heights are float32.  The "first zero" words, needed only when a
// cell's maximum is a zero, share storage with the epilogue's arrays.
template <int OW, int OH>
struct MapTileSmem {
    static constexpr int KW = OW + 4, KH = OH + 4, FW = OW + 2, FH = OH + 2;
    static constexpr int NK = KW * KH, NF = FW * FH;
    unsigned keys[NK];
    union {
        unsigned zw[NK];                    // (2^28 - 1 - first zero's pixel) << 1 | its sign
        struct {
            float fk[FH][FW];               // hole-filled values: the blur's input
            unsigned short holes[NF];       // empty in-grid cells of the blur input
        } e;
    } u;
    long long item;
    int view, r0, c0, ia, ib, ja, jb;
    int n_holes, has_zero;
    unsigned char specrow[FH];              // a NaN or a zero in this row of the blur input
};

// Row/column estimate from the difference d (contained grid: the origin-binade test is
// implied, since d is monotone in the coordinate and every coordinate outside the
// origin's binade lies at least two cells outside [0, tmax); one unsigned compare covers
// d < 0).  The estimate is not clamped into the grid: the key tile's own bounds test
// drops any row or column outside it, and the rare correction clamps first.
__device__ __forceinline__ bool axis_tile(const FastAxis &a, long long d, int &r, bool &sure) {
    const bool ok = static_cast<unsigned long long>(d) < static_cast<unsigned long long>(a.tmax);
    axis_estimate(a, static_cast<unsigned>(static_cast<unsigned long long>(d) >> a.shift), r, sure);
    return ok;
}

// One pass over the item's pixel box [ia, ib] x [ja, jb] (ja a multiple of 4 for float4
// rows).  Every pixel is binned exactly as the per-view path bins its FP64 point (the
// integer/FP32 axis test and the threshold correction); pixels whose cell lies outside
// the key tile are dropped.  ZERO = false: the nanmax keys, zeros as kMapKeyZero;
// ZERO = true: for cells whose maximum is a zero, the first zero pixel and its sign.
template <int OW, int OH, bool ZERO>
__device__ __forceinline__ void map_tile_pass(const MapViewDev &mv, const FastAxis &R, const FastAxis &C, int rbase,
                                              int cbase, int ia, int ib, int ja, int jb, MapTileSmem<OW, OH> &sm) {
    using S = MapTileSmem<OW, OH>;
    constexpr int P = kMapUnitPx;
    const int G = (jb - ja) / P + 1;                    // P-pixel groups per box row
    const int units = (ib - ia + 1) * G;
    int row = threadIdx.x / G, g = threadIdx.x - row * G;
    const int rstep = kMapThreads / G, gstep = kMapThreads - rstep * G;
    const long long scol = 2 * mv.dc_dj, srow = 2 * mv.dr_dj;   // per pixel along a row
    bool zero_seen = false;
    for (int unit = threadIdx.x; unit < units; unit += kMapThreads) {
        const int i = ia + row, j0 = ja + g * P;
        const float *src = mv.map + static_cast<long long>(i) * mv.stride + j0;
        unsigned hb[P];
        if (mv.vec && j0 + P <= mv.W) {
#pragma unroll
            for (int q = 0; q < P / 4; ++q) {
                const float4 v4 = __ldg(reinterpret_cast<const float4 *>(src) + q);
                hb[4 * q] = __float_as_uint(v4.x); hb[4 * q + 1] = __float_as_uint(v4.y);
                hb[4 * q + 2] = __float_as_uint(v4.z); hb[4 * q + 3] = __float_as_uint(v4.w);
            }
        } else {
#pragma unroll
            for (int k = 0; k < P; ++k) hb[k] = j0 + k < mv.W ? __float_as_uint(__ldg(src + k)) : 0x7fc00000u;
        }
        const int di2 = 2 * i + 1 - mv.H, dj0 = 2 * j0 + 1 - mv.W;
        long long dcol = mv.dc0 + mv.dc_di * di2 + mv.dc_dj * dj0;
        long long drow = mv.dr0 + mv.dr_di * di2 + mv.dr_dj * dj0;
        // rows: d is affine along the unit, and the exact row monotone in d, so when the
        // first and the last pixel fall in the same row with sure estimates, all do
        int ra, rb;
        bool sa, sb;
        const bool oka = axis_tile(R, drow, ra, sa), okb = axis_tile(R, drow + (P - 1) * srow, rb, sb);
        const bool row_fixed = oka & okb & sa & sb & (ra == rb);
        const unsigned lr_fixed = static_cast<unsigned>(ra - rbase);
        int cell[P];
        unsigned key[P];
#pragma unroll
        for (int k = 0; k < P; ++k, dcol += scol, drow += srow) {
            const unsigned mag = hb[k] & 0x7fffffffu;
            int c;
            bool sc;
            bool ok = ZERO ? mag == 0u : mag <= 0x7f800000u;    // not NaN
            unsigned lr = lr_fixed;
            if (!row_fixed) {
                int r;
                bool sr;
                ok &= axis_tile(R, drow, r, sr);
                if (ok && !sr) r = axis_correct(R.thr, min(max(r, 0), R.nm1), drow);
                lr = static_cast<unsigned>(r - rbase);
            }
            ok &= axis_tile(C, dcol, c, sc);
            if (ok && !sc) c = axis_correct(C.thr, min(max(c, 0), C.nm1), dcol);
            const unsigned lc = static_cast<unsigned>(c - cbase);
            ok &= (lr < static_cast<unsigned>(S::KH)) & (lc < static_cast<unsigned>(S::KW));
            cell[k] = ok ? static_cast<int>(lr) * S::KW + static_cast<int>(lc) : -1;
            if (ZERO) {
                const unsigned idx = static_cast<unsigned>(i) * static_cast<unsigned>(mv.W) + static_cast<unsigned>(j0 + k);
                key[k] = ((static_cast<unsigned>(kMapIdxLimit) - 1u - idx) << 1) | (hb[k] >> 31);
            } else {
                zero_seen |= ok & (mag == 0u);
                key[k] = mag == 0u ? kMapKeyZero : ((hb[k] >> 31) ? ~hb[k] : (hb[k] | 0x80000000u));
            }
        }
        if (ZERO) {
#pragma unroll
            for (int k = 0; k < P; ++k)
                if (cell[k] >= 0 && sm.keys[cell[k]] == kMapKeyZero) atomicMax(&sm.u.zw[cell[k]], key[k]);
        } else {
#pragma unroll
            for (int k = 1; k < P; ++k) {     // merge runs of consecutive pixels in one cell
                const bool same = (cell[k] >= 0) & (cell[k] == cell[k - 1]);
                key[k] = same ? max(key[k], key[k - 1]) : key[k];
                cell[k - 1] = same ? -1 : cell[k - 1];
            }
#pragma unroll
            for (int k = 0; k < P; ++k)
                if (cell[k] >= 0) atomicMax(&sm.keys[cell[k]], key[k]);
        }
        g += gstep;
        row += rstep;
        if (g >= G) {
            g -= G;
            ++row;
        }
    }
    if (!ZERO && zero_seen) sm.has_zero = 1;
}

// cswap on 32-bit keys.
__device__ __forceinline__ void cswap32(unsigned &a, unsigned &b) {
    const unsigned lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}

__device__ __forceinline__ unsigned select8_32(const unsigned (&s)[8], int idx) {
    const bool b0 = idx & 1, b1 = idx & 2, b2 = idx & 4;
    const unsigned a0 = b0 ? s[1] : s[0], a1 = b0 ? s[3] : s[2];
    const unsigned a2 = b0 ? s[5] : s[4], a3 = b0 ? s[7] : s[6];
    const unsigned c0 = b1 ? a1 : a0, c1 = b1 ? a3 : a2;
    return b2 ? c1 : c0;
}

// 64-bit double order key of a non-zero 32-bit float order key.
__device__ __forceinline__ unsigned long long key64_of_key32(unsigned k) {
    return key_from_double(f32_to_f64(float_from_key(k)));
}

// numpy's median of the non-empty 32-bit keys among 8 (at least one), as float32: the
// float keys order like the double keys of the same values, so the 8-input network runs
// on 32-bit keys and only the middle ones are widened for the FP64 mean.
__device__ __forceinline__ float median8_keys32(unsigned (&s)[8]) {
    int n = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        n += s[i] != 0u;
        s[i] = s[i] ? s[i] : ~0u;                      // empty sorts last
    }
    cswap32(s[0], s[1]); cswap32(s[2], s[3]); cswap32(s[4], s[5]); cswap32(s[6], s[7]);
    cswap32(s[0], s[2]); cswap32(s[1], s[3]); cswap32(s[4], s[6]); cswap32(s[5], s[7]);
    cswap32(s[1], s[2]); cswap32(s[5], s[6]);
    cswap32(s[0], s[4]); cswap32(s[1], s[5]); cswap32(s[2], s[6]); cswap32(s[3], s[7]);
    cswap32(s[2], s[4]); cswap32(s[3], s[5]);
    cswap32(s[1], s[2]); cswap32(s[3], s[4]); cswap32(s[5], s[6]);
    const unsigned lo = select8_32(s, (n - 1) >> 1), hi = select8_32(s, n >> 1);
    if (n & 1) return float_from_key(hi == 0x7fffffffu ? kMapKeyZero : hi);   // -0 + 0 = +0
    return f64_to_f32(median_from_middle(key64_of_key32(lo), key64_of_key32(hi), n));
}

// The tile's epilogue from shared memory: nanmax keys -> hole fill (non-propagating,
// median of the non-empty 3x3 neighbours) -> float32 -> 3x3 median blur, written to the
// view's DSM; the same arithmetic as epilogue_tile.  Output rows whose 3x3 windows hold
// no NaN and no zero take the sorted-column median (bit-identical there); the others run
// OpenCV's network per cell.  Clears the key tile for the next item.
template <int OW, int OH>
__device__ __forceinline__ void map_tile_finish(MapTileSmem<OW, OH> &sm, float *__restrict__ out, int H, int W,
                                                int r0, int c0) {
    using S = MapTileSmem<OW, OH>;
    const int tid = threadIdx.x, lane = tid & 31;
    const float qnan = __uint_as_float(0x7fffffffu);
    for (int base = 0; base < S::NF; base += kMapThreads) {
        const int idx = base + tid;
        const bool in = idx < S::NF;
        const int ly = idx / S::FW, lx = idx - ly * S::FW;
        const bool grid = in && static_cast<unsigned>(r0 - 1 + ly) < static_cast<unsigned>(H) &&
                          static_cast<unsigned>(c0 - 1 + lx) < static_cast<unsigned>(W);
        const unsigned k = in ? sm.keys[(ly + 1) * S::KW + lx + 1] : 1u;
        if (in) {
            const float f = k ? float_from_key(k) : qnan;
            sm.u.e.fk[ly][lx] = f;
            if (grid && k && f == 0.0f) sm.specrow[ly] = 1;
        }
        const unsigned empty = __ballot_sync(0xffffffffu, grid && k == 0u);
        if (empty) {
            int slot = 0;
            if (lane == __ffs(empty) - 1) slot = atomicAdd(&sm.n_holes, __popc(empty));
            slot = __shfl_sync(0xffffffffu, slot, __ffs(empty) - 1);
            if (grid && k == 0u) sm.u.e.holes[slot + __popc(empty & ((1u << lane) - 1u))] = static_cast<unsigned short>(idx);
        }
    }
    __syncthreads();
    for (int h = tid; h < sm.n_holes; h += kMapThreads) {
        const int idx = sm.u.e.holes[h];
        const int ly = idx / S::FW, lx = idx - ly * S::FW;
        unsigned s8[8];
        int m = 0;
#pragma unroll
        for (int dj = 0; dj < 3; ++dj)
#pragma unroll
            for (int dk = 0; dk < 3; ++dk)
                if (dj != 1 || dk != 1) s8[m++] = sm.keys[(ly + dj) * S::KW + lx + dk];
        const unsigned any = s8[0] | s8[1] | s8[2] | s8[3] | s8[4] | s8[5] | s8[6] | s8[7];
        const float f = any ? median8_keys32(s8) : qnan;
        sm.u.e.fk[ly][lx] = f;
        if (isnan(f) || f == 0.0f) sm.specrow[ly] = 1;
    }
    __syncthreads();
    for (int i = tid; i < S::NK; i += kMapThreads) sm.keys[i] = 0u;   // dead until the next item
    const bool line = H == 1 || W == 1;
    constexpr int HALVES = OW / 32;
    const float(&fk)[S::FH][S::FW] = sm.u.e.fk;
    for (int p = tid >> 5; p < OH * HALVES; p += kMapThreads / 32) {
        const int oy = p / HALVES, h = p - oy * HALVES;
        const int r = r0 + oy, c = c0 + 32 * h + lane;
        const int fx = 32 * h + lane + 1;
        int ya = oy, yb = oy + 1, yc = oy + 2;
        if (r == 0) ya = yb;
        if (r == H - 1) yc = yb;
        if (!line && !(sm.specrow[oy] | sm.specrow[oy + 1] | sm.specrow[oy + 2])) {
            // sorted-column median: lane owns one column of a 32-column half row; lanes 0
            // and 31 also sort the halo columns
            const int xe = lane == 0 ? 32 * h : (lane == 31 ? 32 * h + 33 : fx);
            float lo, mid, hi, elo, emid, ehi;
            sort3f(fk[ya][fx], fk[yb][fx], fk[yc][fx], lo, mid, hi);
            sort3f(fk[ya][xe], fk[yb][xe], fk[yc][xe], elo, emid, ehi);
            float llo = __shfl_up_sync(0xffffffffu, lo, 1), lmid = __shfl_up_sync(0xffffffffu, mid, 1),
                  lhi = __shfl_up_sync(0xffffffffu, hi, 1);
            float rlo = __shfl_down_sync(0xffffffffu, lo, 1), rmid = __shfl_down_sync(0xffffffffu, mid, 1),
                  rhi = __shfl_down_sync(0xffffffffu, hi, 1);
            if (lane == 0) { llo = elo; lmid = emid; lhi = ehi; }
            if (lane == 31) { rlo = elo; rmid = emid; rhi = ehi; }
            if (c == 0) { llo = lo; lmid = mid; lhi = hi; }           // replicate border
            if (c == W - 1) { rlo = lo; rmid = mid; rhi = hi; }
            if (c < W && r < H)
                out[static_cast<long long>(r) * W + c] =
                    med3f(fmaxf(fmaxf(llo, lo), rlo), med3f(lmid, mid, rmid), fminf(fminf(lhi, hi), rhi));
            continue;
        }
        if (r >= H || c >= W) continue;
        int xa = fx - 1, xb = fx, xc = fx + 1;
        if (c == 0) xa = xb;
        if (c == W - 1) xc = xb;
        float v;
        if (H == 1) {
            v = cv_median3_line(fk[yb][xa], fk[yb][xb], fk[yb][xc]);
        } else if (W == 1) {
            v = cv_median3_line(fk[ya][xb], fk[yb][xb], fk[yc][xb]);
        } else {
            const float p0 = fk[ya][xa], p1 = fk[ya][xb], p2 = fk[ya][xc], p3 = fk[yb][xa], p4 = fk[yb][xb],
                        p5 = fk[yb][xc], p6 = fk[yc][xa], p7 = fk[yc][xb], p8 = fk[yc][xc];
            // all nine NaN (the epilogue's own NaN): every exchange moves equal bits
            const bool all_nan = isnan(p0) & isnan(p1) & isnan(p2) & isnan(p3) & isnan(p4) & isnan(p5) & isnan(p6) &
                                 isnan(p7) & isnan(p8);
            v = all_nan ? qnan : cv_median9(cv_vector_column(c, W), p0, p1, p2, p3, p4, p5, p6, p7, p8);
        }
        out[static_cast<long long>(r) * W + c] = v;
    }
}

// Pixel box [ia, ib] x [ja, jb] of the pixels whose cells can fall in rows [rlo, rhi) and
// columns [clo, chi) of the grid: the affine pixel <- cell map at the region's corners,
// widened by a quarter cell and by bmarg pixels (one pixel plus a bound of the FP64
// rounding of the map), clipped to the map.  ja is rounded down to a multiple of 4 for float4 rows.
__device__ __forceinline__ void map_pixel_box(const MapViewDev &mv, int rlo, int rhi, int clo, int chi, int &ia, int &ib,
                                              int &ja, int &jb) {
    if (mv.box_all) {
        ia = 0; ib = mv.H - 1; ja = 0; jb = mv.W - 1;
    } else {
        const double sr[2] = {rlo - 0.25, rhi + 0.25}, sc[2] = {clo - 0.25, chi + 0.25};
        double imin = 1e300, imax = -1e300, jmin = 1e300, jmax = -1e300;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                const double pi = __fma_rn(mv.bir, sr[a], __fma_rn(mv.bic, sc[b], mv.bi0));
                const double pj = __fma_rn(mv.bjr, sr[a], __fma_rn(mv.bjc, sc[b], mv.bj0));
                imin = fmin(imin, pi); imax = fmax(imax, pi);
                jmin = fmin(jmin, pj); jmax = fmax(jmax, pj);
            }
        // clamp before converting (a far-away tile maps far outside the map)
        ia = static_cast<int>(fmin(fmax(floor(imin - mv.bmarg), 0.0), mv.H));
        ib = static_cast<int>(fmax(fmin(ceil(imax + mv.bmarg), mv.H - 1.0), -1.0));
        ja = static_cast<int>(fmin(fmax(floor(jmin - mv.bmarg), 0.0), mv.W));
        jb = static_cast<int>(fmax(fmin(ceil(jmax + mv.bmarg), mv.W - 1.0), -1.0));
        if (!(imin <= imax && jmin <= jmax)) { ia = 1; ib = 0; }    // NaN: nothing
    }
    if (mv.vec) ja &= ~3;      // float4 rows: groups start 16-byte aligned
}

// The batched rasterisation of many views, one fused kernel: a CTA takes work items (one
// OW x OH tile of one view's DSM) from a device counter, bins the pixels of the tile's
// pixel box into its shared-memory key tile, and runs the epilogue from shared memory, so
// no key grid exists in device memory.  Items [item_begin, item_end) of the plan's item
// list (views in order, tiles row-major within a view).
template <int OW, int OH>
__global__ void __launch_bounds__(kMapThreads, 4) map_tile_kernel(
    const MapViewDev *__restrict__ views, const AoiDev *__restrict__ aois, const long long *__restrict__ tile_start,
    int v_lo, int v_hi, long long item_begin, long long item_end, float *__restrict__ dsm,
    unsigned long long *__restrict__ counter) {
    using S = MapTileSmem<OW, OH>;
    __shared__ S sm;
    for (int i = threadIdx.x; i < S::NK; i += kMapThreads) sm.keys[i] = 0u;
    int vlast = v_lo;      // thread 0: the view of this CTA's previous item (items only grow)
    for (;;) {
        if (threadIdx.x == 0) {
            const long long it = item_begin + static_cast<long long>(atomicAdd(counter, 1ull));
            sm.item = it;
            sm.n_holes = 0;
            sm.has_zero = 0;
            if (it < item_end) {
                int v = vlast;
                for (int step = 0; step < 8 && v < v_hi && __ldg(tile_start + v + 1) <= it; ++step) ++v;
                if (v < v_hi && __ldg(tile_start + v + 1) <= it) v = find_range(tile_start, v, v_hi, it);
                vlast = v;
                const MapViewDev &mv = views[v];
                const AoiDev &ad = aois[mv.aoi];
                const int tiles_x = (ad.xsize + OW - 1) / OW;
                const int local = static_cast<int>(it - __ldg(tile_start + v));
                const int ty = local / tiles_x, tx = local - ty * tiles_x;
                const int r0 = ty * OH, c0 = tx * OW;
                int ia, ib, ja, jb;
                map_pixel_box(mv, max(r0 - 2, 0), min(r0 + OH + 2, ad.ysize), max(c0 - 2, 0),
                              min(c0 + OW + 2, ad.xsize), ia, ib, ja, jb);
                sm.view = v; sm.r0 = r0; sm.c0 = c0;
                sm.ia = ia; sm.ib = ib; sm.ja = ja; sm.jb = jb;
            }
        }
        __syncthreads();
        if (sm.item >= item_end) return;
        const int v = sm.view, r0 = sm.r0, c0 = sm.c0, ia = sm.ia, ib = sm.ib, ja = sm.ja, jb = sm.jb;
        for (int i = threadIdx.x; i < S::FH; i += kMapThreads) sm.specrow[i] = 0;
        const MapViewDev &mv = views[v];
        const AoiDev &ad = aois[mv.aoi];
        const FastAxis R = ad.row, C = ad.col;
        if (ia <= ib && ja <= jb) map_tile_pass<OW, OH, false>(mv, R, C, r0 - 2, c0 - 2, ia, ib, ja, jb, sm);
        __syncthreads();
        if (sm.has_zero) {       // rare: resolve the sign of cells whose maximum is a zero
            for (int i = threadIdx.x; i < S::NK; i += kMapThreads) sm.u.zw[i] = 0u;
            __syncthreads();
            map_tile_pass<OW, OH, true>(mv, R, C, r0 - 2, c0 - 2, ia, ib, ja, jb, sm);
            __syncthreads();
            for (int i = threadIdx.x; i < S::NK; i += kMapThreads)
                if (sm.keys[i] == kMapKeyZero) sm.keys[i] = (sm.u.zw[i] & 1u) ? 0x7fffffffu : kMapKeyZero;
            __syncthreads();
        }
        map_tile_finish<OW, OH>(sm, mv.out ? mv.out : dsm + mv.off, ad.ysize, ad.xsize, r0, c0);
    }
}

int clear(void *p, size_t bytes, cudaStream_t st) {
    if (cudaMemsetAsync(p, 0, bytes, st) != cudaSuccess) {
        set_error("cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
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
    return carve_raster(nullptr, xsize, ysize, false).bytes + sizeof(double) * xsize * ysize + 512;
}

static bool grid_ok(int64_t xsize, int64_t ysize) {
    return xsize > 0 && ysize > 0 && xsize < (1LL << 31) && ysize < (1LL << 31);
}

extern "C" int vs_proj_to_grid(const double *points, int64_t n, double xoff, double yoff,
                               double xresolution, double yresolution, int64_t xsize, int64_t ysize,
                               double *dsm, void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n >= 0 && n < (1LL << 40) && grid_ok(xsize, ysize), "vs_proj_to_grid: bad sizes n=%lld grid=%lldx%lld",
               (long long)n, (long long)xsize, (long long)ysize);
    VS_REQUIRE(dsm && (points || n == 0) && workspace, "vs_proj_to_grid: null pointer");
    const size_t need = vs_proj_to_grid_workspace_size(xsize, ysize);
    if (workspace_bytes < need) {
        set_error("vs_proj_to_grid: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    RasterWs w = carve_raster(workspace, xsize, ysize, false);
    Carver cv(workspace);
    cv.used = w.bytes;
    double *nanmax = cv.take<double>(static_cast<size_t>(xsize) * ysize);
    Tables tb;
    const long long cells = xsize * ysize;
    int s = make_tables(xoff, yoff, xresolution, yresolution, xsize, ysize, w, tb, st);
    if (s == VS_OK) s = clear(w.keys[0], sizeof(unsigned long long) * cells, st);
    if (s == VS_OK) s = clear(w.first, sizeof(unsigned long long) * cells, st);
    if (s == VS_OK) s = bin_launch(points, nullptr, 0, n, n, tb, w.keys[0], w.first, st);
    if (s != VS_OK) return s;
    const int threads = 256;
    unsigned g = static_cast<unsigned>(std::min<long long>(ceil_div(cells, threads), sm_count() * 16LL));
    decode_kernel<<<g, threads, 0, st>>>(w.keys[0], w.first, points, nanmax, cells);
    VS_LAUNCH_CHECK("decode_kernel");
    hole_fill_kernel<<<g, threads, 0, st>>>(nanmax, dsm, ysize, xsize, cells);
    VS_LAUNCH_CHECK("hole_fill_kernel");
    return VS_OK;
}

extern "C" size_t vs_dsm_from_points_workspace_size(int n_views, int64_t xsize, int64_t ysize) {
    if (n_views <= 0 || xsize <= 0 || ysize <= 0) return 0;
    return carve_raster(nullptr, xsize, ysize, true).bytes + 256;
}

extern "C" int vs_dsm_from_points(const double *points, const int64_t *offsets, int n_views, double xoff,
                                  double yoff, double xresolution, double yresolution, int64_t xsize,
                                  int64_t ysize, float *dsm, void *workspace, size_t workspace_bytes,
                                  void *stream) {
    VS_REQUIRE(n_views > 0 && n_views < (1 << 23) && grid_ok(xsize, ysize),
               "vs_dsm_from_points: bad sizes views=%d grid=%lldx%lld", n_views, (long long)xsize, (long long)ysize);
    VS_REQUIRE(points && offsets && dsm && workspace, "vs_dsm_from_points: null pointer");
    const size_t need = vs_dsm_from_points_workspace_size(n_views, xsize, ysize);
    if (workspace_bytes < need) {
        set_error("vs_dsm_from_points: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    RasterWs w = carve_raster(workspace, xsize, ysize, true);
    Tables tb;
    const long long cells = xsize * ysize;
    int s = make_tables(xoff, yoff, xresolution, yresolution, xsize, ysize, w, tb, st);
    if (s == VS_OK) s = clear(w.keys[0], sizeof(unsigned long long) * cells, st);
    if (s == VS_OK) s = clear(w.first, sizeof(unsigned long long) * cells, st);
    if (s != VS_OK) return s;
    // per-view counts live on the device: launch for a full GPU and let the grid stride
    const long long launch_points = static_cast<long long>(sm_count()) * 8 * 256 * kPts;
    const dim3 egrid(static_cast<unsigned>(ceil_div(xsize, TX)), static_cast<unsigned>(ceil_div(ysize, TILE_Y)));
    for (int v = 0; v < n_views; ++v) {
        unsigned long long *cur = w.keys[v & 1], *nxt = (v + 1 < n_views) ? w.keys[(v + 1) & 1] : nullptr;
        s = bin_launch(points, reinterpret_cast<const long long *>(offsets), v, 0, launch_points, tb, cur, w.first, st);
        if (s != VS_OK) return s;
        dsm_epilogue_kernel<<<egrid, dim3(TX, TY), 0, st>>>(cur, w.first, points, dsm + v * cells, nxt,
                                                            static_cast<int>(ysize), static_cast<int>(xsize));
        VS_LAUNCH_CHECK("dsm_epilogue_kernel");
    }
    return VS_OK;
}

// Overlapped form: view v's epilogue (issue-bound, L2-resident keys) runs on a second
// stream while view v+1's points are binned (HBM-bound).  Three key grids rotate: bin(v)
// fills K[v%3]; epilogue(v) reads K[v%3] and clears K[(v+2)%3] for bin(v+2), which waits
// for it.  The "first zero" words alternate between two arrays (bin(v+1) posts to the one
// epilogue(v) does not read); their epoch tags make stale words lose without clearing.
namespace vs {
namespace {
struct OverlapWs {
    unsigned long long *keys[3];
    unsigned long long *first[2];
    long long *row_thr, *col_thr;
    size_t bytes;
};

OverlapWs carve_overlap(void *ws, long long xsize, long long ysize) {
    Carver cv(ws);
    OverlapWs r;
    const size_t cells = static_cast<size_t>(xsize) * ysize;
    for (auto &k : r.keys) k = cv.take<unsigned long long>(cells);
    for (auto &f : r.first) f = cv.take<unsigned long long>(cells);
    r.row_thr = cv.take<long long>(ysize + 1);
    r.col_thr = cv.take<long long>(xsize + 1);
    r.bytes = cv.used;
    return r;
}

// Per-thread, per-device ring of ordering events (created once; no device memory).
struct EventRing {
    int device = -1;
    cudaEvent_t bin[3] = {}, epi[3] = {};
};

int event_ring(EventRing *&out) {
    static thread_local EventRing ring;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        set_error("cudaGetDevice failed");
        return VS_ERR_CUDA;
    }
    if (ring.device != dev) {
        for (int i = 0; i < 3; ++i) {
            if (cudaEventCreateWithFlags(&ring.bin[i], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&ring.epi[i], cudaEventDisableTiming) != cudaSuccess) {
                set_error("cudaEventCreateWithFlags failed");
                return VS_ERR_CUDA;
            }
        }
        ring.device = dev;
    }
    out = &ring;
    return VS_OK;
}
}  // namespace
}  // namespace vs

// Points in host memory: view v's points are copied into staging buffer v % ring on
// copy_stream while earlier views are binned on `stream`; an event per buffer orders the
// copy after the previous user of the buffer (its binning and epilogue) and the binning
// after the copy.  Per view the binning runs on the buffer as a one-view list (local point
// indices, the view's epoch tag), the epilogue resolves zeros from the same buffer, so the
// results equal vs_dsm_from_points.
static size_t host_ring_bytes(int64_t max_view_points, int ring) {
    return static_cast<size_t>(ring) * ((static_cast<size_t>(max_view_points) * 24 + 255) & ~size_t(255));
}

extern "C" size_t vs_dsm_from_points_host_workspace_size(int64_t max_view_points, int ring, int64_t xsize,
                                                          int64_t ysize) {
    if (max_view_points < 0 || ring < 1 || xsize <= 0 || ysize <= 0) return 0;
    return carve_raster(nullptr, xsize, ysize, true).bytes + 256 + host_ring_bytes(max_view_points, ring);
}

extern "C" int vs_dsm_from_points_host(const double *host_points, const int64_t *host_offsets, int n_views,
                                       double xoff, double yoff, double xresolution, double yresolution,
                                       int64_t xsize, int64_t ysize, float *dsm, int ring, void *workspace,
                                       size_t workspace_bytes, void *stream, void *copy_stream) {
    VS_REQUIRE(n_views > 0 && n_views < (1 << 23) && grid_ok(xsize, ysize) && ring >= 1 && ring <= 8,
               "vs_dsm_from_points_host: bad sizes views=%d grid=%lldx%lld ring=%d", n_views, (long long)xsize,
               (long long)ysize, ring);
    VS_REQUIRE(host_offsets && dsm && workspace, "vs_dsm_from_points_host: null pointer");
    long long max_pts = 0;
    for (int v = 0; v < n_views; ++v) {
        const long long cnt = host_offsets[v + 1] - host_offsets[v];
        VS_REQUIRE(cnt >= 0 && host_offsets[v] >= 0 && cnt < (1LL << 40), "vs_dsm_from_points_host: bad offsets");
        max_pts = std::max(max_pts, cnt);
    }
    VS_REQUIRE(host_points || max_pts == 0, "vs_dsm_from_points_host: null points");
    const size_t need = vs_dsm_from_points_host_workspace_size(max_pts, ring, xsize, ysize);
    if (workspace_bytes < need) {
        set_error("vs_dsm_from_points_host: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream), cs = as_stream(copy_stream);
    RasterWs w = carve_raster(workspace, xsize, ysize, true);
    const size_t slot = (static_cast<size_t>(max_pts) * 24 + 255) & ~size_t(255);
    char *ring_base = static_cast<char *>(workspace) + ((w.bytes + 255) & ~size_t(255));
    Tables tb;
    const long long cells = xsize * ysize;
    int s = make_tables(xoff, yoff, xresolution, yresolution, xsize, ysize, w, tb, st);
    if (s == VS_OK) s = clear(w.keys[0], sizeof(unsigned long long) * cells, st);
    if (s == VS_OK) s = clear(w.first, sizeof(unsigned long long) * cells, st);
    if (s != VS_OK) return s;
    cudaEvent_t freed[8], landed[8];
    int made = 0;
    for (; made < ring; ++made) {
        if (cudaEventCreateWithFlags(&freed[made], cudaEventDisableTiming) != cudaSuccess) break;
        if (cudaEventCreateWithFlags(&landed[made], cudaEventDisableTiming) != cudaSuccess) {
            cudaEventDestroy(freed[made]);
            break;
        }
    }
    if (made < ring) {
        for (int i = 0; i < made; ++i) {
            cudaEventDestroy(freed[i]);
            cudaEventDestroy(landed[i]);
        }
        set_error("vs_dsm_from_points_host: cudaEventCreate failed");
        return VS_ERR_CUDA;
    }
    const dim3 egrid(static_cast<unsigned>(ceil_div(xsize, TX)), static_cast<unsigned>(ceil_div(ysize, TILE_Y)));
    // the copy stream starts after the work already queued on `stream` (tables, clears)
    if (cudaEventRecord(freed[0], st) != cudaSuccess || cudaStreamWaitEvent(cs, freed[0], 0) != cudaSuccess)
        s = VS_ERR_CUDA;
    for (int v = 0; v < n_views && s == VS_OK; ++v) {
        const int b = v % ring;
        const long long cnt = host_offsets[v + 1] - host_offsets[v];
        double *buf = reinterpret_cast<double *>(ring_base + b * slot);
        if (v >= ring && cudaStreamWaitEvent(cs, freed[b], 0) != cudaSuccess) s = VS_ERR_CUDA;
        if (s == VS_OK && cnt > 0 &&
            cudaMemcpyAsync(buf, host_points + 3 * host_offsets[v], static_cast<size_t>(cnt) * 24,
                            cudaMemcpyHostToDevice, cs) != cudaSuccess)
            s = VS_ERR_CUDA;
        if (s == VS_OK && (cudaEventRecord(landed[b], cs) != cudaSuccess ||
                           cudaStreamWaitEvent(st, landed[b], 0) != cudaSuccess))
            s = VS_ERR_CUDA;
        if (s != VS_OK) {
            set_error("vs_dsm_from_points_host: copy or event call failed at view %d", v);
            break;
        }
        unsigned long long *cur = w.keys[v & 1], *nxt = (v + 1 < n_views) ? w.keys[(v + 1) & 1] : nullptr;
        if ((s = bin_launch(buf, nullptr, v, cnt, cnt, tb, cur, w.first, st)) != VS_OK) break;
        dsm_epilogue_kernel<<<egrid, dim3(TX, TY), 0, st>>>(cur, w.first, buf, dsm + v * cells, nxt,
                                                            static_cast<int>(ysize), static_cast<int>(xsize));
        if ((s = check_launch("dsm_epilogue_kernel")) != VS_OK) break;
        if (cudaEventRecord(freed[b], st) != cudaSuccess) {
            set_error("vs_dsm_from_points_host: cudaEventRecord failed");
            s = VS_ERR_CUDA;
        }
    }
    // `stream` covers the copies too (every copy is waited for by a binning on `stream`)
    for (int i = 0; i < ring; ++i) {
        cudaEventDestroy(freed[i]);
        cudaEventDestroy(landed[i]);
    }
    return s;
}

extern "C" size_t vs_dsm_from_points_overlap_workspace_size(int n_views, int64_t xsize, int64_t ysize) {
    if (n_views <= 0 || xsize <= 0 || ysize <= 0) return 0;
    return carve_overlap(nullptr, xsize, ysize).bytes + 256;
}

extern "C" int vs_dsm_from_points_overlap(const double *points, const int64_t *offsets, int n_views, double xoff,
                                          double yoff, double xresolution, double yresolution, int64_t xsize,
                                          int64_t ysize, float *dsm, void *workspace, size_t workspace_bytes,
                                          void *stream, void *epilogue_stream, void *const *bin_events) {
    VS_REQUIRE(n_views > 0 && n_views < (1 << 23) && grid_ok(xsize, ysize),
               "vs_dsm_from_points_overlap: bad sizes views=%d grid=%lldx%lld", n_views, (long long)xsize,
               (long long)ysize);
    VS_REQUIRE(points && offsets && dsm && workspace, "vs_dsm_from_points_overlap: null pointer");
    const size_t need = vs_dsm_from_points_overlap_workspace_size(n_views, xsize, ysize);
    if (workspace_bytes < need) {
        set_error("vs_dsm_from_points_overlap: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream), es = as_stream(epilogue_stream);
    EventRing *ev = nullptr;
    int s = event_ring(ev);
    if (s != VS_OK) return s;
    OverlapWs w = carve_overlap(workspace, xsize, ysize);
    RasterWs tw;                       // threshold tables only
    tw.row_thr = w.row_thr;
    tw.col_thr = w.col_thr;
    Tables tb;
    const long long cells = xsize * ysize;
    s = make_tables(xoff, yoff, xresolution, yresolution, xsize, ysize, tw, tb, st);
    for (int i = 0; i < 2 && s == VS_OK; ++i) s = clear(w.keys[i], sizeof(unsigned long long) * cells, st);
    for (int i = 0; i < 2 && s == VS_OK; ++i) s = clear(w.first[i], sizeof(unsigned long long) * cells, st);
    if (s != VS_OK) return s;
    const long long launch_points = static_cast<long long>(sm_count()) * 8 * 256 * kPts;
    const dim3 egrid(static_cast<unsigned>(ceil_div(xsize, TX)), static_cast<unsigned>(ceil_div(ysize, TILE_Y)));
    auto cuda_ok = [](cudaError_t e) {
        if (e == cudaSuccess) return true;
        set_error("stream ordering failed: %s", cudaGetErrorString(e));
        return false;
    };
    for (int v = 0; v < n_views; ++v) {
        if (v >= 2 && !cuda_ok(cudaStreamWaitEvent(st, ev->epi[(v - 2) % 3], 0))) return VS_ERR_CUDA;
        if (bin_events && !cuda_ok(cudaEventRecord(static_cast<cudaEvent_t>(bin_events[2 * v]), st))) return VS_ERR_CUDA;
        s = bin_launch(points, reinterpret_cast<const long long *>(offsets), v, 0, launch_points, tb, w.keys[v % 3],
                       w.first[v & 1], st);
        if (s != VS_OK) return s;
        if (bin_events && !cuda_ok(cudaEventRecord(static_cast<cudaEvent_t>(bin_events[2 * v + 1]), st)))
            return VS_ERR_CUDA;
        if (!cuda_ok(cudaEventRecord(ev->bin[v % 3], st)) || !cuda_ok(cudaStreamWaitEvent(es, ev->bin[v % 3], 0)))
            return VS_ERR_CUDA;
        // with an L2 set-aside the epilogue's clear of bin(v+2)'s grid is marked persisting:
        // the zeros then stay in L2 while view v+1's points stream through, instead of being
        // written back and fetched again by bin(v+2)'s first atomics
        unsigned long long *nxt = (v + 2 < n_views) ? w.keys[(v + 2) % 3] : nullptr;
        const unsigned long long *cur = w.keys[v % 3], *fz = w.first[v & 1];
        if (launch_with_key_window(dsm_epilogue_kernel, egrid, dim3(TX, TY), es, nxt,
                                   nxt ? sizeof(unsigned long long) * static_cast<size_t>(cells) : 0, cur, fz, points,
                                   dsm + v * cells, nxt, static_cast<int>(ysize), static_cast<int>(xsize)) != cudaSuccess)
            return check_launch("dsm_epilogue_kernel");
        VS_LAUNCH_CHECK("dsm_epilogue_kernel");
        if (!cuda_ok(cudaEventRecord(ev->epi[v % 3], es))) return VS_ERR_CUDA;
    }
    // the caller's stream covers the last epilogues
    if (!cuda_ok(cudaStreamWaitEvent(st, ev->epi[(n_views - 1) % 3], 0))) return VS_ERR_CUDA;
    return VS_OK;
}

// Pipelined form: launch v (v = 0..V) bins view v and runs view v-1's epilogue
// (raster_pipe_kernel), all on one stream.  Key grids rotate as in the overlapped form:
// bin(v) fills K[v%3]; epilogue(v-1) reads K[(v-1)%3] and clears K[(v+1)%3], which
// epilogue(v-2) finished reading in the previous launch; the first-zero words alternate.
// One counter per launch (cleared once per call) hands out the work items.
template <int MINB>
static void launch_pipe(bool flip_row, bool flip_col, unsigned gx, cudaStream_t st, const double *points,
                        const vs::PipeBin &b, const vs::PipeEpi &e, unsigned *counter, size_t key_bytes) {
    using namespace vs;
    auto kern = flip_row ? (flip_col ? raster_pipe_kernel<true, true, MINB> : raster_pipe_kernel<true, false, MINB>)
                         : (flip_col ? raster_pipe_kernel<false, true, MINB> : raster_pipe_kernel<false, false, MINB>);
    launch_with_key_window(kern, dim3(gx), dim3(TX, TY), st, b.keys, b.active ? key_bytes : 0, points, b, e, counter);
}

static size_t pipelined_counters_offset(int64_t xsize, int64_t ysize) {
    return (vs::carve_overlap(nullptr, xsize, ysize).bytes + 255) & ~size_t(255);
}

extern "C" size_t vs_dsm_from_points_pipelined_workspace_size(int n_views, int64_t xsize, int64_t ysize) {
    if (n_views <= 0 || xsize <= 0 || ysize <= 0) return 0;
    return pipelined_counters_offset(xsize, ysize) + sizeof(unsigned) * (static_cast<size_t>(n_views) + 1) + 256;
}

extern "C" int vs_dsm_from_points_pipelined(const double *points, const int64_t *offsets, int n_views, double xoff,
                                            double yoff, double xresolution, double yresolution, int64_t xsize,
                                            int64_t ysize, float *dsm, void *workspace, size_t workspace_bytes,
                                            void *stream, void *const *launch_events) {
    using namespace vs;
    VS_REQUIRE(n_views > 0 && n_views < (1 << 23) && grid_ok(xsize, ysize),
               "vs_dsm_from_points_pipelined: bad sizes views=%d grid=%lldx%lld", n_views, (long long)xsize,
               (long long)ysize);
    VS_REQUIRE(points && offsets && dsm && workspace, "vs_dsm_from_points_pipelined: null pointer");
    const size_t need = vs_dsm_from_points_pipelined_workspace_size(n_views, xsize, ysize);
    if (workspace_bytes < need) {
        set_error("vs_dsm_from_points_pipelined: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    OverlapWs w = carve_overlap(workspace, xsize, ysize);
    unsigned *counters = reinterpret_cast<unsigned *>(static_cast<char *>(workspace) +
                                                      pipelined_counters_offset(xsize, ysize));
    RasterWs tw;                       // threshold tables only
    tw.row_thr = w.row_thr;
    tw.col_thr = w.col_thr;
    Tables tb;
    const long long cells = xsize * ysize;
    int s = make_tables(xoff, yoff, xresolution, yresolution, xsize, ysize, tw, tb, st);
    for (int i = 0; i < 2 && s == VS_OK; ++i) s = clear(w.keys[i], sizeof(unsigned long long) * cells, st);
    for (int i = 0; i < 2 && s == VS_OK; ++i) s = clear(w.first[i], sizeof(unsigned long long) * cells, st);
    if (s == VS_OK) s = clear(counters, sizeof(unsigned) * (static_cast<size_t>(n_views) + 1), st);
    if (s != VS_OK) return s;
    const int tiles_x = static_cast<int>(ceil_div(xsize, TX));
    const long long n_tiles = static_cast<long long>(tiles_x) * ceil_div(ysize, TILE_Y);
    if (!fast_binning(tb)) {
        // points outside the fast path's precondition: the literal FP64 binning, then the
        // epilogue, view by view (same results)
        const long long launch_points = static_cast<long long>(sm_count()) * 8 * 256 * kPts;
        const dim3 egrid(static_cast<unsigned>(tiles_x), static_cast<unsigned>(ceil_div(ysize, TILE_Y)));
        for (int v = 0; v < n_views; ++v) {
            s = bin_launch(points, reinterpret_cast<const long long *>(offsets), v, 0, launch_points, tb, w.keys[v % 3],
                           w.first[v & 1], st);
            if (s != VS_OK) return s;
            unsigned long long *nxt = (v + 2 < n_views) ? w.keys[(v + 2) % 3] : nullptr;
            dsm_epilogue_kernel<<<egrid, dim3(TX, TY), 0, st>>>(w.keys[v % 3], w.first[v & 1], points,
                                                                dsm + v * cells, nxt, static_cast<int>(ysize),
                                                                static_cast<int>(xsize));
            VS_LAUNCH_CHECK("dsm_epilogue_kernel");
        }
        return VS_OK;
    }
    FastAxis fa[2];
    fast_axes(tb, fa);
    const bool flip_row = !tb.row.neg, flip_col = tb.col.neg != 0;
    // a cap of 5 or fewer CTAs per SM takes the 48-register build, which spills nothing
    const bool narrow = g_bin_ctas_per_sm > 0 && g_bin_ctas_per_sm <= 5;
    static int resident[2] = {0, 0};
    if (!resident[narrow]) {
        int per_sm = 0;
        const cudaError_t e = narrow ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                           &per_sm, raster_pipe_kernel<true, false, 5>, TX * TY, 0)
                                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                           &per_sm, raster_pipe_kernel<true, false, 6>, TX * TY, 0);
        resident[narrow] = (e == cudaSuccess && per_sm > 0) ? per_sm : 4;
    }
    const int per_sm = g_bin_ctas_per_sm > 0 ? std::min(g_bin_ctas_per_sm, resident[narrow]) : resident[narrow];
    // the views' point counts stay on the device: every launch is one resident wave, and
    // its CTAs derive the chunk count from the offsets
    const unsigned gx = static_cast<unsigned>(sm_count() * per_sm);
    for (int v = 0; v <= n_views; ++v) {
        PipeBin b{};
        b.offsets = reinterpret_cast<const long long *>(offsets);
        b.v = v < n_views ? v : 0;
        b.active = v < n_views;
        b.row = fa[0];
        b.col = fa[1];
        if (v < n_views) {
            b.keys = w.keys[v % 3];
            b.first = w.first[v & 1];
        }
        PipeEpi e{};
        e.H = static_cast<int>(ysize);
        e.W = static_cast<int>(xsize);
        e.tiles_x = tiles_x;
        if (v > 0) {
            e.keys = w.keys[(v - 1) % 3];
            e.first = w.first[(v - 1) & 1];
            e.out = dsm + (v - 1) * cells;
            e.clear = (v + 1 < n_views) ? w.keys[(v + 1) % 3] : nullptr;
            e.n_tiles = n_tiles;
        }
        if (launch_events && cudaEventRecord(static_cast<cudaEvent_t>(launch_events[2 * v]), st) != cudaSuccess) {
            set_error("vs_dsm_from_points_pipelined: cudaEventRecord failed");
            return VS_ERR_CUDA;
        }
        const size_t key_bytes = sizeof(unsigned long long) * static_cast<size_t>(cells);
        if (narrow)
            launch_pipe<5>(flip_row, flip_col, gx, st, points, b, e, counters + v, key_bytes);
        else
            launch_pipe<6>(flip_row, flip_col, gx, st, points, b, e, counters + v, key_bytes);
        VS_LAUNCH_CHECK("raster_pipe_kernel");
        if (launch_events && cudaEventRecord(static_cast<cudaEvent_t>(launch_events[2 * v + 1]), st) != cudaSuccess) {
            set_error("vs_dsm_from_points_pipelined: cudaEventRecord failed");
            return VS_ERR_CUDA;
        }
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

// ---- batched form: plan and run ------------------------------------------------------------
struct VsAoiBatch {
    int n_aois = 0, n_views = 0, tile = 0;
    std::vector<VsAoi> aois;
    std::vector<long long> view_off, fused_off, tile_start;
    long long view_cells = 0, fused_cells = 0, max_fuse_cells = 0;
    bool all_direct = true;                // every view has its own DSM output
    vs::MapViewDev *d_views = nullptr;
    vs::AoiDev *d_aois = nullptr;
    long long *d_tile_start = nullptr;
    unsigned long long *d_counter = nullptr;
    std::vector<vs::MapViewDev> h_views;   // host copies, alive while their upload runs
    std::vector<vs::AoiDev> h_aois;
};

namespace vs {
namespace {

struct PlanLayout {
    MapViewDev *views;
    AoiDev *aois;
    long long *tile_start;
    unsigned long long *counter;
    long long *thr;
    size_t bytes;
};

PlanLayout carve_plan(void *ws, const VsAoi *aois, int n_aois, int n_views) {
    Carver cv(ws);
    PlanLayout p;
    p.views = cv.take<MapViewDev>(n_views);
    p.aois = cv.take<AoiDev>(n_aois);
    p.tile_start = cv.take<long long>(n_views + 1);
    p.counter = cv.take<unsigned long long>(2);
    size_t thr = 0;
    for (int a = 0; a < n_aois; ++a) thr += static_cast<size_t>(aois[a].xsize + 1) + static_cast<size_t>(aois[a].ysize + 1);
    p.thr = cv.take<long long>(thr);
    p.bytes = cv.used;
    return p;
}

// Fixed-point view coordinates stay exact doubles and shifted bit patterns stay in range.
bool map_axis_ok(long long o, int sj, int si, int W, int H, int sh) {
    const long long lim = 1LL << 52;
    if (o <= -lim || o >= lim) return false;
    const long long dj = W - 1, di = H - 1;
    for (int a = -1; a <= 1; a += 2)
        for (int b = -1; b <= 1; b += 2) {
            const long long v = o + static_cast<long long>(sj) * dj * a + static_cast<long long>(si) * di * b;
            if (v <= -lim || v >= lim) return false;
            const long long mag = v < 0 ? -v : v;
            if (mag >= (1LL << (62 - sh))) return false;
        }
    return true;
}

}  // namespace
}  // namespace vs

extern "C" size_t vs_aoi_batch_plan_workspace_size(const VsAoi *aois, int n_aois, int n_views) {
    if (!aois || n_aois <= 0 || n_views <= 0) return 0;
    for (int a = 0; a < n_aois; ++a)
        if (aois[a].xsize <= 0 || aois[a].ysize <= 0) return 0;
    return carve_plan(nullptr, aois, n_aois, n_views).bytes + 256;
}

extern "C" int vs_aoi_batch_plan(const VsAoi *aois, int n_aois, const VsMapView *views, int n_views,
                                 int tile, void *workspace, size_t workspace_bytes, VsAoiBatch **plan,
                                 void *stream) {
    VS_REQUIRE(aois && views && plan && workspace && n_aois > 0 && n_views > 0 && n_views < (1 << 30) &&
                   (tile == 32 || tile == 64),
               "vs_aoi_batch_plan: bad arguments (tile must be 32 or 64)");
    *plan = nullptr;
    const size_t need = vs_aoi_batch_plan_workspace_size(aois, n_aois, n_views);
    VS_REQUIRE(need > 0, "vs_aoi_batch_plan: empty grid");
    if (workspace_bytes < need) {
        set_error("vs_aoi_batch_plan: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    PlanLayout L = carve_plan(workspace, aois, n_aois, n_views);
    VsAoiBatch *p = new VsAoiBatch();
    p->n_aois = n_aois;
    p->n_views = n_views;
    p->tile = tile;
    p->aois.assign(aois, aois + n_aois);
    p->h_aois.resize(n_aois);
    p->h_views.resize(n_views);
    p->view_off.resize(n_views + 1);
    p->tile_start.resize(n_views + 1);
    p->fused_off.resize(n_aois + 1);
    auto fail = [&](int code) {
        delete p;
        return code;
    };
    long long *thr = L.thr;
    std::vector<double> sig_c(n_aois), sig_r(n_aois);   // cell coordinate per ulp of difference
    p->fused_off[0] = 0;
    int expect_view = 0;
    for (int a = 0; a < n_aois; ++a) {
        const VsAoi &A = aois[a];
        // cells below 2^31: the binning kernel indexes cells with 32-bit integers
        if (!(grid_ok(A.xsize, A.ysize) && A.xsize < (1LL << 22) && A.ysize < (1LL << 22) &&
              A.xsize * A.ysize < (1LL << 31) && A.n_views > 0 && A.first_view == expect_view && A.xoff > 0.0 &&
              A.yoff > 0.0)) {
            set_error("vs_aoi_batch_plan: AOI %d: bad grid (at most 2^31 - 1 cells) or view range (views must be "
                      "consecutive, origin positive)", a);
            return fail(VS_ERR_ARG);
        }
        expect_view += A.n_views;
        Tables tb;
        int s = make_axis(tb.row, A.yoff, A.xres, A.ysize, -1, thr, st);
        thr += A.ysize + 1;
        if (s == VS_OK) s = make_axis(tb.col, A.xoff, A.yres, A.xsize, +1, thr, st);
        thr += A.xsize + 1;
        if (s != VS_OK) return fail(s);
        if (!(tb.row.fast && tb.row.contained && tb.col.fast && tb.col.contained)) {
            set_error("vs_aoi_batch_plan: AOI %d: grid extent crosses a power of two of its origin", a);
            return fail(VS_ERR_ARG);
        }
        AoiDev &ad = p->h_aois[a];
        ad.row = fast_axis_of(tb.row);
        ad.col = fast_axis_of(tb.col);
        int ex = 0, ey = 0;
        frexp(A.xoff, &ex);
        frexp(A.yoff, &ey);
        ex -= 1;   // 2^ex <= xoff < 2^(ex+1)
        ey -= 1;
        if (ex < 0 || ex > 24 || ey < 0 || ey > 24) {
            set_error("vs_aoi_batch_plan: AOI %d: origin outside [1, 2^25) m", a);
            return fail(VS_ERR_ARG);
        }
        ad.shx = 24 - ex;
        ad.shy = 24 - ey;
        sig_c[a] = ldexp(1.0, ex - 52) / A.yres;    // columns divide by yres, rows by xres
        sig_r[a] = ldexp(1.0, ey - 52) / A.xres;    // (lib/proj_to_grid.py's own pairing)
        ad.bx = (static_cast<long long>(ex + 1023) << 52) - (1LL << 52);
        ad.by = (static_cast<long long>(ey + 1023) << 52) - (1LL << 52);
        ad.xsize = static_cast<int>(A.xsize);
        ad.ysize = static_cast<int>(A.ysize);
        const long long cells = A.xsize * A.ysize;
        p->fused_off[a + 1] = p->fused_off[a] + cells;
        p->max_fuse_cells = std::max(p->max_fuse_cells, cells);
    }
    if (expect_view != n_views) {
        set_error("vs_aoi_batch_plan: the AOIs cover %d views, %d given", expect_view, n_views);
        return fail(VS_ERR_ARG);
    }
    p->view_off[0] = p->tile_start[0] = 0;
    for (int v = 0; v < n_views; ++v) {
        const VsMapView &V = views[v];
        const bool aoi_ok = V.aoi >= 0 && V.aoi < n_aois && v >= aois[V.aoi].first_view &&
                            v < aois[V.aoi].first_view + aois[V.aoi].n_views;
        if (!(aoi_ok && V.heights && V.width > 0 && V.height > 0 && V.row_stride >= V.width &&
              static_cast<unsigned long long>(V.width) * static_cast<unsigned long long>(V.height) <= kMapIdxLimit)) {
            set_error("vs_aoi_batch_plan: view %d: bad size, stride, map or AOI index", v);
            return fail(VS_ERR_ARG);
        }
        const AoiDev &ad = p->h_aois[V.aoi];
        if (!map_axis_ok(V.e0, V.ej, V.ei, V.width, V.height, ad.shx) ||
            !map_axis_ok(V.n0, V.nj, V.ni, V.width, V.height, ad.shy)) {
            set_error("vs_aoi_batch_plan: view %d: fixed-point coordinates out of the exact range", v);
            return fail(VS_ERR_ARG);
        }
        MapViewDev &d = p->h_views[v];
        d.map = V.heights;
        d.stride = V.row_stride;
        d.e0 = V.e0;
        d.n0 = V.n0;
        d.ej = V.ej;
        d.ei = V.ei;
        d.nj = V.nj;
        d.ni = V.ni;
        d.W = V.width;
        d.H = V.height;
        d.aoi = V.aoi;
        d.vec = ((reinterpret_cast<uintptr_t>(V.heights) & 15) == 0) && (V.row_stride % 4 == 0);
        d.off = p->view_off[v];
        d.out = V.dsm;
        // d = bits(x) - bits(xoff) = (bx - bits(xoff)) + (x_fx << shx), x_fx affine in the
        // pixel indices (the shifts are exact: the plan checked |x_fx| << sh < 2^62)
        {
            const long long cb = ad.bx - ad.col.off_bits, rb = ad.row.off_bits - ad.by;
            d.dc0 = cb + (V.e0 << ad.shx);
            d.dc_di = static_cast<long long>(V.ei) << ad.shx;
            d.dc_dj = static_cast<long long>(V.ej) << ad.shx;
            d.dr0 = rb - (V.n0 << ad.shy);
            d.dr_di = -(static_cast<long long>(V.ni) << ad.shy);
            d.dr_dj = -(static_cast<long long>(V.nj) << ad.shy);
        }
        // pixel <- cell map for the tiles' pixel boxes: (s_col, s_row) = sig * (d_col, d_row)
        // with d = d0 + M (u, w), u = 2i+1-H, w = 2j+1-W; inverted in FP64, with a margin for
        // its rounding; a singular (or numerically hopeless) map reads the whole map per tile
        {
            const double a = static_cast<double>(d.dc_di), b = static_cast<double>(d.dc_dj);
            const double c = static_cast<double>(d.dr_di), e = static_cast<double>(d.dr_dj);
            const double dc0 = static_cast<double>(d.dc0), dr0 = static_cast<double>(d.dr0);
            const double det = a * e - b * c;
            const double sc = sig_c[V.aoi], sr = sig_r[V.aoi];
            d.bic = e / (sc * det) * 0.5;
            d.bir = -b / (sr * det) * 0.5;
            d.bi0 = ((b * dr0 - e * dc0) / det + (V.height - 1)) * 0.5;
            d.bjc = -c / (sc * det) * 0.5;
            d.bjr = a / (sr * det) * 0.5;
            d.bj0 = ((c * dc0 - a * dr0) / det + (V.width - 1)) * 0.5;
            const double span = fabs(d.bic) * (static_cast<double>(aois[V.aoi].xsize) + 4.0) + fabs(d.bir) * (static_cast<double>(aois[V.aoi].ysize) + 4.0) +
                                fabs(d.bjc) * (static_cast<double>(aois[V.aoi].xsize) + 4.0) + fabs(d.bjr) * (static_cast<double>(aois[V.aoi].ysize) + 4.0);
            const double big = (fabs(e * dc0) + fabs(b * dr0) + fabs(c * dc0) + fabs(a * dr0)) / fabs(det);
            d.bmarg = 1.0 + 1e-12 * (big + span + fabs(d.bi0) + fabs(d.bj0));
            const bool finite = std::isfinite(d.bic) && std::isfinite(d.bir) && std::isfinite(d.bi0) &&
                                std::isfinite(d.bjc) && std::isfinite(d.bjr) && std::isfinite(d.bj0) &&
                                std::isfinite(d.bmarg);
            d.box_all = !(det != 0.0 && finite && d.bmarg < 64.0);
        }
        if (!V.dsm) p->all_direct = false;
        const VsAoi &A = aois[V.aoi];
        const long long cells = A.xsize * A.ysize;
        p->view_off[v + 1] = p->view_off[v] + cells;
        p->tile_start[v + 1] = p->tile_start[v] + ceil_div(A.xsize, tile) * ceil_div(A.ysize, tile);
    }
    p->view_cells = p->view_off[n_views];
    p->fused_cells = p->fused_off[n_aois];
    p->d_views = L.views;
    p->d_aois = L.aois;
    p->d_tile_start = L.tile_start;
    p->d_counter = L.counter;
    bool ok = cudaMemcpyAsync(L.views, p->h_views.data(), sizeof(MapViewDev) * n_views, cudaMemcpyHostToDevice, st) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(L.aois, p->h_aois.data(), sizeof(AoiDev) * n_aois, cudaMemcpyHostToDevice, st) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(L.tile_start, p->tile_start.data(), sizeof(long long) * (n_views + 1),
                               cudaMemcpyHostToDevice, st) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) {
        set_error("vs_aoi_batch_plan: descriptor upload failed: %s", cudaGetErrorString(cudaGetLastError()));
        return fail(VS_ERR_CUDA);
    }
    *plan = p;
    return VS_OK;
}

extern "C" int vs_aoi_batch_query(const VsAoiBatch *plan, int64_t *view_cells, int64_t *fused_cells,
                                  size_t *scratch_bytes) {
    VS_REQUIRE(plan, "vs_aoi_batch_query: null plan");
    if (view_cells) *view_cells = plan->view_cells;
    if (fused_cells) *fused_cells = plan->fused_cells;
    if (scratch_bytes) *scratch_bytes = vs_fuse_dsms_workspace_size(1, plan->max_fuse_cells) + 256;
    return VS_OK;
}

namespace vs {
namespace {

template <int T>
int launch_map_tiles(const VsAoiBatch *plan, int view_begin, int view_end, int blocks_per_sm, float *view_dsm,
                     cudaStream_t st) {
    static int resident = 0;       // CTAs per SM the kernel fits (registers, shared memory)
    if (!resident) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, map_tile_kernel<T, T>, kMapThreads, 0) !=
                cudaSuccess ||
            per_sm <= 0)
            per_sm = 1;
        resident = per_sm;
    }
    const long long t0 = plan->tile_start[view_begin], t1 = plan->tile_start[view_end];
    const long long blocks = std::min<long long>(t1 - t0, 1LL * sm_count() * std::min(blocks_per_sm, resident));
    map_tile_kernel<T, T><<<static_cast<unsigned>(blocks), kMapThreads, 0, st>>>(
        plan->d_views, plan->d_aois, plan->d_tile_start, view_begin, view_end - 1, t0, t1, view_dsm, plan->d_counter);
    return check_launch("map_tile_kernel");
}

}  // namespace
}  // namespace vs

extern "C" int vs_aoi_batch_run(const VsAoiBatch *plan, int view_begin, int view_end, int blocks_per_sm,
                                float *view_dsm, void *stream) {
    VS_REQUIRE(plan && (view_dsm || plan->all_direct), "vs_aoi_batch_run: null pointer");
    VS_REQUIRE(0 <= view_begin && view_begin < view_end && view_end <= plan->n_views && blocks_per_sm > 0 &&
                   blocks_per_sm <= 64,
               "vs_aoi_batch_run: bad view range [%d, %d) or blocks per SM %d", view_begin, view_end, blocks_per_sm);
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(plan->d_counter, 0, sizeof(unsigned long long), st) != cudaSuccess) {
        set_error("vs_aoi_batch_run: cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
    return plan->tile == 64 ? launch_map_tiles<64>(plan, view_begin, view_end, blocks_per_sm, view_dsm, st)
                            : launch_map_tiles<32>(plan, view_begin, view_end, blocks_per_sm, view_dsm, st);
}

extern "C" int vs_aoi_batch_fuse(const VsAoiBatch *plan, int aoi_begin, int aoi_end, const float *view_dsm,
                                 float *fused, int median_blur, void *scratch, size_t scratch_bytes, void *stream) {
    VS_REQUIRE(plan && view_dsm && fused && scratch, "vs_aoi_batch_fuse: null pointer");
    VS_REQUIRE(0 <= aoi_begin && aoi_begin < aoi_end && aoi_end <= plan->n_aois, "vs_aoi_batch_fuse: bad AOI range");
    for (int a = aoi_begin; a < aoi_end; ++a) {
        const VsAoi &A = plan->aois[a];
        const int s = vs_fuse_dsms(view_dsm + plan->view_off[A.first_view], VS_LAYOUT_VHW, A.n_views, A.ysize, A.xsize,
                                   fused + plan->fused_off[a], median_blur, scratch, scratch_bytes, stream);
        if (s != VS_OK) return s;
    }
    return VS_OK;
}

extern "C" void vs_aoi_batch_destroy(VsAoiBatch *plan) { delete plan; }

// ---- (f1) depth maps -> DSM, without materialising the points ------------------------------
// Each pixel's (easting, northing, altitude) is computed as vs_depth_to_points does (the same
// shared device code, so the same bits) and binned at once with the fast binning.  Zeros of
// the nanmax keep the first-of-equal rule through the "first zero" words, which here carry
// the pixel index (monotone in the point index) and the zero's sign in bit 0.
namespace vs {
namespace {

constexpr unsigned long long kDepthIdxLimit = 1ull << 39;

struct SignZeroDecoder {
    const unsigned long long *first;
    __device__ __forceinline__ unsigned long long operator()(unsigned long long k, long long cell) const {
        if (k != kZeroKey) return k;
        return (first[cell] & 1ull) ? 0x7fffffffffffffffull : kZeroKey;
    }
};

template <bool FLIP_ROW, bool FLIP_COL>
__global__ void __launch_bounds__(256) depth_bin_kernel(const float *__restrict__ depth, long long H, long long W,
                                                        DepthView v, GeoFast f, const GeoFrame *g, int mode,
                                                        int south, FastAxis ra, FastAxis ca, int view,
                                                        unsigned long long *__restrict__ vk,
                                                        unsigned long long *__restrict__ first, int *flags) {
    __shared__ double smd[16];
    stage_matrix(v, smd);
    const long long total = H * W;
    const unsigned long long tag = epoch_tag(view);
    const unsigned long long ncols = static_cast<unsigned>(ca.nm1 + 1);
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x * kDepthPix;
    // pixel (row, col) of p kept incrementally in 32 bits (H, W < 2^24): no 64-bit division
    // or 64-bit int -> float conversion per pixel
    const long long p0 = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) * kDepthPix;
    const int Wi = static_cast<int>(W);
    const int stride_r = static_cast<int>(stride / W), stride_c = static_cast<int>(stride - (stride / W) * W);
    int r0 = static_cast<int>(p0 / W), c0 = static_cast<int>(p0 - (p0 / W) * W);
    for (long long p = p0; p < total; p += stride) {
        int r = r0, c = c0;
        float rf = __int2float_rn(r), cf = __int2float_rn(c);
        r0 += stride_r;
        c0 += stride_c;
        if (c0 >= Wi) {
            c0 -= Wi;
            ++r0;
        }
        long long run_cell = -1;
        unsigned long long run_key = kEmptyKey;
#pragma unroll 1
        for (int k = 0; k < kDepthPix; ++k) {
            const float dk = p + k < total ? __ldcs(depth + p + k) : -1.0f;
            df w;
            const int cls = pixel_class(v, cf, rf, dk, w);
            unsigned long long bits[3];
            if (cls != 0 && pixel_point(v, smd, f, g, mode, cls, w, cf, rf, dk, south, bits, flags)) {
                int rr, cc;
                long long dr, dc;
                bool sr, sc;
                bool ok = axis_fast<FLIP_ROW>(ra, static_cast<long long>(bits[1]), rr, dr, sr);
                ok &= axis_fast<FLIP_COL>(ca, static_cast<long long>(bits[0]), cc, dc, sc);
                ok &= !is_nan_bits(bits[2]);
                if (ok) {
                    if (!sr) rr = axis_correct(ra.thr, rr, dr);
                    if (!sc) cc = axis_correct(ca.thr, cc, dc);
                    const long long cell =
                        static_cast<long long>(static_cast<unsigned long long>(static_cast<unsigned>(rr)) * ncols) + cc;
                    const unsigned long long zb = bits[2];
                    unsigned long long key;
                    if ((zb << 1) == 0) {
                        key = kZeroKey;
                        const unsigned long long idx = static_cast<unsigned long long>(p + k);
                        atomicMax(first + cell, tag | ((kDepthIdxLimit - 1ull - idx) << 1) | (zb >> 63));
                    } else {
                        key = (zb >> 63) ? ~zb : (zb | 0x8000000000000000ull);
                    }
                    if (cell == run_cell) {
                        run_key = max(run_key, key);
                    } else {
                        if (run_key != kEmptyKey) atomicMax(vk + run_cell, run_key);
                        run_cell = cell;
                        run_key = key;
                    }
                }
            }
            cf = __fadd_rn(cf, 1.0f);
            if (++c == Wi) {
                c = 0;
                cf = 0.0f;
                ++r;
                rf = __fadd_rn(rf, 1.0f);
            }
        }
        if (run_key != kEmptyKey) atomicMax(vk + run_cell, run_key);
    }
}

__global__ void __launch_bounds__(TX *TY) depth_epilogue_kernel(const unsigned long long *__restrict__ vk,
                                                               const unsigned long long *__restrict__ first,
                                                               float *__restrict__ out,
                                                               unsigned long long *__restrict__ next_keys, int H,
                                                               int W) {
    __shared__ EpilogueSmem sm;
    epilogue_tile(vk, SignZeroDecoder{first}, out, next_keys, H, W, blockIdx.y * TILE_Y, blockIdx.x * TX, sm);
}

}  // namespace
}  // namespace vs

extern "C" size_t vs_dsm_from_depth_maps_workspace_size(int64_t xsize, int64_t ysize) {
    if (xsize <= 0 || ysize <= 0) return 0;
    return carve_raster(nullptr, xsize, ysize, true).bytes + 256;
}

extern "C" int vs_dsm_from_depth_maps(const float *const *depths, const int64_t *heights, const int64_t *widths,
                                      int n_views, const double *inv_projs, const VsGeoPlan *plan, int32_t mode,
                                      double xoff, double yoff, double xresolution, double yresolution, int64_t xsize,
                                      int64_t ysize, float *dsm, int32_t *flags, void *workspace,
                                      size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n_views > 0 && n_views < (1 << 23) && grid_ok(xsize, ysize),
               "vs_dsm_from_depth_maps: bad sizes views=%d grid=%lldx%lld", n_views, (long long)xsize,
               (long long)ysize);
    VS_REQUIRE(depths && heights && widths && inv_projs && plan && dsm && workspace,
               "vs_dsm_from_depth_maps: null pointer");
    VS_REQUIRE(mode == VS_GEO_EXACT || mode == VS_GEO_FAST, "vs_dsm_from_depth_maps: bad mode %d", mode);
    for (int v = 0; v < n_views; ++v)
        VS_REQUIRE(depths[v] && heights[v] > 0 && widths[v] > 0 && heights[v] * widths[v] < (1LL << 39) &&
                       heights[v] < (1 << 24) && widths[v] < (1 << 24),
                   "vs_dsm_from_depth_maps: bad view %d", v);
    const size_t need = vs_dsm_from_depth_maps_workspace_size(xsize, ysize);
    if (workspace_bytes < need) {
        set_error("vs_dsm_from_depth_maps: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    RasterWs w = carve_raster(workspace, xsize, ysize, true);
    Tables tb;
    const long long cells = xsize * ysize;
    int s = make_tables(xoff, yoff, xresolution, yresolution, xsize, ysize, w, tb, st);
    if (s != VS_OK) return s;
    VS_REQUIRE(tb.row.fast && tb.row.contained && tb.col.fast && tb.col.contained && xoff > 0 && yoff > 0,
               "vs_dsm_from_depth_maps: the grid must be positive and inside its origins' binades");
    if ((s = clear(w.keys[0], sizeof(unsigned long long) * cells, st)) != VS_OK) return s;
    if ((s = clear(w.first, sizeof(unsigned long long) * cells, st)) != VS_OK) return s;
    const FastAxis fr = fast_axis_of(tb.row), fc = fast_axis_of(tb.col);
    const GeoFast &gf = geo_plan_fast(plan);
    const GeoFrame *gfr = geo_plan_frame(plan);
    const int south = geo_plan_south(plan);
    const dim3 egrid(static_cast<unsigned>(ceil_div(xsize, TX)), static_cast<unsigned>(ceil_div(ysize, TILE_Y)));
    int *fl = reinterpret_cast<int *>(flags);
    for (int v = 0; v < n_views; ++v) {
        DepthView dv;
        VS_REQUIRE(make_depth_view(inv_projs + 16 * v, dv), "vs_dsm_from_depth_maps: non-finite matrix of view %d", v);
        unsigned long long *cur = w.keys[v & 1], *nxt = (v + 1 < n_views) ? w.keys[(v + 1) & 1] : nullptr;
        const long long total = heights[v] * widths[v];
        const unsigned gx = static_cast<unsigned>(
            std::max<long long>(1, std::min<long long>(ceil_div(ceil_div(total, kDepthPix), 256), sm_count() * 8LL)));
        // rows: a = off - v for the positive origin; columns: a = v - off
        depth_bin_kernel<true, false><<<gx, 256, 0, st>>>(depths[v], heights[v], widths[v], dv, gf, gfr, mode, south,
                                                          fr, fc, v, cur, w.first, fl);
        VS_LAUNCH_CHECK("depth_bin_kernel");
        depth_epilogue_kernel<<<egrid, dim3(TX, TY), 0, st>>>(cur, w.first, dsm + v * cells, nxt,
                                                              static_cast<int>(ysize), static_cast<int>(xsize));
        VS_LAUNCH_CHECK("depth_epilogue_kernel");
    }
    return VS_OK;
}

extern "C" void vs_set_binning_ctas_per_sm(int ctas) { vs::g_bin_ctas_per_sm = ctas > 0 ? ctas : 0; }

extern "C" int vs_set_l2_persisting(size_t bytes) {
    using namespace vs;
    int dev = 0, maxp = 0, maxw = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, dev) != cudaSuccess) {
        set_error("vs_set_l2_persisting: device query failed");
        return VS_ERR_CUDA;
    }
    const size_t want = std::min(bytes, static_cast<size_t>(std::max(maxp, 0)));
    if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) {
        set_error("vs_set_l2_persisting: cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, %zu) failed", want);
        return VS_ERR_CUDA;
    }
    if (want == 0 && cudaCtxResetPersistingL2Cache() != cudaSuccess) {
        set_error("vs_set_l2_persisting: cudaCtxResetPersistingL2Cache failed");
        return VS_ERR_CUDA;
    }
    g_l2_persist = want;
    g_l2_window_max = static_cast<size_t>(std::max(maxw, 0));
    return VS_OK;
}

extern "C" int vs_map_upload(const float *host_heights, int64_t host_row_stride, int width, int height, float *heights,
                             int64_t row_stride, void *stream) {
    VS_REQUIRE(host_heights && heights && width > 0 && height > 0 && host_row_stride >= width && row_stride >= width,
               "vs_map_upload: bad arguments (%dx%d, strides %lld / %lld)", width, height, (long long)host_row_stride,
               (long long)row_stride);
    const size_t f = sizeof(float);
    if (cudaMemcpy2DAsync(heights, static_cast<size_t>(row_stride) * f, host_heights,
                          static_cast<size_t>(host_row_stride) * f, static_cast<size_t>(width) * f,
                          static_cast<size_t>(height), cudaMemcpyHostToDevice, as_stream(stream)) != cudaSuccess) {
        set_error("vs_map_upload: cudaMemcpy2DAsync failed: %s", cudaGetErrorString(cudaGetLastError()));
        return VS_ERR_CUDA;
    }
    return VS_OK;
}

extern "C" int vs_map_points(const float *heights, int64_t row_stride, int width, int height, int64_t e0, int64_t n0,
                             int64_t ej, int64_t ei, int64_t nj, int64_t ni, double *points, void *stream) {
    VS_REQUIRE(heights && points && width > 0 && height > 0 && row_stride >= width,
               "vs_map_points: bad arguments (%dx%d, stride %lld)", width, height, (long long)row_stride);
    const long long total = static_cast<long long>(width) * height;
    // every coordinate integer e0 + ej (2j+1-W) + ei (2i+1-H) must stay below 2^53 (an exact
    // double, and no 64-bit overflow): bound |e0| + |ej| W + |ei| H in FP64 with margin
    auto bound = [&](long long c0, long long cj, long long ci) {
        return std::fabs(static_cast<double>(c0)) + std::fabs(static_cast<double>(cj)) * width +
               std::fabs(static_cast<double>(ci)) * height;
    };
    VS_REQUIRE(bound(e0, ej, ei) < 0x1p52 && bound(n0, nj, ni) < 0x1p52,
               "vs_map_points: affine map out of the exact range");
    const int threads = 256;
    const unsigned g = static_cast<unsigned>(std::min<long long>(ceil_div(total, threads), sm_count() * 16LL));
    map_points_kernel<<<g, threads, 0, as_stream(stream)>>>(heights, row_stride, width, height, e0, n0, ej, ei, nj, ni,
                                                            points);
    VS_LAUNCH_CHECK("map_points_kernel");
    return VS_OK;
}
