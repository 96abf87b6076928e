// (a)+(b) RPC projection and the RPC -> perspective fit:
//   RPCModel.projection        lib/rpc_model.py:160-168
//   solve_perspective          lib/solve_perspective.py:82-126  (+ factorize :38-79)
//   check_perspective_error    lib/check_error.py:37-121
//   the per-view loop          camera_approx.py:166-189
//
// The fit solves the reference's problem -- the unit vector p minimising |A p| for the
// 2N x 12 DLT matrix A -- without forming A.  A^T A only depends on 40 point moments
// (sum X X^T weighted by 1, c, r, c^2 + r^2 with X = [x y z 1]), so one streaming pass
// accumulates them in coordinates centred and scaled per view (FP32 sums over at most 16
// points per thread and across a warp, FP64 beyond).  The 12x12 problem is then solved in
// FP64 by inverse iteration on the normalised Gram matrix, with the centring/scaling map M
// applied exactly, so the minimiser is the reference's un-normalised one.  Factorisation is
// a positive-diagonal RQ (Gram-Schmidt from the last row), which is unique and equals the
// reference's sign-fixed scipy RQ.
//
// GB300 executes FP64 arithmetic, FP64 compares and every conversion instruction on a
// narrow pipe (~1/64 of FP32), so the per-point passes use integer bit manipulation for
// conversions and double-float (two-FP32) arithmetic where FP32 is not accurate enough.
#include <algorithm>
#include <math.h>

#include "common.cuh"
#include "rpc.cuh"

namespace vs {
namespace {

// ---------------------------------------------------------------------------------------
// (a) projection
// ---------------------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(256) rpc_project_kernel(const VsRpcCamera *__restrict__ cams,
                                                          const double *__restrict__ lat,
                                                          const double *__restrict__ lon,
                                                          const double *__restrict__ alt, long long n,
                                                          long long stride, double *__restrict__ col,
                                                          double *__restrict__ row,
                                                          uint8_t *__restrict__ keep) {
    __shared__ VsRpcCamera cam;
    __shared__ RpcFast fast;
    const int c = blockIdx.y;
    {
        const double *src = reinterpret_cast<const double *>(cams + c);
        double *dst = reinterpret_cast<double *>(&cam);
        for (int i = threadIdx.x; i < static_cast<int>(sizeof(VsRpcCamera) / 8); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    if (MODE == VS_PROJ_FAST && threadIdx.x == 0) prepare_fast(cam, fast);
    __syncthreads();
    const double *la = lat + c * stride, *lo = lon + c * stride, *al = alt + c * stride;
    double *oc = col + c * n, *orow = row + c * n;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        double cc, rr;
        bool k;
        if (MODE == VS_PROJ_EXACT) {
            project_exact(cam, __ldcs(la + i), __ldcs(lo + i), __ldcs(al + i), cc, rr);
            k = cc >= 0.0 && rr >= 0.0 && cc < cam.width && rr < cam.height;
        } else {
            df dc, dr;
            project_fast(fast, split_double(__ldcs(la + i)), split_double(__ldcs(lo + i)),
                         split_double(__ldcs(al + i)), dc, dr);
            cc = df_to_double(dc);
            rr = df_to_double(dr);
            k = df_ge0(dc) && df_ge0(dr) && df_lt(dc, fast.width) && df_lt(dr, fast.height);
        }
        __stcs(oc + i, cc);
        __stcs(orow + i, rr);
        if (keep) keep[c * n + i] = k;
    }
}

// ---------------------------------------------------------------------------------------
// (b) fit: normalisation, moments, solve
// ---------------------------------------------------------------------------------------
// Per-view normalisation: X' = (X - centre) / s, c' = (col - c0) / sp, r' = (row - r0) / sp
struct Norm {
    double cx, cy, cz, s, c0, r0, sp;
};

// Points sampled per view for the normalisation box: each sample costs a DRAM sector per
// coordinate array, and 8192 of them bound the data's extent well enough for scaling.
constexpr int kBoxSamples = 8192;

// Min/max of x, y, z (and col, row when given) over a strided sample of the kept points,
// as order-preserving keys (the min through the complemented key).  Any centre and scale
// serve the normalisation; it only has to keep the moments well scaled.
__global__ void bbox_init_kernel(unsigned long long *bb, int n_views) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_views * 10) bb[i] = 0ull;
}

__global__ void __launch_bounds__(256) bbox_kernel(const double *__restrict__ x, const double *__restrict__ y,
                                                   const double *__restrict__ z, long long xyz_stride,
                                                   const double *__restrict__ col, const double *__restrict__ row,
                                                   const uint8_t *__restrict__ keep, long long n, long long step,
                                                   unsigned long long *__restrict__ bb) {
    const int v = blockIdx.y;
    const double *src[5] = {x + v * xyz_stride, y + v * xyz_stride, z + v * xyz_stride, col ? col + v * n : nullptr,
                            row ? row + v * n : nullptr};
    unsigned long long hi[5], lo[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) hi[j] = lo[j] = 0ull;
    for (long long i = (blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x) * step; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x * step) {
        if (keep && !keep[v * n + i]) continue;
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            if (!src[j]) continue;
            const unsigned long long k = key_from_double(src[j][i]);
            hi[j] = max(hi[j], k);
            lo[j] = max(lo[j], ~k);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            hi[j] = max(hi[j], __shfl_xor_sync(0xffffffffu, hi[j], off));
            lo[j] = max(lo[j], __shfl_xor_sync(0xffffffffu, lo[j], off));
        }
    if ((threadIdx.x & 31) == 0) {
        unsigned long long *b = bb + v * 10;
        for (int j = 0; j < 5; ++j) {
            if (hi[j]) atomicMax(b + j, hi[j]);
            if (lo[j]) atomicMax(b + 5 + j, lo[j]);
        }
    }
}

__device__ __forceinline__ double finite_or(double v, double fallback) {
    return (isfinite(v)) ? v : fallback;
}

// Per-view normalisation in the forms the per-point kernels use.
struct NormF {
    df cx, cy, cz, inv_s, c0, r0, inv_sp;
    float sp;
};

__device__ __forceinline__ NormF make_normf(const Norm &nm) {
    NormF f;
    f.cx = df_from_double(nm.cx);
    f.cy = df_from_double(nm.cy);
    f.cz = df_from_double(nm.cz);
    f.inv_s = df_from_double(1.0 / nm.s);
    f.c0 = df_from_double(nm.c0);
    f.r0 = df_from_double(nm.r0);
    f.inv_sp = df_from_double(1.0 / nm.sp);
    f.sp = static_cast<float>(nm.sp);
    return f;
}

// Normalisation from the sampled boxes.  For the fused camera path the pixel frame is the
// RPC's own (colOff/rowOff, larger scale).
__global__ void norm_kernel(const unsigned long long *__restrict__ bb, const VsRpcCamera *__restrict__ cams,
                            int n_views, Norm *__restrict__ norm, NormF *__restrict__ normf) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    const unsigned long long *b = bb + v * 10;
    double mx[5], mn[5];
    for (int j = 0; j < 5; ++j) {
        mx[j] = b[j] ? double_from_key(b[j]) : 0.0;
        mn[j] = b[5 + j] ? double_from_key(~b[5 + j]) : 0.0;
    }
    Norm nm;
    nm.cx = finite_or(0.5 * (mn[0] + mx[0]), 0.0);
    nm.cy = finite_or(0.5 * (mn[1] + mx[1]), 0.0);
    nm.cz = finite_or(0.5 * (mn[2] + mx[2]), 0.0);
    double s = fmax(fmax(mx[0] - mn[0], mx[1] - mn[1]), mx[2] - mn[2]) * 0.5;
    nm.s = (s > 0.0 && isfinite(s)) ? s : 1.0;
    if (cams) {
        nm.c0 = cams[v].col_off;
        nm.r0 = cams[v].row_off;
        nm.sp = fmax(fabs(cams[v].col_scale), fabs(cams[v].row_scale));
        if (!(nm.sp > 0.0) || !isfinite(nm.sp)) nm.sp = 1.0;
    } else {
        nm.c0 = finite_or(0.5 * (mn[3] + mx[3]), 0.0);
        nm.r0 = finite_or(0.5 * (mn[4] + mx[4]), 0.0);
        double sp = fmax(mx[3] - mn[3], mx[4] - mn[4]) * 0.5;
        nm.sp = (sp > 0.0 && isfinite(sp)) ? sp : 1.0;
    }
    norm[v] = nm;
    normf[v] = make_normf(nm);     // once per view: the per-point kernels read it (no FP64 there)
}

constexpr int kMom = 40;            // 4 weights x 10 unique entries of X X^T
constexpr int kSlots = 41;          // + kept-point count
constexpr int kMomThreads = 128;
constexpr int kChunk = 16;          // points per thread (FP32 partial sums)

// Accumulates one point's 40 moment terms into FP32 partial sums held as FP32x2 pairs:
// ma[k] = (m[k], m[10 + k]) with weights (1, c), mb[k] = (m[20 + k], m[30 + k]) with
// weights (r, c^2 + r^2) -- one FFMA2 per pair; 1 * e + m is exactly the plain sum, so
// every lane rounds as the scalar accumulation does.
__device__ __forceinline__ void add_moments(float2 (&ma)[10], float2 (&mb)[10], float x, float y, float z, float c,
                                            float r) {
    const float xx = x * x, xy = x * y, xz = x * z, yy = y * y, yz = y * z, zz = z * z;
    const float e[10] = {xx, xy, xz, x, yy, yz, y, zz, z, 1.0f};
    const float2 wa = make_float2(1.0f, c), wb = make_float2(r, __fmaf_rn(c, c, r * r));
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        const float2 ek = make_float2(e[k], e[k]);
        ma[k] = __ffma2_rn(wa, ek, ma[k]);
        mb[k] = __ffma2_rn(wb, ek, mb[k]);
    }
}

// Warp sums in FP32, warps combined in FP64 in a fixed order (deterministic):
// partial[kSlots] of this block.
__device__ __forceinline__ void store_block_moments(float (&m)[kMom], float count, double *partial, double *red) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // moments 0..31: a reduce-scatter -- at the step of offset h a lane keeps the half of
    // its remaining sums selected by lane bit h and adds its partner's copy of that half --
    // so lane l ends with the warp sum of moment l after 31 shuffles instead of 160.  Each
    // sum is formed as own + partner's at every step, as the butterfly below forms it, so
    // the values are the butterfly's bit for bit.
#pragma unroll
    for (int h = 16; h > 0; h >>= 1) {
        const bool up = (lane & h) != 0;
#pragma unroll
        for (int j = 0; j < h; ++j) {
            const float send = up ? m[j] : m[j + h];
            const float keep = up ? m[j + h] : m[j];
            m[j] = keep + __shfl_xor_sync(0xffffffffu, send, h);
        }
    }
    // moments 32..39 and the count: butterflies (every lane ends with the sum)
#pragma unroll
    for (int k = 32; k < kMom; ++k)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) m[k] += __shfl_xor_sync(0xffffffffu, m[k], off);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) count += __shfl_xor_sync(0xffffffffu, count, off);
    red[warp * kSlots + lane] = f32_to_f64(m[0]);
    if (lane == 0) {
#pragma unroll
        for (int k = 32; k < kMom; ++k) red[warp * kSlots + k] = f32_to_f64(m[k]);
        red[warp * kSlots + kMom] = f32_to_f64(count);
    }
    __syncthreads();
    if (threadIdx.x < kSlots) {
        double s = 0.0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) s += red[w * kSlots + threadIdx.x];
        partial[threadIdx.x] = s;
    }
}

// Normalised coordinates of one kept point from FP64 ENU and double-float pixels (FP32 is
// enough here: the rounding acts like data noise of ~1e-4 px that the fit averages out).
__device__ __forceinline__ void normalised_point(const NormF &nf, long long X, long long Y, long long Z, df c, df r,
                                                 float &px, float &py, float &pz, float &pc, float &pr) {
    const df x = split_double(__longlong_as_double(X)), y = split_double(__longlong_as_double(Y)),
             z = split_double(__longlong_as_double(Z));
    px = ((x.hi - nf.cx.hi) + (x.lo - nf.cx.lo)) * nf.inv_s.hi;
    py = ((y.hi - nf.cy.hi) + (y.lo - nf.cy.lo)) * nf.inv_s.hi;
    pz = ((z.hi - nf.cz.hi) + (z.lo - nf.cz.lo)) * nf.inv_s.hi;
    pc = ((c.hi - nf.c0.hi) + (c.lo - nf.c0.lo)) * nf.inv_sp.hi;
    pr = ((r.hi - nf.r0.hi) + (r.lo - nf.r0.lo)) * nf.inv_sp.hi;
}

// Moments of the kept points of view v.  Block b owns points [b * 128 * kChunk, ...);
// (col, row) come as FP64 arrays (drop-in fit) or as the double-floats of the projection
// pass (fused camera path, in-image mask from the image size).
__global__ void __launch_bounds__(kMomThreads, 6) moments_kernel(
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z, long long xyz_stride,
    const double *__restrict__ col, const double *__restrict__ row, const float4 *__restrict__ colrow,
    const uint8_t *__restrict__ keep, const float *__restrict__ wh, long long n, const NormF *__restrict__ normf,
    double *__restrict__ partial) {
    __shared__ double red[(kMomThreads / 32) * kSlots];
    const int v = blockIdx.y;
    const NormF nf = normf[v];
    const double *xv = x + v * xyz_stride, *yv = y + v * xyz_stride, *zv = z + v * xyz_stride;
    const float w = wh ? wh[2 * v] : 0.f, h = wh ? wh[2 * v + 1] : 0.f;
    float2 ma[10], mb[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) ma[k] = mb[k] = make_float2(0.0f, 0.0f);
    float count = 0.0f;
    const long long base = static_cast<long long>(blockIdx.x) * kMomThreads * kChunk + threadIdx.x;
    // groups of kAhead points: all loads of a group are issued before its arithmetic
    constexpr int kAhead = 2;
#pragma unroll 1
    for (int j0 = 0; j0 < kChunk; j0 += kAhead) {
        // coordinates as raw 64-bit patterns: double-typed registers would be moved and
        // selected by FP64 instructions, which GB300 runs on a narrow pipe
        long long X[kAhead], Y[kAhead], Z[kAhead];
        df c[kAhead], r[kAhead];
        bool ok[kAhead];
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
            const long long i = base + static_cast<long long>(j0 + u) * kMomThreads;
            ok[u] = i < n;
            X[u] = Y[u] = Z[u] = 0;
            c[u] = r[u] = df{0.0f, 0.0f};
            if (ok[u]) {
                X[u] = __ldg(reinterpret_cast<const long long *>(xv) + i);
                Y[u] = __ldg(reinterpret_cast<const long long *>(yv) + i);
                Z[u] = __ldg(reinterpret_cast<const long long *>(zv) + i);
                if (colrow) {
                    const float4 cr = colrow[static_cast<long long>(v) * n + i];
                    c[u] = {cr.x, cr.y};
                    r[u] = {cr.z, cr.w};
                    ok[u] = df_ge0(c[u]) && df_ge0(r[u]) && df_lt(c[u], w) && df_lt(r[u], h);
                } else {
                    ok[u] = !keep || keep[v * n + i];
                    c[u] = split_double(col[v * n + i]);
                    r[u] = split_double(row[v * n + i]);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
            if (!ok[u]) continue;
            float px, py, pz, pc, pr;
            normalised_point(nf, X[u], Y[u], Z[u], c[u], r[u], px, py, pz, pc, pr);
            add_moments(ma, mb, px, py, pz, pc, pr);
            count += 1.0f;
        }
    }
    float m[kMom];
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        m[k] = ma[k].x;
        m[10 + k] = ma[k].y;
        m[20 + k] = mb[k].x;
        m[30 + k] = mb[k].y;
    }
    store_block_moments(m, count, partial + (static_cast<long long>(v) * gridDim.x + blockIdx.x) * kSlots, red);
}

// Double-float form of every view's camera, prepared once per call (one thread per view)
// rather than by the first thread of every projection block.
__global__ void prepare_views_kernel(const VsRpcCamera *__restrict__ cams, int n_views, RpcFast *__restrict__ fast,
                                     float *__restrict__ wh) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    RpcFast f;
    prepare_fast(cams[v], f);
    fast[v] = f;
    wh[2 * v] = f.width;
    wh[2 * v + 1] = f.height;
}

// Projection pass of the fused camera path: (col, row) of every grid point through view
// v's RPC camera as double-floats.
template <int MODE>
__global__ void __launch_bounds__(256) project_view_kernel(const VsRpcCamera *__restrict__ cams,
                                                           const RpcFast *__restrict__ fasts,
                                                           const double *__restrict__ lat,
                                                           const double *__restrict__ lon,
                                                           const double *__restrict__ alt, long long n,
                                                           long long stride, float4 *__restrict__ colrow) {
    __shared__ VsRpcCamera cam;
    __shared__ RpcFast fast;
    const int v = blockIdx.y;
    {
        const unsigned *src = MODE == VS_PROJ_EXACT ? reinterpret_cast<const unsigned *>(cams + v)
                                                    : reinterpret_cast<const unsigned *>(fasts + v);
        unsigned *dst = MODE == VS_PROJ_EXACT ? reinterpret_cast<unsigned *>(&cam) : reinterpret_cast<unsigned *>(&fast);
        const int words = MODE == VS_PROJ_EXACT ? static_cast<int>(sizeof(VsRpcCamera) / 4)
                                                : static_cast<int>(sizeof(RpcFast) / 4);
        for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const long long off = v * stride;
    const long long step = static_cast<long long>(gridDim.x) * blockDim.x;
    // the next point's coordinates (raw 64-bit patterns) are loaded before the current
    // point's few hundred instructions, so their latency is hidden behind them
    const long long *la = reinterpret_cast<const long long *>(lat + off);
    const long long *lo = reinterpret_cast<const long long *>(lon + off);
    const long long *al = reinterpret_cast<const long long *>(alt + off);
    long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    long long a0 = 0, a1 = 0, a2 = 0;
    if (i < n) {
        a0 = __ldcs(la + i);
        a1 = __ldcs(lo + i);
        a2 = __ldcs(al + i);
    }
    for (; i < n; i += step) {
        long long b0 = 0, b1 = 0, b2 = 0;
        if (i + step < n) {
            b0 = __ldcs(la + i + step);
            b1 = __ldcs(lo + i + step);
            b2 = __ldcs(al + i + step);
        }
        df dc, dr;
        if (MODE == VS_PROJ_EXACT) {
            double cc, rr;
            project_exact(cam, __longlong_as_double(a0), __longlong_as_double(a1), __longlong_as_double(a2), cc, rr);
            dc = split_double(cc);
            dr = split_double(rr);
        } else {
            project_fast(fast, split_double(__longlong_as_double(a0)), split_double(__longlong_as_double(a1)),
                         split_double(__longlong_as_double(a2)), dc, dr);
        }
        colrow[static_cast<long long>(v) * n + i] = make_float4(dc.hi, dc.lo, dr.hi, dr.lo);
        a0 = b0;
        a1 = b1;
        a2 = b2;
    }
}

// ---- 12x12 solve (one thread per view; FP64) -------------------------------------------
struct Mmap {     // the exact map between normalised (q) and original (p) camera vectors
    double cx, cy, cz, s, c0, r0, sp;
};

// u = T^-1 w, T = [[s,0,0,cx],[0,s,0,cy],[0,0,s,cz],[0,0,0,1]]
__device__ __forceinline__ void t_inv(const Mmap &m, const double *w, double *u) {
    u[0] = (w[0] - m.cx * w[3]) / m.s;
    u[1] = (w[1] - m.cy * w[3]) / m.s;
    u[2] = (w[2] - m.cz * w[3]) / m.s;
    u[3] = w[3];
}
// u = T^-T w
__device__ __forceinline__ void tt_inv(const Mmap &m, const double *w, double *u) {
    u[0] = w[0] / m.s;
    u[1] = w[1] / m.s;
    u[2] = w[2] / m.s;
    u[3] = w[3] - m.cx * u[0] - m.cy * u[1] - m.cz * u[2];
}
// solve M^T u = v   (q = M p with q1 = T^T(p1 - c0 p3)/sp, q2 = T^T(p2 - r0 p3)/sp, q3 = T^T p3)
__device__ void solve_mt(const Mmap &m, const double *v, double *u) {
    double w[4];
    t_inv(m, v, u);
    t_inv(m, v + 4, u + 4);
    for (int i = 0; i < 8; ++i) u[i] *= m.sp;
    for (int i = 0; i < 4; ++i) w[i] = v[8 + i] + m.c0 * v[i] + m.r0 * v[4 + i];
    t_inv(m, w, u + 8);
}
// solve M u = v
__device__ void solve_m(const Mmap &m, const double *v, double *u) {
    double w[4];
    tt_inv(m, v + 8, u + 8);
    for (int i = 0; i < 4; ++i) w[i] = m.sp * v[i] + m.c0 * v[8 + i];
    tt_inv(m, w, u);
    for (int i = 0; i < 4; ++i) w[i] = m.sp * v[4 + i] + m.r0 * v[8 + i];
    tt_inv(m, w, u + 4);
}

__device__ double det3(const double *a) {
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
}

__device__ __forceinline__ bool isclose(double a, double b) {   // numpy defaults
    return fabs(a - b) <= 1e-8 + 1e-5 * fabs(b);
}

// rotation -> quaternion (w, x, y, z), M. Day's branch-on-trace method applied to R^T
// (the convention of pyquaternion's Quaternion(matrix=R), camera_approx.py:178)
__device__ void quaternion(const double *R, double *q) {
    double m[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m[3 * i + j] = R[3 * j + i];
    double t;
    if (m[8] < 0) {
        if (m[0] > m[4]) {
            t = 1 + m[0] - m[4] - m[8];
            q[0] = m[5] - m[7]; q[1] = t; q[2] = m[1] + m[3]; q[3] = m[6] + m[2];
        } else {
            t = 1 - m[0] + m[4] - m[8];
            q[0] = m[6] - m[2]; q[1] = m[1] + m[3]; q[2] = t; q[3] = m[5] + m[7];
        }
    } else {
        if (m[0] < -m[4]) {
            t = 1 - m[0] - m[4] + m[8];
            q[0] = m[1] - m[3]; q[1] = m[6] + m[2]; q[2] = m[5] + m[7]; q[3] = t;
        } else {
            t = 1 + m[0] + m[4] + m[8];
            q[0] = t; q[1] = m[5] - m[7]; q[2] = m[6] - m[2]; q[3] = m[1] - m[3];
        }
    }
    const double f = 0.5 / sqrt(t);
    for (int i = 0; i < 4; ++i) q[i] *= f;
}

// Positive-diagonal RQ of the left 3x3 block of P by Gram-Schmidt from the last row (with
// one re-orthogonalisation), then the reference's normalisations.  Returns a status.
__device__ int factorize(double *P, double *K, double *R, double *t) {
    const double *a0 = P, *a1 = P + 4, *a2 = P + 8;
    double r0[3], r1[3], r2[3], u[3];
    for (int i = 0; i < 9; ++i) K[i] = 0.0;
    double n2 = sqrt(a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2]);
    if (!(n2 > 0.0) || !isfinite(n2)) return VS_ERR_DEGENERATE;
    for (int i = 0; i < 3; ++i) r2[i] = a2[i] / n2;
    K[8] = n2;
    double k12 = a1[0] * r2[0] + a1[1] * r2[1] + a1[2] * r2[2];
    for (int i = 0; i < 3; ++i) u[i] = a1[i] - k12 * r2[i];
    double d = u[0] * r2[0] + u[1] * r2[1] + u[2] * r2[2];
    for (int i = 0; i < 3; ++i) u[i] -= d * r2[i];
    k12 += d;
    double n1 = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    if (!(n1 > 0.0)) return VS_ERR_DEGENERATE;
    for (int i = 0; i < 3; ++i) r1[i] = u[i] / n1;
    K[4] = n1;
    K[5] = k12;
    double k02 = a0[0] * r2[0] + a0[1] * r2[1] + a0[2] * r2[2];
    double k01 = a0[0] * r1[0] + a0[1] * r1[1] + a0[2] * r1[2];
    for (int i = 0; i < 3; ++i) u[i] = a0[i] - k02 * r2[i] - k01 * r1[i];
    double d2 = u[0] * r2[0] + u[1] * r2[1] + u[2] * r2[2];
    double d1 = u[0] * r1[0] + u[1] * r1[1] + u[2] * r1[2];
    for (int i = 0; i < 3; ++i) u[i] -= d2 * r2[i] + d1 * r1[i];
    k02 += d2;
    k01 += d1;
    double n0 = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    if (!(n0 > 0.0)) return VS_ERR_DEGENERATE;
    for (int i = 0; i < 3; ++i) r0[i] = u[i] / n0;
    K[0] = n0;
    K[1] = k01;
    K[2] = k02;
    for (int i = 0; i < 3; ++i) R[i] = r0[i], R[3 + i] = r1[i], R[6 + i] = r2[i];
    // K /= K[2,2], P /= K[2,2]
    const double sc = K[8];
    for (int i = 0; i < 9; ++i) K[i] /= sc;
    for (int i = 0; i < 12; ++i) P[i] /= sc;
    if (det3(R) < 0.0) {
        for (int i = 0; i < 9; ++i) R[i] = -R[i];
        for (int i = 0; i < 12; ++i) P[i] = -P[i];
    }
    // t = K^-1 P[:, 3] (upper triangular)
    t[2] = P[11] / K[8];
    t[1] = (P[7] - K[5] * t[2]) / K[4];
    t[0] = (P[3] - K[1] * t[1] - K[2] * t[2]) / K[0];
    // the reference's assertions: det R ~ 1 and K [R | t] ~ P
    if (!isclose(det3(R), 1.0)) return VS_ERR_FACTORIZE;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 4; ++j) {
            double kr = 0.0;
            for (int l = 0; l < 3; ++l) kr += K[3 * i + l] * (j < 3 ? R[3 * l + j] : t[l]);
            if (!isclose(P[4 * i + j], kr)) return VS_ERR_FACTORIZE;
        }
    return VS_OK;
}

// What the error pass needs of one view's camera: the camera in the normalised frame
// (q = M p, rescaled) as double-floats, the normalisation, and K^-1.
struct ErrCam {
    df q[12];
    float2 q01_hi[4], q01_lo[4];   // rows 0 and 1 of q paired, for the packed dot products
    NormF nf;
    float qscale;      // q = qscale * M p
    float kinv[9];
    float w, h;
    int ok;
};

__device__ void make_errcam(const double *K, const double *R, const double *t, const Norm &nm, float w, float h,
                            int ok, ErrCam &ec) {
    double P[12];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int l = 0; l < 3; ++l) s += K[3 * i + l] * (j < 3 ? R[3 * l + j] : t[l]);
            P[4 * i + j] = s;
        }
    double u[3][4];
    for (int i = 0; i < 3; ++i) {   // T^T p_i
        const double *p = P + 4 * i;
        u[i][0] = nm.s * p[0];
        u[i][1] = nm.s * p[1];
        u[i][2] = nm.s * p[2];
        u[i][3] = nm.cx * p[0] + nm.cy * p[1] + nm.cz * p[2] + p[3];
    }
    double q[12], mx = 0.0;
    for (int j = 0; j < 4; ++j) {
        q[j] = (u[0][j] - nm.c0 * u[2][j]) / nm.sp;
        q[4 + j] = (u[1][j] - nm.r0 * u[2][j]) / nm.sp;
        q[8 + j] = u[2][j];
    }
    for (int i = 0; i < 12; ++i) mx = fmax(mx, fabs(q[i]));
    const double sc = (mx > 0.0 && isfinite(mx)) ? 1.0 / mx : 1.0;
    for (int i = 0; i < 12; ++i) ec.q[i] = df_from_double(q[i] * sc);
    for (int j = 0; j < 4; ++j) {
        ec.q01_hi[j] = make_float2(ec.q[j].hi, ec.q[4 + j].hi);
        ec.q01_lo[j] = make_float2(ec.q[j].lo, ec.q[4 + j].lo);
    }
    ec.qscale = static_cast<float>(sc);
    ec.nf = make_normf(nm);
    const double a = K[0], b = K[1], c = K[2], d = K[3], e = K[4], f = K[5], g = K[6], hh = K[7], i9 = K[8];
    const double det = a * (e * i9 - f * hh) - b * (d * i9 - f * g) + c * (d * hh - e * g);
    const double ki[9] = {(e * i9 - f * hh) / det, (c * hh - b * i9) / det, (b * f - c * e) / det,
                          (f * g - d * i9) / det,  (a * i9 - c * g) / det,  (c * d - a * f) / det,
                          (d * hh - e * g) / det,  (b * g - a * hh) / det,  (a * e - b * d) / det};
    for (int k = 0; k < 9; ++k) ec.kinv[k] = static_cast<float>(ki[k]);
    ec.w = w;
    ec.h = h;
    ec.ok = ok;
}

// One CTA per view: sum the block partials in a fixed order, solve, factorise.
__global__ void __launch_bounds__(64) solve_kernel(const double *__restrict__ partial, int n_blocks,
                                                   const Norm *__restrict__ norm,
                                                   const VsRpcCamera *__restrict__ cams, double *__restrict__ K_out,
                                                   double *__restrict__ R_out, double *__restrict__ t_out,
                                                   double *__restrict__ params, ErrCam *__restrict__ errcam,
                                                   int32_t *__restrict__ status) {
    __shared__ double mom[kSlots];
    const int v = blockIdx.x;
    if (threadIdx.x < kSlots) {
        double s = 0.0;
        const double *p = partial + static_cast<long long>(v) * n_blocks * kSlots + threadIdx.x;
        for (int b = 0; b < n_blocks; ++b) s += p[b * kSlots];
        mom[threadIdx.x] = s;
    }
    __syncthreads();
    // warp 0 solves; lane 0 keeps the serial parts (maps, factorisation, outputs), the
    // Cholesky factor and the triangular solves run across lanes 0..11 (one row each)
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    __shared__ double G[12][12];
    __shared__ double vec[3][12];          // p, u, w
    __shared__ double s_floor;
    const Norm nm = norm[v];
    const double count = mom[kMom];
    double K[9], R[9], t[3];
    for (int i = 0; i < 9; ++i) K[i] = R[i] = 0.0;
    t[0] = t[1] = t[2] = 0.0;
    int st = VS_OK;
    if (count < 6.0) st = VS_ERR_DEGENERATE;
    double P[12];
    if (st == VS_OK) {
        // normalised Gram matrix G = [[S0,0,-Sc],[0,S0,-Sr],[-Sc,-Sr,Sq]]
        if (lane == 0) {
            const int ent[10][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 3}, {1, 1}, {1, 2}, {1, 3}, {2, 2}, {2, 3}, {3, 3}};
            for (int i = 0; i < 12; ++i)
                for (int j = 0; j < 12; ++j) G[i][j] = 0.0;
            for (int e = 0; e < 10; ++e) {
                const int a = ent[e][0], b = ent[e][1];
                const double s0 = mom[e], sc = mom[10 + e], sr = mom[20 + e], sq = mom[30 + e];
                G[a][b] = G[b][a] = s0;
                G[4 + a][4 + b] = G[4 + b][4 + a] = s0;
                G[a][8 + b] = G[b][8 + a] = G[8 + a][b] = G[8 + b][a] = -sc;
                G[4 + a][8 + b] = G[4 + b][8 + a] = G[8 + a][4 + b] = G[8 + b][4 + a] = -sr;
                G[8 + a][8 + b] = G[8 + b][8 + a] = sq;
            }
            double dmax = 0.0;
            for (int i = 0; i < 12; ++i) dmax = fmax(dmax, G[i][i]);
            s_floor = dmax * 1e-30 + 1e-300;
        }
        __syncwarp();
        // Cholesky G = L L^T, column by column (a non-positive pivot -- an exactly
        // consistent system -- is floored; the inverse iteration then lands on the null
        // vector).  Every element keeps the serial operation order.
        const double floor_piv = s_floor;
        for (int j = 0; j < 12; ++j) {
            if (lane == j) {
                double d = G[j][j];
                for (int k = 0; k < j; ++k) d -= G[j][k] * G[j][k];
                d = d > floor_piv ? d : floor_piv;
                G[j][j] = sqrt(d);
            }
            __syncwarp();
            if (lane > j && lane < 12) {
                double sum = G[lane][j];
                for (int k = 0; k < j; ++k) sum -= G[lane][k] * G[j][k];
                G[lane][j] = sum / G[j][j];
            }
            __syncwarp();
        }
        const Mmap mm{nm.cx, nm.cy, nm.cz, nm.s, nm.c0, nm.r0, nm.sp};
        if (lane < 12) vec[0][lane] = 0.28867513459481287;   // 1/sqrt(12)
        __syncwarp();
        for (int it = 0; it < 6; ++it) {
            if (lane == 0) solve_mt(mm, vec[0], vec[1]);
            __syncwarp();
            // L w = u: lane i subtracts w[j] L[i][j] as each w[j] is formed
            double sum = lane < 12 ? vec[1][lane] : 0.0;
            for (int j = 0; j < 12; ++j) {
                if (lane == j) vec[2][j] = sum / G[j][j];
                __syncwarp();
                if (lane > j && lane < 12) sum -= G[lane][j] * vec[2][j];
            }
            __syncwarp();
            // L^T u = w
            sum = lane < 12 ? vec[2][lane] : 0.0;
            for (int j = 11; j >= 0; --j) {
                if (lane == j) vec[1][j] = sum / G[j][j];
                __syncwarp();
                if (lane < j) sum -= G[j][lane] * vec[1][j];
            }
            __syncwarp();
            if (lane == 0) {
                double pp[12];
                solve_m(mm, vec[1], pp);
                double nrm = 0.0;
                for (int i = 0; i < 12; ++i) nrm += pp[i] * pp[i];
                nrm = 1.0 / sqrt(nrm);
                for (int i = 0; i < 12; ++i) vec[0][i] = pp[i] * nrm;
            }
            __syncwarp();
        }
        if (lane != 0) return;
        double p[12];
        for (int i = 0; i < 12; ++i) p[i] = vec[0][i];
        for (int i = 0; i < 12; ++i) P[i] = p[i];
        bool finite = true;
        for (int i = 0; i < 12; ++i) finite &= isfinite(P[i]);
        st = finite ? factorize(P, K, R, t) : VS_ERR_DEGENERATE;
    }
    if (lane != 0) return;
    for (int i = 0; i < 9; ++i) K_out[v * 9 + i] = K[i], R_out[v * 9 + i] = R[i];
    for (int i = 0; i < 3; ++i) t_out[v * 3 + i] = t[i];
    status[v] = st;
    if (errcam)
        make_errcam(K, R, t, nm, cams ? static_cast<float>(cams[v].width) : 0.f,
                    cams ? static_cast<float>(cams[v].height) : 0.f, st == VS_OK, errcam[v]);
    if (params) {
        double q[4] = {0, 0, 0, 0};
        if (st == VS_OK) quaternion(R, q);
        double *o = params + v * VS_CAMERA_PARAMS;
        o[0] = cams ? cams[v].width : 0.0;
        o[1] = cams ? cams[v].height : 0.0;
        o[2] = K[0]; o[3] = K[4]; o[4] = K[2]; o[5] = K[5]; o[6] = K[1];
        o[7] = q[0]; o[8] = q[1]; o[9] = q[2]; o[10] = q[3];
        o[11] = t[0]; o[12] = t[1]; o[13] = t[2];
    }
}

// ---------------------------------------------------------------------------------------
// error statistics (check_perspective_error)
// ---------------------------------------------------------------------------------------
// ErrCam for given K, R, t (the drop-in statistics entry)
__global__ void errcam_kernel(const double *K, const double *R, const double *t, const Norm *norm, int n_views,
                              ErrCam *ec) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    make_errcam(K + 9 * v, R + 9 * v, t + 3 * v, norm[v], 0.f, 0.f, 1, ec[v]);
}

// Radix selection over the float bits of the per-point errors (non-negative floats, so
// the bits order like the values), 11 + 11 + 10 bits.  Targets per view: 0/1 = the
// low/high middle order statistic of the pixel errors, 2/3 = of the metric errors.
__host__ __device__ constexpr int digit_bits(int pass) { return pass == 2 ? 10 : 11; }
__host__ __device__ constexpr int digit_shift(int pass) { return pass == 0 ? 21 : (pass == 1 ? 10 : 0); }
constexpr int kBins = 2048;

struct ErrWs {
    unsigned *keys;          // [2][V][n] float bits of the per-point errors (kept points only)
    double *sums;            // [V][blocks][3]: pixel sum, metric sum, count
    unsigned *maxk;          // [V][2]
    unsigned *hist;          // [V][2][kBins] histogram of the current digit (pixel, metric)
    unsigned *sel;           // [V][4][3]: prefix, mask, rank
    double *cnt;             // [V]
};

constexpr int kErrThreads = 256;

// compensated dot product of a double-float 4-vector with (x, y, z, 1), FP32 exact inputs
__device__ __forceinline__ df dot2(const df *q, float x, float y, float z) {
    df p0 = two_prod(q[0].hi, x), p1 = two_prod(q[1].hi, y), p2 = two_prod(q[2].hi, z);
    float err = __fmaf_rn(q[0].lo, x, p0.lo) + __fmaf_rn(q[1].lo, y, p1.lo) + __fmaf_rn(q[2].lo, z, p2.lo) + q[3].lo;
    df s = two_sum(p0.hi, p1.hi);
    err += s.lo;
    s = two_sum(s.hi, p2.hi);
    err += s.lo;
    s = two_sum(s.hi, q[3].hi);
    err += s.lo;
    return fast_two_sum(s.hi, err);
}

// dot2 for rows 0 and 1 of q at once (FP32x2 lanes; each lane performs dot2's operations)
__device__ __forceinline__ df2 dot2_rows01(const ErrCam &ec, float x, float y, float z) {
    const float2 X = f2s(x), Y = f2s(y), Z = f2s(z), nX = f2s(-x), nY = f2s(-y), nZ = f2s(-z);
    const float2 h0 = ec.q01_hi[0], h1 = ec.q01_hi[1], h2 = ec.q01_hi[2];
    const df2 p0 = {__fmul2_rn(h0, X), __ffma2_rn(h0, X, __fmul2_rn(h0, nX))};
    const df2 p1 = {__fmul2_rn(h1, Y), __ffma2_rn(h1, Y, __fmul2_rn(h1, nY))};
    const df2 p2 = {__fmul2_rn(h2, Z), __ffma2_rn(h2, Z, __fmul2_rn(h2, nZ))};
    float2 err = __fadd2_rn(__fadd2_rn(__fadd2_rn(__ffma2_rn(ec.q01_lo[0], X, p0.lo), __ffma2_rn(ec.q01_lo[1], Y, p1.lo)),
                                       __ffma2_rn(ec.q01_lo[2], Z, p2.lo)),
                            ec.q01_lo[3]);
    df2 s = two_sum2(p0.hi, p1.hi);
    err = __fadd2_rn(err, s.lo);
    s = two_sum2(s.hi, p2.hi);
    err = __fadd2_rn(err, s.lo);
    s = two_sum2(s.hi, ec.q01_hi[3]);
    err = __fadd2_rn(err, s.lo);
    return fast_two_sum2(s.hi, err);
}

// Per kept point: pixel reprojection error and metric inverse-projection error, written
// as float bits for the median selection, plus block sums/maxima and the histogram of
// the leading digit.
//  * reprojection: in the fit's normalised frame, with the ENU point rounded to FP32
//    (|error| <~ 1e-4 px): h = q.X' by compensated dot products, residual
//    (h0 - c' h2) / h2 with c' the double-float normalised observation;
//  * inverse projection: the reference's |scale*ray - cam| is the distance from the
//    camera-frame point to the ray d = K^-1 [c r 1].  The point lies on the ray through
//    its own projection, cam = h2 K^-1 [c^ r^ 1], so the distance is
//    |h2| |delta x d| / |d| with delta = K^-1 [c^ - c, r^ - r, 0]: the pixel residual
//    enters directly and nothing of the camera's ~1e5-1e6 m depth cancels.
__global__ void __launch_bounds__(kErrThreads, 4) error_points_kernel(
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z, long long xyz_stride,
    const double *__restrict__ col, const double *__restrict__ row, const float4 *__restrict__ colrow,
    const uint8_t *__restrict__ keep, long long n, const ErrCam *__restrict__ cams, ErrWs w) {
    __shared__ ErrCam ec;
    __shared__ double red[3][kErrThreads / 32];
    __shared__ unsigned hist[2][kBins];
    const int v = blockIdx.y;
    const int V = gridDim.y;
    if (threadIdx.x == 0) ec = cams[v];
    for (int i = threadIdx.x; i < 2 * kBins; i += blockDim.x) (&hist[0][0])[i] = 0;
    __syncthreads();
    float ps = 0.0f, is = 0.0f, cnt = 0.0f;
    unsigned pmax = 0, imax = 0;
    const double *xv = x + v * xyz_stride, *yv = y + v * xyz_stride, *zv = z + v * xyz_stride;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        // the point's coordinates are requested with its pixels, not after the in-image
        // test on them: one memory round trip per point instead of two
        const long long RX = __ldg(reinterpret_cast<const long long *>(xv) + i);
        const long long RY = __ldg(reinterpret_cast<const long long *>(yv) + i);
        const long long RZ = __ldg(reinterpret_cast<const long long *>(zv) + i);
        df c, r;
        bool k;
        if (colrow) {
            const float4 cr = colrow[static_cast<long long>(v) * n + i];
            c = {cr.x, cr.y};
            r = {cr.z, cr.w};
            k = df_ge0(c) && df_ge0(r) && df_lt(c, ec.w) && df_lt(r, ec.h);
        } else {
            c = split_double(col[v * n + i]);
            r = split_double(row[v * n + i]);
            k = keep ? keep[v * n + i] != 0 : true;
        }
        unsigned pk = 0xffffffffu, ik = 0xffffffffu;
        if (k && ec.ok) {
            float X, Y, Z, cf_, rf_;
            normalised_point(ec.nf, RX, RY, RZ, c, r, X, Y, Z, cf_, rf_);
            // rows 0 and 1 of the camera (h0, h1) and the observations (c, r) travel as FP32x2
            // pairs; every lane performs the scalar double-float operations
            const df2 h01 = dot2_rows01(ec, X, Y, Z);
            const df h2 = dot2(ec.q + 8, X, Y, Z);
            // observation in the normalised frame as a double-float: (c - c0) / sp
            const df2 crn = df_mul2(df_add2({f2(c.hi, r.hi), f2(c.lo, r.lo)},
                                            {f2(-ec.nf.c0.hi, -ec.nf.r0.hi), f2(-ec.nf.c0.lo, -ec.nf.r0.lo)}),
                                    {f2s(ec.nf.inv_sp.hi), f2s(ec.nf.inv_sp.lo)}, f2s(-ec.nf.inv_sp.hi));
            const df2 ncr = df_add2(h01, df_mul2({sub2(f2s(0.0f), crn.hi), sub2(f2s(0.0f), crn.lo)},
                                                 {f2s(h2.hi), f2s(h2.lo)}, f2s(-h2.hi)));
            const float h2f = h2.hi + h2.lo;
            const float2 nsum = __fadd2_rn(ncr.hi, ncr.lo);
            const float dc = ec.nf.sp * (nsum.x / h2f), dr = ec.nf.sp * (nsum.y / h2f);
            const float pe = sqrtf(__fmaf_rn(dr, dr, dc * dc));
            const float *ki = ec.kinv;
            const float cf = c.hi, rf = r.hi;
            const float d0 = __fmaf_rn(ki[0], cf, __fmaf_rn(ki[1], rf, ki[2]));
            const float d1 = __fmaf_rn(ki[3], cf, __fmaf_rn(ki[4], rf, ki[5]));
            const float d2 = __fmaf_rn(ki[6], cf, __fmaf_rn(ki[7], rf, ki[8]));
            const float e0 = __fmaf_rn(ki[0], dc, ki[1] * dr);
            const float e1 = __fmaf_rn(ki[3], dc, ki[4] * dr);
            const float e2 = __fmaf_rn(ki[6], dc, ki[7] * dr);
            const float x0 = e1 * d2 - e2 * d1, x1 = e2 * d0 - e0 * d2, x2 = e0 * d1 - e1 * d0;
            const float hz = fabsf(h2f / ec.qscale);
            const float ie = hz * sqrtf((x0 * x0 + x1 * x1 + x2 * x2) / (d0 * d0 + d1 * d1 + d2 * d2));
            ps += pe;
            is += ie;
            cnt += 1.0f;
            pk = __float_as_uint(pe);
            ik = __float_as_uint(ie);
            pmax = max(pmax, pk);
            imax = max(imax, ik);
            atomicAdd(&hist[0][pk >> digit_shift(0)], 1u);
            atomicAdd(&hist[1][ik >> digit_shift(0)], 1u);
        }
        w.keys[static_cast<long long>(v) * n + i] = pk;
        w.keys[(static_cast<long long>(V) + v) * n + i] = ik;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ps += __shfl_xor_sync(0xffffffffu, ps, off);
        is += __shfl_xor_sync(0xffffffffu, is, off);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
        pmax = max(pmax, __shfl_xor_sync(0xffffffffu, pmax, off));
        imax = max(imax, __shfl_xor_sync(0xffffffffu, imax, off));
    }
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][warp] = f32_to_f64(ps);
        red[1][warp] = f32_to_f64(is);
        red[2][warp] = f32_to_f64(cnt);
        if (pmax) atomicMax(w.maxk + 2 * v, pmax);
        if (imax) atomicMax(w.maxk + 2 * v + 1, imax);
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int i = 0; i < kErrThreads / 32; ++i) s += red[threadIdx.x][i];
        w.sums[(static_cast<long long>(v) * gridDim.x + blockIdx.x) * 3 + threadIdx.x] = s;
    }
    for (int i = threadIdx.x; i < 2 * kBins; i += blockDim.x) {
        const unsigned c = (&hist[0][0])[i];
        if (c) atomicAdd(w.hist + static_cast<long long>(v) * 2 * kBins + i, c);
    }
}

// per-view totals of the block sums (fixed order) and the selection ranks
__global__ void error_count_kernel(ErrWs w, int n_views, int n_blocks) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    double c = 0.0;
    for (int b = 0; b < n_blocks; ++b) c += w.sums[(static_cast<long long>(v) * n_blocks + b) * 3 + 2];
    w.cnt[v] = c;
    const unsigned long long n = static_cast<unsigned long long>(c);
    for (int t = 0; t < 4; ++t) {
        const int i = v * 4 + t;
        w.sel[3 * i] = 0;       // prefix
        w.sel[3 * i + 1] = 0;   // mask
        w.sel[3 * i + 2] = n ? static_cast<unsigned>((t & 1) ? n / 2 : (n - 1) / 2) : 0u;
    }
}

// Histograms of digit `pass` (1, 2) of the keys matching each target's prefix.
__global__ void __launch_bounds__(256) select_hist_kernel(ErrWs w, long long n, int pass) {
    __shared__ unsigned h[4][kBins];
    const int v = blockIdx.y, V = gridDim.y;
    const int shift = digit_shift(pass);
    const unsigned dmask = (1u << digit_bits(pass)) - 1u;
    for (int i = threadIdx.x; i < 4 * kBins; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    unsigned pre[4], msk[4];
    for (int t = 0; t < 4; ++t) pre[t] = w.sel[3 * (v * 4 + t)], msk[t] = w.sel[3 * (v * 4 + t) + 1];
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const unsigned kp = w.keys[static_cast<long long>(v) * n + i];
        const unsigned kq = w.keys[(static_cast<long long>(V) + v) * n + i];
        const unsigned dp = (kp >> shift) & dmask, dq = (kq >> shift) & dmask;
        if ((kp & msk[0]) == pre[0]) atomicAdd(&h[0][dp], 1u);
        if ((kp & msk[1]) == pre[1] && pre[1] != pre[0]) atomicAdd(&h[1][dp], 1u);
        if ((kq & msk[2]) == pre[2]) atomicAdd(&h[2][dq], 1u);
        if ((kq & msk[3]) == pre[3] && pre[3] != pre[2]) atomicAdd(&h[3][dq], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * kBins; i += blockDim.x) {
        const unsigned c = (&h[0][0])[i];
        if (c) atomicAdd(w.hist + static_cast<long long>(v) * 4 * kBins + i, c);
    }
}

// Picks the digit of the four targets of one view: one block per view, one warp per
// target, the bins scanned 32 at a time with warp prefix sums.  Every prefix is read
// before the barrier and written after it.  Pass 0 reads the two histograms the error
// kernel built (pixel, metric); later passes read one histogram per target, except that
// the high target shares its low partner's histogram while their prefixes agree.
__global__ void __launch_bounds__(128) select_step_kernel(ErrWs w, int pass) {
    const int v = blockIdx.x;
    const int t = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = v * 4 + t;
    __shared__ unsigned pre[4];
    if (lane == 0) pre[t] = w.sel[3 * i];
    __syncthreads();
    const unsigned *hist;
    if (pass == 0) {
        hist = w.hist + static_cast<long long>(v) * 2 * kBins + (t >> 1) * kBins;
    } else {
        const bool shared_h = (t & 1) && pre[t] == pre[t ^ 1];
        hist = w.hist + static_cast<long long>(v) * 4 * kBins + (shared_h ? (t ^ 1) : t) * kBins;
    }
    const int bins = 1 << digit_bits(pass);
    const unsigned k = w.sel[3 * i + 2];
    unsigned below = 0;          // count of keys in earlier chunks
    int digit = -1;
    unsigned skip = 0;
    for (int base = 0; base < bins; base += 32) {
        const unsigned c = hist[base + lane];
        unsigned incl = c;       // inclusive warp scan
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += u;
        }
        const unsigned excl = incl - c;
        const unsigned hit = __ballot_sync(0xffffffffu, below + incl > k);
        if (hit) {
            const int l = __ffs(hit) - 1;
            digit = base + l;
            skip = below + __shfl_sync(0xffffffffu, excl, l);
            break;
        }
        below += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (digit < 0) {             // rank beyond the counts (no kept points): the last bin
        digit = bins - 1;
        skip = below - hist[bins - 1];
    }
    __syncthreads();
    if (lane == 0) {
        w.sel[3 * i] = pre[t] | (static_cast<unsigned>(digit) << digit_shift(pass));
        w.sel[3 * i + 1] |= static_cast<unsigned>(bins - 1) << digit_shift(pass);
        w.sel[3 * i + 2] = k - skip;
    }
}

__global__ void error_final_kernel(ErrWs w, int n_views, int n_blocks, double *err) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    const double cnt = w.cnt[v];
    double s[2] = {0.0, 0.0};
    for (int b = 0; b < n_blocks; ++b) {
        s[0] += w.sums[(static_cast<long long>(v) * n_blocks + b) * 3];
        s[1] += w.sums[(static_cast<long long>(v) * n_blocks + b) * 3 + 1];
    }
    double *o = err + v * VS_ERROR_STATS;
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    for (int q = 0; q < 2; ++q) {
        const double lo = __uint_as_float(w.sel[3 * (v * 4 + 2 * q)]);
        const double hi = __uint_as_float(w.sel[3 * (v * 4 + 2 * q + 1)]);
        o[3 * q] = cnt > 0 ? s[q] / cnt : nan;
        o[3 * q + 1] = cnt > 0 ? ((0.0 + lo) + hi) / 2.0 : nan;
        o[3 * q + 2] = cnt > 0 ? static_cast<double>(__uint_as_float(w.maxk[2 * v + q])) : nan;
    }
}

int err_blocks(long long n) {
    long long want = ceil_div(n, kErrThreads * 4);
    return static_cast<int>(std::max<long long>(1, std::min<long long>(want, sm_count() * 2LL)));
}

ErrWs carve_err(Carver &cv, int V, long long n, int blocks) {
    ErrWs w;
    w.keys = cv.take<unsigned>(2 * static_cast<size_t>(V) * n);
    w.sums = cv.take<double>(static_cast<size_t>(V) * blocks * 3);
    w.maxk = cv.take<unsigned>(2 * V);
    w.hist = cv.take<unsigned>(static_cast<size_t>(V) * 4 * kBins);
    w.sel = cv.take<unsigned>(static_cast<size_t>(V) * 12);
    w.cnt = cv.take<double>(V);
    return w;
}

int run_error_stats(const double *x, const double *y, const double *z, long long xyz_stride, const double *col,
                    const double *row, const float4 *colrow, const uint8_t *keep, int V, long long n,
                    const ErrCam *cams, double *err, ErrWs &w, cudaStream_t st) {
    const int blocks = err_blocks(n);
    const size_t hist_bytes = sizeof(unsigned) * 4 * kBins * V;
    if (cudaMemsetAsync(w.maxk, 0, sizeof(unsigned) * 2 * V, st) != cudaSuccess ||
        cudaMemsetAsync(w.hist, 0, hist_bytes, st) != cudaSuccess) {
        set_error("cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
    if (n > 0) {
        error_points_kernel<<<dim3(blocks, V), kErrThreads, 0, st>>>(x, y, z, xyz_stride, col, row, colrow, keep, n,
                                                                      cams, w);
        VS_LAUNCH_CHECK("error_points_kernel");
    } else if (cudaMemsetAsync(w.sums, 0, sizeof(double) * V * blocks * 3, st) != cudaSuccess) {
        set_error("cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
    const unsigned vg = static_cast<unsigned>(ceil_div(V, 128));
    error_count_kernel<<<vg, 128, 0, st>>>(w, V, blocks);
    VS_LAUNCH_CHECK("error_count_kernel");
    for (int pass = 0; pass < 3 && n > 0; ++pass) {
        if (pass > 0) {
            if (cudaMemsetAsync(w.hist, 0, hist_bytes, st) != cudaSuccess) {
                set_error("cudaMemsetAsync failed");
                return VS_ERR_CUDA;
            }
            select_hist_kernel<<<dim3(blocks, V), 256, 0, st>>>(w, n, pass);
            VS_LAUNCH_CHECK("select_hist_kernel");
        }
        select_step_kernel<<<V, 128, 0, st>>>(w, pass);
        VS_LAUNCH_CHECK("select_step_kernel");
    }
    error_final_kernel<<<vg, 128, 0, st>>>(w, V, blocks, err);
    VS_LAUNCH_CHECK("error_final_kernel");
    return VS_OK;
}

int mom_blocks(long long n) {
    return static_cast<int>(std::max<long long>(1, ceil_div(n, static_cast<long long>(kMomThreads) * kChunk)));
}

long long box_step(long long n) { return std::max<long long>(1, n / kBoxSamples); }

int box_blocks(long long n) {
    long long samples = ceil_div(n, box_step(n));
    return static_cast<int>(std::max<long long>(1, std::min<long long>(ceil_div(samples, 256), 64)));
}

struct FitWs {
    unsigned long long *bb;
    Norm *norm;
    NormF *normf;
    double *partial;
    ErrCam *errcam;
    float4 *colrow;
    float *wh;
    RpcFast *fast;
};

FitWs carve_fit(Carver &cv, int V, long long n, bool fused) {
    FitWs f;
    f.bb = cv.take<unsigned long long>(static_cast<size_t>(V) * 10);
    f.norm = cv.take<Norm>(V);
    f.normf = cv.take<NormF>(V);
    f.partial = cv.take<double>(static_cast<size_t>(V) * mom_blocks(n) * kSlots);
    f.errcam = cv.take<ErrCam>(V);
    f.colrow = fused ? cv.take<float4>(static_cast<size_t>(V) * n) : nullptr;
    f.wh = cv.take<float>(2 * static_cast<size_t>(V));
    f.fast = fused ? cv.take<RpcFast>(V) : nullptr;
    return f;
}

int launch_norm(const double *x, const double *y, const double *z, long long xyz_stride, const double *col,
                const double *row, const uint8_t *keep, const VsRpcCamera *cams, int V, long long n, FitWs &f,
                cudaStream_t st) {
    bbox_init_kernel<<<static_cast<unsigned>(ceil_div(V * 10, 128)), 128, 0, st>>>(f.bb, V);
    VS_LAUNCH_CHECK("bbox_init_kernel");
    if (n > 0) {
        bbox_kernel<<<dim3(box_blocks(n), V), 256, 0, st>>>(x, y, z, xyz_stride, col, row, keep, n, box_step(n), f.bb);
        VS_LAUNCH_CHECK("bbox_kernel");
    }
    norm_kernel<<<static_cast<unsigned>(ceil_div(V, 64)), 64, 0, st>>>(f.bb, cams, V, f.norm, f.normf);
    VS_LAUNCH_CHECK("norm_kernel");
    return VS_OK;
}

}  // namespace
}  // namespace vs

using namespace vs;

extern "C" int vs_rpc_project(const VsRpcCamera *cams, int n_cams, const double *lat, const double *lon,
                              const double *alt, int64_t n, int64_t point_stride, double *col, double *row,
                              uint8_t *keep, int mode, void *stream) {
    VS_REQUIRE(n_cams > 0 && n_cams <= 65535 && n >= 0 && point_stride >= 0, "vs_rpc_project: bad sizes");
    VS_REQUIRE(mode == VS_PROJ_EXACT || mode == VS_PROJ_FAST, "vs_rpc_project: bad mode %d", mode);
    if (n == 0) return VS_OK;
    VS_REQUIRE(cams && lat && lon && alt && col && row, "vs_rpc_project: null pointer");
    const int threads = 256;
    long long want = ceil_div(n, threads);
    unsigned gx = static_cast<unsigned>(std::min<long long>(want, std::max(1LL, sm_count() * 8LL / n_cams + 1)));
    dim3 grid(gx, n_cams);
    cudaStream_t st = as_stream(stream);
    if (mode == VS_PROJ_EXACT)
        rpc_project_kernel<VS_PROJ_EXACT><<<grid, threads, 0, st>>>(cams, lat, lon, alt, n, point_stride, col, row, keep);
    else
        rpc_project_kernel<VS_PROJ_FAST><<<grid, threads, 0, st>>>(cams, lat, lon, alt, n, point_stride, col, row, keep);
    VS_LAUNCH_CHECK("rpc_project_kernel");
    return VS_OK;
}

extern "C" size_t vs_dlt_fit_workspace_size(int n_views, int64_t n) {
    if (n_views <= 0 || n < 0) return 0;
    Carver cv(nullptr);
    carve_fit(cv, n_views, n, false);
    return cv.used + 256;
}

extern "C" int vs_dlt_fit(const double *x, const double *y, const double *z, int64_t xyz_stride, const double *col,
                          const double *row, const uint8_t *keep, int n_views, int64_t n, double *K, double *R,
                          double *t, int32_t *status, void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n_views > 0 && n_views <= 65535 && n >= 0 && xyz_stride >= 0, "vs_dlt_fit: bad sizes");
    VS_REQUIRE(x && y && z && col && row && K && R && t && status && workspace, "vs_dlt_fit: null pointer");
    const size_t need = vs_dlt_fit_workspace_size(n_views, n);
    if (workspace_bytes < need) {
        set_error("vs_dlt_fit: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace);
    FitWs f = carve_fit(cv, n_views, n, false);
    int s = launch_norm(x, y, z, xyz_stride, col, row, keep, nullptr, n_views, n, f, st);
    if (s != VS_OK) return s;
    const int blocks = mom_blocks(n);
    moments_kernel<<<dim3(blocks, n_views), kMomThreads, 0, st>>>(x, y, z, xyz_stride, col, row, nullptr, keep,
                                                                   nullptr, n, f.normf, f.partial);
    VS_LAUNCH_CHECK("moments_kernel");
    solve_kernel<<<n_views, 64, 0, st>>>(f.partial, blocks, f.norm, nullptr, K, R, t, nullptr, nullptr, status);
    VS_LAUNCH_CHECK("solve_kernel");
    return VS_OK;
}

extern "C" size_t vs_perspective_error_workspace_size(int n_views, int64_t n) {
    if (n_views <= 0 || n < 0) return 0;
    Carver cv(nullptr);
    carve_fit(cv, n_views, 0, false);
    carve_err(cv, n_views, n, err_blocks(n));
    return cv.used + 256;
}

extern "C" int vs_perspective_error(const double *x, const double *y, const double *z, int64_t xyz_stride,
                                    const double *col, const double *row, const uint8_t *keep, int n_views,
                                    int64_t n, const double *K, const double *R, const double *t, double *err,
                                    void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n_views > 0 && n_views <= 65535 && n >= 0 && xyz_stride >= 0, "vs_perspective_error: bad sizes");
    VS_REQUIRE(x && y && z && col && row && K && R && t && err && workspace, "vs_perspective_error: null pointer");
    const size_t need = vs_perspective_error_workspace_size(n_views, n);
    if (workspace_bytes < need) {
        set_error("vs_perspective_error: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace);
    FitWs f = carve_fit(cv, n_views, 0, false);
    ErrWs w = carve_err(cv, n_views, n, err_blocks(n));
    int s = launch_norm(x, y, z, xyz_stride, col, row, keep, nullptr, n_views, n, f, st);
    if (s != VS_OK) return s;
    errcam_kernel<<<static_cast<unsigned>(ceil_div(n_views, 64)), 64, 0, st>>>(K, R, t, f.norm, n_views, f.errcam);
    VS_LAUNCH_CHECK("errcam_kernel");
    return run_error_stats(x, y, z, xyz_stride, col, row, nullptr, keep, n_views, n, f.errcam, err, w, st);
}

extern "C" size_t vs_camera_approx_workspace_size(int n_views, int64_t n) {
    if (n_views <= 0 || n < 0) return 0;
    Carver cv(nullptr);
    carve_fit(cv, n_views, n, true);
    cv.take<double>(static_cast<size_t>(n_views) * 9);    // K
    cv.take<double>(static_cast<size_t>(n_views) * 9);    // R
    cv.take<double>(static_cast<size_t>(n_views) * 3);    // t
    carve_err(cv, n_views, n, err_blocks(n));
    return cv.used + 256;
}

extern "C" int vs_camera_approx_perspective(const VsRpcCamera *cams, int n_views, const double *lat,
                                            const double *lon, const double *alt, const double *x, const double *y,
                                            const double *z, int64_t n, int64_t point_stride, int proj_mode,
                                            double *params, double *err, int32_t *status, void *workspace,
                                            size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n_views > 0 && n_views <= 65535 && n >= 0 && point_stride >= 0,
               "vs_camera_approx_perspective: bad sizes");
    VS_REQUIRE(proj_mode == VS_PROJ_EXACT || proj_mode == VS_PROJ_FAST, "vs_camera_approx_perspective: bad mode");
    VS_REQUIRE(cams && lat && lon && alt && x && y && z && params && status && workspace,
               "vs_camera_approx_perspective: null pointer");
    const size_t need = vs_camera_approx_workspace_size(n_views, n);
    if (workspace_bytes < need) {
        set_error("vs_camera_approx_perspective: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace);
    FitWs f = carve_fit(cv, n_views, n, true);
    double *K = cv.take<double>(static_cast<size_t>(n_views) * 9);
    double *R = cv.take<double>(static_cast<size_t>(n_views) * 9);
    double *t = cv.take<double>(static_cast<size_t>(n_views) * 3);
    ErrWs ew = carve_err(cv, n_views, n, err_blocks(n));
    // ENU box (sampled) -> normalisation; pixel frame from each RPC
    int s = launch_norm(x, y, z, point_stride, nullptr, nullptr, nullptr, cams, n_views, n, f, st);
    if (s != VS_OK) return s;
    const int blocks = mom_blocks(n);
    prepare_views_kernel<<<static_cast<unsigned>(ceil_div(n_views, 64)), 64, 0, st>>>(cams, n_views, f.fast, f.wh);
    VS_LAUNCH_CHECK("prepare_views_kernel");
    if (n > 0) {
        const unsigned pg = static_cast<unsigned>(std::min<long long>(ceil_div(n, 256), sm_count() * 8LL / n_views + 8));
        if (proj_mode == VS_PROJ_EXACT)
            project_view_kernel<VS_PROJ_EXACT><<<dim3(pg, n_views), 256, 0, st>>>(cams, f.fast, lat, lon, alt, n,
                                                                                  point_stride, f.colrow);
        else
            project_view_kernel<VS_PROJ_FAST><<<dim3(pg, n_views), 256, 0, st>>>(cams, f.fast, lat, lon, alt, n,
                                                                                 point_stride, f.colrow);
        VS_LAUNCH_CHECK("project_view_kernel");
    }
    moments_kernel<<<dim3(blocks, n_views), kMomThreads, 0, st>>>(x, y, z, point_stride, nullptr, nullptr, f.colrow,
                                                                   nullptr, f.wh, n, f.normf, f.partial);
    VS_LAUNCH_CHECK("moments_kernel");
    solve_kernel<<<n_views, 64, 0, st>>>(f.partial, blocks, f.norm, cams, K, R, t, params, f.errcam, status);
    VS_LAUNCH_CHECK("solve_kernel");
    if (!err) return VS_OK;
    return run_error_stats(x, y, z, point_stride, nullptr, nullptr, f.colrow, nullptr, n_views, n, f.errcam, err, ew,
                           st);
}
