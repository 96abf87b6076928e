// (a)+(b) RPC projection and the RPC -> perspective fit:
//   RPCModel.projection        lib/rpc_model.py:160-168
//   solve_perspective          lib/solve_perspective.py:82-126  (+ factorize :38-79)
//   check_perspective_error    lib/check_error.py:37-121
//   the per-view loop          camera_approx.py:166-189
//
// The fit solves the reference's problem -- the unit vector p minimising |A p| for the
// 2N x 12 DLT matrix A -- without forming A.  A^T A only depends on 40 point moments
// (sum X X^T weighted by 1, c, r, c^2 + r^2 with X = [x y z 1]), so one streaming pass
// accumulates them in coordinates centred and scaled per view (FP32 partial sums over 32
// points, FP64 beyond).  The 12x12 problem is then solved in FP64 by inverse iteration on
// the normalised Gram matrix, with the centring/scaling map M applied exactly, so the
// minimiser is the reference's un-normalised one.  Factorisation is a positive-diagonal
// RQ (Gram-Schmidt from the last row), which is unique and equals the reference's
// sign-fixed scipy RQ.
#include <algorithm>
#include <math.h>

#include "common.cuh"
#include "rpc.cuh"

namespace vs {
namespace {

constexpr int kMom = 40;            // 4 weights x 10 unique entries of X X^T
constexpr int kMomThreads = 128;
constexpr int kChunk = 32;          // points per FP32 partial sum

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
    double cx, cy, cz, s, c0, r0, sp, count;
};

// Min/max of x, y, z, col, row over the kept points of each view, as order-preserving
// keys (min via the complemented key so everything is an atomicMax).
__global__ void bbox_init_kernel(unsigned long long *bb, int n_views) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_views * 11) bb[i] = 0ull;
}

__global__ void __launch_bounds__(256) bbox_kernel(const double *__restrict__ x, const double *__restrict__ y,
                                                   const double *__restrict__ z, long long xyz_stride,
                                                   const double *__restrict__ col, const double *__restrict__ row,
                                                   const uint8_t *__restrict__ keep, long long n,
                                                   unsigned long long *__restrict__ bb) {
    const int v = blockIdx.y;
    const double *src[5] = {x + v * xyz_stride, y + v * xyz_stride, z + v * xyz_stride, col ? col + v * n : nullptr,
                            row ? row + v * n : nullptr};
    unsigned long long hi[5], lo[5];
    unsigned long long cnt = 0;
#pragma unroll
    for (int j = 0; j < 5; ++j) hi[j] = lo[j] = 0ull;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (keep && !keep[v * n + i]) continue;
        ++cnt;
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            if (!src[j]) continue;
            unsigned long long k = key_from_double(src[j][i]);
            hi[j] = max(hi[j], k);
            lo[j] = max(lo[j], ~k);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            hi[j] = max(hi[j], __shfl_xor_sync(0xffffffffu, hi[j], off));
            lo[j] = max(lo[j], __shfl_xor_sync(0xffffffffu, lo[j], off));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        unsigned long long *b = bb + v * 11;
        for (int j = 0; j < 5; ++j) {
            atomicMax(b + j, hi[j]);
            atomicMax(b + 5 + j, lo[j]);
        }
        atomicAdd(b + 10, cnt);
    }
}

// Normalisation from the bounding boxes.  For the fused camera path the pixel frame is the
// RPC's own (colOff/rowOff, max scale) and the count is filled in by the moments pass.
__global__ void norm_kernel(const unsigned long long *__restrict__ bb, const VsRpcCamera *__restrict__ cams,
                            int n_views, Norm *__restrict__ norm) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    const unsigned long long *b = bb + v * 11;
    double mx[5], mn[5];
    for (int j = 0; j < 5; ++j) {
        mx[j] = b[j] ? double_from_key(b[j]) : 0.0;
        mn[j] = b[5 + j] ? double_from_key(~b[5 + j]) : 0.0;
    }
    Norm nm;
    nm.cx = 0.5 * (mn[0] + mx[0]);
    nm.cy = 0.5 * (mn[1] + mx[1]);
    nm.cz = 0.5 * (mn[2] + mx[2]);
    double s = fmax(fmax(mx[0] - mn[0], mx[1] - mn[1]), mx[2] - mn[2]) * 0.5;
    nm.s = (s > 0.0 && isfinite(s)) ? s : 1.0;
    if (cams) {
        nm.c0 = cams[v].col_off;
        nm.r0 = cams[v].row_off;
        nm.sp = fmax(fabs(cams[v].col_scale), fabs(cams[v].row_scale));
        if (!(nm.sp > 0.0)) nm.sp = 1.0;
    } else {
        nm.c0 = 0.5 * (mn[3] + mx[3]);
        nm.r0 = 0.5 * (mn[4] + mx[4]);
        double sp = fmax(mx[3] - mn[3], mx[4] - mn[4]) * 0.5;
        nm.sp = (sp > 0.0 && isfinite(sp)) ? sp : 1.0;
    }
    nm.count = static_cast<double>(b[10]);
    norm[v] = nm;
}

struct NormF {
    float cx, cy, cz, inv_s, c0, r0, inv_sp;
};

__device__ __forceinline__ NormF to_f32(const Norm &nm) {
    return {static_cast<float>(nm.cx), static_cast<float>(nm.cy), static_cast<float>(nm.cz),
            static_cast<float>(1.0 / nm.s), static_cast<float>(nm.c0), static_cast<float>(nm.r0),
            static_cast<float>(1.0 / nm.sp)};
}

// Accumulates one point's 40 moment terms into FP32 partial sums.
__device__ __forceinline__ void add_moments(float (&m)[kMom], float x, float y, float z, float c, float r) {
    const float xx = x * x, xy = x * y, xz = x * z, yy = y * y, yz = y * z, zz = z * z;
    const float e[10] = {xx, xy, xz, x, yy, yz, y, zz, z, 1.0f};
    const float q = __fmaf_rn(c, c, r * r);
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        m[k] += e[k];
        m[10 + k] = __fmaf_rn(c, e[k], m[10 + k]);
        m[20 + k] = __fmaf_rn(r, e[k], m[20 + k]);
        m[30 + k] = __fmaf_rn(q, e[k], m[30 + k]);
    }
}

// Block reduction of the per-thread FP64 accumulators into partial[v][blockIdx.x][40].
__device__ __forceinline__ void store_block_moments(double (&acc)[kMom], double *partial, double *red) {
    // warp shuffle, then across warps through shared memory (fixed order: deterministic)
#pragma unroll
    for (int k = 0; k < kMom; ++k) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], off);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < kMom; ++k) red[warp * kMom + k] = acc[k];
    __syncthreads();
    if (threadIdx.x < kMom) {
        double s = 0.0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) s += red[w * kMom + threadIdx.x];
        partial[threadIdx.x] = s;
    }
}

// Moments of the drop-in fit: points and (col, row) are given (FP64).
__global__ void __launch_bounds__(kMomThreads) moments_kernel(
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z, long long xyz_stride,
    const double *__restrict__ col, const double *__restrict__ row, const uint8_t *__restrict__ keep, long long n,
    const Norm *__restrict__ norm, double *__restrict__ partial) {
    __shared__ double red[(kMomThreads / 32) * kMom];
    const int v = blockIdx.y;
    const NormF nf = to_f32(norm[v]);
    const double *xv = x + v * xyz_stride, *yv = y + v * xyz_stride, *zv = z + v * xyz_stride;
    const double *cv = col + v * n, *rv = row + v * n;
    double acc[kMom];
    float m[kMom];
#pragma unroll
    for (int k = 0; k < kMom; ++k) acc[k] = 0.0, m[k] = 0.0f;
    int in_chunk = 0;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (keep && !keep[v * n + i]) continue;
        const float px = (__double2float_rn(xv[i]) - nf.cx) * nf.inv_s;
        const float py = (__double2float_rn(yv[i]) - nf.cy) * nf.inv_s;
        const float pz = (__double2float_rn(zv[i]) - nf.cz) * nf.inv_s;
        const df dc = split_double(cv[i]), dr = split_double(rv[i]);
        const float pc = ((dc.hi - nf.c0) + dc.lo) * nf.inv_sp;
        const float pr = ((dr.hi - nf.r0) + dr.lo) * nf.inv_sp;
        add_moments(m, px, py, pz, pc, pr);
        if (++in_chunk == kChunk) {
#pragma unroll
            for (int k = 0; k < kMom; ++k) acc[k] += m[k], m[k] = 0.0f;
            in_chunk = 0;
        }
    }
#pragma unroll
    for (int k = 0; k < kMom; ++k) acc[k] += m[k];
    store_block_moments(acc, partial + (static_cast<long long>(v) * gridDim.x + blockIdx.x) * kMom, red);
}

// Fused camera path: project the grid through view v's RPC, apply the in-image mask,
// accumulate the moments and keep the projections (double-float) for the error pass.
template <int MODE>
__global__ void __launch_bounds__(kMomThreads) project_moments_kernel(
    const VsRpcCamera *__restrict__ cams, const double *__restrict__ lat, const double *__restrict__ lon,
    const double *__restrict__ alt, const double *__restrict__ x, const double *__restrict__ y,
    const double *__restrict__ z, long long n, long long stride, const Norm *__restrict__ norm,
    double *__restrict__ partial, float4 *__restrict__ colrow, unsigned long long *__restrict__ counts) {
    __shared__ double red[(kMomThreads / 32) * kMom];
    __shared__ VsRpcCamera cam;
    __shared__ RpcFast fast;
    const int v = blockIdx.y;
    {
        const double *src = reinterpret_cast<const double *>(cams + v);
        double *dst = reinterpret_cast<double *>(&cam);
        for (int i = threadIdx.x; i < static_cast<int>(sizeof(VsRpcCamera) / 8); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) prepare_fast(cam, fast);
    __syncthreads();
    const NormF nf = to_f32(norm[v]);
    const long long off = v * stride;
    double acc[kMom];
    float m[kMom];
#pragma unroll
    for (int k = 0; k < kMom; ++k) acc[k] = 0.0, m[k] = 0.0f;
    int in_chunk = 0;
    unsigned long long kept = 0;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        df dc, dr;
        if (MODE == VS_PROJ_EXACT) {
            double cc, rr;
            project_exact(cam, lat[off + i], lon[off + i], alt[off + i], cc, rr);
            dc = split_double(cc);
            dr = split_double(rr);
        } else {
            project_fast(fast, split_double(lat[off + i]), split_double(lon[off + i]), split_double(alt[off + i]),
                         dc, dr);
        }
        const bool k = df_ge0(dc) && df_ge0(dr) && df_lt(dc, fast.width) && df_lt(dr, fast.height);
        colrow[static_cast<long long>(v) * n + i] = make_float4(dc.hi, dc.lo, dr.hi, dr.lo);
        if (!k) continue;
        ++kept;
        const float px = (__double2float_rn(x[off + i]) - nf.cx) * nf.inv_s;
        const float py = (__double2float_rn(y[off + i]) - nf.cy) * nf.inv_s;
        const float pz = (__double2float_rn(z[off + i]) - nf.cz) * nf.inv_s;
        const float pc = ((dc.hi - nf.c0) + dc.lo) * nf.inv_sp;
        const float pr = ((dr.hi - nf.r0) + dr.lo) * nf.inv_sp;
        add_moments(m, px, py, pz, pc, pr);
        if (++in_chunk == kChunk) {
#pragma unroll
            for (int k2 = 0; k2 < kMom; ++k2) acc[k2] += m[k2], m[k2] = 0.0f;
            in_chunk = 0;
        }
    }
#pragma unroll
    for (int k = 0; k < kMom; ++k) acc[k] += m[k];
#pragma unroll
    for (int off2 = 16; off2 > 0; off2 >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, off2);
    if ((threadIdx.x & 31) == 0) atomicAdd(counts + v, kept);
    store_block_moments(acc, partial + (static_cast<long long>(v) * gridDim.x + blockIdx.x) * kMom, red);
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

// One CTA per view: sum the block partials in a fixed order, solve, factorise.
__global__ void __launch_bounds__(64) solve_kernel(const double *__restrict__ partial, int n_blocks,
                                                   const Norm *__restrict__ norm,
                                                   const unsigned long long *__restrict__ counts,
                                                   const VsRpcCamera *__restrict__ cams, double *__restrict__ K_out,
                                                   double *__restrict__ R_out, double *__restrict__ t_out,
                                                   double *__restrict__ params, double *__restrict__ pinfo,
                                                   int32_t *__restrict__ status) {
    __shared__ double mom[kMom];
    const int v = blockIdx.x;
    if (threadIdx.x < kMom) {
        double s = 0.0;
        const double *p = partial + static_cast<long long>(v) * n_blocks * kMom + threadIdx.x;
        for (int b = 0; b < n_blocks; ++b) s += p[b * kMom];
        mom[threadIdx.x] = s;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const Norm nm = norm[v];
    const double count = counts ? static_cast<double>(counts[v]) : nm.count;
    double K[9], R[9], t[3];
    for (int i = 0; i < 9; ++i) K[i] = R[i] = 0.0;
    t[0] = t[1] = t[2] = 0.0;
    int st = VS_OK;
    if (count < 6.0) st = VS_ERR_DEGENERATE;
    double P[12];
    if (st == VS_OK) {
        // normalised Gram matrix G = [[S0,0,-Sc],[0,S0,-Sr],[-Sc,-Sr,Sq]]
        double G[12][12];
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
        // Cholesky G = L L^T (a non-positive pivot -- an exactly consistent system -- is
        // floored; the inverse iteration then lands on the null vector)
        double dmax = 0.0;
        for (int i = 0; i < 12; ++i) dmax = fmax(dmax, G[i][i]);
        const double floor_piv = dmax * 1e-30 + 1e-300;
        for (int j = 0; j < 12; ++j) {
            double d = G[j][j];
            for (int k = 0; k < j; ++k) d -= G[j][k] * G[j][k];
            d = d > floor_piv ? d : floor_piv;
            const double l = sqrt(d);
            G[j][j] = l;
            for (int i = j + 1; i < 12; ++i) {
                double s = G[i][j];
                for (int k = 0; k < j; ++k) s -= G[i][k] * G[j][k];
                G[i][j] = s / l;
            }
        }
        const Mmap mm{nm.cx, nm.cy, nm.cz, nm.s, nm.c0, nm.r0, nm.sp};
        double p[12], u[12], w[12];
        for (int i = 0; i < 12; ++i) p[i] = 0.28867513459481287;   // 1/sqrt(12)
        for (int it = 0; it < 6; ++it) {
            solve_mt(mm, p, u);
            for (int i = 0; i < 12; ++i) {          // L w = u
                double s = u[i];
                for (int k = 0; k < i; ++k) s -= G[i][k] * w[k];
                w[i] = s / G[i][i];
            }
            for (int i = 11; i >= 0; --i) {         // L^T u = w
                double s = w[i];
                for (int k = i + 1; k < 12; ++k) s -= G[k][i] * u[k];
                u[i] = s / G[i][i];
            }
            solve_m(mm, u, p);
            double nrm = 0.0;
            for (int i = 0; i < 12; ++i) nrm += p[i] * p[i];
            nrm = 1.0 / sqrt(nrm);
            for (int i = 0; i < 12; ++i) p[i] *= nrm;
        }
        for (int i = 0; i < 12; ++i) P[i] = p[i];
        bool finite = true;
        for (int i = 0; i < 12; ++i) finite &= isfinite(P[i]);
        st = finite ? factorize(P, K, R, t) : VS_ERR_DEGENERATE;
    }
    for (int i = 0; i < 9; ++i) K_out[v * 9 + i] = K[i], R_out[v * 9 + i] = R[i];
    for (int i = 0; i < 3; ++i) t_out[v * 3 + i] = t[i];
    status[v] = st;
    if (pinfo) {       // K[R|t] and K^-1 for the error pass
        double *pi = pinfo + v * 21;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 4; ++j) {
                double s = 0.0;
                for (int l = 0; l < 3; ++l) s += K[3 * i + l] * (j < 3 ? R[3 * l + j] : t[l]);
                pi[4 * i + j] = s;
            }
        // K^-1 of an upper-triangular K
        const double a = K[0], b = K[1], c = K[2], d = K[4], e = K[5], f = K[8];
        double *ki = pi + 12;
        ki[0] = 1 / a; ki[1] = -b / (a * d); ki[2] = (b * e - c * d) / (a * d * f);
        ki[3] = 0; ki[4] = 1 / d; ki[5] = -e / (d * f);
        ki[6] = 0; ki[7] = 0; ki[8] = 1 / f;
    }
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
// P^ = K[R|t] and K^-1 for given K, R, t
__global__ void pinfo_kernel(const double *K, const double *R, const double *t, int n_views, double *pinfo) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    const double *k = K + v * 9, *r = R + v * 9, *tt = t + v * 3;
    double *pi = pinfo + v * 21;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int l = 0; l < 3; ++l) s += k[3 * i + l] * (j < 3 ? r[3 * l + j] : tt[l]);
            pi[4 * i + j] = s;
        }
    // general 3x3 inverse (np.linalg.inv(K.T) is used transposed: ray = K^-1 [c r 1])
    const double a = k[0], b = k[1], c = k[2], d = k[3], e = k[4], f = k[5], g = k[6], h = k[7], i9 = k[8];
    const double det = a * (e * i9 - f * h) - b * (d * i9 - f * g) + c * (d * h - e * g);
    double *ki = pi + 12;
    ki[0] = (e * i9 - f * h) / det; ki[1] = (c * h - b * i9) / det; ki[2] = (b * f - c * e) / det;
    ki[3] = (f * g - d * i9) / det; ki[4] = (a * i9 - c * g) / det; ki[5] = (c * d - a * f) / det;
    ki[6] = (d * h - e * g) / det; ki[7] = (b * g - a * h) / det; ki[8] = (a * e - b * d) / det;
}

struct ErrWs {
    unsigned *keys;          // [2][V][n] float bits of the per-point errors (kept points only)
    double *sums;            // [V][blocks][2]
    unsigned *maxk;          // [V][2]
    unsigned long long *cnt; // [V]
    unsigned *hist;          // [V][4][256]
    unsigned *sel;           // [V][4][3]: prefix, mask, k
};

constexpr int kErrThreads = 256;

// Per kept point: pixel reprojection error and metric inverse-projection error.
// colrow_df (fused path) or col/row (FP64) supply the observations.
__global__ void __launch_bounds__(kErrThreads) error_points_kernel(
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z, long long xyz_stride,
    const double *__restrict__ col, const double *__restrict__ row, const float4 *__restrict__ colrow,
    const uint8_t *__restrict__ keep, const float *__restrict__ wh, long long n, const double *__restrict__ pinfo,
    const double *__restrict__ Rm, const double *__restrict__ tv, ErrWs w) {
    __shared__ double red[2][kErrThreads / 32];
    const int v = blockIdx.y;
    const int V = gridDim.y;
    const double *pi = pinfo + v * 21, *ki = pi + 12, *R = Rm + v * 9, *t = tv + v * 3;
    double ps = 0.0, is = 0.0;
    unsigned pmax = 0, imax = 0;
    unsigned long long cnt = 0;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        double c, r;
        bool k;
        if (colrow) {
            const float4 cr = colrow[static_cast<long long>(v) * n + i];
            const df dc{cr.x, cr.y}, dr{cr.z, cr.w};
            k = df_ge0(dc) && df_ge0(dr) && df_lt(dc, wh[2 * v]) && df_lt(dr, wh[2 * v + 1]);
            c = df_to_double(dc);
            r = df_to_double(dr);
        } else {
            c = col[v * n + i];
            r = row[v * n + i];
            k = keep ? keep[v * n + i] != 0 : true;
        }
        unsigned pk = 0xffffffffu, ik = 0xffffffffu;
        if (k) {
            const double X = x[v * xyz_stride + i], Y = y[v * xyz_stride + i], Z = z[v * xyz_stride + i];
            const double cx = R[0] * X + R[1] * Y + R[2] * Z + t[0];
            const double cy = R[3] * X + R[4] * Y + R[5] * Z + t[1];
            const double cz = R[6] * X + R[7] * Y + R[8] * Z + t[2];
            const double h0 = pi[0] * X + pi[1] * Y + pi[2] * Z + pi[3];
            const double h1 = pi[4] * X + pi[5] * Y + pi[6] * Z + pi[7];
            const double h2 = pi[8] * X + pi[9] * Y + pi[10] * Z + pi[11];
            const double ec = h0 / h2 - c, er = h1 / h2 - r;
            const double pe = sqrt(er * er + ec * ec);
            const double rx = ki[0] * c + ki[1] * r + ki[2];
            const double ry = ki[3] * c + ki[4] * r + ki[5];
            const double rz = ki[6] * c + ki[7] * r + ki[8];
            const double sc = (cx * rx + cy * ry + cz * rz) / (rx * rx + ry * ry + rz * rz);
            const double dx = rx * sc - cx, dy = ry * sc - cy, dz = rz * sc - cz;
            const double ie = sqrt(dx * dx + dy * dy + dz * dz);
            ps += pe;
            is += ie;
            pk = __float_as_uint(__double2float_rn(pe));
            ik = __float_as_uint(__double2float_rn(ie));
            pmax = max(pmax, pk);
            imax = max(imax, ik);
            ++cnt;
        }
        w.keys[static_cast<long long>(v) * n + i] = pk;
        w.keys[(static_cast<long long>(V) + v) * n + i] = ik;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ps += __shfl_xor_sync(0xffffffffu, ps, off);
        is += __shfl_xor_sync(0xffffffffu, is, off);
        pmax = max(pmax, __shfl_xor_sync(0xffffffffu, pmax, off));
        imax = max(imax, __shfl_xor_sync(0xffffffffu, imax, off));
        cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    }
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][warp] = ps;
        red[1][warp] = is;
        atomicMax(w.maxk + 2 * v, pmax);
        atomicMax(w.maxk + 2 * v + 1, imax);
        atomicAdd(w.cnt + v, cnt);
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        double s = 0.0;
        for (int i = 0; i < kErrThreads / 32; ++i) s += red[threadIdx.x][i];
        w.sums[(static_cast<long long>(v) * gridDim.x + blockIdx.x) * 2 + threadIdx.x] = s;
    }
}

// Radix selection of the two middle order statistics of both error arrays, 8 bits a pass.
// Targets per view: 0/1 = low/high middle of the pixel errors, 2/3 = of the metric errors.
__global__ void select_init_kernel(ErrWs w, int n_views) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_views * 4) return;
    const int v = i / 4;
    const unsigned long long n = w.cnt[v];
    const int t = i % 4;
    unsigned k = 0;
    if (n > 0) k = static_cast<unsigned>((t & 1) ? n / 2 : (n - 1) / 2);
    w.sel[3 * i] = 0;       // prefix
    w.sel[3 * i + 1] = 0;   // mask
    w.sel[3 * i + 2] = k;   // rank still to skip inside the prefix bucket
}

__global__ void __launch_bounds__(256) select_hist_kernel(ErrWs w, long long n, int shift) {
    __shared__ unsigned h[4][256];
    const int v = blockIdx.y, V = gridDim.y;
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    unsigned pre[4], msk[4];
    for (int t = 0; t < 4; ++t) pre[t] = w.sel[3 * (v * 4 + t)], msk[t] = w.sel[3 * (v * 4 + t) + 1];
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const unsigned kp = w.keys[static_cast<long long>(v) * n + i];
        const unsigned kq = w.keys[(static_cast<long long>(V) + v) * n + i];
        const unsigned dp = (kp >> shift) & 255u, dq = (kq >> shift) & 255u;
        if ((kp & msk[0]) == pre[0]) atomicAdd(&h[0][dp], 1u);
        if ((kp & msk[1]) == pre[1]) atomicAdd(&h[1][dp], 1u);
        if ((kq & msk[2]) == pre[2]) atomicAdd(&h[2][dq], 1u);
        if ((kq & msk[3]) == pre[3]) atomicAdd(&h[3][dq], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) {
        const unsigned c = (&h[0][0])[i];
        if (c) atomicAdd(w.hist + v * 1024 + i, c);
    }
}

__global__ void select_step_kernel(ErrWs w, int n_views, int shift) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_views * 4) return;
    unsigned *hist = w.hist + i * 256;
    unsigned k = w.sel[3 * i + 2];
    unsigned d = 0, below = 0;
    for (; d < 255; ++d) {
        if (below + hist[d] > k) break;
        below += hist[d];
    }
    w.sel[3 * i] |= d << shift;
    w.sel[3 * i + 1] |= 255u << shift;
    w.sel[3 * i + 2] = k - below;
    for (int j = 0; j < 256; ++j) hist[j] = 0;
}

__global__ void error_final_kernel(ErrWs w, int n_views, int n_blocks, double *err) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    const double cnt = static_cast<double>(w.cnt[v]);
    double s[2] = {0.0, 0.0};
    for (int b = 0; b < n_blocks; ++b) {
        s[0] += w.sums[(static_cast<long long>(v) * n_blocks + b) * 2];
        s[1] += w.sums[(static_cast<long long>(v) * n_blocks + b) * 2 + 1];
    }
    double *o = err + v * VS_ERROR_STATS;
    for (int q = 0; q < 2; ++q) {
        const double lo = __uint_as_float(w.sel[3 * (v * 4 + 2 * q)]);
        const double hi = __uint_as_float(w.sel[3 * (v * 4 + 2 * q + 1)]);
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        o[3 * q] = cnt > 0 ? s[q] / cnt : nan;
        o[3 * q + 1] = cnt > 0 ? ((0.0 + lo) + hi) / 2.0 : nan;
        o[3 * q + 2] = cnt > 0 ? static_cast<double>(__uint_as_float(w.maxk[2 * v + q])) : nan;
    }
}

ErrWs carve_err(Carver &cv, int V, long long n, int blocks) {
    ErrWs w;
    w.keys = cv.take<unsigned>(2 * static_cast<size_t>(V) * n);
    w.sums = cv.take<double>(static_cast<size_t>(V) * blocks * 2);
    w.maxk = cv.take<unsigned>(2 * V);
    w.cnt = cv.take<unsigned long long>(V);
    w.hist = cv.take<unsigned>(static_cast<size_t>(V) * 1024);
    w.sel = cv.take<unsigned>(static_cast<size_t>(V) * 12);
    return w;
}

int err_blocks(long long n) {
    long long want = ceil_div(n, kErrThreads);
    return static_cast<int>(std::max<long long>(1, std::min<long long>(want, sm_count() * 4LL)));
}

int run_error_stats(const double *x, const double *y, const double *z, long long xyz_stride, const double *col,
                    const double *row, const float4 *colrow, const uint8_t *keep, const float *wh, int V,
                    long long n, const double *pinfo, const double *R, const double *t, double *err, ErrWs &w,
                    cudaStream_t st) {
    const int blocks = err_blocks(n);
    if (cudaMemsetAsync(w.maxk, 0, sizeof(unsigned) * 2 * V, st) != cudaSuccess ||
        cudaMemsetAsync(w.cnt, 0, sizeof(unsigned long long) * V, st) != cudaSuccess ||
        cudaMemsetAsync(w.hist, 0, sizeof(unsigned) * 1024 * V, st) != cudaSuccess) {
        set_error("cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
    error_points_kernel<<<dim3(blocks, V), kErrThreads, 0, st>>>(x, y, z, xyz_stride, col, row, colrow, keep, wh, n,
                                                                  pinfo, R, t, w);
    VS_LAUNCH_CHECK("error_points_kernel");
    const unsigned sg = static_cast<unsigned>(ceil_div(V * 4, 128));
    select_init_kernel<<<sg, 128, 0, st>>>(w, V);
    VS_LAUNCH_CHECK("select_init_kernel");
    for (int shift = 24; shift >= 0; shift -= 8) {
        select_hist_kernel<<<dim3(blocks, V), 256, 0, st>>>(w, n, shift);
        VS_LAUNCH_CHECK("select_hist_kernel");
        select_step_kernel<<<sg, 128, 0, st>>>(w, V, shift);
        VS_LAUNCH_CHECK("select_step_kernel");
    }
    error_final_kernel<<<static_cast<unsigned>(ceil_div(V, 128)), 128, 0, st>>>(w, V, blocks, err);
    VS_LAUNCH_CHECK("error_final_kernel");
    return VS_OK;
}

int mom_blocks(long long n) {
    long long want = ceil_div(n, kMomThreads * 8);
    return static_cast<int>(std::max<long long>(1, std::min<long long>(want, sm_count() * 2LL)));
}

struct FitWs {
    unsigned long long *bb;
    Norm *norm;
    double *partial;
    double *pinfo;
    unsigned long long *counts;
    float *wh;
    float4 *colrow;
};

FitWs carve_fit(Carver &cv, int V, long long n, bool fused) {
    FitWs f;
    f.bb = cv.take<unsigned long long>(static_cast<size_t>(V) * 11);
    f.norm = cv.take<Norm>(V);
    f.partial = cv.take<double>(static_cast<size_t>(V) * mom_blocks(n) * kMom);
    f.pinfo = cv.take<double>(static_cast<size_t>(V) * 21);
    f.counts = cv.take<unsigned long long>(V);
    f.wh = cv.take<float>(2 * static_cast<size_t>(V));
    f.colrow = fused ? cv.take<float4>(static_cast<size_t>(V) * n) : nullptr;
    return f;
}

__global__ void wh_kernel(const VsRpcCamera *cams, int V, float *wh) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < V) wh[2 * v] = static_cast<float>(cams[v].width), wh[2 * v + 1] = static_cast<float>(cams[v].height);
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
    bbox_init_kernel<<<static_cast<unsigned>(ceil_div(n_views * 11, 128)), 128, 0, st>>>(f.bb, n_views);
    VS_LAUNCH_CHECK("bbox_init_kernel");
    const int blocks = mom_blocks(n);
    if (n > 0) {
        bbox_kernel<<<dim3(blocks, n_views), 256, 0, st>>>(x, y, z, xyz_stride, col, row, keep, n, f.bb);
        VS_LAUNCH_CHECK("bbox_kernel");
    }
    norm_kernel<<<static_cast<unsigned>(ceil_div(n_views, 64)), 64, 0, st>>>(f.bb, nullptr, n_views, f.norm);
    VS_LAUNCH_CHECK("norm_kernel");
    moments_kernel<<<dim3(blocks, n_views), kMomThreads, 0, st>>>(x, y, z, xyz_stride, col, row, keep, n, f.norm,
                                                                   f.partial);
    VS_LAUNCH_CHECK("moments_kernel");
    solve_kernel<<<n_views, 64, 0, st>>>(f.partial, blocks, f.norm, nullptr, nullptr, K, R, t, nullptr, nullptr,
                                         status);
    VS_LAUNCH_CHECK("solve_kernel");
    return VS_OK;
}

extern "C" size_t vs_perspective_error_workspace_size(int n_views, int64_t n) {
    if (n_views <= 0 || n < 0) return 0;
    Carver cv(nullptr);
    cv.take<double>(static_cast<size_t>(n_views) * 21);
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
    double *pinfo = cv.take<double>(static_cast<size_t>(n_views) * 21);
    ErrWs w = carve_err(cv, n_views, n, err_blocks(n));
    pinfo_kernel<<<static_cast<unsigned>(ceil_div(n_views, 64)), 64, 0, st>>>(K, R, t, n_views, pinfo);
    VS_LAUNCH_CHECK("pinfo_kernel");
    return run_error_stats(x, y, z, xyz_stride, col, row, nullptr, keep, nullptr, n_views, n, pinfo, R, t, err, w, st);
}

extern "C" size_t vs_camera_approx_workspace_size(int n_views, int64_t n) {
    if (n_views <= 0 || n < 0) return 0;
    Carver cv(nullptr);
    carve_fit(cv, n_views, n, true);
    cv.take<double>(static_cast<size_t>(n_views) * 21);   // K
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
    double *K = cv.take<double>(static_cast<size_t>(n_views) * 21);
    double *R = cv.take<double>(static_cast<size_t>(n_views) * 9);
    double *t = cv.take<double>(static_cast<size_t>(n_views) * 3);
    ErrWs ew = carve_err(cv, n_views, n, err_blocks(n));
    // ENU bounding box (all points) -> normalisation; pixel frame from each RPC
    bbox_init_kernel<<<static_cast<unsigned>(ceil_div(n_views * 11, 128)), 128, 0, st>>>(f.bb, n_views);
    VS_LAUNCH_CHECK("bbox_init_kernel");
    const int blocks = mom_blocks(n);
    if (n > 0) {
        bbox_kernel<<<dim3(blocks, n_views), 256, 0, st>>>(x, y, z, point_stride, nullptr, nullptr, nullptr, n, f.bb);
        VS_LAUNCH_CHECK("bbox_kernel");
    }
    norm_kernel<<<static_cast<unsigned>(ceil_div(n_views, 64)), 64, 0, st>>>(f.bb, cams, n_views, f.norm);
    VS_LAUNCH_CHECK("norm_kernel");
    if (cudaMemsetAsync(f.counts, 0, sizeof(unsigned long long) * n_views, st) != cudaSuccess) {
        set_error("cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
    if (proj_mode == VS_PROJ_EXACT)
        project_moments_kernel<VS_PROJ_EXACT><<<dim3(blocks, n_views), kMomThreads, 0, st>>>(
            cams, lat, lon, alt, x, y, z, n, point_stride, f.norm, f.partial, f.colrow, f.counts);
    else
        project_moments_kernel<VS_PROJ_FAST><<<dim3(blocks, n_views), kMomThreads, 0, st>>>(
            cams, lat, lon, alt, x, y, z, n, point_stride, f.norm, f.partial, f.colrow, f.counts);
    VS_LAUNCH_CHECK("project_moments_kernel");
    solve_kernel<<<n_views, 64, 0, st>>>(f.partial, blocks, f.norm, f.counts, cams, K, R, t, params, f.pinfo, status);
    VS_LAUNCH_CHECK("solve_kernel");
    if (!err) return VS_OK;
    wh_kernel<<<static_cast<unsigned>(ceil_div(n_views, 64)), 64, 0, st>>>(cams, n_views, f.wh);
    VS_LAUNCH_CHECK("wh_kernel");
    return run_error_stats(x, y, z, point_stride, nullptr, nullptr, f.colrow, nullptr, f.wh, n_views, n, f.pinfo, R,
                           t, err, ew, st);
}
