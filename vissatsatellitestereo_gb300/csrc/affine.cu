// Affine camera fit: solve_affine (lib/solve_affine.py:37-72) for many views, and the
// per-view loop of CameraApprox.approx_affine_latlonalt (camera_approx.py:112-137).
//
// The reference solves the 2N x 8 least-squares system [x y z 1 0 0 0 0; 0 0 0 0 x y z 1]
// p = [col; row] with LAPACK.  Its two halves share the 4 x 4 Gram matrix of [x y z 1],
// so here every view accumulates, over its kept points, that Gram matrix and the two
// right-hand sides in FP64, in coordinates centred and scaled per axis (the reference
// passes lat/lon/alt, whose axes differ by four orders of magnitude), solves both systems
// by Cholesky and maps the solution back to the raw coordinates.  The result equals the
// full-rank least-squares solution up to rounding (well below 1e-6 px on the fitted
// camera's predictions).
#include <algorithm>

#include "common.cuh"

namespace vs {
namespace {

constexpr int kAffThreads = 256;
constexpr int kAffChunk = 16;            // points per thread per block
constexpr int kAffSums = 18;             // 10 Gram entries + 4 col + 4 row
constexpr int kAffSamples = 65536;       // strided sample for the normalisation box

struct AffNorm {
    double c[3], s[3];                   // centre and 1/half-extent per axis
};

// order-preserving 64-bit keys of doubles (NaN excluded by the callers)
__device__ __forceinline__ unsigned long long dkey(double v) { return key_from_double(v); }

__global__ void aff_box_init_kernel(unsigned long long *box, int n_views) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_views * 6) box[i] = (i % 6) < 3 ? ~0ull : 0ull;   // mins, then maxs
}

// min/max per axis over a strided sample of each view's points (grid y = view)
__global__ void aff_box_kernel(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                               long long stride, long long n, long long step, unsigned long long *__restrict__ box) {
    const int v = blockIdx.y;
    const double *src[3] = {x + v * stride, y + v * stride, z + v * stride};
    unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0ull, 0ull, 0ull};
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k * step < n;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long i = k * step;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double val = src[a][i];
            if (val == val && fabs(val) < 1e300) {
                const unsigned long long kk = dkey(val);
                mn[a] = min(mn[a], kk);
                mx[a] = max(mx[a], kk);
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        for (int off = 16; off > 0; off >>= 1) {
            mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], off));
            mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], off));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(box + v * 6 + a, mn[a]);
            atomicMax(box + v * 6 + 3 + a, mx[a]);
        }
    }
}

__global__ void aff_norm_kernel(const unsigned long long *__restrict__ box, int n_views, AffNorm *__restrict__ norm) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    AffNorm nm;
    for (int a = 0; a < 3; ++a) {
        const unsigned long long lo = box[v * 6 + a], hi = box[v * 6 + 3 + a];
        double c = 0.0, s = 1.0;
        if (lo <= hi && hi != 0ull) {
            const double l = double_from_key(lo), h = double_from_key(hi);
            c = 0.5 * (l + h);
            const double half = 0.5 * (h - l);
            s = half > 0.0 ? 1.0 / half : 1.0;
        }
        nm.c[a] = c;
        nm.s[a] = s;
    }
    norm[v] = nm;
}

// FP64 sums of the kept points of view v: Gram of [u v w 1] (upper triangle, 10 entries),
// col * [u v w 1] and row * [u v w 1].  Block partials land in a fixed slot (deterministic).
__global__ void __launch_bounds__(kAffThreads) aff_moments_kernel(
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z, long long stride,
    const double *__restrict__ col, const double *__restrict__ row, const uint8_t *__restrict__ keep, long long n,
    const AffNorm *__restrict__ norm, double *__restrict__ partial) {
    __shared__ double red[kAffThreads / 32][kAffSums];
    const int v = blockIdx.y;
    const AffNorm nm = norm[v];
    const double *xv = x + v * stride, *yv = y + v * stride, *zv = z + v * stride;
    const double *cv = col + v * n, *rv = row + v * n;
    const uint8_t *kv = keep ? keep + v * n : nullptr;
    double m[kAffSums];
#pragma unroll
    for (int k = 0; k < kAffSums; ++k) m[k] = 0.0;
    const long long base = static_cast<long long>(blockIdx.x) * kAffThreads * kAffChunk + threadIdx.x;
#pragma unroll 1
    for (int j = 0; j < kAffChunk; ++j) {
        const long long i = base + static_cast<long long>(j) * kAffThreads;
        if (i >= n) break;
        if (kv && !kv[i]) continue;
        const double u = (xv[i] - nm.c[0]) * nm.s[0], w1 = (yv[i] - nm.c[1]) * nm.s[1];
        const double w2 = (zv[i] - nm.c[2]) * nm.s[2];
        const double e[4] = {u, w1, w2, 1.0};
        const double c = cv[i], r = rv[i];
        int q = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = a; b < 4; ++b) m[q++] += e[a] * e[b];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            m[10 + a] += c * e[a];
            m[14 + a] += r * e[a];
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < kAffSums; ++k) {
        for (int off = 16; off > 0; off >>= 1) m[k] += __shfl_xor_sync(0xffffffffu, m[k], off);
        if (lane == 0) red[warp][k] = m[k];
    }
    __syncthreads();
    if (threadIdx.x < kAffSums) {
        double s = 0.0;
        for (int w = 0; w < kAffThreads / 32; ++w) s += red[w][threadIdx.x];
        partial[(static_cast<long long>(v) * gridDim.x + blockIdx.x) * kAffSums + threadIdx.x] = s;
    }
}

// One thread per view: sum the block partials in order, Cholesky-solve both systems,
// map back to raw coordinates.  P row-major [2][4]; params (optional) [w, h, P].
__global__ void aff_solve_kernel(const double *__restrict__ partial, int blocks, int n_views,
                                 const AffNorm *__restrict__ norm, const VsRpcCamera *__restrict__ cams,
                                 double *__restrict__ P, double *__restrict__ params, int32_t *__restrict__ status) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views) return;
    double m[kAffSums];
    for (int k = 0; k < kAffSums; ++k) m[k] = 0.0;
    for (int b = 0; b < blocks; ++b)
        for (int k = 0; k < kAffSums; ++k) m[k] += partial[(static_cast<long long>(v) * blocks + b) * kAffSums + k];
    double G[4][4];
    int q = 0;
    for (int a = 0; a < 4; ++a)
        for (int b = a; b < 4; ++b) {
            G[a][b] = m[q];
            G[b][a] = m[q];
            ++q;
        }
    // Cholesky G = L L^T
    double L[4][4] = {};
    bool ok = m[9] >= 4.0;   // G[3][3] is the kept-point count
    for (int i = 0; i < 4 && ok; ++i) {
        for (int j = 0; j <= i; ++j) {
            double s = G[i][j];
            for (int k = 0; k < j; ++k) s -= L[i][k] * L[j][k];
            if (i == j) {
                if (!(s > 1e-12 * (G[i][i] > 0.0 ? G[i][i] : 1.0))) { ok = false; break; }
                L[i][i] = sqrt(s);
            } else {
                L[i][j] = s / L[j][j];
            }
        }
    }
    const AffNorm nm = norm[v];
    double out[8];
    for (int rhs = 0; rhs < 2; ++rhs) {
        double a[4];
        if (ok) {
            double t[4];
            for (int i = 0; i < 4; ++i) {
                double s = m[10 + 4 * rhs + i];
                for (int k = 0; k < i; ++k) s -= L[i][k] * t[k];
                t[i] = s / L[i][i];
            }
            for (int i = 3; i >= 0; --i) {
                double s = t[i];
                for (int k = i + 1; k < 4; ++k) s -= L[k][i] * a[k];
                a[i] = s / L[i][i];
            }
        } else {
            for (int i = 0; i < 4; ++i) a[i] = __longlong_as_double(0x7ff8000000000000ll);
        }
        // value = a0 (x - c0) s0 + a1 (y - c1) s1 + a2 (z - c2) s2 + a3
        double off = a[3];
        for (int k = 0; k < 3; ++k) {
            out[4 * rhs + k] = a[k] * nm.s[k];
            off -= a[k] * nm.s[k] * nm.c[k];
        }
        out[4 * rhs + 3] = off;
    }
    for (int k = 0; k < 8; ++k) P[v * 8 + k] = out[k];
    if (params) {
        params[v * 10 + 0] = cams ? cams[v].width : 0.0;
        params[v * 10 + 1] = cams ? cams[v].height : 0.0;
        for (int k = 0; k < 8; ++k) params[v * 10 + 2 + k] = out[k];
    }
    if (status) status[v] = ok ? VS_OK : VS_ERR_DEGENERATE;
}

struct AffWs {
    unsigned long long *box;
    AffNorm *norm;
    double *partial;
    double *P;
    double *col, *row;     // camera path: projections
    uint8_t *keep;
};

int aff_blocks(long long n) { return static_cast<int>(std::max<long long>(1, ceil_div(n, 1LL * kAffThreads * kAffChunk))); }

AffWs carve_affine(Carver &cv, int n_views, long long n, bool camera_path) {
    AffWs w;
    w.box = cv.take<unsigned long long>(6 * static_cast<size_t>(n_views));
    w.norm = cv.take<AffNorm>(n_views);
    w.partial = cv.take<double>(static_cast<size_t>(n_views) * aff_blocks(n) * kAffSums);
    w.P = cv.take<double>(8 * static_cast<size_t>(n_views));
    w.col = w.row = nullptr;
    w.keep = nullptr;
    if (camera_path) {
        w.col = cv.take<double>(static_cast<size_t>(n_views) * n);
        w.row = cv.take<double>(static_cast<size_t>(n_views) * n);
        w.keep = cv.take<uint8_t>(static_cast<size_t>(n_views) * n);
    }
    return w;
}

int run_affine(const double *x, const double *y, const double *z, long long stride, const double *col, const double *row,
               const uint8_t *keep, int n_views, long long n, const VsRpcCamera *cams, double *P, double *params,
               int32_t *status, AffWs &w, cudaStream_t st) {
    aff_box_init_kernel<<<static_cast<unsigned>(ceil_div(6LL * n_views, 256)), 256, 0, st>>>(w.box, n_views);
    VS_LAUNCH_CHECK("aff_box_init_kernel");
    const long long step = std::max<long long>(1, n / kAffSamples);
    const long long samples = ceil_div(n, step);
    aff_box_kernel<<<dim3(static_cast<unsigned>(std::max<long long>(1, std::min<long long>(ceil_div(samples, 256), 64))),
                          n_views),
                     256, 0, st>>>(x, y, z, stride, n, step, w.box);
    VS_LAUNCH_CHECK("aff_box_kernel");
    aff_norm_kernel<<<static_cast<unsigned>(ceil_div(n_views, 128)), 128, 0, st>>>(w.box, n_views, w.norm);
    VS_LAUNCH_CHECK("aff_norm_kernel");
    const int blocks = aff_blocks(n);
    aff_moments_kernel<<<dim3(blocks, n_views), kAffThreads, 0, st>>>(x, y, z, stride, col, row, keep, n, w.norm,
                                                                      w.partial);
    VS_LAUNCH_CHECK("aff_moments_kernel");
    aff_solve_kernel<<<static_cast<unsigned>(ceil_div(n_views, 64)), 64, 0, st>>>(w.partial, blocks, n_views, w.norm,
                                                                                  cams, P ? P : w.P, params, status);
    VS_LAUNCH_CHECK("aff_solve_kernel");
    return VS_OK;
}

}  // namespace
}  // namespace vs

using namespace vs;

extern "C" size_t vs_affine_fit_workspace_size(int n_views, int64_t n) {
    if (n_views <= 0 || n < 0) return 0;
    Carver cv(nullptr);
    carve_affine(cv, n_views, n, false);
    return cv.used + 256;
}

extern "C" int vs_affine_fit(const double *x, const double *y, const double *z, int64_t xyz_stride, const double *col,
                             const double *row, const uint8_t *keep, int n_views, int64_t n, double *P,
                             int32_t *status, void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n_views > 0 && n_views <= 65535 && n > 0 && xyz_stride >= 0, "vs_affine_fit: bad sizes");
    VS_REQUIRE(x && y && z && col && row && P && workspace, "vs_affine_fit: null pointer");
    const size_t need = vs_affine_fit_workspace_size(n_views, n);
    if (workspace_bytes < need) {
        set_error("vs_affine_fit: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    Carver cv(workspace);
    AffWs w = carve_affine(cv, n_views, n, false);
    return run_affine(x, y, z, xyz_stride, col, row, keep, n_views, n, nullptr, P, nullptr, status, w,
                      as_stream(stream));
}

extern "C" size_t vs_camera_approx_affine_workspace_size(int n_views, int64_t n) {
    if (n_views <= 0 || n < 0) return 0;
    Carver cv(nullptr);
    carve_affine(cv, n_views, n, true);
    return cv.used + 256;
}

extern "C" int vs_camera_approx_affine(const VsRpcCamera *cams, int n_views, const double *lat, const double *lon,
                                       const double *alt, int64_t n, int64_t point_stride, double *params,
                                       int32_t *status, void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n_views > 0 && n_views <= 65535 && n > 0 && point_stride >= 0, "vs_camera_approx_affine: bad sizes");
    VS_REQUIRE(cams && lat && lon && alt && params && workspace, "vs_camera_approx_affine: null pointer");
    const size_t need = vs_camera_approx_affine_workspace_size(n_views, n);
    if (workspace_bytes < need) {
        set_error("vs_camera_approx_affine: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace);
    AffWs w = carve_affine(cv, n_views, n, true);
    // the reference projects the grid with RPCModel.projection (FP64) and keeps the points
    // inside the image (camera_approx.py:121-128)
    const int s = vs_rpc_project(cams, n_views, lat, lon, alt, n, point_stride, w.col, w.row, w.keep, VS_PROJ_EXACT,
                                 stream);
    if (s != VS_OK) return s;
    return run_affine(lat, lon, alt, point_stride, w.col, w.row, w.keep, n_views, n, cams, nullptr, params, status, w,
                      st);
}
