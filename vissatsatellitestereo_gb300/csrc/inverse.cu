// RPCModel.inverse_projection (lib/rpc_model.py:170-249) for many cameras and points.
//
// The reference iterates all points of one camera together: from lon = lat = -1 (in the
// normalised frame) it projects the point and two finite-difference neighbours (steps 2,
// then 0.1), moves lon/lat by the projections of the image residual on the two difference
// vectors, and stops when EVERY point reprojects within sqrt(1e-18) of its target.  A
// point's result therefore depends on its camera's global iteration count, so the device
// keeps each point's state in the workspace and the host runs the per-camera global loop:
// one update launch per iteration for the cameras still running, each block counting its
// unconverged points.  Every FP64 operation is the reference's (no contraction into FMA),
// so the results are bit-identical.
#include <vector>

#include "common.cuh"
#include "rpc.cuh"

namespace vs {
namespace {

constexpr int kInvThreads = 256;
constexpr int kStateFields = 11;   // lon lat x0 y0 x1 y1 x2 y2 c_col c_row c_alt

struct InvState {
    double *f[kStateFields];
};

__device__ __forceinline__ double rfm(const double *num, const double *den, double lat, double lon, double alt) {
    return __ddiv_rn(poly_exact(num, lat, lon, alt), poly_exact(den, lat, lon, alt));
}

// the reference's three projections: at (lat, lon), (lat, lon + eps), (lat + eps, lon)
__device__ __forceinline__ void frames(const VsRpcCamera &c, double lat, double lon, double alt, double eps,
                                       double (&o)[6]) {
    const double lon_e = __dadd_rn(lon, eps), lat_e = __dadd_rn(lat, eps);
    o[0] = rfm(c.col_num, c.col_den, lat, lon, alt);
    o[1] = rfm(c.row_num, c.row_den, lat, lon, alt);
    o[2] = rfm(c.col_num, c.col_den, lat, lon_e, alt);
    o[3] = rfm(c.row_num, c.row_den, lat, lon_e, alt);
    o[4] = rfm(c.col_num, c.col_den, lat_e, lon, alt);
    o[5] = rfm(c.row_num, c.row_den, lat_e, lon, alt);
}

// (x0 - c_col)^2 + (y0 - c_row)^2 < 1e-18 (false for NaN)
__device__ __forceinline__ bool converged(double x0, double y0, double cc, double cr) {
    const double dx = __dsub_rn(x0, cc), dy = __dsub_rn(y0, cr);
    return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)) < 1e-18;
}

__device__ __forceinline__ void count_block(bool unconverged, int *count) {
    __shared__ int s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    const unsigned b = __ballot_sync(0xffffffffu, unconverged);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(&s, __popc(b));
    __syncthreads();
    if (threadIdx.x == 0 && s) atomicAdd(count, s);
}

// grid (points, cameras)
__global__ void __launch_bounds__(kInvThreads) inverse_init_kernel(
    const VsRpcCamera *__restrict__ cams, const double *__restrict__ col, const double *__restrict__ row,
    const double *__restrict__ alt, long long n, long long stride, InvState st, int *__restrict__ count) {
    const int c = blockIdx.y;
    const long long i = blockIdx.x * static_cast<long long>(kInvThreads) + threadIdx.x;
    bool unc = false;
    if (i < n) {
        const VsRpcCamera &cam = cams[c];
        const long long p = c * stride + i, s = c * n + i;
        const double cc = __ddiv_rn(__dsub_rn(col[p], cam.col_off), cam.col_scale);
        const double cr = __ddiv_rn(__dsub_rn(row[p], cam.row_off), cam.row_scale);
        const double ca = __ddiv_rn(__dsub_rn(alt[p], cam.alt_off), cam.alt_scale);
        double o[6];
        frames(cam, -1.0, -1.0, ca, 2.0, o);
        st.f[0][s] = -1.0;
        st.f[1][s] = -1.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) st.f[2 + k][s] = o[k];
        st.f[8][s] = cc;
        st.f[9][s] = cr;
        st.f[10][s] = ca;
        unc = !converged(o[0], o[1], cc, cr);
    }
    count_block(unc, count + c);
}

// One global iteration for the cameras with iter[c] >= 0 (iter[c] = iterations done).
__global__ void __launch_bounds__(kInvThreads) inverse_step_kernel(const VsRpcCamera *__restrict__ cams,
                                                                   const int *__restrict__ iter, long long n,
                                                                   InvState st, int *__restrict__ count) {
    const int c = blockIdx.y;
    const int k = iter[c];
    if (k < 0) return;
    const long long i = blockIdx.x * static_cast<long long>(kInvThreads) + threadIdx.x;
    bool unc = false;
    if (i < n) {
        const VsRpcCamera &cam = cams[c];
        const long long s = c * n + i;
        double lon = st.f[0][s], lat = st.f[1][s];
        const double x0 = st.f[2][s], y0 = st.f[3][s], x1 = st.f[4][s], y1 = st.f[5][s], x2 = st.f[6][s],
                     y2 = st.f[7][s];
        const double cc = st.f[8][s], cr = st.f[9][s], ca = st.f[10][s];
        const double e1x = __dsub_rn(x1, x0), e1y = __dsub_rn(y1, y0);
        const double e2x = __dsub_rn(x2, x0), e2y = __dsub_rn(y2, y0);
        const double ux = __dsub_rn(cc, x0), uy = __dsub_rn(cr, y0);
        const double a1 = __ddiv_rn(__dadd_rn(__dmul_rn(ux, e1x), __dmul_rn(uy, e1y)),
                                    __dadd_rn(__dmul_rn(e1x, e1x), __dmul_rn(e1y, e1y)));
        const double a2 = __ddiv_rn(__dadd_rn(__dmul_rn(ux, e2x), __dmul_rn(uy, e2y)),
                                    __dadd_rn(__dmul_rn(e2x, e2x), __dmul_rn(e2y, e2y)));
        const double eps = k == 0 ? 2.0 : 0.1;
        lon = __dadd_rn(lon, __dmul_rn(a1, eps));
        lat = __dadd_rn(lat, __dmul_rn(a2, eps));
        double o[6];
        frames(cam, lat, lon, ca, 0.1, o);
        st.f[0][s] = lon;
        st.f[1][s] = lat;
#pragma unroll
        for (int q = 0; q < 6; ++q) st.f[2 + q][s] = o[q];
        unc = !converged(o[0], o[1], cc, cr);
    }
    count_block(unc, count + c);
}

__global__ void inverse_final_kernel(const VsRpcCamera *__restrict__ cams, const double *__restrict__ alt,
                                     long long n, long long stride, int normalized, InvState st,
                                     double *__restrict__ lon_out, double *__restrict__ lat_out,
                                     double *__restrict__ alt_out) {
    const int c = blockIdx.y;
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const VsRpcCamera &cam = cams[c];
    const long long s = c * n + i;
    const double lon = st.f[0][s], lat = st.f[1][s];
    if (normalized) {
        lon_out[s] = lon;
        lat_out[s] = lat;
        if (alt_out) alt_out[s] = st.f[10][s];
    } else {
        lon_out[s] = __dadd_rn(__dmul_rn(lon, cam.lon_scale), cam.lon_off);
        lat_out[s] = __dadd_rn(__dmul_rn(lat, cam.lat_scale), cam.lat_off);
        if (alt_out) alt_out[s] = alt[c * stride + i];
    }
}

InvState carve_inverse(Carver &cv, int n_cams, long long n, int *&count, int *&iter) {
    InvState st;
    for (auto &f : st.f) f = cv.take<double>(static_cast<size_t>(n_cams) * n);
    count = cv.take<int>(n_cams);
    iter = cv.take<int>(n_cams);
    return st;
}

}  // namespace
}  // namespace vs

using namespace vs;

extern "C" size_t vs_rpc_inverse_project_workspace_size(int n_cams, int64_t n) {
    if (n_cams <= 0 || n < 0) return 0;
    Carver cv(nullptr);
    int *a, *b;
    carve_inverse(cv, n_cams, n, a, b);
    return cv.used + 256;
}

extern "C" int vs_rpc_inverse_project(const VsRpcCamera *cams, int n_cams, const double *col, const double *row,
                                      const double *alt, int64_t n, int64_t point_stride, int normalized,
                                      double *lon, double *lat, double *alt_out, int max_iter, int32_t *iterations,
                                      void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n_cams > 0 && n_cams <= 65535 && n >= 0 && point_stride >= 0 && max_iter > 0,
               "vs_rpc_inverse_project: bad sizes");
    VS_REQUIRE(cams && workspace && (n == 0 || (col && row && alt && lon && lat)),
               "vs_rpc_inverse_project: null pointer");
    const size_t need = vs_rpc_inverse_project_workspace_size(n_cams, n);
    if (workspace_bytes < need) {
        set_error("vs_rpc_inverse_project: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    std::vector<int> it(n_cams, 0), cnt(n_cams, 0);
    if (n == 0) {
        if (iterations)
            for (int c = 0; c < n_cams; ++c) iterations[c] = 0;
        return VS_OK;
    }
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace);
    int *d_count = nullptr, *d_iter = nullptr;
    const InvState state = carve_inverse(cv, n_cams, n, d_count, d_iter);
    const dim3 grid(static_cast<unsigned>(ceil_div(n, kInvThreads)), static_cast<unsigned>(n_cams));
    auto fetch = [&]() -> int {
        if (cudaMemcpyAsync(cnt.data(), d_count, sizeof(int) * n_cams, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            set_error("vs_rpc_inverse_project: %s", cudaGetErrorString(cudaGetLastError()));
            return VS_ERR_CUDA;
        }
        return VS_OK;
    };
    if (cudaMemsetAsync(d_count, 0, sizeof(int) * n_cams, st) != cudaSuccess) {
        set_error("vs_rpc_inverse_project: cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
    inverse_init_kernel<<<grid, kInvThreads, 0, st>>>(cams, col, row, alt, n, point_stride, state, d_count);
    VS_LAUNCH_CHECK("inverse_init_kernel");
    int s = fetch();
    if (s != VS_OK) return s;
    // per camera: iterations done, or -1 once all of its points have converged
    std::vector<int> state_iter(n_cams);
    for (int c = 0; c < n_cams; ++c) state_iter[c] = cnt[c] > 0 ? 0 : -1;
    for (;;) {
        bool any = false;
        for (int c = 0; c < n_cams; ++c) any |= state_iter[c] >= 0;
        if (!any) break;
        for (int c = 0; c < n_cams; ++c)
            if (state_iter[c] >= max_iter) {
                set_error("vs_rpc_inverse_project: camera %d did not converge in %d iterations", c, max_iter);
                return VS_ERR_DEGENERATE;
            }
        if (cudaMemcpyAsync(d_iter, state_iter.data(), sizeof(int) * n_cams, cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaMemsetAsync(d_count, 0, sizeof(int) * n_cams, st) != cudaSuccess) {
            set_error("vs_rpc_inverse_project: upload failed");
            return VS_ERR_CUDA;
        }
        inverse_step_kernel<<<grid, kInvThreads, 0, st>>>(cams, d_iter, n, state, d_count);
        VS_LAUNCH_CHECK("inverse_step_kernel");
        if ((s = fetch()) != VS_OK) return s;
        for (int c = 0; c < n_cams; ++c) {
            if (state_iter[c] < 0) continue;
            ++it[c];
            state_iter[c] = cnt[c] > 0 ? state_iter[c] + 1 : -1;
        }
    }
    inverse_final_kernel<<<grid, kInvThreads, 0, st>>>(cams, alt, n, point_stride, normalized, state, lon, lat,
                                                        alt_out);
    VS_LAUNCH_CHECK("inverse_final_kernel");
    if (iterations)
        for (int c = 0; c < n_cams; ++c) iterations[c] = it[c];
    return VS_OK;
}
