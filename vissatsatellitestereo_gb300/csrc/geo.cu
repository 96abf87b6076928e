// Geodesy entry points and the depth map -> UTM points path (aggregate_2p5d_util.py:75-98).
//
//  * vs_geo_plan_create: frame constants, then on the device the 5^3 exact Chebyshev nodes
//    over the caller's ENU box, the truncated total-degree-4 fit, and its validation against
//    the exact chain at 17^3 grid + 16384 quasi-random points of the box.  The fast path is
//    enabled only if the largest difference is within VS_GEO_FAST_TOL_M.
//  * vs_enu_to_geodetic / vs_geodetic_to_utm: the exact chain per point (local_to_global,
//    latlon_to_eastnorh).
//  * vs_depth_to_points: count valid pixels per 2048-pixel block, scan, write the valid
//    pixels' (easting, northing, altitude) in pixel order -- the reference's
//    points = tmp[:, valid_mask].T followed by the geodesy.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>

#include "geo.cuh"

namespace vs {
namespace {

constexpr double kPi = 3.141592653589793;
constexpr int kNodes = 5;                      // Chebyshev nodes per axis
constexpr int kNodeCount = kNodes * kNodes * kNodes;
constexpr int kCheb = 35;                      // (a, b, c) with a + b + c <= 4
constexpr int kValGrid = 17;                   // validation grid per axis
constexpr int kValRandom = 16384;
constexpr int kPixThreads = 256, kPixPerThread = kDepthPix, kPixPerBlock = kPixThreads * kPixPerThread;

// Device-resident part of a plan (the exact path reads the frame through a pointer).
struct GeoPlanDev {
    GeoFrame frame;
    GeoFast fast;
    double nodes[3][kNodeCount];
    unsigned max_err_bits;                     // float bits of the largest |fast - exact| (m)
    int lat_sign[2];                           // validation points seen south / north
};

__host__ __device__ inline void cheb_index(int k, int &a, int &b, int &c) {
    int i = 0;
    for (int deg = 0; deg <= 4; ++deg)
        for (int x = deg; x >= 0; --x)
            for (int y = deg - x; y >= 0; --y) {
                if (i == k) {
                    a = x;
                    b = y;
                    c = deg - x - y;
                    return;
                }
                ++i;
            }
    a = b = c = 0;
}

// Coefficient of s^p in the Chebyshev polynomial T_a (a <= 4).
__host__ __device__ inline double cheb_mono(int a, int p) {
    const double t[5][5] = {{1, 0, 0, 0, 0}, {0, 1, 0, 0, 0}, {-1, 0, 2, 0, 0}, {0, -3, 0, 4, 0}, {1, 0, -8, 0, 8}};
    return t[a][p];
}

__device__ __forceinline__ double node_x(int j) {       // cos(pi (j + 1/2) / 5), the middle one exactly 0
    return j == 2 ? 0.0 : cos(kPi * (j + 0.5) / kNodes);
}

__global__ void geo_nodes_kernel(GeoPlanDev *p) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kNodeCount) return;
    const int j0 = k / (kNodes * kNodes), j1 = (k / kNodes) % kNodes, j2 = k % kNodes;
    const GeoFast &f = p->fast;
    const double e = static_cast<double>(f.cen[0]) + static_cast<double>(f.half[0]) * node_x(j0);
    const double n = static_cast<double>(f.cen[1]) + static_cast<double>(f.half[1]) * node_x(j1);
    const double u = static_cast<double>(f.cen[2]) + static_cast<double>(f.half[2]) * node_x(j2);
    double east, north, alt, lat;
    geo_exact(&p->frame, e, n, u, east, north, alt, lat);
    p->nodes[0][k] = east;
    p->nodes[1][k] = north;
    p->nodes[2][k] = alt;
}

// One block: Chebyshev coefficients of (value - centre value), truncated to total degree 4,
// converted to monomials of the normalised coordinates.
__global__ void geo_fit_kernel(GeoPlanDev *p) {
    __shared__ double cheb[3][kCheb];
    __shared__ double mono[3][kCheb];
    __shared__ double tj[kNodes][kNodes];        // T_a(x_j) = cos(a theta_j)
    const int centre = (2 * kNodes + 2) * kNodes + 2;
    const int t = threadIdx.x;
    if (t < kNodes * kNodes) tj[t / kNodes][t % kNodes] = cos((t / kNodes) * kPi * ((t % kNodes) + 0.5) / kNodes);
    __syncthreads();
    if (t < 3 * kCheb) {
        const int o = t / kCheb, k = t % kCheb;
        int a, b, c;
        cheb_index(k, a, b, c);
        const double ref = p->nodes[o][centre];
        double s = 0.0;
        for (int q = 0; q < kNodeCount; ++q) {
            const int j0 = q / (kNodes * kNodes), j1 = (q / kNodes) % kNodes, j2 = q % kNodes;
            s += (p->nodes[o][q] - ref) * tj[a][j0] * tj[b][j1] * tj[c][j2];
        }
        const double w = (a ? 2.0 : 1.0) * (b ? 2.0 : 1.0) * (c ? 2.0 : 1.0) / kNodeCount;
        cheb[o][k] = s * w;
    }
    __syncthreads();
    if (t < 3 * kCheb) {
        const int o = t / kCheb, k = t % kCheb;
        int pp, q, r;
        cheb_index(k, pp, q, r);
        double s = 0.0;
        for (int i = 0; i < kCheb; ++i) {
            int a, b, c;
            cheb_index(i, a, b, c);
            if (a < pp || b < q || c < r) continue;
            s += cheb[o][i] * cheb_mono(a, pp) * cheb_mono(b, q) * cheb_mono(c, r);
        }
        mono[o][k] = s;
    }
    __syncthreads();
    if (t < 3) {
        const int o = t;
        GeoFast &f = p->fast;
        const double ref = p->nodes[o][centre];
        const double scale = 1073741824.0;    // 2^30
        f.c0[o] = llrint(ref * scale) + llrint(mono[o][0] * scale);
        for (int i = 0; i < 3; ++i) f.lin[o][i] = df_from_double(mono[o][1 + i]);
        for (int j = 0; j < kGeoNl; ++j) {
            int a, b, c;
            geo_monomial(j, a, b, c);
            int k = 0;
            for (; k < kCheb; ++k) {
                int x, y, z;
                cheb_index(k, x, y, z);
                if (x == a && y == b && z == c) break;
            }
            f.nl[o][j] = static_cast<float>(mono[o][k]);
        }
        f.enabled = 1;
    }
}

__device__ __forceinline__ double bits_to_double(unsigned long long b) { return __longlong_as_double(static_cast<long long>(b)); }

// Largest |fast - exact| over the validation set (grid points, then a Kronecker sequence).
__global__ void geo_validate_kernel(GeoPlanDev *p) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_grid = kValGrid * kValGrid * kValGrid;
    if (k >= n_grid + kValRandom) return;
    const GeoFast &f = p->fast;
    double s[3];
    if (k < n_grid) {
        const int g[3] = {k / (kValGrid * kValGrid), (k / kValGrid) % kValGrid, k % kValGrid};
        for (int i = 0; i < 3; ++i) s[i] = -1.0 + 2.0 * g[i] / (kValGrid - 1);
    } else {
        const double phi[3] = {0.8191725133961645, 0.6710436067037893, 0.5497004779019703};   // R3 sequence
        const int q = k - n_grid + 1;
        for (int i = 0; i < 3; ++i) {
            const double v = q * phi[i];
            s[i] = 2.0 * (v - floor(v)) - 1.0;
        }
    }
    df enu[3];
    double ed[3];
    for (int i = 0; i < 3; ++i) {
        const double v = static_cast<double>(f.cen[i]) + s[i] * static_cast<double>(f.half[i]) * 0.999;
        enu[i] = df_from_double(v);
        ed[i] = static_cast<double>(enu[i].hi) + static_cast<double>(enu[i].lo);
    }
    double east, north, alt, lat;
    geo_exact(&p->frame, ed[0], ed[1], ed[2], east, north, alt, lat);
    atomicOr(&p->lat_sign[lat < 0.0 ? 0 : 1], 1);
    unsigned long long bits[3];
    float err;
    if (!geo_fast(f, enu, bits)) {
        err = __int_as_float(0x7f800000);
    } else {
        const double d0 = fabs(bits_to_double(bits[0]) - east);
        const double d1 = fabs(bits_to_double(bits[1]) - north);
        const double d2 = fabs(bits_to_double(bits[2]) - alt);
        const double d = fmax(fmax(d0, d1), d2);
        err = d == d ? static_cast<float>(d) : __int_as_float(0x7f800000);
    }
    atomicMax(&p->max_err_bits, __float_as_uint(err));
}

// ---- standalone conversions ---------------------------------------------------------------
__global__ void enu_to_geodetic_kernel(const GeoFrame *g, const double *__restrict__ enu, long long n, long long stride,
                                       double *__restrict__ lat, double *__restrict__ lon, double *__restrict__ alt) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double *q = enu + i * stride;
        double x, y, z, la, lo, al;
        enu_to_ecef(*g, q[0], q[1], q[2], x, y, z);
        ecef_to_geodetic(*g, x, y, z, la, lo, al);
        lat[i] = gm(la, 180.0 / kPi);
        lon[i] = gm(lo, 180.0 / kPi);
        alt[i] = al;
    }
}

__global__ void geodetic_to_utm_kernel(const GeoFrame *g, const double *__restrict__ lat, const double *__restrict__ lon,
                                       long long n, double *__restrict__ east, double *__restrict__ north,
                                       int *__restrict__ flags, int south) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double la = lat[i];
        if (flags && ((la < 0.0) != (south != 0))) atomicOr(flags, VS_GEO_FLAG_HEMISPHERE);
        double e, nn;
        geodetic_to_tm(*g, gm(la, kPi / 180.0), gm(lon[i], kPi / 180.0), e, nn);
        east[i] = e;
        north[i] = nn;
    }
}

// ---- depth map -> points ------------------------------------------------------------------
// Valid-pixel mask of a thread's 8 pixels (bit k: pixel p + k).
__device__ __forceinline__ unsigned valid_mask(const DepthView &v, const double *smd, const float (&d)[kPixPerThread],
                                               long long p, long long W) {
    int r = static_cast<int>(p / W), c = static_cast<int>(p - (p / W) * W);
    const int Wi = static_cast<int>(W);
    unsigned mask = 0;
#pragma unroll
    for (int k = 0; k < kPixPerThread; ++k) {
        const float cf = __int2float_rn(c), rf = __int2float_rn(r);
        const int cls = pixel_class(v, cf, rf, d[k]);
        bool ok = cls == 1;
        if (cls == 2) ok = pixel_valid_exact(smd, cf, rf, d[k]);
        mask |= ok ? (1u << k) : 0u;
        if (++c == Wi) {
            c = 0;
            ++r;
        }
    }
    return mask;
}

__global__ void __launch_bounds__(kPixThreads) depth_count_kernel(const float *__restrict__ depth, long long H,
                                                                  long long W, DepthView v, int *__restrict__ counts) {
    __shared__ int warp_sum[kPixThreads / 32];
    __shared__ double smd[16];
    stage_matrix(v, smd);
    const long long total = H * W;
    const long long p = static_cast<long long>(blockIdx.x) * kPixPerBlock + threadIdx.x * kPixPerThread;
    float d[kPixPerThread];
    load_depths(depth, p, total, d);
    int n = __popc(valid_mask(v, smd, d, p, W));
#pragma unroll
    for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < kPixThreads / 32; ++w) s += warp_sum[w];
        counts[blockIdx.x] = s;
    }
}

// Exclusive scan of the block counts (one block); total into n_points.
__global__ void __launch_bounds__(1024) count_scan_kernel(const int *__restrict__ counts, int n_blocks,
                                                         long long *__restrict__ offsets, int64_t *__restrict__ n_points) {
    __shared__ long long part[1024];
    const int per = (n_blocks + 1023) / 1024;
    const int b0 = threadIdx.x * per;
    long long s = 0;
    for (int i = 0; i < per && b0 + i < n_blocks; ++i) s += counts[b0 + i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {               // Hillis-Steele inclusive scan
        const long long add = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += add;
        __syncthreads();
    }
    long long run = part[threadIdx.x] - s;
    for (int i = 0; i < per && b0 + i < n_blocks; ++i) {
        offsets[b0 + i] = run;
        run += counts[b0 + i];
    }
    if (threadIdx.x == 1023) *n_points = part[1023];
}

__global__ void __launch_bounds__(kPixThreads) depth_points_kernel(
    const float *__restrict__ depth, long long H, long long W, DepthView v, GeoFast f, const GeoFrame *g, int mode,
    int south, const long long *__restrict__ offsets, unsigned long long *__restrict__ out, int *flags) {
    __shared__ int warp_sum[kPixThreads / 32];
    __shared__ double smd[16];
    stage_matrix(v, smd);
    const long long total = H * W;
    const long long p = static_cast<long long>(blockIdx.x) * kPixPerBlock + threadIdx.x * kPixPerThread;
    float d[kPixPerThread];
    load_depths(depth, p, total, d);
    const unsigned mask = valid_mask(v, smd, d, p, W);
    // block-exclusive prefix of the per-thread counts
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int n = __popc(mask);
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sum[wid] = incl;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < wid; ++w) before += warp_sum[w];
    long long slot = offsets[blockIdx.x] + before + incl - n;
    int r = static_cast<int>(p / W), c = static_cast<int>(p - (p / W) * W);
    const int Wi = static_cast<int>(W);
#pragma unroll 1
    for (int k = 0; k < kPixPerThread; ++k) {
        if (mask & (1u << k)) {
            unsigned long long bits[3];
            const float cf = __int2float_rn(c), rf = __int2float_rn(r);
            const float dk = depth[p + k];
            df w;
            const int cls = pixel_class(v, cf, rf, dk, w);
            pixel_point(v, smd, f, g, mode, cls, w, cf, rf, dk, south, bits, flags);
            unsigned long long *dst = out + 3 * slot;
            dst[0] = bits[0];
            dst[1] = bits[1];
            dst[2] = bits[2];
            ++slot;
        }
        if (++c == Wi) {
            c = 0;
            ++r;
        }
    }
}

}  // namespace

// ---- host helpers shared with the fused rasteriser ------------------------------------------
void build_geo_frame(const VsGeoFrame &in, GeoFrame &g) {
    const double a = 6378137.0, fl = 1.0 / 298.257223563;
    const double b = a * (1.0 - fl), e2 = fl * (2.0 - fl);
    const double phi = in.lat0 * (kPi / 180.0), lam = in.lon0 * (kPi / 180.0);
    const double sp = sin(phi), nu = a / sqrt(1.0 - e2 * sp * sp);
    g.x0 = (nu + in.alt0) * cos(phi) * cos(lam);
    g.y0 = (nu + in.alt0) * cos(phi) * sin(lam);
    g.z0 = (nu * (1.0 - e2) + in.alt0) * sp;
    g.sphi = sp;
    g.cphi = cos(phi);
    g.slam = sin(lam);
    g.clam = cos(lam);
    g.a = a;
    g.b = b;
    g.a2 = a * a;
    g.b2 = b * b;
    g.esq = a * a - b * b;
    g.E = sqrt(g.esq);
    g.ecc = sqrt(e2);
    g.a_over_b = a / b;
    g.lam0 = ((in.utm_zone - 1) * 6 - 180 + 3) * (kPi / 180.0);
    const double n = fl / (2.0 - fl), n2 = n * n, n3 = n2 * n, n4 = n3 * n, n5 = n4 * n, n6 = n5 * n;
    g.alpha[0] = n / 2 - 2 * n2 / 3 + 5 * n3 / 16 + 41 * n4 / 180 - 127 * n5 / 288 + 7891 * n6 / 37800;
    g.alpha[1] = 13 * n2 / 48 - 3 * n3 / 5 + 557 * n4 / 1440 + 281 * n5 / 630 - 1983433 * n6 / 1935360;
    g.alpha[2] = 61 * n3 / 240 - 103 * n4 / 140 + 15061 * n5 / 26880 + 167603 * n6 / 181440;
    g.alpha[3] = 49561 * n4 / 161280 - 179 * n5 / 168 + 6601661 * n6 / 7257600;
    g.alpha[4] = 34729 * n5 / 80640 - 3418889 * n6 / 1995840;
    g.alpha[5] = 212378941 * n6 / 319334400;
    const double A = a / (1 + n) * (1 + n2 / 4 + n4 / 64 + n6 / 256);
    g.k0A = 0.9996 * A;
    g.fe = 500000.0;
    g.fn = in.south ? 10000000.0 : 0.0;
}

bool make_depth_view(const double *m, DepthView &v) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            const double x = m[4 * i + j];
            if (!isfinite(x)) return false;
            v.md[i][j] = x;
            v.m[i][j] = df_from_double(x);
        }
    return true;
}

}  // namespace vs

using namespace vs;

struct VsGeoPlan {
    GeoPlanDev *dev;          // caller's device buffer
    GeoFast fast;             // host copy, passed to kernels by value
    int zone, south;
    float max_err;
    int straddles;            // the box reaches both hemispheres
};

extern "C" size_t vs_geo_plan_device_bytes(void) { return (sizeof(GeoPlanDev) + 255) & ~size_t(255); }

extern "C" int vs_geo_plan_create(const VsGeoFrame *frame, void *device_buffer, size_t device_bytes,
                                  VsGeoPlan **plan_out, void *stream) {
    VS_REQUIRE(frame && device_buffer && plan_out, "vs_geo_plan_create: null pointer");
    VS_REQUIRE(device_bytes >= vs_geo_plan_device_bytes(), "vs_geo_plan_create: device buffer %zu < %zu bytes",
               device_bytes, vs_geo_plan_device_bytes());
    VS_REQUIRE(frame->utm_zone >= 1 && frame->utm_zone <= 60 && (frame->south == 0 || frame->south == 1),
               "vs_geo_plan_create: zone %d / south %d", frame->utm_zone, frame->south);
    VS_REQUIRE(isfinite(frame->lat0) && isfinite(frame->lon0) && isfinite(frame->alt0) && fabs(frame->lat0) <= 90.0,
               "vs_geo_plan_create: bad origin");
    *plan_out = nullptr;
    cudaStream_t st = as_stream(stream);
    GeoPlanDev *host = static_cast<GeoPlanDev *>(calloc(1, sizeof(GeoPlanDev)));
    VsGeoPlan *plan = new (std::nothrow) VsGeoPlan();
    if (!host || !plan) {
        free(host);
        delete plan;
        set_error("vs_geo_plan_create: host allocation failed");
        return VS_ERR_ARG;
    }
    build_geo_frame(*frame, host->frame);
    // box: centre rounded to a float, half-widths rounded up to powers of two (>= 1 m)
    bool box_ok = true;
    for (int i = 0; i < 3; ++i) {
        const double lo = frame->box_lo[i], hi = frame->box_hi[i];
        if (!(isfinite(lo) && isfinite(hi) && hi > lo)) box_ok = false;
        const float cen = static_cast<float>(0.5 * (lo + hi));
        const double need = fmax(fmax(hi - cen, cen - lo), 1.0);
        int k = static_cast<int>(ceil(log2(need)));
        if (k > 16) box_ok = false;                // beyond +-64 km: the fit is not used
        k = k < 0 ? 0 : (k > 16 ? 16 : k);
        host->fast.cen[i] = box_ok ? cen : 0.0f;
        host->fast.half[i] = ldexpf(1.0f, k);
        host->fast.inv_half[i] = ldexpf(1.0f, -k);
    }
    int s = VS_OK;
    if (cudaMemcpyAsync(device_buffer, host, sizeof(GeoPlanDev), cudaMemcpyHostToDevice, st) != cudaSuccess) {
        set_error("vs_geo_plan_create: copy to device failed");
        s = VS_ERR_CUDA;
    }
    GeoPlanDev *dev = static_cast<GeoPlanDev *>(device_buffer);
    if (s == VS_OK && box_ok) {
        geo_nodes_kernel<<<1, 128, 0, st>>>(dev);
        s = check_launch("geo_nodes_kernel");
        if (s == VS_OK) {
            geo_fit_kernel<<<1, 128, 0, st>>>(dev);
            s = check_launch("geo_fit_kernel");
        }
        if (s == VS_OK) {
            const int n = kValGrid * kValGrid * kValGrid + kValRandom;
            geo_validate_kernel<<<(n + 127) / 128, 128, 0, st>>>(dev);
            s = check_launch("geo_validate_kernel");
        }
    }
    if (s == VS_OK) {
        if (cudaMemcpyAsync(host, device_buffer, sizeof(GeoPlanDev), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            set_error("vs_geo_plan_create: plan readback failed");
            s = VS_ERR_CUDA;
        }
    }
    if (s != VS_OK) {
        free(host);
        delete plan;
        return s;
    }
    plan->dev = dev;
    plan->fast = host->fast;
    plan->zone = frame->utm_zone;
    plan->south = frame->south;
    float err;
    memcpy(&err, &host->max_err_bits, sizeof err);
    plan->max_err = box_ok ? err : INFINITY;
    plan->straddles = host->lat_sign[0] && host->lat_sign[1];
    plan->fast.enabled = box_ok && err <= VS_GEO_FAST_TOL_M && !plan->straddles &&
                         (host->lat_sign[frame->south ? 0 : 1] != 0);
    free(host);
    *plan_out = plan;
    return VS_OK;
}

extern "C" int vs_geo_plan_query(const VsGeoPlan *plan, double *max_err_m, int32_t *fast_enabled) {
    VS_REQUIRE(plan, "vs_geo_plan_query: null plan");
    if (max_err_m) *max_err_m = plan->max_err;
    if (fast_enabled) *fast_enabled = plan->fast.enabled;
    return VS_OK;
}

extern "C" void vs_geo_plan_destroy(VsGeoPlan *plan) { delete plan; }

namespace vs {
// Accessors for the fused rasteriser (raster.cu).
const GeoFast &geo_plan_fast(const VsGeoPlan *p) { return p->fast; }
const GeoFrame *geo_plan_frame(const VsGeoPlan *p) { return &p->dev->frame; }
int geo_plan_south(const VsGeoPlan *p) { return p->south; }
}  // namespace vs

extern "C" int vs_enu_to_geodetic(const VsGeoPlan *plan, const double *enu, int64_t n, int64_t point_stride,
                                  double *lat, double *lon, double *alt, void *stream) {
    VS_REQUIRE(plan && n >= 0 && point_stride >= 3, "vs_enu_to_geodetic: bad arguments");
    VS_REQUIRE(n == 0 || (enu && lat && lon && alt), "vs_enu_to_geodetic: null pointer");
    if (n == 0) return VS_OK;
    const unsigned g = static_cast<unsigned>(std::min<long long>(ceil_div(n, 128), sm_count() * 16LL));
    enu_to_geodetic_kernel<<<g, 128, 0, as_stream(stream)>>>(&plan->dev->frame, enu, n, point_stride, lat, lon, alt);
    return check_launch("enu_to_geodetic_kernel");
}

extern "C" int vs_geodetic_to_utm(const VsGeoPlan *plan, const double *lat, const double *lon, int64_t n,
                                  double *east, double *north, int32_t *flags, void *stream) {
    VS_REQUIRE(plan && n >= 0, "vs_geodetic_to_utm: bad arguments");
    VS_REQUIRE(n == 0 || (lat && lon && east && north), "vs_geodetic_to_utm: null pointer");
    if (n == 0) return VS_OK;
    const unsigned g = static_cast<unsigned>(std::min<long long>(ceil_div(n, 128), sm_count() * 16LL));
    geodetic_to_utm_kernel<<<g, 128, 0, as_stream(stream)>>>(&plan->dev->frame, lat, lon, n, east, north,
                                                              reinterpret_cast<int *>(flags), plan->south);
    return check_launch("geodetic_to_utm_kernel");
}

extern "C" size_t vs_depth_to_points_workspace_size(int64_t height, int64_t width) {
    if (height <= 0 || width <= 0) return 0;
    const long long blocks = ceil_div(height * width, kPixPerBlock);
    return static_cast<size_t>(blocks) * (sizeof(int) + sizeof(long long)) + 1024;
}

extern "C" int vs_depth_to_points(const float *depth, int64_t height, int64_t width, const double *inv_proj,
                                  const VsGeoPlan *plan, int32_t mode, double *points, int64_t *n_points,
                                  int32_t *flags, void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(height > 0 && width > 0 && height * width < (1LL << 39) && height < (1 << 24) && width < (1 << 24),
               "vs_depth_to_points: bad size %lldx%lld", (long long)height, (long long)width);
    VS_REQUIRE(depth && inv_proj && plan && points && n_points && workspace, "vs_depth_to_points: null pointer");
    VS_REQUIRE(mode == VS_GEO_EXACT || mode == VS_GEO_FAST, "vs_depth_to_points: bad mode %d", mode);
    const size_t need = vs_depth_to_points_workspace_size(height, width);
    if (workspace_bytes < need) {
        set_error("vs_depth_to_points: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    DepthView v;
    VS_REQUIRE(make_depth_view(inv_proj, v), "vs_depth_to_points: non-finite inverse projection");
    cudaStream_t st = as_stream(stream);
    const long long blocks = ceil_div(height * width, kPixPerBlock);
    VS_REQUIRE(blocks < (1LL << 31), "vs_depth_to_points: too many pixels");
    Carver cv(workspace);
    int *counts = cv.take<int>(blocks);
    long long *offsets = cv.take<long long>(blocks);
    depth_count_kernel<<<static_cast<unsigned>(blocks), kPixThreads, 0, st>>>(depth, height, width, v, counts);
    VS_LAUNCH_CHECK("depth_count_kernel");
    count_scan_kernel<<<1, 1024, 0, st>>>(counts, static_cast<int>(blocks), offsets, n_points);
    VS_LAUNCH_CHECK("count_scan_kernel");
    depth_points_kernel<<<static_cast<unsigned>(blocks), kPixThreads, 0, st>>>(
        depth, height, width, v, plan->fast, &plan->dev->frame, mode, plan->south, offsets,
        reinterpret_cast<unsigned long long *>(points), reinterpret_cast<int *>(flags));
    return check_launch("depth_points_kernel");
}
