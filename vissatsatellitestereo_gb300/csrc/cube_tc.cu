// Precision form of the RPC projection (BF16X3 split products) on the 5th-generation
// tensor cores: tcgen05.mma with both operands in shared memory and the FP32 accumulators
// in tensor memory.
//
// A CTA of 128 threads owns a tile of 128 points at a time.  Each thread computes its
// point's 20 monomials, splits them into bf16 pieces and writes its row of A into shared
// memory; the coefficient pieces B (all cameras' 4 polynomials, N = 4 cameras rounded up
// to 16 columns) are loaded into shared memory once.  One thread issues the K = 64
// contraction as four 128 x N x 16 MMAs into a TMEM accumulator and commits them to an
// mbarrier; the four warps then read their 32 lanes (points) back with tcgen05.ld, form
// num/den, denormalise and stream the col/row planes out (consecutive threads write
// consecutive points, so the stores coalesce).
//
// Measured (16 M points x 50 cameras): correct to the bit pattern of BF16X3's error
// (max 0.0376 px) but 3.3 ms against 1.75 ms for the warp-level mma.sync kernel.  The
// contraction is tiny (K = 64) and the kernel is bound by its output stream; here every
// tile runs A-build, MMA and epilogue back to back behind CTA barriers (8 warps per SM),
// while the warp-level kernel keeps 24 independent warps per SM.  A 256-thread variant
// (two warps per lane quadrant) measured 3.75 ms.  Overlapping the phases would need a
// warp-specialised producer/consumer pipeline over two TMEM accumulators.
//
// Reduction axis: slot k' = 3q + p for monomial q (0..19) and split product p: A holds
// (hi, lo, hi)[p] of the monomial, B holds (hi, hi, lo)[p] of the coefficient, so the sum
// over k' is hh + lh + hl; slots 60..63 are zero.
//
// Operand layout (no swizzle, K-major): 8-row x 16-byte core matrices, rows of a core
// 16 bytes apart; cores adjacent along K 128 bytes apart (leading byte offset), cores
// adjacent along M/N 1024 bytes apart (stride byte offset).
//
// Every wait is bounded: a CTA that times out sets the error word, still waits (bounded)
// for its committed MMAs, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"

namespace vs {
namespace {

constexpr int kTcThreads = 128;     // one warpgroup: thread = TMEM lane = point of the tile
constexpr int kTcK = 64;            // padded reduction length (bf16)
constexpr int kTcRowBytes = kTcK * 2;
constexpr int kTcTmemCols = 256;
constexpr unsigned kWaitLimit = 1u << 24;

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte offsets,
// descriptor version 1, no swizzle
__device__ __forceinline__ unsigned long long umma_desc(unsigned addr, unsigned lbo, unsigned sbo) {
    return (static_cast<unsigned long long>((addr >> 4) & 0x3fffu)) |
           (static_cast<unsigned long long>((lbo >> 4) & 0x3fffu) << 16) |
           (static_cast<unsigned long long>((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// instruction descriptor: FP32 accumulate, bf16 A and B, both K-major, M = 128, N = n
__host__ __device__ constexpr unsigned umma_idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<unsigned>(n >> 3) << 17) | (static_cast<unsigned>(128 >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned phase) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(phase)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned phase, unsigned limit = kWaitLimit) {
    for (unsigned it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// Polls of the completion wait before a CTA gives up (vs_set_tc_wait_limit; 0 makes every
// CTA give up at once, which exercises the timeout path).
unsigned g_tc_wait_limit = kWaitLimit;

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void umma_bf16(unsigned d_tmem, unsigned long long a, unsigned long long b, unsigned idesc,
                                          unsigned accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(unsigned bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float bf16_round(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// byte offset of element (row, k) in the canonical layout: [row/8][k/8][row%8][k%8]
__host__ __device__ __forceinline__ unsigned canon_offset(int row, int k) {
    return static_cast<unsigned>(((row >> 3) * (kTcK / 8) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ float tc_quotient(float num, float den) {
    if (fabsf(den) > 1e-30f && fabsf(den) < 1e30f && fabsf(num) < 1e30f) {
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(den));
        const float q0 = num * r;
        return __fmaf_rn(__fmaf_rn(-den, q0, num), r, q0);
    }
    return __fdiv_rn(num, den);
}

// B (canonical layout, bf16) and the denormalisation of every output plane
__global__ void cube_tc_prepare_kernel(const VsRpcCamera *__restrict__ cams, int n_cams, int n_pad,
                                       __nv_bfloat16 *__restrict__ b, float2 *__restrict__ denorm) {
    const int total = n_pad * kTcK;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int col = i / kTcK, k = i - col * kTcK;
        const int cam = col >> 2, p = col & 3;
        float v = 0.0f;
        if (cam < n_cams && k < 60) {
            const VsRpcCamera &c = cams[cam];
            const double *poly = p == 0 ? c.col_num : p == 1 ? c.col_den : p == 2 ? c.row_num : c.row_den;
            const double coef = poly[k / 3];
            const float hi = bf16_round(static_cast<float>(coef));
            const float lo = bf16_round(static_cast<float>(coef - static_cast<double>(hi)));
            v = (k % 3 == 2) ? lo : hi;
        }
        b[canon_offset(col, k) / 2] = __float2bfloat16_rn(v);
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * n_cams; i += gridDim.x * blockDim.x) {
        const VsRpcCamera &c = cams[i >> 1];
        denorm[i] = (i & 1) == 0 ? make_float2(static_cast<float>(c.col_scale), static_cast<float>(c.col_off))
                                 : make_float2(static_cast<float>(c.row_scale), static_cast<float>(c.row_off));
    }
}

__global__ void __launch_bounds__(kTcThreads) cube_tc_kernel(const float *__restrict__ xyz, long long n, int n_cams,
                                                            int n_pad, const uint4 *__restrict__ bglob,
                                                            const float2 *__restrict__ denorm, float *__restrict__ out,
                                                            int *__restrict__ error, unsigned wait_limit) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sa = smem;                                  // A: 128 x 64 bf16 (16 KB)
    unsigned char *sb = smem + 128 * kTcRowBytes;              // B: n_pad x 64 bf16
    float2 *sden = reinterpret_cast<float2 *>(sb + n_pad * kTcRowBytes);
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ unsigned tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    // B and the denormalisation into shared memory (visible to the tensor cores' proxy)
    for (int i = tid; i < n_pad * kTcRowBytes / 16; i += kTcThreads) reinterpret_cast<uint4 *>(sb)[i] = bglob[i];
    for (int i = tid; i < 2 * n_cams; i += kTcThreads) sden[i] = denorm[i];
    const unsigned bar = smem_addr(&mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = tmem_base;
    const unsigned idesc = umma_idesc_bf16(n_pad);
    const unsigned a_base = smem_addr(sa), b_base = smem_addr(sb);
    const long long tiles = (n + 127) / 128;
    unsigned phase = 0;
    bool failed = false;
    for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        // ---- A row of this thread's point: 20 monomials -> (hi, lo, hi) bf16 pieces
        const long long p = tile * 128 + tid;
        float x = 0.0f, y = 0.0f, z = 0.0f;
        if (p < n) {
            x = __ldg(xyz + p);
            y = __ldg(xyz + n + p);
            z = __ldg(xyz + 2 * n + p);
        }
        const float yx = y * x, yz = y * z, xz = x * z, yy = y * y, xx = x * x, zz = z * z;
        const float m[20] = {1.0f,   y,      x,      z,      yx,     yz,     xz,     yy,     xx,     zz,
                             yx * z, yy * y, y * xx, y * zz, yy * x, xx * x, x * zz, yy * z, xx * z, zz * z};
        unsigned words[kTcK / 2];
#pragma unroll
        for (int w = 0; w < kTcK / 2; ++w) {
            float e[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = 2 * w + h;
                if (k < 60) {
                    const float mv = m[k / 3];
                    const float hi = bf16_round(mv);
                    e[h] = (k % 3 == 1) ? bf16_round(mv - hi) : hi;
                } else {
                    e[h] = 0.0f;
                }
            }
            words[w] = __byte_perm(__float_as_uint(e[0]), __float_as_uint(e[1]), 0x7632);
        }
#pragma unroll
        for (int c = 0; c < kTcK / 8; ++c)
            *reinterpret_cast<uint4 *>(sa + canon_offset(tid, 8 * c)) =
                make_uint4(words[4 * c], words[4 * c + 1], words[4 * c + 2], words[4 * c + 3]);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        // ---- one thread issues the contraction
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kTcK / 16; ++ks) {
                const unsigned long long da = umma_desc(a_base + ks * 256, 128, 1024);
                const unsigned long long db = umma_desc(b_base + ks * 256, 128, 1024);
                umma_bf16(tmem, da, db, idesc, ks > 0 ? 1u : 0u);
            }
            umma_commit(bar);
        }
        // the outcome of the wait is made block-uniform before anyone leaves the loop
        const bool done = mbar_wait_bounded(bar, phase, wait_limit);
        if (__syncthreads_or(!done)) {
            failed = true;
            break;
        }
        phase ^= 1u;
        tc_fence_after();
        // ---- epilogue: warp w reads lanes 32w..32w+31 (its points), 16 columns at a time
        const unsigned lane_base = tmem + (static_cast<unsigned>(warp * 32) << 16);
        for (int c0 = 0; c0 < n_pad; c0 += 16) {
            float v[16];
            tmem_ld16(lane_base + c0, v);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int cam = (c0 >> 2) + q;
                if (cam < n_cams && p < n) {
                    const float2 dc = sden[2 * cam], dr = sden[2 * cam + 1];
                    __stcs(out + (2LL * cam) * n + p, __fmaf_rn(tc_quotient(v[4 * q], v[4 * q + 1]), dc.x, dc.y));
                    __stcs(out + (2LL * cam + 1) * n + p,
                           __fmaf_rn(tc_quotient(v[4 * q + 2], v[4 * q + 3]), dr.x, dr.y));
                }
            }
        }
        tc_fence_before();
        __syncthreads();   // TMEM and the A tile are free for the next tile
        tc_fence_after();
    }
    if (failed) {
        if (tid == 0) atomicExch(error, 1);
        mbar_wait_bounded(bar, phase);     // the committed MMAs (full limit) before TMEM is freed
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols) : "memory");
}

}  // namespace

size_t cube_tc_workspace_bytes(int n_cams) {
    const int n_pad = ((4 * n_cams + 15) / 16) * 16;
    return static_cast<size_t>(n_pad) * kTcRowBytes + 256 + sizeof(float2) * 2 * n_cams + 256 + 256;
}

// The workspace layout of the tcgen05 variant: coefficient pieces, denormalisation, error word.
struct CubeTcWs {
    __nv_bfloat16 *b;
    float2 *den;
    int *err;
};
static CubeTcWs carve_cube_tc(void *ws, int n_cams) {
    const int n_pad = ((4 * n_cams + 15) / 16) * 16;
    Carver cv(ws);
    CubeTcWs w;
    w.b = cv.take<__nv_bfloat16>(static_cast<size_t>(n_pad) * kTcK);
    w.den = cv.take<float2>(2 * static_cast<size_t>(n_cams));
    w.err = cv.take<int>(1);
    return w;
}

// Reads back the error word of the last tcgen05 launch that used `ws` (synchronises `st`).
int cube_tc_status(const void *ws, int n_cams, cudaStream_t st) {
    const CubeTcWs w = carve_cube_tc(const_cast<void *>(ws), n_cams);
    int h = 0;
    if (cudaMemcpyAsync(&h, w.err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("vs_rpc_project_cube_status: reading the error word failed");
        return VS_ERR_CUDA;
    }
    if (h) {
        set_error("vs_rpc_project_cube: a CTA of the tcgen05 kernel gave up waiting for its tensor-core work; "
                  "its tiles of colrow were not written");
        return VS_ERR_TIMEOUT;
    }
    return VS_OK;
}

int launch_cube_tc(const VsRpcCamera *cams, int n_cams, const float *xyz, long long n, float *colrow, void *ws,
                   cudaStream_t st) {
    const int n_pad = ((4 * n_cams + 15) / 16) * 16;
    if (n_pad > 256) {
        set_error("vs_rpc_project_cube: the tcgen05 variant takes at most 64 cameras (%d given)", n_cams);
        return VS_ERR_ARG;
    }
    const CubeTcWs w = carve_cube_tc(ws, n_cams);
    __nv_bfloat16 *b = w.b;
    float2 *den = w.den;
    int *err = w.err;
    if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) {
        set_error("vs_rpc_project_cube: cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
    cube_tc_prepare_kernel<<<static_cast<unsigned>(ceil_div(static_cast<int64_t>(n_pad) * kTcK, 256)), 256, 0, st>>>(
        cams, n_cams, n_pad, b, den);
    VS_LAUNCH_CHECK("cube_tc_prepare_kernel");
    // at least 100 KB of shared memory: at most two CTAs per SM, which share its 512 TMEM
    // columns (256 each), so no allocation has to wait for another CTA to finish
    const size_t need_sh = static_cast<size_t>(128 + n_pad) * kTcRowBytes + sizeof(float2) * 2 * n_cams + 1024;
    const size_t sh = std::max<size_t>(need_sh, 100 * 1024);
    if (cudaFuncSetAttribute(cube_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sh)) !=
        cudaSuccess) {
        set_error("vs_rpc_project_cube: shared memory request of %zu bytes refused", sh);
        return VS_ERR_CUDA;
    }
    // two CTAs per SM share its 512 TMEM columns
    const long long tiles = ceil_div(n, 128);
    const unsigned grid = static_cast<unsigned>(std::max(1LL, std::min<long long>(tiles, 2LL * sm_count())));
    cube_tc_kernel<<<grid, kTcThreads, sh, st>>>(xyz, n, n_cams, n_pad, reinterpret_cast<const uint4 *>(b), den,
                                                 colrow, err, g_tc_wait_limit);
    VS_LAUNCH_CHECK("cube_tc_kernel");
    return VS_OK;
}

}  // namespace vs

extern "C" void vs_set_tc_wait_limit(unsigned polls) { vs::g_tc_wait_limit = polls; }
