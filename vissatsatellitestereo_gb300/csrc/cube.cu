// Precision form of the RPC projection: C cameras evaluated over one set of points given
// in the normalised frame (x = latitude', y = longitude', z = altitude', as in
// lib/rpc_model.py:40-63), posed as the contraction
//     [N x 20 monomials] x [20 x 4C coefficients]   (col num/den, row num/den per camera)
// followed by the ratio and the denormalisation of RPCModel.projection
// (lib/rpc_model.py:164-168).  Outputs are FP32 col/row planes.
//
// Variants (all accumulate in FP32):
//   VS_CUBE_FP32    CUDA cores, plain FP32 (the comparator of the split forms);
//   VS_CUBE_BF16X3  tensor cores, both factors split into 2 bf16 pieces, products
//                   hh + lh + hl (mma.sync m16n8k16);
//   VS_CUBE_TF32X3  tensor cores, 2 tf32 pieces, the same 3 products (m16n8k8);
//   VS_CUBE_BF16X6  tensor cores, 3 bf16 pieces, the 6 products of order <= 2;
//   VS_CUBE_BF16X3_LIN  BF16X3 for the 16 higher-order terms only, the constant and the
//                   three linear terms in FP32 on the CUDA cores, added in the epilogue.
//                   The split forms' error comes from the large linear coefficients
//                   (|c| ~ 1 at line/sample scale 2048: 2^-16 relative is 0.03 px); the
//                   higher-order coefficients are ~1e-3, so bf16 pieces are ample there.
//                   The linear monomials are the last reduction slots of every lane
//                   (owned monomial q = 0), so one of the four k-steps is dropped.
//
// Contraction layout.  A lane (g = lane/4, t = lane%4) of an m16n8 MMA only ever sees the
// reduction indices k' with k' % 4 == t (tf32 m16n8k8) or k' % 8 in {2t, 2t+1} (bf16
// m16n8k16).  The reduction axis is therefore laid out per lane: lane t owns the five
// monomials k = t, t+4, t+8, t+12, t+16, and its 16 (or 32) reduction slots hold, for each
// owned monomial, one slot per split product (A piece, B piece).  The A fragments of a
// point are then built in registers by the lane itself from the point's coordinates, and
// the B fragments of a column tile are a per-lane contiguous record in shared memory
// prepared once per call from the FP64 coefficients.
//
// Column tile j (8 columns) covers cameras 2j and 2j+1; the accumulator pair of lane t is
// (numerator, denominator) of output plane 4j + t (camera 2j + t/2, col for even t, row
// for odd t), so the epilogue finishes col/row in registers and streams them out.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"

namespace vs {
namespace {

constexpr int kTerms = 20;
constexpr int kCubeWarps = 8;           // warps per CTA of the tensor-core kernels
constexpr int kFp32Threads = 256;
constexpr int kFp32Pts = 4;             // points per thread of the FP32 kernel

template <int V>
struct CubeCfg;
template <>
struct CubeCfg<VS_CUBE_BF16X3> {
    static constexpr bool kBf16 = true, kLin = false;
    static constexpr int kProducts = 3, kPieces = 2, kSlots = 16, kMTiles = 2, kMinBlocks = 3;
};
template <>
struct CubeCfg<VS_CUBE_BF16X3_LIN> {
    static constexpr bool kBf16 = true, kLin = true;
    static constexpr int kProducts = 3, kPieces = 2, kSlots = 16, kMTiles = 2, kMinBlocks = 3;
};
template <>
struct CubeCfg<VS_CUBE_BF16X6> {
    static constexpr bool kBf16 = true, kLin = false;
    static constexpr int kProducts = 6, kPieces = 3, kSlots = 32, kMTiles = 2, kMinBlocks = 2;
};
template <>
struct CubeCfg<VS_CUBE_TF32X3> {
    static constexpr bool kBf16 = false, kLin = false;
    static constexpr int kProducts = 3, kPieces = 2, kSlots = 16, kMTiles = 2, kMinBlocks = 2;
};

// Split products: (A piece, B piece) of product p.  Order-1 terms for 3 products, order-2
// terms for 6 (piece 0 is the largest).
__host__ __device__ constexpr int prod_a(int n_products, int p) {
    return n_products == 3 ? (p == 1 ? 1 : 0) : (p == 2 ? 1 : p == 4 ? 2 : p == 5 ? 1 : 0);
}
__host__ __device__ constexpr int prod_b(int n_products, int p) {
    return n_products == 3 ? (p == 2 ? 1 : 0) : (p == 1 ? 1 : p == 3 ? 2 : p == 5 ? 1 : 0);
}

// Reduction slot s (< 5 * n_products) of a lane: owned monomial index q (monomial
// t + 4q) and split product p.  Small contributions come first and the leading product of
// the constant and linear monomials (q = 0) last, so the FP32 running sums stay small
// until the final k-steps and round at the magnitude of the result only there.
__host__ __device__ constexpr int slot_q(int n_products, int s) { return 4 - s / n_products; }
__host__ __device__ constexpr int slot_p(int n_products, int s) { return n_products - 1 - s % n_products; }

// monomials 0..19 in RPC order from FP32 normalised coordinates
__device__ __forceinline__ void rpc_monomials(float x, float y, float z, float (&m)[kTerms]) {
    const float yx = y * x, yz = y * z, xz = x * z, yy = y * y, xx = x * x, zz = z * z;
    m[0] = 1.0f; m[1] = y; m[2] = x; m[3] = z;
    m[4] = yx; m[5] = yz; m[6] = xz; m[7] = yy; m[8] = xx; m[9] = zz;
    m[10] = yx * z; m[11] = yy * y; m[12] = y * xx; m[13] = y * zz; m[14] = yy * x;
    m[15] = xx * x; m[16] = x * zz; m[17] = yy * z; m[18] = xx * z; m[19] = zz * z;
}

__device__ __forceinline__ float round_tf32(float v) {
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return __uint_as_float(r);
}

template <bool BF16>
__device__ __forceinline__ float round_piece(float v) {
    if constexpr (BF16) return __bfloat162float(__float2bfloat16_rn(v));
    else return round_tf32(v);
}

// n pieces of an FP32 value; each residual is exact in FP32
template <bool BF16, int N>
__device__ __forceinline__ void split_f32(float v, float (&pc)[N]) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
        pc[i] = round_piece<BF16>(v);
        v -= pc[i];
    }
}

// n pieces of an FP64 coefficient (residuals in FP64)
template <bool BF16, int N>
__device__ void split_f64(double v, float (&pc)[N]) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
        pc[i] = round_piece<BF16>(static_cast<float>(v));
        v -= static_cast<double>(pc[i]);
    }
}

// two bf16-exact floats -> one bf16x2 register (lower k in the low half)
__device__ __forceinline__ unsigned pack_bf16x2(float lo, float hi) {
    return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// num / den outside the range of the fast form: IEEE division
__device__ __noinline__ float quotient_ieee(float num, float den) { return __fdiv_rn(num, den); }

// Operands for which the fast quotient below is accurate: |den| in [1e-30, 1e30] keeps the
// approximate reciprocal finite and normal, |num| < 1e30 keeps the residual finite.
__device__ __forceinline__ bool quotient_fast_ok(float num, float den) {
    return fabsf(den) > 1e-30f && fabsf(den) < 1e30f && fabsf(num) < 1e30f;
}

// num / den: approximate reciprocal refined by one residual correction (Markstein's
// q1 = q0 + r (num - den q0)); valid where quotient_fast_ok holds.
__device__ __forceinline__ float quotient_fast(float num, float den) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(den));
    const float q0 = num * r;
    return __fmaf_rn(__fmaf_rn(-den, q0, num), r, q0);
}

// -(num / den) for two values at once with packed FP32x2 operations: quotient_fast's steps
// with the reciprocal's sign flipped (nr = -r, q0n = -q0), so the residual
// num - den q0 = fma(den, q0n, num) and -(q0 + e r) = fma(e, nr, q0n) need no negated
// operand; each lane's products and sums are the scalar form's, negated exactly.
__device__ __forceinline__ float2 quotient2_neg(float2 num, float2 den) {
    float2 nr;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(nr.x) : "f"(-den.x));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(nr.y) : "f"(-den.y));
    const float2 q0n = __fmul2_rn(num, nr);
    const float2 e = __ffma2_rn(den, q0n, num);
    return __ffma2_rn(e, nr, q0n);
}

__device__ __forceinline__ float quotient(float num, float den) {
    if (__builtin_expect(!quotient_fast_ok(num, den), 0)) return quotient_ieee(num, den);
    return quotient_fast(num, den);
}

// The coefficient polynomial of column col = 4*camera + {colNum, colDen, rowNum, rowDen}.
__device__ __forceinline__ const double *column_poly(const VsRpcCamera &cam, int p) {
    return p == 0 ? cam.col_num : p == 1 ? cam.col_den : p == 2 ? cam.row_num : cam.row_den;
}

// Per-call constants, carved from the caller workspace.
struct CubeWs {
    uint4 *bfrag;             // [n_ctiles][W/4][32 lanes] uint4: per-lane B slot records
    float *fcoef;             // [20][4C] FP32 coefficients (FP32 variant)
    float2 *denorm;           // [4 n_ctiles]: (scale, offset) of output plane 2*camera + coord
    float4 *lincoef;          // [n_ctiles][4 lanes][num, den]: constant + linear coefficients (LIN)
};

inline __host__ __device__ int n_col_tiles(int n_cams) { return (n_cams + 1) / 2; }

template <int V>
__global__ void cube_prepare_mma_kernel(const VsRpcCamera *__restrict__ cams, int n_cams, CubeWs w) {
    using C = CubeCfg<V>;
    constexpr int W = C::kBf16 ? C::kSlots / 2 : C::kSlots;     // 32-bit words per lane
    const int n_ct = n_col_tiles(n_cams);
    const int total = n_ct * 32 * W;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        // i = ((j * W/4 + chunk) * 32 + lane) * 4 + e, word = 4 * chunk + e
        const int e = i & 3, lane = (i >> 2) & 31, rest = i >> 7;
        const int chunk = rest % (W / 4), j = rest / (W / 4);
        const int word = 4 * chunk + e;
        const int g = lane >> 2, t = lane & 3;
        const int col = 8 * j + g, cam = col >> 2;
        float slot_val[2] = {0.0f, 0.0f};
        const int n_slot = C::kBf16 ? 2 : 1;
        for (int h = 0; h < n_slot; ++h) {
            const int s = C::kBf16 ? 2 * word + h : word;
            if (cam < n_cams && s < 5 * C::kProducts && !(C::kLin && slot_q(C::kProducts, s) == 0)) {
                const int q = slot_q(C::kProducts, s), p = slot_p(C::kProducts, s);
                float pc[C::kPieces];
                split_f64<C::kBf16, C::kPieces>(column_poly(cams[cam], col & 3)[t + 4 * q], pc);
                const int b = prod_b(C::kProducts, p);
                slot_val[h] = b == 0 ? pc[0] : b == 1 ? pc[1] : pc[C::kPieces - 1];
            }
        }
        unsigned *dst = reinterpret_cast<unsigned *>(w.bfrag);
        dst[i] = C::kBf16 ? pack_bf16x2(slot_val[0], slot_val[1]) : __float_as_uint(slot_val[0]);
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * n_ct; i += gridDim.x * blockDim.x) {
        const int cam = i >> 1, coord = i & 1;
        float2 v = make_float2(1.0f, 0.0f);
        if (cam < n_cams)
            v = coord == 0 ? make_float2(static_cast<float>(cams[cam].col_scale), static_cast<float>(cams[cam].col_off))
                           : make_float2(static_cast<float>(cams[cam].row_scale), static_cast<float>(cams[cam].row_off));
        w.denorm[i] = v;
    }
    if constexpr (C::kLin) {
        // lane t of column tile j: plane 4j + t = camera 2j + t/2, col (t even) or row (t odd)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 8 * n_ct; i += gridDim.x * blockDim.x) {
            const int j = i >> 3, t = (i >> 1) & 3, den = i & 1;
            const int cam = 2 * j + (t >> 1);
            float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (cam < n_cams) {
                const double *poly = column_poly(cams[cam], 2 * (t & 1) + den);
                c = make_float4(static_cast<float>(poly[0]), static_cast<float>(poly[1]), static_cast<float>(poly[2]),
                                static_cast<float>(poly[3]));
            }
            w.lincoef[i] = c;
        }
    }
}

__global__ void cube_prepare_fp32_kernel(const VsRpcCamera *__restrict__ cams, int n_cams, CubeWs w) {
    const int ncol = 4 * n_cams;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kTerms * ncol; i += gridDim.x * blockDim.x) {
        const int k = i / ncol, col = i - k * ncol;
        w.fcoef[i] = static_cast<float>(column_poly(cams[col >> 2], col & 3)[k]);
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * n_cams; i += gridDim.x * blockDim.x) {
        const VsRpcCamera &c = cams[i >> 1];
        w.denorm[i] = (i & 1) == 0 ? make_float2(static_cast<float>(c.col_scale), static_cast<float>(c.col_off))
                                   : make_float2(static_cast<float>(c.row_scale), static_cast<float>(c.row_off));
    }
}

// ---- FP32 CUDA-core variant -----------------------------------------------------------
// Thread: kFp32Pts points (stride blockDim.x); per camera the 4 polynomials of a monomial
// are one float4 of shared memory.
__global__ void __launch_bounds__(kFp32Threads) cube_fp32_kernel(const float *__restrict__ xyz, long long n,
                                                                 int n_cams, CubeWs w, float *__restrict__ out) {
    extern __shared__ float4 coef4[];                  // [20][n_cams]
    float2 *dn = reinterpret_cast<float2 *>(coef4 + kTerms * n_cams);
    for (int i = threadIdx.x; i < kTerms * n_cams; i += blockDim.x) coef4[i] = reinterpret_cast<const float4 *>(w.fcoef)[i];
    for (int i = threadIdx.x; i < 2 * n_cams; i += blockDim.x) dn[i] = w.denorm[i];
    __syncthreads();
    const long long per_block = static_cast<long long>(kFp32Threads) * kFp32Pts;
    for (long long base = blockIdx.x * per_block; base < n; base += static_cast<long long>(gridDim.x) * per_block) {
        float m[kFp32Pts][kTerms];
#pragma unroll
        for (int i = 0; i < kFp32Pts; ++i) {
            const long long p = base + threadIdx.x + i * kFp32Threads;
            float x = 0.0f, y = 0.0f, z = 0.0f;
            if (p < n) {
                x = __ldg(xyz + p);
                y = __ldg(xyz + n + p);
                z = __ldg(xyz + 2 * n + p);
            }
            rpc_monomials(x, y, z, m[i]);
        }
        for (int c = 0; c < n_cams; ++c) {
            float acc[kFp32Pts][4];
#pragma unroll
            for (int i = 0; i < kFp32Pts; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
            // high-order (small) terms first, the constant and linear terms last
#pragma unroll
            for (int k = kTerms - 1; k >= 0; --k) {
                const float4 cf = coef4[k * n_cams + c];
#pragma unroll
                for (int i = 0; i < kFp32Pts; ++i) {
                    acc[i][0] = __fmaf_rn(cf.x, m[i][k], acc[i][0]);
                    acc[i][1] = __fmaf_rn(cf.y, m[i][k], acc[i][1]);
                    acc[i][2] = __fmaf_rn(cf.z, m[i][k], acc[i][2]);
                    acc[i][3] = __fmaf_rn(cf.w, m[i][k], acc[i][3]);
                }
            }
            const float2 dc = dn[2 * c], dr = dn[2 * c + 1];
            float *oc = out + (2LL * c) * n, *orow = oc + n;
#pragma unroll
            for (int i = 0; i < kFp32Pts; ++i) {
                const long long p = base + threadIdx.x + i * kFp32Threads;
                if (p < n) {
                    __stcs(oc + p, __fmaf_rn(quotient(acc[i][0], acc[i][1]), dc.x, dc.y));
                    __stcs(orow + p, __fmaf_rn(quotient(acc[i][2], acc[i][3]), dr.x, dr.y));
                }
            }
        }
    }
}

// ---- tensor-core variants --------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
    asm(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
    asm(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

template <int V>
__host__ __device__ constexpr int cube_words() { return CubeCfg<V>::kBf16 ? CubeCfg<V>::kSlots / 2 : CubeCfg<V>::kSlots; }

// A slot record of one point for lane t: the pieces of monomials t, t+4, ..., t+16 placed
// per split product, packed into 32-bit words.
template <int V>
__device__ __forceinline__ void a_record(float x, float y, float z, int t, unsigned (&a)[cube_words<V>()]) {
    using C = CubeCfg<V>;
    float m[kTerms];
    rpc_monomials(x, y, z, m);
    float pc[5][C::kPieces];
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const float v = t == 0 ? m[4 * q] : t == 1 ? m[4 * q + 1] : t == 2 ? m[4 * q + 2] : m[4 * q + 3];
        split_f32<C::kBf16, C::kPieces>(v, pc[q]);
    }
    float sv[C::kSlots];
#pragma unroll
    for (int s = 0; s < C::kSlots; ++s) {
        const int q = s < 5 * C::kProducts ? slot_q(C::kProducts, s) : 0;
        sv[s] = s < 5 * C::kProducts ? pc[q][prod_a(C::kProducts, slot_p(C::kProducts, s))] : 0.0f;
    }
    if constexpr (C::kBf16) {
#pragma unroll
        for (int wd = 0; wd < C::kSlots / 2; ++wd) a[wd] = pack_bf16x2(sv[2 * wd], sv[2 * wd + 1]);
    } else {
#pragma unroll
        for (int wd = 0; wd < C::kSlots; ++wd) a[wd] = __float_as_uint(sv[wd]);
    }
}

template <int V>
__global__ void __launch_bounds__(kCubeWarps * 32, CubeCfg<V>::kMinBlocks) cube_mma_kernel(const float *__restrict__ xyz, long long n,
                                                                   int n_cams, CubeWs w, float *__restrict__ out) {
    using C = CubeCfg<V>;
    constexpr int W = cube_words<V>();
    constexpr int MT = C::kMTiles;
    constexpr int PTS = 16 * MT;                       // points per warp iteration
    extern __shared__ uint4 bsh[];                     // [n_ct][W/4][32]
    const int n_ct = n_col_tiles(n_cams);
    float2 *dn = reinterpret_cast<float2 *>(bsh + n_ct * (W / 4) * 32);
    float4 *lc = reinterpret_cast<float4 *>(dn + 4 * n_ct);   // LIN: [n_ct][4][2]
    for (int i = threadIdx.x; i < n_ct * (W / 4) * 32; i += blockDim.x) bsh[i] = w.bfrag[i];
    for (int i = threadIdx.x; i < 4 * n_ct; i += blockDim.x) dn[i] = w.denorm[i];
    if constexpr (C::kLin)
        for (int i = threadIdx.x; i < 8 * n_ct; i += blockDim.x) lc[i] = w.lincoef[i];
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int planes = 2 * n_cams;
    const long long groups = (n + PTS - 1) / PTS;
    for (long long grp = static_cast<long long>(blockIdx.x) * kCubeWarps + warp; grp < groups;
         grp += static_cast<long long>(gridDim.x) * kCubeWarps) {
        const long long p0 = grp * PTS;
        const bool full = p0 + PTS <= n;
        unsigned a[MT][2][W];
        float px[MT][2], py[MT][2], pz[MT][2];          // the points, for the LIN epilogue
#pragma unroll
        for (int mt = 0; mt < MT; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const long long p = p0 + 16 * mt + 8 * h + g;
                float x = 0.0f, y = 0.0f, z = 0.0f;
                if (p < n) {
                    x = __ldg(xyz + p);
                    y = __ldg(xyz + n + p);
                    z = __ldg(xyz + 2 * n + p);
                }
                px[mt][h] = x;
                py[mt][h] = y;
                pz[mt][h] = z;
                a_record<V>(x, y, z, t, a[mt][h]);
            }
        float *o = out + static_cast<long long>(t) * n + p0 + g;
        for (int j = 0; j < n_ct; ++j, o += 4 * n) {
            unsigned b[W];
#pragma unroll
            for (int c = 0; c < W / 4; ++c) {
                const uint4 v = bsh[(j * (W / 4) + c) * 32 + lane];
                b[4 * c] = v.x; b[4 * c + 1] = v.y; b[4 * c + 2] = v.z; b[4 * c + 3] = v.w;
            }
            const float2 sc = dn[4 * j + t];
            const bool plane_ok = 4 * j + t < planes;
            // MT independent accumulator chains, interleaved per k-step
            float d[MT][4];
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) d[mt][0] = d[mt][1] = d[mt][2] = d[mt][3] = 0.0f;
#pragma unroll
            for (int s = 0; s < W / 2 - (C::kLin ? 1 : 0); ++s)   // LIN: the q = 0 k-step is dropped
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) {
                    if constexpr (C::kBf16)
                        mma_bf16(d[mt], a[mt][0][2 * s], a[mt][1][2 * s], a[mt][0][2 * s + 1], a[mt][1][2 * s + 1],
                                 b[2 * s], b[2 * s + 1]);
                    else
                        mma_tf32(d[mt], a[mt][0][2 * s], a[mt][1][2 * s], a[mt][0][2 * s + 1], a[mt][1][2 * s + 1],
                                 b[2 * s], b[2 * s + 1]);
                }
            // the two points of an accumulator row pair (g, g + 8) travel as one FP32x2 pair
            // through the linear terms (LIN), the quotient and the denormalisation; one
            // warp-uniform range test (min/max reductions, which NaN cannot trip and an
            // infinity always does) sends rare operands to the per-value test and IEEE division
            float2 num[MT], den[MT];
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                num[mt] = make_float2(d[mt][0], d[mt][2]);
                den[mt] = make_float2(d[mt][1], d[mt][3]);
            }
            if constexpr (C::kLin) {     // constant + linear terms (RPC order 1, y, x, z): z, x, y, then 1
                const float4 cn = lc[(4 * j + t) * 2], cd = lc[(4 * j + t) * 2 + 1];
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) {
                    const float2 X = make_float2(px[mt][0], px[mt][1]), Y = make_float2(py[mt][0], py[mt][1]),
                                 Z = make_float2(pz[mt][0], pz[mt][1]);
                    num[mt] = __ffma2_rn(make_float2(cn.w, cn.w), Z, num[mt]);
                    den[mt] = __ffma2_rn(make_float2(cd.w, cd.w), Z, den[mt]);
                    num[mt] = __ffma2_rn(make_float2(cn.z, cn.z), X, num[mt]);
                    den[mt] = __ffma2_rn(make_float2(cd.z, cd.z), X, den[mt]);
                    num[mt] = __ffma2_rn(make_float2(cn.y, cn.y), Y, num[mt]);
                    den[mt] = __ffma2_rn(make_float2(cd.y, cd.y), Y, den[mt]);
                    num[mt] = __fadd2_rn(num[mt], make_float2(cn.x, cn.x));
                    den[mt] = __fadd2_rn(den[mt], make_float2(cd.x, cd.x));
                }
            }
            float dlo = 1.0f, dhi = 1.0f, nhi = 0.0f;
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                dlo = fminf(dlo, fminf(fabsf(den[mt].x), fabsf(den[mt].y)));
                dhi = fmaxf(dhi, fmaxf(fabsf(den[mt].x), fabsf(den[mt].y)));
                nhi = fmaxf(nhi, fmaxf(fabsf(num[mt].x), fabsf(num[mt].y)));
            }
            float2 qn[MT];                                   // -(num / den)
            if (__builtin_expect(__all_sync(0xffffffffu, dlo > 1e-30f && dhi < 1e30f && nhi < 1e30f), 1)) {
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) qn[mt] = quotient2_neg(num[mt], den[mt]);
            } else {
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) {
                    qn[mt].x = -quotient(num[mt].x, den[mt].x);
                    qn[mt].y = -quotient(num[mt].y, den[mt].y);
                }
            }
            if (plane_ok) {
                const float2 nsc = make_float2(-sc.x, -sc.x), off = make_float2(sc.y, sc.y);
                if (full) {
#pragma unroll
                    for (int mt = 0; mt < MT; ++mt) {
                        const float2 v = __ffma2_rn(qn[mt], nsc, off);
                        __stcs(o + 16 * mt, v.x);
                        __stcs(o + 16 * mt + 8, v.y);
                    }
                } else {
#pragma unroll
                    for (int mt = 0; mt < MT; ++mt) {
                        const long long p = p0 + 16 * mt + g;
                        const float2 v = __ffma2_rn(qn[mt], nsc, off);
                        if (p < n) __stcs(o + 16 * mt, v.x);
                        if (p + 8 < n) __stcs(o + 16 * mt + 8, v.y);
                    }
                }
            }
        }
    }
}

CubeWs carve_cube(Carver &cv, int n_cams) {
    CubeWs w;
    w.bfrag = cv.take<uint4>(static_cast<size_t>(n_col_tiles(n_cams)) * 4 * 32);   // up to 16 words per lane
    w.fcoef = cv.take<float>(static_cast<size_t>(kTerms) * 4 * n_cams);
    w.denorm = cv.take<float2>(4 * static_cast<size_t>(n_col_tiles(n_cams)));
    w.lincoef = cv.take<float4>(8 * static_cast<size_t>(n_col_tiles(n_cams)));
    return w;
}

template <int V>
int launch_mma(const VsRpcCamera *cams, int n_cams, const float *xyz, long long n, float *colrow, CubeWs w,
               cudaStream_t st) {
    using C = CubeCfg<V>;
    constexpr int W = cube_words<V>();
    const int n_ct = n_col_tiles(n_cams);
    cube_prepare_mma_kernel<V><<<static_cast<unsigned>(ceil_div(static_cast<int64_t>(n_ct) * 32 * W, 256)), 256, 0, st>>>(
        cams, n_cams, w);
    VS_LAUNCH_CHECK("cube_prepare_mma_kernel");
    const size_t sh = sizeof(uint4) * n_ct * (W / 4) * 32 + sizeof(float2) * 4 * n_ct + (C::kLin ? sizeof(float4) * 8 * n_ct : 0);
    if (cudaFuncSetAttribute(cube_mma_kernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sh)) !=
        cudaSuccess) {
        set_error("vs_rpc_project_cube: shared memory request of %zu bytes refused", sh);
        return VS_ERR_CUDA;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cube_mma_kernel<V>, kCubeWarps * 32, sh) != cudaSuccess ||
        per_sm <= 0)
        per_sm = 1;
    const long long groups = ceil_div(n, 16LL * C::kMTiles);
    const long long blocks = std::max(1LL, std::min<long long>(ceil_div(groups, kCubeWarps), 1LL * sm_count() * per_sm));
    cube_mma_kernel<V><<<static_cast<unsigned>(blocks), kCubeWarps * 32, sh, st>>>(xyz, n, n_cams, w, colrow);
    VS_LAUNCH_CHECK("cube_mma_kernel");
    return VS_OK;
}

}  // namespace

size_t cube_tc_workspace_bytes(int n_cams);
int cube_tc_status(const void *ws, int n_cams, cudaStream_t st);
int launch_cube_tc(const VsRpcCamera *cams, int n_cams, const float *xyz, long long n, float *colrow, void *ws,
                   cudaStream_t st, bool lin);

}  // namespace vs

using namespace vs;

extern "C" size_t vs_rpc_project_cube_workspace_size(int n_cams) {
    if (n_cams <= 0) return 0;
    Carver cv(nullptr);
    carve_cube(cv, n_cams);
    return std::max(cv.used + 256, cube_tc_workspace_bytes(n_cams));
}

extern "C" int vs_rpc_project_cube(const VsRpcCamera *cams, int n_cams, const float *xyz, int64_t n, float *colrow,
                                   int variant, void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(n_cams > 0 && n_cams <= VS_CUBE_MAX_CAMERAS && n >= 0,
               "vs_rpc_project_cube: bad sizes (cameras %d, max %d; n %lld)", n_cams, VS_CUBE_MAX_CAMERAS, (long long)n);
    VS_REQUIRE(variant == VS_CUBE_FP32 || variant == VS_CUBE_BF16X3 || variant == VS_CUBE_TF32X3 ||
                   variant == VS_CUBE_BF16X6 || variant == VS_CUBE_BF16X3_TC || variant == VS_CUBE_BF16X3_LIN ||
                   variant == VS_CUBE_BF16X3_LIN_TC,
               "vs_rpc_project_cube: bad variant %d", variant);
    VS_REQUIRE(cams && workspace && (n == 0 || (xyz && colrow)), "vs_rpc_project_cube: null pointer");
    const size_t need = vs_rpc_project_cube_workspace_size(n_cams);
    if (workspace_bytes < need) {
        set_error("vs_rpc_project_cube: workspace %zu < %zu bytes", workspace_bytes, need);
        return VS_ERR_WORKSPACE;
    }
    if (n == 0) return VS_OK;
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace);
    const CubeWs w = carve_cube(cv, n_cams);
    switch (variant) {
        case VS_CUBE_BF16X3: return launch_mma<VS_CUBE_BF16X3>(cams, n_cams, xyz, n, colrow, w, st);
        case VS_CUBE_TF32X3: return launch_mma<VS_CUBE_TF32X3>(cams, n_cams, xyz, n, colrow, w, st);
        case VS_CUBE_BF16X6: return launch_mma<VS_CUBE_BF16X6>(cams, n_cams, xyz, n, colrow, w, st);
        case VS_CUBE_BF16X3_LIN: return launch_mma<VS_CUBE_BF16X3_LIN>(cams, n_cams, xyz, n, colrow, w, st);
        case VS_CUBE_BF16X3_TC: return launch_cube_tc(cams, n_cams, xyz, n, colrow, workspace, st, false);
        case VS_CUBE_BF16X3_LIN_TC: return launch_cube_tc(cams, n_cams, xyz, n, colrow, workspace, st, true);
        default: break;
    }
    cube_prepare_fp32_kernel<<<static_cast<unsigned>(ceil_div(static_cast<int64_t>(kTerms) * 4 * n_cams, 256)), 256, 0,
                               st>>>(cams, n_cams, w);
    VS_LAUNCH_CHECK("cube_prepare_fp32_kernel");
    const size_t sh = sizeof(float4) * kTerms * n_cams + sizeof(float2) * 2 * n_cams;
    if (cudaFuncSetAttribute(cube_fp32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sh)) !=
        cudaSuccess) {
        set_error("vs_rpc_project_cube: shared memory request of %zu bytes refused", sh);
        return VS_ERR_CUDA;
    }
    const long long blocks =
        std::max(1LL, std::min<long long>(ceil_div(n, 1LL * kFp32Threads * kFp32Pts), 1LL * sm_count() * 4));
    cube_fp32_kernel<<<static_cast<unsigned>(blocks), kFp32Threads, sh, st>>>(xyz, n, n_cams, w, colrow);
    VS_LAUNCH_CHECK("cube_fp32_kernel");
    return VS_OK;
}

extern "C" int vs_rpc_project_cube_status(const void *workspace, int n_cams, int variant, void *stream) {
    VS_REQUIRE(workspace && n_cams > 0 && n_cams <= VS_CUBE_MAX_CAMERAS, "vs_rpc_project_cube_status: bad arguments");
    if (variant != VS_CUBE_BF16X3_TC && variant != VS_CUBE_BF16X3_LIN_TC)
        return VS_OK;                                    // the other variants have no device-side waits
    return cube_tc_status(workspace, n_cams, as_stream(stream));
}
