// Precision form of the RPC projection on the 5th-generation tensor cores (tcgen05):
// the contraction [N x monomials] x [monomials x 4C coefficients] of lib/rpc_model.py:40-79
// with split bf16 products, FP32 accumulators in tensor memory, and the ratio and
// denormalisation of RPCModel.projection (lib/rpc_model.py:164-168) in the epilogue.
//
// Split schemes (reduction slot s = 3 j + p of the scheme's j-th monomial, product p):
//   X3   (VS_CUBE_BF16X3_TC): all 20 monomials, A pieces (hi, lo, hi) x B pieces
//        (hi, hi, lo) = hh + lh + hl; K = 60 slots padded to 64.
//   LIN  (VS_CUBE_BF16X3_LIN_TC): the 16 higher-order monomials only (K = 48); the
//        constant and linear terms -- whose large coefficients carry the split forms'
//        error -- are added in FP32 in the epilogue (z, x, y, then the constant).
// Monomials enter the reduction from the highest order down, so the large terms come last.
//
// One persistent CTA per SM, warp-specialised, tiles of 128 points (the TMEM lanes):
//   * 2 producer warps: each thread builds two points' A rows (bf16 pieces, canonical
//     no-swizzle K-major layout) into a 4-stage shared-memory ring;
//   * 1 MMA warp: its lane 0 issues the K/16 MMAs (M = 128, N = 4C rounded up to 16) of
//     a tile into one of two TMEM accumulators and commits them to the stage's "empty" and
//     the accumulator's "full" mbarriers;
//   * 28 epilogue warps (seven warpgroups, each a seventh of the cameras): a warp reads its
//     32 lanes (points) with tcgen05.ld, forms the quotients (the fast form for a chunk of
//     4 cameras at once, one warp-uniform check for rare operands), denormalises, streams
//     the col/row planes out (32 consecutive points of a plane per store) and releases the
//     accumulator.
// No CTA-wide barrier inside the tile loop: the producers run up to four tiles ahead, the
// tensor cores work on tile k+1 while the epilogue finishes tile k.  The coefficient tile
// B (all cameras' pieces, prepared once per call) is copied into shared memory once per
// CTA by the bulk-copy (TMA) engine.
//
// Operand layout (no swizzle, K-major): 8-row x 16-byte core matrices; cores adjacent along
// K are 128 bytes apart (leading byte offset), along M/N K/8 * 128 bytes (stride offset).
//
// Every wait is bounded.  A warp that gives up sets the error word and a shared abort flag
// that ends the other roles' waits; before freeing its tensor memory the CTA waits
// (bounded) for the coefficient copy and for every MMA it committed.
// vs_rpc_project_cube_status reads the word back.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"

namespace vs {
namespace {

constexpr int kTcProducerWarps = 2;                 // two point rows of A per thread
constexpr int kTcMmaWarp = kTcProducerWarps;        // allocates TMEM; its lane 0 issues the MMAs
constexpr int kTcEpiWarps = 28;                     // seven epilogue warpgroups
constexpr int kTcGroups = kTcEpiWarps / 4;          // camera groups of the epilogue
constexpr int kTcThreads = 32 * (kTcProducerWarps + 1 + kTcEpiWarps);
constexpr int kTcStages = 4;                        // A ring
constexpr int kTcTile = 128;        // points per tile = TMEM lanes
constexpr int kTcTmemCols = 512;    // two accumulators of up to 256 columns
constexpr int kTcMaxN = 256;
constexpr int kTcMaxCams = kTcMaxN / 4;
constexpr unsigned kWaitLimit = 1u << 24;

template <bool LIN>
struct TcScheme {
    static constexpr int kFirst = LIN ? 4 : 0;            // first monomial in the contraction
    static constexpr int kMonos = 20 - kFirst;
    static constexpr int kK = LIN ? 48 : 64;              // slots, padded to whole K=16 steps
    static constexpr int kRowBytes = kK * 2;
    // monomial of contraction slot group j (highest order first)
    static __host__ __device__ constexpr int mono(int j) { return 19 - j; }
};

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

// Bounded wait that also gives up once another warp of the CTA has raised `abort`.
__device__ __forceinline__ bool mbar_wait_abortable(unsigned bar, unsigned phase, unsigned limit,
                                                    const volatile int *abort) {
    for (unsigned it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, phase)) return true;
        if ((it & 63u) == 63u && *abort) return false;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

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

// 8 consecutive accumulator columns of this thread's lane (complete after tmem_wait)
__device__ __forceinline__ void tmem_ld8(unsigned taddr, unsigned (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tmem_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ float bf16_round(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ unsigned pack_bf16x2(float lo, float hi) {
    return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// byte offset of element (row, k) in the canonical layout of a K-slot operand:
// [row/8][k/8][row%8][k%8]
__host__ __device__ __forceinline__ unsigned canon_offset(int row, int k, int K) {
    return static_cast<unsigned>(((row >> 3) * (K / 8) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// num / den: approximate reciprocal refined by one residual correction; IEEE division
// outside the range where that is accurate
__device__ __noinline__ float tc_quotient_ieee(float num, float den) { return __fdiv_rn(num, den); }

__device__ __forceinline__ const double *column_poly(const VsRpcCamera &cam, int p) {
    return p == 0 ? cam.col_num : p == 1 ? cam.col_den : p == 2 ? cam.row_num : cam.row_den;
}

// The per-call constants in the workspace: B pieces (canonical layout), per camera the
// negated scales and the offsets of its two planes, (LIN) per camera and term k the FP32
// constant + linear coefficients of the four polynomials, paired (col, row) for the packed
// FP32x2 epilogue, and the error word.
struct CubeTcWs {
    __nv_bfloat16 *b;          // [n_pad x K]
    float4 *den;               // [C]: (-col_scale, -row_scale, col_off, row_off)
    float4 *lin;               // [C][4 terms]: (colNum_k, rowNum_k, colDen_k, rowDen_k)
    int *err;
};

inline int tc_n_pad(int n_cams) { return ((4 * n_cams + 15) / 16) * 16; }

CubeTcWs carve_cube_tc(void *ws, int n_cams) {
    Carver cv(ws);
    CubeTcWs w;
    w.b = cv.take<__nv_bfloat16>(static_cast<size_t>(kTcMaxN) * 64);
    w.den = cv.take<float4>(static_cast<size_t>(n_cams));
    w.lin = cv.take<float4>(4 * static_cast<size_t>(n_cams));
    w.err = cv.take<int>(1);
    return w;
}

template <bool LIN>
__global__ void cube_tc_prepare_kernel(const VsRpcCamera *__restrict__ cams, int n_cams, int n_pad, CubeTcWs w) {
    using S = TcScheme<LIN>;
    const int total = n_pad * S::kK;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int col = i / S::kK, k = i - col * S::kK;
        const int cam = col >> 2, p = col & 3;
        float v = 0.0f;
        if (cam < n_cams && k < 3 * S::kMonos) {
            const double coef = column_poly(cams[cam], p)[S::mono(k / 3)];
            const float hi = bf16_round(static_cast<float>(coef));
            const float lo = bf16_round(static_cast<float>(coef - static_cast<double>(hi)));
            v = (k % 3 == 2) ? lo : hi;           // B pieces (hi, hi, lo)
        }
        w.b[canon_offset(col, k, S::kK) / 2] = __float2bfloat16_rn(v);
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_cams; i += gridDim.x * blockDim.x) {
        const VsRpcCamera &c = cams[i];
        w.den[i] = make_float4(-static_cast<float>(c.col_scale), -static_cast<float>(c.row_scale),
                               static_cast<float>(c.col_off), static_cast<float>(c.row_off));
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * n_cams; i += gridDim.x * blockDim.x) {
        const VsRpcCamera &c = cams[i >> 2];
        const int k = i & 3;
        w.lin[i] = make_float4(static_cast<float>(c.col_num[k]), static_cast<float>(c.row_num[k]),
                               static_cast<float>(c.col_den[k]), static_cast<float>(c.row_den[k]));
    }
}

// A point's A row: all K/8 16-byte chunks (8 slots each).
template <bool LIN>
__device__ __forceinline__ void build_a_row(unsigned char *a_tile, int row, float x, float y, float z) {
    using S = TcScheme<LIN>;
    const float yx = y * x, yz = y * z, xz = x * z, yy = y * y, xx = x * x, zz = z * z;
    const float m[20] = {1.0f,   y,      x,      z,      yx,     yz,     xz,     yy,     xx,     zz,
                         yx * z, yy * y, y * xx, y * zz, yy * x, xx * x, x * zz, yy * z, xx * z, zz * z};
#pragma unroll
    for (int c = 0; c < S::kK / 8; ++c) {
        unsigned words[4];
#pragma unroll
        for (int wd = 0; wd < 4; ++wd) {
            float e[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int k = 8 * c + 2 * wd + q;
                float v = 0.0f;
                if (k < 3 * S::kMonos) {
                    const float mv = m[S::mono(k / 3)];
                    const float hi = bf16_round(mv);
                    v = (k % 3 == 1) ? bf16_round(mv - hi) : hi;   // A pieces (hi, lo, hi)
                }
                e[q] = v;
            }
            words[wd] = pack_bf16x2(e[0], e[1]);
        }
        *reinterpret_cast<uint4 *>(a_tile + canon_offset(row, 8 * c, S::kK)) =
            make_uint4(words[0], words[1], words[2], words[3]);
    }
}

// Operands for which the fast quotient is accurate.  An RPC denominator is 1 plus small
// terms inside the normalised cube, so the test is |den - 1| < 1/2 (rcp.approx is then
// well inside its accurate range) and |num| < 1e30 (finite residual); anything else --
// points far outside the cube, NaN, infinities -- takes IEEE division.
__device__ __forceinline__ bool quotient_fast_ok(float num, float den) {
    return fabsf(den - 1.0f) < 0.5f && fabsf(num) < 1e30f;
}
__device__ __forceinline__ float quotient_fast(float num, float den) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(den));
    const float q0 = num * r;
    return __fmaf_rn(__fmaf_rn(-den, q0, num), r, q0);
}

// -(num / den) for a (col, row) pair with packed FP32x2 operations: the same steps as
// quotient_fast with the reciprocal's sign flipped (nr = -r, q0n = -q0), so the residual
// num - den q0 = fma(den, q0n, num) and the result -(q0 + e r) = fma(e, nr, q0n) need no
// negated operand -- every product and sum is the scalar form's, negated exactly.
__device__ __forceinline__ float2 quotient2_neg(float2 num, float2 den) {
    float2 nr;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(nr.x) : "f"(-den.x));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(nr.y) : "f"(-den.y));
    const float2 q0n = __fmul2_rn(num, nr);
    const float2 e = __ffma2_rn(den, q0n, num);
    return __ffma2_rn(e, nr, q0n);
}

// The epilogue of one tile for one warp: its lanes are 32 points of the tile (the TMEM
// lanes of the warp's quarter), its cameras [c_begin, c_end) those of its warpgroup, taken
// CH at a time (CH even: a tcgen05.ld of 8 columns covers two cameras).  A camera's col and
// row travel as one FP32x2 pair through the linear terms (LIN), the quotient and the
// denormalisation (packed FFMA2/FMUL2/FADD2, IEEE round-to-nearest per lane, so the
// values equal the scalar form's); one warp-uniform range test per chunk (denominators in
// (1/2, 3/2), numerators below 1e30: min/max reductions, which NaN cannot trip and an
// infinity always does) sends a chunk holding a rare operand to the per-lane test and
// IEEE division.
template <bool LIN, int CH>
__device__ __forceinline__ void tc_epilogue(unsigned lane_base, int c_begin, int c_end, long long p, long long n,
                                            float2 x2, float2 y2, float2 z2, const float4 *sdn, const float4 *slin,
                                            float *__restrict__ out) {
    for (int cb = c_begin; cb < c_end; cb += CH) {
        unsigned r[CH / 2][8];
#pragma unroll
        for (int j = 0; j < CH / 2; ++j) {
            if (cb + 2 * j < c_end) {
                tmem_ld8(lane_base + 4 * (cb + 2 * j), r[j]);   // warp-uniform
            } else {
#pragma unroll
                for (int k = 0; k < 8; ++k) r[j][k] = 0u;
            }
        }
        tmem_wait();
        const int nc = min(CH, c_end - cb);
        float2 num[CH], den[CH];
        float dmin = 1.0f, dmax = 1.0f, nmax = 0.0f;
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            const unsigned *w4 = &r[c >> 1][4 * (c & 1)];     // colNum, colDen, rowNum, rowDen
            float2 nu = make_float2(__uint_as_float(w4[0]), __uint_as_float(w4[2]));
            float2 de = make_float2(__uint_as_float(w4[1]), __uint_as_float(w4[3]));
            if (LIN) {      // + z, + x, + y terms, then the constant (within slin's 64 cameras)
                const float4 *lc = slin + 4 * (cb + c);
                const float4 l3 = lc[3], l2 = lc[2], l1 = lc[1], l0 = lc[0];
                nu = __ffma2_rn(make_float2(l3.x, l3.y), z2, nu);
                de = __ffma2_rn(make_float2(l3.z, l3.w), z2, de);
                nu = __ffma2_rn(make_float2(l2.x, l2.y), x2, nu);
                de = __ffma2_rn(make_float2(l2.z, l2.w), x2, de);
                nu = __ffma2_rn(make_float2(l1.x, l1.y), y2, nu);
                de = __ffma2_rn(make_float2(l1.z, l1.w), y2, de);
                nu = __fadd2_rn(nu, make_float2(l0.x, l0.y));
                de = __fadd2_rn(de, make_float2(l0.z, l0.w));
            }
            if (c < nc) {
                dmin = fminf(dmin, fminf(de.x, de.y));
                dmax = fmaxf(dmax, fmaxf(de.x, de.y));
                nmax = fmaxf(nmax, fmaxf(fabsf(nu.x), fabsf(nu.y)));
            }
            num[c] = nu;
            den[c] = de;
        }
        float2 qn[CH];                                   // -(num / den)
        if (__builtin_expect(__all_sync(0xffffffffu, dmin > 0.5f && dmax < 1.5f && nmax < 1e30f), 1)) {
#pragma unroll
            for (int c = 0; c < CH; ++c) qn[c] = quotient2_neg(num[c], den[c]);
        } else {
#pragma unroll
            for (int c = 0; c < CH; ++c) {
                qn[c].x = -(quotient_fast_ok(num[c].x, den[c].x) ? quotient_fast(num[c].x, den[c].x)
                                                                 : tc_quotient_ieee(num[c].x, den[c].x));
                qn[c].y = -(quotient_fast_ok(num[c].y, den[c].y) ? quotient_fast(num[c].y, den[c].y)
                                                                 : tc_quotient_ieee(num[c].y, den[c].y));
            }
        }
        if (p < n) {
            float *o = out + (2LL * cb) * n + p;     // camera cb's col plane; its row plane follows
#pragma unroll
            for (int c = 0; c < CH; ++c, o += 2 * n) {
                if (c < nc) {
                    const float4 sd = sdn[cb + c];   // (-col_scale, -row_scale, col_off, row_off)
                    const float2 v = __ffma2_rn(qn[c], make_float2(sd.x, sd.y), make_float2(sd.z, sd.w));
                    __stcs(o, v.x);
                    __stcs(o + n, v.y);
                }
            }
        }
    }
}

template <bool LIN>
__global__ void __launch_bounds__(kTcThreads, 1) cube_tc_kernel(const float *__restrict__ xyz, long long n, int n_cams,
                                                               int n_pad, CubeTcWs w, float *__restrict__ out,
                                                               unsigned wait_limit) {
    using S = TcScheme<LIN>;
    constexpr unsigned kStageBytes = kTcTile * S::kRowBytes;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sb = smem;                                           // B: n_pad x K
    unsigned char *sa = sb + kTcMaxN * S::kRowBytes;                    // A ring: kTcStages x 128 x K
    float4 *sden = reinterpret_cast<float4 *>(sa + kTcStages * kStageBytes);
    float4 *slin = sden + kTcMaxCams;
    // mbarriers: A full / empty per stage, accumulator full / empty, B landed, final drain
    __shared__ __align__(8) unsigned long long bars[2 * kTcStages + 6];
    __shared__ unsigned tmem_base;
    __shared__ volatile int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const unsigned bar0 = smem_addr(&bars[0]);
    auto a_full = [&](int st) { return bar0 + 8u * st; };
    auto a_empty = [&](int st) { return bar0 + 8u * (kTcStages + st); };
    auto acc_full = [&](int a) { return bar0 + 8u * (2 * kTcStages + a); };
    auto acc_empty = [&](int a) { return bar0 + 8u * (2 * kTcStages + 2 + a); };
    const unsigned bar_b = bar0 + 8u * (2 * kTcStages + 4), bar_drain = bar0 + 8u * (2 * kTcStages + 5);
    const unsigned b_bytes = static_cast<unsigned>(n_pad * S::kRowBytes);
    if (tid == 0) {
        for (int st = 0; st < kTcStages; ++st) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a_full(st)), "r"(kTcProducerWarps * 32) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a_empty(st)) : "memory");
        }
        for (int a = 0; a < 2; ++a) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(acc_full(a)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(acc_empty(a)), "r"(kTcEpiWarps) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_b) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_drain) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        abort_flag = 0;
        // B into shared memory by the bulk-copy engine (16-byte aligned, size a multiple of 16)
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_b), "r"(b_bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_addr(sb)),
            "l"(w.b), "r"(b_bytes), "r"(bar_b)
            : "memory");
    }
    for (int i = tid; i < n_cams; i += kTcThreads) sden[i] = w.den[i];
    if (LIN)
        for (int i = tid; i < 4 * n_cams; i += kTcThreads) slin[i] = w.lin[i];
    if (warp == kTcMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = tmem_base;
    const long long tiles = (n + kTcTile - 1) / kTcTile;
    const long long my_tiles = tiles > blockIdx.x ? (tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    bool failed = false;
    if (warp < kTcProducerWarps) {
        // ---- producers: thread t builds rows t and t + 64 of every tile's A operand
        constexpr int kRows = kTcTile / (32 * kTcProducerWarps);
        float nx[kRows], ny[kRows], nz[kRows];
#pragma unroll
        for (int h = 0; h < kRows; ++h) {
            const long long p = static_cast<long long>(blockIdx.x) * kTcTile + tid + 32 * kTcProducerWarps * h;
            nx[h] = ny[h] = nz[h] = 0.0f;
            if (p < n) {
                nx[h] = __ldg(xyz + p);
                ny[h] = __ldg(xyz + n + p);
                nz[h] = __ldg(xyz + 2 * n + p);
            }
        }
        for (long long k = 0; k < my_tiles; ++k) {
            const int st = static_cast<int>(k % kTcStages);
            const unsigned ph = static_cast<unsigned>((k / kTcStages) & 1);
            float cx[kRows], cy[kRows], cz[kRows];
#pragma unroll
            for (int h = 0; h < kRows; ++h) {
                cx[h] = nx[h];
                cy[h] = ny[h];
                cz[h] = nz[h];
                const long long p = (blockIdx.x + (k + 1) * gridDim.x) * kTcTile + tid + 32 * kTcProducerWarps * h;
                nx[h] = ny[h] = nz[h] = 0.0f;                // the next tile's points, in flight meanwhile
                if (p < n) {
                    nx[h] = __ldg(xyz + p);
                    ny[h] = __ldg(xyz + n + p);
                    nz[h] = __ldg(xyz + 2 * n + p);
                }
            }
            const bool ok = __all_sync(0xffffffffu, mbar_wait_abortable(a_empty(st), ph ^ 1u, wait_limit, &abort_flag));
            if (!ok) {
                failed = true;
                break;
            }
#pragma unroll
            for (int h = 0; h < kRows; ++h)
                build_a_row<LIN>(sa + st * kStageBytes, tid + 32 * kTcProducerWarps * h, cx[h], cy[h], cz[h]);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // visible to the tensor cores
            mbar_arrive(a_full(st));
        }
    } else if (warp == kTcMmaWarp) {
        // ---- MMA issuer (lane 0)
        if (lane == 0) {
            const unsigned idesc = umma_idesc_bf16(n_pad);
            const unsigned sbo = static_cast<unsigned>(S::kK / 8 * 128);
            const unsigned b_base = smem_addr(sb), a_base0 = smem_addr(sa);
            failed = !mbar_wait_abortable(bar_b, 0, wait_limit, &abort_flag);
            for (long long k = 0; !failed && k < my_tiles; ++k) {
                const int st = static_cast<int>(k % kTcStages), acc = static_cast<int>(k & 1);
                const unsigned ph = static_cast<unsigned>((k / kTcStages) & 1), aph = static_cast<unsigned>((k >> 1) & 1);
                if (!mbar_wait_abortable(a_full(st), ph, wait_limit, &abort_flag) ||
                    !mbar_wait_abortable(acc_empty(acc), aph ^ 1u, wait_limit, &abort_flag)) {
                    failed = true;
                    break;
                }
                tc_fence_after();
                const unsigned d = tmem + static_cast<unsigned>(acc * 256);
                const unsigned a_base = a_base0 + static_cast<unsigned>(st) * kStageBytes;
#pragma unroll
                for (int ks = 0; ks < S::kK / 16; ++ks)
                    umma_bf16(d, umma_desc(a_base + ks * 256, 128, sbo), umma_desc(b_base + ks * 256, 128, sbo), idesc,
                              ks > 0 ? 1u : 0u);
                umma_commit(a_empty(st));          // the stage is free once these MMAs have read it
                umma_commit(acc_full(acc));        // and the accumulator holds the tile
            }
        }
        __syncwarp();
    } else {
        // ---- epilogue: warp e handles TMEM lane quarter (warp % 4) for camera group e / 4
        const int e = warp - kTcProducerWarps - 1, quad = warp & 3, grp = e >> 2;
        const int c_begin = min(((grp * n_cams / kTcGroups) + 1) & ~1, n_cams);
        const int c_end = min((((grp + 1) * n_cams / kTcGroups) + 1) & ~1, n_cams);
        const int row = quad * 32 + lane;
        float nx = 0.0f, ny = 0.0f, nz = 0.0f;
        if (LIN) {
            const long long p = static_cast<long long>(blockIdx.x) * kTcTile + row;
            if (p < n) {
                nx = __ldg(xyz + p);
                ny = __ldg(xyz + n + p);
                nz = __ldg(xyz + 2 * n + p);
            }
        }
        for (long long k = 0; k < my_tiles; ++k) {
            const int acc = static_cast<int>(k & 1);
            const unsigned aph = static_cast<unsigned>((k >> 1) & 1);
            const long long tile = blockIdx.x + k * gridDim.x;
            const float cx = nx, cy = ny, cz = nz;
            if (LIN) {
                const long long p = (tile + gridDim.x) * kTcTile + row;   // next tile's point
                nx = ny = nz = 0.0f;
                if (p < n) {
                    nx = __ldg(xyz + p);
                    ny = __ldg(xyz + n + p);
                    nz = __ldg(xyz + 2 * n + p);
                }
            }
            const bool ok = __all_sync(0xffffffffu, mbar_wait_abortable(acc_full(acc), aph, wait_limit, &abort_flag));
            if (!ok) {
                failed = true;
                break;
            }
            tc_fence_after();
            const unsigned lane_base = tmem + (static_cast<unsigned>(quad * 32) << 16) + static_cast<unsigned>(acc * 256);
            tc_epilogue<LIN, 4>(lane_base, c_begin, c_end, tile * kTcTile + row, n, make_float2(cx, cx),
                                make_float2(cy, cy), make_float2(cz, cz), sden, slin, out);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty(acc));
        }
    }
    if (failed) {
        abort_flag = 1;
        atomicExch(w.err, 1);
    }
    // the coefficient copy and every committed MMA have completed before the CTA's shared
    // and tensor memory are released (bounded waits, full limit)
    tc_fence_before();
    __syncthreads();
    if (tid == kTcMmaWarp * 32) {
        mbar_wait_bounded(bar_b, 0);
        umma_commit(bar_drain);
        mbar_wait_bounded(bar_drain, 0);
    }
    __syncthreads();
    tc_fence_after();
    if (warp == kTcMmaWarp)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols) : "memory");
}

template <bool LIN>
size_t cube_tc_smem() {
    using S = TcScheme<LIN>;
    // at least half of the SM's shared memory: one CTA per SM, which owns all 512 TMEM columns
    const size_t need = static_cast<size_t>(kTcMaxN + kTcStages * kTcTile) * S::kRowBytes + sizeof(float4) * kTcMaxCams +
                        sizeof(float4) * 4 * kTcMaxCams + 1024;
    return std::max<size_t>(need, 120 * 1024);
}

}  // namespace

// Polls of a completion wait before a thread gives up (vs_set_tc_wait_limit; 0 makes the
// first wait of every CTA give up at once, which exercises the timeout path).
unsigned g_tc_wait_limit = kWaitLimit;

size_t cube_tc_workspace_bytes(int n_cams) {
    Carver cv(nullptr);
    cv.take<__nv_bfloat16>(static_cast<size_t>(kTcMaxN) * 64);
    cv.take<float4>(static_cast<size_t>(n_cams));
    cv.take<float4>(4 * static_cast<size_t>(n_cams));
    cv.take<int>(1);
    return cv.used + 256;
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

template <bool LIN>
static int launch_tc(const VsRpcCamera *cams, int n_cams, const float *xyz, long long n, float *colrow, void *ws,
                     cudaStream_t st) {
    const int n_pad = tc_n_pad(n_cams);
    if (n_cams > kTcMaxCams) {
        set_error("vs_rpc_project_cube: the tcgen05 variants take at most %d cameras (%d given)", kTcMaxCams, n_cams);
        return VS_ERR_ARG;
    }
    const CubeTcWs w = carve_cube_tc(ws, n_cams);
    if (cudaMemsetAsync(w.err, 0, sizeof(int), st) != cudaSuccess) {
        set_error("vs_rpc_project_cube: cudaMemsetAsync failed");
        return VS_ERR_CUDA;
    }
    cube_tc_prepare_kernel<LIN><<<static_cast<unsigned>(ceil_div(static_cast<int64_t>(n_pad) * TcScheme<LIN>::kK, 256)),
                                   256, 0, st>>>(cams, n_cams, n_pad, w);
    VS_LAUNCH_CHECK("cube_tc_prepare_kernel");
    const size_t sh = cube_tc_smem<LIN>();
    if (cudaFuncSetAttribute(cube_tc_kernel<LIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sh)) !=
        cudaSuccess) {
        set_error("vs_rpc_project_cube: shared memory request of %zu bytes refused", sh);
        return VS_ERR_CUDA;
    }
    const long long tiles = ceil_div(n, static_cast<long long>(kTcTile));
    const unsigned grid = static_cast<unsigned>(std::max(1LL, std::min<long long>(tiles, sm_count())));
    cube_tc_kernel<LIN><<<grid, kTcThreads, sh, st>>>(xyz, n, n_cams, n_pad, w, colrow, g_tc_wait_limit);
    VS_LAUNCH_CHECK("cube_tc_kernel");
    return VS_OK;
}

int launch_cube_tc(const VsRpcCamera *cams, int n_cams, const float *xyz, long long n, float *colrow, void *ws,
                   cudaStream_t st, bool lin) {
    return lin ? launch_tc<true>(cams, n_cams, xyz, n, colrow, ws, st)
               : launch_tc<false>(cams, n_cams, xyz, n, colrow, ws, st);
}

}  // namespace vs

extern "C" void vs_set_tc_wait_limit(unsigned polls) { vs::g_tc_wait_limit = polls; }
