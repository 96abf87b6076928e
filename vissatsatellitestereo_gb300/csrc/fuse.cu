// (d) Fusion of per-view DSMs: the inline block of run_fuse (aggregate_2p5d.py:65-81).
//
// Per cell over the V views (float32, NaN = no measurement):
//   n = #valid; n <= 2 -> NaN                                    (aggregate_2p5d.py:69-71)
//   med = nanmedian: sorted s, ((0 + s[(n-1)/2]) + s[n/2]) / 2    (:74, numpy masked median)
//   mad = nanmedian(|x - med|)                                    (:75)
//   drop x with |x - med| > mad                                   (:76-77)
//   mean = nanmean: NaN -> 0, numpy's float32 pairwise sum over the V slots in view order
//          (8 accumulators for 8 <= V <= 128, halving above), started from 0, then the
//          float32 division by the kept count                     (:78)
// then optionally the 3x3 median blur (:81), launched from raster.cu's blur kernel.
// Views beyond 64 use a local-memory path with the same arithmetic.
#include <algorithm>
#include <math.h>
#include <mutex>

#include "common.cuh"

namespace vs {
int launch_blur_f32(const float *in, float *out, long long h, long long w, cudaStream_t st);

namespace {

__device__ __forceinline__ float median_of_sorted(unsigned lo_key, unsigned hi_key) {
    const float lo = float_from_key(lo_key), hi = float_from_key(hi_key);
    return __fdiv_rn(__fadd_rn(__fadd_rn(0.0f, lo), hi), 2.0f);
}

// ---- V > 64: same arithmetic with local arrays -----------------------------------------
// numpy's pairwise block of n <= 128 values: 8 accumulators, combined in a tree, then the
// tail (n < 8: a plain sequential sum from 0).
__device__ __forceinline__ float pairwise_block(const float *x, int n) {
    float res;
    if (n < 8) {
        res = 0.0f;
        for (int i = 0; i < n; ++i) res = __fadd_rn(res, x[i]);
        return res;
    }
    float r[8];
    for (int j = 0; j < 8; ++j) r[j] = x[j];
    int i = 8;
    for (; i < n - (n % 8); i += 8)
        for (int j = 0; j < 8; ++j) r[j] = __fadd_rn(r[j], x[i + j]);
    res = __fadd_rn(__fadd_rn(__fadd_rn(r[0], r[1]), __fadd_rn(r[2], r[3])),
                    __fadd_rn(__fadd_rn(r[4], r[5]), __fadd_rn(r[6], r[7])));
    for (; i < n; ++i) res = __fadd_rn(res, x[i]);
    return res;
}

// numpy's halving recursion above 128 values, unrolled at compile time (no call stack):
// D levels of halving cover n <= 128 * 2^D.
template <int D>
__device__ __forceinline__ float pairwise_any(const float *x, int n) {
    if constexpr (D == 0) {
        return pairwise_block(x, n);
    } else {
        if (n <= 128) return pairwise_block(x, n);
        int n2 = n / 2;
        n2 -= n2 % 8;
        return __fadd_rn(pairwise_any<D - 1>(x, n2), pairwise_any<D - 1>(x + n2, n - n2));
    }
}

constexpr int kMaxViewsLocal = 512;

__device__ void insertion_sort(unsigned *a, int n) {
    for (int i = 1; i < n; ++i) {
        unsigned v = a[i];
        int j = i - 1;
        while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
        a[j + 1] = v;
    }
}

__global__ void fuse_kernel_large(const float *__restrict__ dsm, int layout, int V, long long cells,
                                  float *__restrict__ out) {
    float x[kMaxViewsLocal];
    unsigned k[kMaxViewsLocal];
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < cells;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        int n = 0;
        for (int i = 0; i < V; ++i) {
            x[i] = layout == VS_LAYOUT_VHW ? dsm[i * cells + c] : dsm[c * V + i];
            if (!isnan(x[i])) k[n++] = key_from_float(x[i]);
        }
        if (n <= 2) { out[c] = __int_as_float(0x7fffffff); continue; }
        insertion_sort(k, n);
        const float med = median_of_sorted(k[(n - 1) >> 1], k[n >> 1]);
        int nd = 0;
        for (int i = 0; i < V; ++i)
            if (!isnan(x[i])) {
                float d = fabsf(__fsub_rn(x[i], med));
                if (!isnan(d)) k[nd++] = key_from_float(d);
            }
        float mad = __int_as_float(0x7fffffff);
        if (nd > 0) {
            insertion_sort(k, nd);
            mad = median_of_sorted(k[(nd - 1) >> 1], k[nd >> 1]);
        }
        int cnt = 0;
        for (int i = 0; i < V; ++i) {
            bool keep = !isnan(x[i]) && !(fabsf(__fsub_rn(x[i], med)) > mad);
            cnt += keep;
            x[i] = keep ? x[i] : 0.0f;
        }
        const float tot = __fadd_rn(0.0f, pairwise_any<4>(x, V));   // 4 levels: V <= 2048
        out[c] = __fdiv_rn(tot, static_cast<float>(cnt));
    }
}

// ---- fusion for V <= 64 -------------------------------------------------------------------
// One thread fuses one cell:
//   * its V values as float32 with NaN replaced by +inf: the valid values are the n
//     smallest slots (ties with a valid +inf are the same value), so no key conversion is
//     needed, and the sign of a zero cannot change ((0 + lo) + hi) / 2, |x - med| or the
//     mask;
//   * Batcher's odd-even merge sort on N = V rounded up to 4 slots, derived from the
//     64-slot network by dropping the comparators that touch a slot >= N (those slots hold
//     +inf and every comparator puts its maximum on the higher slot, so they never change);
//   * the sorted values go to a per-thread column of shared memory, from which the
//     median's two middle order statistics are read;
//   * with a finite median m, the deviations of the sorted values split into two sorted
//     runs: fl(med - s) for the values left of the middle (ascending from the middle out)
//     and fl(s - med) for those right of it (fl(x - med) is monotone in x).  The MAD's
//     order statistics are the k-th and (k+1)-th smallest of the two runs: a binary search
//     over how many come from the left run (merge path), reading the column;
//   * the keep mask and numpy's pairwise mean read the values again in view order.
// The main kernel stages each tile of 128 cells (its V view rows, or its 128 x V block in
// the [H][W][V] layout) in shared memory with cp.async (the hardware tracks completion:
// no spin waits); each thread sorts its cell into its column of a view-major scratch
// block beside the tile (conflict-free) and reads the originals for the mean from the
// tile.  Stacks whose view rows are not 16-byte aligned are staged with 4-byte copies.
constexpr int kTileCells = 128;

__device__ __forceinline__ void cp_async16(float *smem_dst, const float *gmem_src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async4(float *smem_dst, const float *gmem_src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cmpx(float (&a)[N], int i, int l) {
    const float lo = fminf(a[i], a[l]);
    a[l] = fmaxf(a[i], a[l]);
    a[i] = lo;
}

constexpr int pow2_ceil(int n) { return n <= 1 ? 1 : 2 * pow2_ceil((n + 1) / 2); }

// Batcher's odd-even merge sort network for N slots as a compile-time comparator list: the
// power-of-two network without the comparators that touch a slot >= N.
template <int N>
struct OemsNet {
    static constexpr int kP2 = pow2_ceil(N);
    static constexpr int kMax = 544;          // comparators of the 64-slot network
    int n = 0;
    unsigned char i[kMax] = {}, l[kMax] = {};
    constexpr OemsNet() {
        for (int p = 1; p < kP2; p <<= 1)
            for (int k = p; k >= 1; k >>= 1)
                for (int j = k % p; j + k <= kP2 - 1; j += 2 * k)
                    for (int q = 0; q < k; ++q)
                        if (q + j + k < N && (q + j) / (2 * p) == (q + j + k) / (2 * p)) {
                            i[n] = static_cast<unsigned char>(q + j);
                            l[n] = static_cast<unsigned char>(q + j + k);
                            ++n;
                        }
    }
};

// Sorts a[0..N) ascending (slots beyond the valid count hold +inf).
template <int N>
__device__ __forceinline__ void oems_sort(float (&a)[N]) {
    constexpr OemsNet<N> net{};
    constexpr int kCount = net.n;
#pragma unroll
    for (int c = 0; c < kCount; ++c) cmpx(a, net.i[c], net.l[c]);
}

__device__ __forceinline__ float median_pair(float lo, float hi) {
    return __fdiv_rn(__fadd_rn(__fadd_rn(0.0f, lo), hi), 2.0f);
}

// The cell's values: value i at xs[i * si] (shared memory or global); sorted values are
// written to srt[i * ss] (shared memory); the values are read again, in view order, at
// xg[i * sg].
template <int N>
__device__ __forceinline__ float fuse_cell_v64(const float *xs, long long si, int V, float *srt, int ss,
                                               const float *__restrict__ xg, long long sg) {
    const float inf = __int_as_float(0x7f800000);
    float a[N];
    int n = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        float v = inf;
        if (i < V) {
            const float x = xs[i * si];
            const bool ok = !isnan(x);
            n += ok;
            v = ok ? x : inf;
        }
        a[i] = v;
    }
    if (n <= 2) return __int_as_float(0x7fffffff);
    oems_sort(a);
#pragma unroll
    for (int i = 0; i < N; ++i)
        if (i < V) srt[i * ss] = a[i];
    const float med = median_pair(srt[((n - 1) >> 1) * ss], srt[(n >> 1) * ss]);
    float mad = __int_as_float(0x7fffffff);
    if (isfinite(med)) {
        // left run A_j = med - s[m-1-j] (j < m), right run B_j = s[m+j] - med (j < n-m)
        const int m = (n & 1) ? (n - 1) >> 1 : n >> 1, nb = n - m;
        const float *left = srt + (m - 1) * ss, *right = srt + m * ss;
        const int k = (n - 1) >> 1;
        int lo = max(0, k + 1 - nb), hi = min(k + 1, m);
        while (lo < hi) {
            const int i = (lo + hi) >> 1, j = k + 1 - i;
            if (__fsub_rn(med, left[-i * ss]) < __fsub_rn(right[(j - 1) * ss], med)) lo = i + 1;
            else hi = i;
        }
        const int i = lo, j = k + 1 - i;
        const float a_last = i > 0 ? __fsub_rn(med, left[-(i - 1) * ss]) : -inf;
        const float b_last = j > 0 ? __fsub_rn(right[(j - 1) * ss], med) : -inf;
        const float kth = fmaxf(a_last, b_last);
        float nxt = kth;
        if (!(n & 1)) {
            const float a_next = i < m ? __fsub_rn(med, left[-i * ss]) : inf;
            const float b_next = j < nb ? __fsub_rn(right[j * ss], med) : inf;
            nxt = fminf(a_next, b_next);
        }
        mad = median_pair(kth, nxt);
    } else {
        // deviations of the original values (inf - inf is NaN: missing)
        int nd = 0;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float v = inf;
            if (i < V) {
                const float d = fabsf(__fsub_rn(xg[i * sg], med));
                const bool ok = !isnan(d);
                nd += ok;
                v = ok ? d : inf;
            }
            a[i] = v;
        }
        if (nd > 0) {
            oems_sort(a);
#pragma unroll
            for (int i = 0; i < N; ++i)
                if (i < V) srt[i * ss] = a[i];
            mad = median_pair(srt[((nd - 1) >> 1) * ss], srt[(nd >> 1) * ss]);
        }
    }
    // keep |x - med| <= mad (NaN compares false), then numpy's float32 pairwise sum of the
    // kept values (others 0) over the V slots in view order, from 0, / kept count
    int cnt = 0;
    auto kept = [&](int i, float &acc) {
        const float x = xg[i * sg];
        const bool keep = !isnan(x) && !(fabsf(__fsub_rn(x, med)) > mad);
        cnt += keep;
        acc = __fadd_rn(acc, keep ? x : 0.0f);
    };
    float res;
    if (V < 8) {
        res = 0.0f;
#pragma unroll
        for (int i = 0; i < (N < 8 ? N : 8); ++i)
            if (i < V) kept(i, res);
    } else {
        float r[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            r[j] = -0.0f;          // -0 + x == x for every x: the first kept value seeds r[j]
            kept(j, r[j]);
        }
        const int full = V - (V % 8);
#pragma unroll
        for (int b = 8; b < N; b += 8)
            if (b < full)
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (b + j < N) kept(b + j, r[j]);
        res = __fadd_rn(__fadd_rn(__fadd_rn(r[0], r[1]), __fadd_rn(r[2], r[3])),
                        __fadd_rn(__fadd_rn(r[4], r[5]), __fadd_rn(r[6], r[7])));
#pragma unroll
        for (int i = 8; i < N; ++i)
            if (i >= full && i < V) kept(i, res);
    }
    return __fdiv_rn(__fadd_rn(0.0f, res), static_cast<float>(cnt));   // cnt == 0 -> 0/0 = NaN
}

template <int N>
__global__ void __launch_bounds__(kTileCells) fuse_tile_kernel(const float *__restrict__ dsm, int layout, int V,
                                                               long long cells, float *__restrict__ out,
                                                               long long n_tiles, int aligned) {
    extern __shared__ __align__(16) float fsm[];           // the tile: V x 128 (VHW) or 128 x V (HWV)
    float *scratch = fsm + V * kTileCells;                 // sorted columns: N x 128
    const int t = threadIdx.x;
    const bool vhw = layout == VS_LAYOUT_VHW;
    for (long long tl = blockIdx.x; tl < n_tiles; tl += gridDim.x) {
        const long long c0 = tl * kTileCells;
        const int len = static_cast<int>(min(static_cast<long long>(kTileCells), cells - c0));   // multiple of 4
        if (aligned) {               // 16-byte copies: rows (VHW) or blocks (HWV) start 16-byte aligned
            if (vhw) {
                const int chunks = len >> 2;
                for (int q = t; q < V * (kTileCells / 4); q += kTileCells) {
                    const int v = q / (kTileCells / 4), ch = q - v * (kTileCells / 4);
                    if (ch < chunks) cp_async16(fsm + v * kTileCells + 4 * ch, dsm + v * cells + c0 + 4 * ch);
                }
            } else {
                const int chunks = (len * V) >> 2;
                for (int q = t; q < chunks; q += kTileCells) cp_async16(fsm + 4 * q, dsm + c0 * V + 4 * q);
            }
        } else if (vhw) {            // 4-byte copies otherwise (a thread per cell, so t < len)
            if (t < len)
                for (int v = 0; v < V; ++v) cp_async4(fsm + v * kTileCells + t, dsm + v * cells + c0 + t);
        } else {
            for (int q = t; q < len * V; q += kTileCells) cp_async4(fsm + q, dsm + c0 * V + q);
        }
        cp_async_commit();
        cp_async_wait_all();
        __syncthreads();
        const long long c = c0 + t;
        if (c < cells) {
            const float *col = vhw ? fsm + t : fsm + t * V;
            const int si = vhw ? kTileCells : 1;
            out[c] = fuse_cell_v64<N>(col, si, V, scratch + t, kTileCells, col, si);
        }
        __syncthreads();                           // the tile is refilled next
    }
}

size_t fuse_tile_smem(int V, int N) { return sizeof(float) * static_cast<size_t>(V + N) * kTileCells; }

template <int N>
bool launch_fuse_v64(const float *dsm, int layout, int V, long long cells, float *out, bool aligned, cudaStream_t st) {
    const size_t sh = fuse_tile_smem(V, N);
    static bool configured = false;     // per instantiation: room for the largest tile (V = N)
    if (!configured) {
        if (cudaFuncSetAttribute(fuse_tile_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(fuse_tile_smem(N, N))) != cudaSuccess)
            return false;
        configured = true;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fuse_tile_kernel<N>, kTileCells, sh) != cudaSuccess ||
        per_sm <= 0)
        return false;
    const long long n_tiles = ceil_div(cells, static_cast<long long>(kTileCells));
    const unsigned g = static_cast<unsigned>(std::min<long long>(n_tiles, 1LL * sm_count() * per_sm));
    fuse_tile_kernel<N><<<g, kTileCells, sh, st>>>(dsm, layout, V, cells, out, n_tiles, aligned ? 1 : 0);
    return true;
}

// 16-byte copies need 16-byte aligned view rows (VHW) or cell blocks (HWV).
bool fuse_tile_aligned(const float *dsm, int layout, int V, long long cells) {
    (void)layout;
    (void)V;
    return (reinterpret_cast<uintptr_t>(dsm) & 15) == 0 && cells % 4 == 0;
}

int launch_fuse_small(const float *dsm, int layout, int V, long long cells, float *out, cudaStream_t st) {
    const bool aligned = fuse_tile_aligned(dsm, layout, V, cells);
    bool ok = false;
    switch ((V + 3) / 4) {
        case 0: case 1: ok = launch_fuse_v64<4>(dsm, layout, V, cells, out, aligned, st); break;
        case 2: ok = launch_fuse_v64<8>(dsm, layout, V, cells, out, aligned, st); break;
        case 3: ok = launch_fuse_v64<12>(dsm, layout, V, cells, out, aligned, st); break;
        case 4: ok = launch_fuse_v64<16>(dsm, layout, V, cells, out, aligned, st); break;
        case 5: ok = launch_fuse_v64<20>(dsm, layout, V, cells, out, aligned, st); break;
        case 6: ok = launch_fuse_v64<24>(dsm, layout, V, cells, out, aligned, st); break;
        case 7: ok = launch_fuse_v64<28>(dsm, layout, V, cells, out, aligned, st); break;
        case 8: ok = launch_fuse_v64<32>(dsm, layout, V, cells, out, aligned, st); break;
        case 9: ok = launch_fuse_v64<36>(dsm, layout, V, cells, out, aligned, st); break;
        case 10: ok = launch_fuse_v64<40>(dsm, layout, V, cells, out, aligned, st); break;
        case 11: ok = launch_fuse_v64<44>(dsm, layout, V, cells, out, aligned, st); break;
        case 12: ok = launch_fuse_v64<48>(dsm, layout, V, cells, out, aligned, st); break;
        case 13: ok = launch_fuse_v64<52>(dsm, layout, V, cells, out, aligned, st); break;
        case 14: ok = launch_fuse_v64<56>(dsm, layout, V, cells, out, aligned, st); break;
        case 15: ok = launch_fuse_v64<60>(dsm, layout, V, cells, out, aligned, st); break;
        default: ok = launch_fuse_v64<64>(dsm, layout, V, cells, out, aligned, st); break;
    }
    if (!ok) {
        set_error("fuse_tile_kernel: launch configuration refused");
        return VS_ERR_CUDA;
    }
    return VS_OK;
}


}  // namespace
}  // namespace vs

using namespace vs;

// Largest grid (cells) the fusion accepts: the float32 grid plus its slack must stay well
// inside int64 (and size_t) arithmetic.
constexpr long long kMaxFuseCells = (1LL << 60) / static_cast<long long>(sizeof(float));

// h * w without overflow: 0 when either side is not positive or the product exceeds `limit`.
static long long checked_cells(int64_t h, int64_t w, long long limit) {
    if (h <= 0 || w <= 0 || h > limit || w > limit / h) return 0;
    return static_cast<long long>(h) * w;
}

extern "C" size_t vs_fuse_dsms_workspace_size(int64_t h, int64_t w) {
    const long long cells = checked_cells(h, w, kMaxFuseCells);
    if (!cells) return 0;
    return sizeof(float) * static_cast<size_t>(cells) + 256;
}

extern "C" int vs_fuse_dsms(const float *dsm, int layout, int64_t n_views, int64_t h, int64_t w, float *out,
                            int median_blur, void *workspace, size_t workspace_bytes, void *stream) {
    VS_REQUIRE(checked_cells(h, w, kMaxFuseCells) > 0 && n_views > 0 && n_views <= kMaxViewsLocal,
               "vs_fuse_dsms: bad sizes views=%lld grid=%lldx%lld", (long long)n_views, (long long)h,
               (long long)w);
    VS_REQUIRE(layout == VS_LAYOUT_HWV || layout == VS_LAYOUT_VHW, "vs_fuse_dsms: bad layout %d", layout);
    VS_REQUIRE(dsm && out, "vs_fuse_dsms: null pointer");
    cudaStream_t st = as_stream(stream);
    const long long cells = h * w;
    float *dst = out;
    if (median_blur) {
        const size_t need = vs_fuse_dsms_workspace_size(h, w);
        VS_REQUIRE(workspace, "vs_fuse_dsms: median_blur needs a workspace");
        if (workspace_bytes < need) {
            set_error("vs_fuse_dsms: workspace %zu < %zu bytes", workspace_bytes, need);
            return VS_ERR_WORKSPACE;
        }
        dst = static_cast<float *>(workspace);
    }
    const int V = static_cast<int>(n_views);
    if (V <= 64) {
        const int s = launch_fuse_small(dsm, layout, V, cells, dst, st);
        if (s != VS_OK) return s;
    } else {
        const int threads = 64;
        unsigned g = static_cast<unsigned>(std::min<long long>(ceil_div(cells, threads), sm_count() * 8LL));
        fuse_kernel_large<<<g, threads, 0, st>>>(dsm, layout, V, cells, dst);
    }
    VS_LAUNCH_CHECK("fuse_kernel");
    if (median_blur) return launch_blur_f32(dst, out, h, w, st);
    return VS_OK;
}

// ---- fusion without any device allocation -------------------------------------------------
// Some callers cannot allocate device memory where they call the fusion: code running in a
// stream-ordered pipeline that forbids allocation after start-up, or a foreign host with no
// device allocator of its own.  vs_fuse_dsms_static keeps the blur's intermediate grid in
// this file-scope array instead of a caller workspace.  Every GPU that loads the library
// holds the array (16 MiB) until the process exits.
static __device__ __align__(256) float g_fuse_scratch[VS_FUSE_STATIC_MAX_CELLS + 64];   // + vs_fuse_dsms' 256 B slack

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
float *g_scratch_ptr[kMaxDevices] = {};
}  // namespace

extern "C" int vs_fuse_dsms_static(const float *dsm, int layout, int64_t n_views, int64_t h, int64_t w, float *out,
                                   int median_blur, void *stream) {
    VS_REQUIRE(h > 0 && w > 0, "vs_fuse_dsms_static: bad grid %lldx%lld", (long long)h, (long long)w);
    // h and w are bounded before they are multiplied, so no product can wrap
    VS_REQUIRE(checked_cells(h, w, VS_FUSE_STATIC_MAX_CELLS) > 0,
               "vs_fuse_dsms_static: grid %lldx%lld exceeds the static scratch of %d cells", (long long)h,
               (long long)w, VS_FUSE_STATIC_MAX_CELLS);
    if (!median_blur) return vs_fuse_dsms(dsm, layout, n_views, h, w, out, 0, nullptr, 0, stream);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_error("vs_fuse_dsms_static: no usable current device");
        return VS_ERR_CUDA;
    }
    float *scratch = nullptr;
    {
        // device address of the array on the current device, looked up once per device
        // (the array's name in host code is only a host-side stand-in)
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_ptr[dev]) {
            const cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void **>(&g_scratch_ptr[dev]), g_fuse_scratch);
            if (e != cudaSuccess) {
                g_scratch_ptr[dev] = nullptr;
                set_error("vs_fuse_dsms_static: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
                return VS_ERR_CUDA;
            }
        }
        scratch = g_scratch_ptr[dev];
    }
    // the fusion kernel writes every cell of the scratch grid before the blur reads it, so
    // nothing has to be cleared between calls
    return vs_fuse_dsms(dsm, layout, n_views, h, w, out, 1, scratch,
                        sizeof(float) * static_cast<size_t>(VS_FUSE_STATIC_MAX_CELLS + 64), stream);
}
