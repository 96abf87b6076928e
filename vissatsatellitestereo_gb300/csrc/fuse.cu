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
//
// One thread owns one cell; the V values live in registers (V padded to a power of two,
// template parameter) and are sorted with a bitonic network on order-preserving integer
// keys (NaN -> all ones, so missing values sort last); the MAD's deviations, taken in
// sorted order, form a bitonic sequence and need only the merge half of the network.
// Views beyond 64 use a local-memory path with the same arithmetic.
#include <algorithm>
#include <math.h>
#include <mutex>

#include "common.cuh"

namespace vs {
int launch_blur_f32(const float *in, float *out, long long h, long long w, cudaStream_t st);

namespace {

constexpr unsigned kMissing = 0xffffffffu;

__device__ __forceinline__ unsigned fkey(float v) { return isnan(v) ? kMissing : key_from_float(v); }

template <int N>
__device__ __forceinline__ void bitonic_sort(unsigned (&a)[N]) {
#pragma unroll
    for (int k = 2; k <= N; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned lo = min(a[i], a[l]), hi = max(a[i], a[l]);
                    if ((i & k) == 0) { a[i] = lo; a[l] = hi; }
                    else { a[i] = hi; a[l] = lo; }
                }
            }
}

// Sorts a bitonic sequence (a cyclic shift of non-decreasing then non-increasing, e.g.
// non-increasing then non-decreasing) ascending: the merge half of the bitonic network.
template <int N>
__device__ __forceinline__ void bitonic_merge(unsigned (&a)[N]) {
#pragma unroll
    for (int j = N >> 1; j > 0; j >>= 1)
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const int l = i ^ j;
            if (l > i) {
                const unsigned lo = min(a[i], a[l]), hi = max(a[i], a[l]);
                a[i] = lo;
                a[l] = hi;
            }
        }
}

// select sorted[idx] with compile-time indexing (keeps the array in registers)
template <int N>
__device__ __forceinline__ unsigned pick(const unsigned (&a)[N], int idx) {
    unsigned r = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) r = (i == idx) ? a[i] : r;
    return r;
}

__device__ __forceinline__ float median_of_sorted(unsigned lo_key, unsigned hi_key) {
    const float lo = float_from_key(lo_key), hi = float_from_key(hi_key);
    return __fdiv_rn(__fadd_rn(__fadd_rn(0.0f, lo), hi), 2.0f);
}

// numpy float32 pairwise sum of the first V entries of x (V <= 128), plus the outer 0.
template <int N>
__device__ __forceinline__ float numpy_sum(const float (&x)[N], int V) {
    float res;
    if (V < 8) {
        res = 0.0f;
#pragma unroll
        for (int i = 0; i < (N < 8 ? N : 8); ++i)
            if (i < V) res = __fadd_rn(res, x[i]);
    } else {
        float r[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = (j < N) ? x[j] : 0.0f;
        const int full = V - (V % 8);
#pragma unroll
        for (int b = 8; b < N; b += 8)
            if (b < full)
#pragma unroll
                for (int j = 0; j < 8; ++j) r[j] = __fadd_rn(r[j], x[(b + j) < N ? b + j : 0]);
        res = __fadd_rn(__fadd_rn(__fadd_rn(r[0], r[1]), __fadd_rn(r[2], r[3])),
                        __fadd_rn(__fadd_rn(r[4], r[5]), __fadd_rn(r[6], r[7])));
#pragma unroll
        for (int i = 8; i < N; ++i)
            if (i >= full && i < V) res = __fadd_rn(res, x[i]);
    }
    return __fadd_rn(0.0f, res);
}

template <int N>
__device__ float fuse_cell(const float (&x)[N], int V) {
    unsigned k[N];
    int n = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        k[i] = (i < V) ? fkey(x[i]) : kMissing;
        n += (k[i] != kMissing);
    }
    if (n <= 2) return __int_as_float(0x7fffffff);
    bitonic_sort(k);
    const float med = median_of_sorted(pick(k, (n - 1) >> 1), pick(k, n >> 1));
    // deviations |x - med| of the valid values; NaN deviations (inf - inf) are missing.
    // With a finite median, the deviations of the sorted values are non-increasing up to
    // the median and non-decreasing after it (fl(x - med) is monotone in x), and the missing
    // slots sort last: a bitonic sequence, so one merge sorts it.
    unsigned dk[N];
    int nd = 0;
    float mad = __int_as_float(0x7fffffff);
    if (isfinite(med)) {
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const float d = fabsf(__fsub_rn(float_from_key(k[i]), med));
            dk[i] = (k[i] != kMissing) ? fkey(d) : kMissing;
        }
        nd = n;
        bitonic_merge(dk);
        mad = median_of_sorted(pick(dk, (nd - 1) >> 1), pick(dk, nd >> 1));
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float d = (i < V && !isnan(x[i])) ? fabsf(__fsub_rn(x[i], med)) : __int_as_float(0x7fffffff);
            dk[i] = fkey(d);
            nd += (dk[i] != kMissing);
        }
        if (nd > 0) {
            bitonic_sort(dk);
            mad = median_of_sorted(pick(dk, (nd - 1) >> 1), pick(dk, nd >> 1));
        }
    }
    float kept[N];
    int cnt = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        bool keep = false;
        if (i < V && !isnan(x[i])) {
            const float d = fabsf(__fsub_rn(x[i], med));
            keep = !(d > mad);
        }
        kept[i] = keep ? x[i] : 0.0f;
        cnt += keep;
    }
    const float tot = numpy_sum(kept, V);
    return __fdiv_rn(tot, static_cast<float>(cnt));   // cnt == 0 -> 0/0 = NaN
}

template <int N>
__global__ void __launch_bounds__(128) fuse_kernel(const float *__restrict__ dsm, int layout, int V,
                                                   long long cells, float *__restrict__ out) {
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < cells;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        float x[N];
        if (layout == VS_LAYOUT_VHW) {
#pragma unroll
            for (int i = 0; i < N; ++i) x[i] = (i < V) ? __ldcs(dsm + i * cells + c) : 0.0f;
        } else {
            const float *p = dsm + c * V;
#pragma unroll
            for (int i = 0; i < N; ++i) x[i] = (i < V) ? __ldcs(p + i) : 0.0f;
        }
        out[c] = fuse_cell(x, V);
    }
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

// ---- tile-staged fusion (V <= 64) ---------------------------------------------------------
// A CTA of 128 threads fuses tiles of 128 consecutive cells.  The tile's V view rows (or, in
// the [H][W][V] layout, its 128 x V block) are copied into shared memory with cp.async,
// double-buffered: the copies of the next tile are in flight while the current one is
// fused.  Each thread then works on its cell's V values in registers:
//   * values as float32 with NaN replaced by +inf: the valid values are the n smallest
//     slots (ties with a valid +inf are the same value), so no key conversion is needed,
//     and the sign of a zero cannot change ((0 + lo) + hi) / 2, |x - med| or the mask;
//   * Batcher's odd-even merge sort on N = V rounded up to 8 slots, derived from the
//     power-of-two network by dropping the comparators that touch a slot >= N (those slots
//     hold +inf and every comparator puts its maximum on the higher slot, so they never
//     change);
//   * the median's two middle order statistics read back from a per-thread row of shared
//     memory (only ranks <= N/2 can be needed, so only those are stored);
//   * with a finite median the deviations of the sorted values, +inf beyond n, form a
//     V shape (fl(x - med) is monotone in x): one bitonic merge sorts them;
//   * the keep mask and numpy's pairwise mean read the values again from the staged tile.
// The copies use the hardware's own completion tracking (cp.async.wait_group): no spin
// waits.
constexpr int kTileCells = 128;

__device__ __forceinline__ void cp_async16(float *smem_dst, const float *gmem_src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
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

// Ascending bitonic merge of a V-shaped a[0..N) (power-of-two half-cleaners, slots >= N
// implicitly +inf).
template <int N>
__device__ __forceinline__ void bitonic_merge_asc(float (&a)[N]) {
    constexpr int P2 = pow2_ceil(N);
#pragma unroll
    for (int j = P2 >> 1; j > 0; j >>= 1)
#pragma unroll
        for (int i = 0; i < P2; ++i)
            if ((i & j) == 0 && (i | j) < N) cmpx(a, i, i | j);
}

constexpr int row_slots(int N) { return ((N / 2 + 1 + 3) / 4) * 4; }   // ranks 0..N/2, whole float4s
constexpr int row_stride(int N) { return row_slots(N) + 4; }          // odd number of float4s: no bank conflicts

template <int N>
__device__ __forceinline__ void store_low_ranks(const float (&a)[N], float *row) {
#pragma unroll
    for (int q = 0; q < row_slots(N) / 4; ++q)
        reinterpret_cast<float4 *>(row)[q] =
            make_float4(a[4 * q], 4 * q + 1 < N ? a[4 * q + 1] : 0.0f, 4 * q + 2 < N ? a[4 * q + 2] : 0.0f,
                        4 * q + 3 < N ? a[4 * q + 3] : 0.0f);
}

template <int N>
__device__ __forceinline__ float fuse_cell_staged(const float *__restrict__ xs, int si, int V, float *row) {
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
    store_low_ranks(a, row);
    const float med = __fdiv_rn(__fadd_rn(__fadd_rn(0.0f, row[(n - 1) >> 1]), row[n >> 1]), 2.0f);
    float mad = __int_as_float(0x7fffffff);
    if (isfinite(med)) {
#pragma unroll
        for (int i = 0; i < N; ++i) a[i] = i < n ? fabsf(__fsub_rn(a[i], med)) : inf;
        bitonic_merge_asc(a);
        store_low_ranks(a, row);
        mad = __fdiv_rn(__fadd_rn(__fadd_rn(0.0f, row[(n - 1) >> 1]), row[n >> 1]), 2.0f);
    } else {
        // deviations of the original values (inf - inf is NaN: missing)
        int nd = 0;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float v = inf;
            if (i < V) {
                const float d = fabsf(__fsub_rn(xs[i * si], med));
                const bool ok = !isnan(d);
                nd += ok;
                v = ok ? d : inf;
            }
            a[i] = v;
        }
        if (nd > 0) {
            oems_sort(a);
            store_low_ranks(a, row);
            mad = __fdiv_rn(__fadd_rn(__fadd_rn(0.0f, row[(nd - 1) >> 1]), row[nd >> 1]), 2.0f);
        }
    }
    // keep |x - med| <= mad (NaN compares false), then numpy's float32 pairwise sum of the
    // kept values (others 0) over the V slots in view order, from 0, / kept count
    int cnt = 0;
    auto kept = [&](int i, float &acc) {
        const float x = xs[i * si];
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
                for (int j = 0; j < 8; ++j) kept(b + j, r[j]);
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
                                                               long long n_tiles) {
    extern __shared__ __align__(16) float fsm[];
    const int t = threadIdx.x;
    const int tile_floats = V * kTileCells;
    float *buf0 = fsm, *buf1 = fsm + tile_floats;
    float *row = fsm + 2 * tile_floats + t * row_stride(N);
    // VHW: value i of cell t at [i][t]; HWV: at [t][i]
    const int sv = layout == VS_LAYOUT_VHW ? 1 : V, si = layout == VS_LAYOUT_VHW ? kTileCells : 1;
    auto issue = [&](long long tl, float *dst) {
        const long long c0 = tl * kTileCells;
        const int len = static_cast<int>(min(static_cast<long long>(kTileCells), cells - c0));   // multiple of 4
        if (layout == VS_LAYOUT_VHW) {
            const int chunks = len >> 2;
            for (int q = t; q < V * (kTileCells / 4); q += kTileCells) {
                const int v = q / (kTileCells / 4), ch = q - v * (kTileCells / 4);
                if (ch < chunks) cp_async16(dst + v * kTileCells + 4 * ch, dsm + v * cells + c0 + 4 * ch);
            }
        } else {
            const int chunks = (len * V) >> 2;
            for (int q = t; q < chunks; q += kTileCells) cp_async16(dst + 4 * q, dsm + c0 * V + 4 * q);
        }
        cp_async_commit();
    };
    long long tl = blockIdx.x;
    if (tl < n_tiles) issue(tl, buf0);
    for (; tl < n_tiles; tl += gridDim.x) {
        const long long nxt = tl + gridDim.x;
        if (nxt < n_tiles) issue(nxt, buf1);
        else cp_async_commit();                    // an empty group keeps "all but the newest" exact
        cp_async_wait_prev();
        __syncthreads();
        const long long c = tl * kTileCells + t;
        if (c < cells) out[c] = fuse_cell_staged<N>(buf0 + t * sv, si, V, row);
        __syncthreads();                           // buf0 is refilled next
        float *tmp = buf0;
        buf0 = buf1;
        buf1 = tmp;
    }
    cp_async_wait_all();
}

size_t fuse_tile_smem(int V, int N) {
    return sizeof(float) * (2 * static_cast<size_t>(V) * kTileCells + static_cast<size_t>(kTileCells) * row_stride(N));
}

template <int N>
bool launch_fuse_tile(const float *dsm, int layout, int V, long long cells, float *out, cudaStream_t st) {
    const size_t sh = fuse_tile_smem(V, N);
    static size_t configured = 0;     // per instantiation: the largest dynamic size set so far
    if (sh > configured) {
        if (cudaFuncSetAttribute(fuse_tile_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(fuse_tile_smem(64, N))) != cudaSuccess)
            return false;
        configured = fuse_tile_smem(64, N);
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fuse_tile_kernel<N>, kTileCells, sh) != cudaSuccess ||
        per_sm <= 0)
        return false;
    const long long n_tiles = ceil_div(cells, static_cast<long long>(kTileCells));
    const unsigned g = static_cast<unsigned>(std::min<long long>(n_tiles, 1LL * sm_count() * per_sm));
    fuse_tile_kernel<N><<<g, kTileCells, sh, st>>>(dsm, layout, V, cells, out, n_tiles);
    return true;
}

// The staged kernel needs 16-byte aligned view rows (VHW) or blocks (HWV).
bool fuse_tile_ok(const float *dsm, int layout, int V, long long cells) {
    if (V > 64 || (reinterpret_cast<uintptr_t>(dsm) & 15)) return false;
    return layout == VS_LAYOUT_VHW ? (cells % 4 == 0) : ((cells % 4 == 0) && ((static_cast<long long>(V) * 4) % 4 == 0));
}

int launch_fuse_staged(const float *dsm, int layout, int V, long long cells, float *out, cudaStream_t st) {
    bool ok = false;
    switch ((V + 7) / 8) {
        case 1: ok = launch_fuse_tile<8>(dsm, layout, V, cells, out, st); break;
        case 2: ok = launch_fuse_tile<16>(dsm, layout, V, cells, out, st); break;
        case 3: ok = launch_fuse_tile<24>(dsm, layout, V, cells, out, st); break;
        case 4: ok = launch_fuse_tile<32>(dsm, layout, V, cells, out, st); break;
        case 5: ok = launch_fuse_tile<40>(dsm, layout, V, cells, out, st); break;
        case 6: ok = launch_fuse_tile<48>(dsm, layout, V, cells, out, st); break;
        case 7: ok = launch_fuse_tile<56>(dsm, layout, V, cells, out, st); break;
        default: ok = launch_fuse_tile<64>(dsm, layout, V, cells, out, st); break;
    }
    if (!ok) {
        set_error("fuse_tile_kernel: launch configuration refused");
        return VS_ERR_CUDA;
    }
    return VS_OK;
}

template <int N>
void launch_fuse(const float *dsm, int layout, int V, long long cells, float *out, cudaStream_t st) {
    const int threads = 128;
    long long want = ceil_div(cells, threads);
    unsigned g = static_cast<unsigned>(std::min<long long>(want, sm_count() * 16LL));
    fuse_kernel<N><<<g, threads, 0, st>>>(dsm, layout, V, cells, out);
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
    if (fuse_tile_ok(dsm, layout, V, cells)) {
        const int s = launch_fuse_staged(dsm, layout, V, cells, dst, st);
        if (s != VS_OK) return s;
    } else if (V <= 8) launch_fuse<8>(dsm, layout, V, cells, dst, st);
    else if (V <= 16) launch_fuse<16>(dsm, layout, V, cells, dst, st);
    else if (V <= 32) launch_fuse<32>(dsm, layout, V, cells, dst, st);
    else if (V <= 64) launch_fuse<64>(dsm, layout, V, cells, dst, st);
    else {
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
