// Stable LSD radix sort, scans and deterministic sums.
//
// Radix sort: 8-bit digits, tiles of 2048 items (256 threads x 8 rounds).
// Per pass: (1) per-tile digit histograms in shared memory, (2) a parallel
// exclusive scan over the digit-major [digit][tile] histogram, (3) a stable
// scatter: each round of 256 items ranks equal digits inside a warp with
// __match_any_sync, then across the 8 warps by a per-digit prefix, on top of
// the tile's running per-digit offsets.  Grid sizes follow the tile count.
#include "sort.cuh"

namespace rigc {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;
constexpr int kWarps = kSortThreads / 32;

template <class Key>
__global__ void k_digit_hist(const Key* __restrict__ keys, int64_t n, int shift,
                             int ntiles, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * kSortTile;
#pragma unroll
    for (int r = 0; r < kSortRounds; r++) {
        int64_t i = base + r * kSortThreads + threadIdx.x;
        if (i < n) {
            uint32_t d = (uint32_t)(keys[i] >> shift) & 0xffu;
            atomicAdd(&cnt[d], 1u);
        }
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

template <class Key>
__global__ void __launch_bounds__(kSortThreads)
k_scatter(const Key* __restrict__ kin, const uint32_t* __restrict__ vin,
          Key* __restrict__ kout, uint32_t* __restrict__ vout, int64_t n,
          int shift, int ntiles, const uint32_t* __restrict__ offsets)
{
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[kWarps][256];
    __shared__ uint32_t woff[kWarps][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base[tid] = offsets[(int64_t)tid * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kWarps; w++) wcnt[w][tid] = 0;
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    int64_t tile0 = (int64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; r++) {
        int64_t i = tile0 + r * kSortThreads + tid;
        bool valid = i < n;
        Key k = valid ? kin[i] : Key(0);
        uint32_t v = valid ? vin[i] : 0u;
        uint32_t d = valid ? ((uint32_t)(k >> shift) & 0xffu) : 256u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = base[tid];
#pragma unroll
            for (int w = 0; w < kWarps; w++) {
                uint32_t c = wcnt[w][tid];
                woff[w][tid] = run;
                run += c;
                wcnt[w][tid] = 0;
            }
            base[tid] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = woff[warp][d] + rank;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
    }
}

int64_t scan_tiles(int64_t n);
int scan_in_place(int32_t* a, int64_t n, int32_t* sums, cudaStream_t stream);

// Inputs of at most one tile (the sorts of small scenes) are sorted by one
// block in one launch: per pass the tile's digit histogram, its exclusive
// scan over the 256 digits and the stable scatter of k_scatter, passes
// separated by block barriers (global writes of a block are visible to it
// after __syncthreads).  Same passes and the same stable order as the
// multi-launch sort.
template <class Key>
__global__ void __launch_bounds__(kSortThreads)
k_sort_tile(const Key* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
            Key* keys_out, uint32_t* vals_out, Key* tmp_k, uint32_t* tmp_v, int n, int passes)
{
    __shared__ uint32_t cnt[256];
    __shared__ uint32_t base[256];
    __shared__ uint32_t wsum[kWarps];
    __shared__ uint32_t wcnt[kWarps][256];
    __shared__ uint32_t woff[kWarps][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const Key* src_k = keys_in;
    const uint32_t* src_v = vals_in;
    for (int p = 0; p < passes; p++) {
        const bool to_out = ((passes - 1 - p) % 2) == 0;
        Key* dk = to_out ? keys_out : tmp_k;
        uint32_t* dv = to_out ? vals_out : tmp_v;
        const int shift = 8 * p;
        cnt[tid] = 0;
#pragma unroll
        for (int w = 0; w < kWarps; w++) wcnt[w][tid] = 0;
        __syncthreads();
        for (int r = 0; r < kSortRounds; r++) {
            const int i = r * kSortThreads + tid;
            if (i < n) atomicAdd(&cnt[(uint32_t)(src_k[i] >> shift) & 0xffu], 1u);
        }
        __syncthreads();
        // exclusive scan of the 256 digit counts
        uint32_t x = cnt[tid];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        uint32_t before = 0;
        for (int w = 0; w < warp; w++) before += wsum[w];
        base[tid] = before + x - cnt[tid];
        __syncthreads();
        for (int r = 0; r < kSortRounds; r++) {
            const int i = r * kSortThreads + tid;
            const bool valid = i < n;
            const Key k = valid ? src_k[i] : Key(0);
            const uint32_t v = valid ? src_v[i] : 0u;
            const uint32_t d = valid ? ((uint32_t)(k >> shift) & 0xffu) : 256u;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            const uint32_t rank = __popc(peers & lt);
            if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
            __syncthreads();
            {
                uint32_t run = base[tid];
#pragma unroll
                for (int w = 0; w < kWarps; w++) {
                    const uint32_t c = wcnt[w][tid];
                    woff[w][tid] = run;
                    run += c;
                    wcnt[w][tid] = 0;
                }
                base[tid] = run;
            }
            __syncthreads();
            if (valid) {
                const uint32_t pos = woff[warp][d] + rank;
                dk[pos] = k;
                dv[pos] = v;
            }
            __syncthreads();
        }
        src_k = dk;
        src_v = dv;
    }
}

} // namespace

template <class Key>
int radix_sort_pairs(const Key* keys_in, const uint32_t* vals_in, Key* keys_out,
                     uint32_t* vals_out, int64_t n, int bits, DevBuf& tmp_keys,
                     DevBuf& tmp_vals, DevBuf& hist, cudaStream_t stream)
{
    if (n <= 0) return RIGC_OK;
    if (bits < 1) bits = 1;
    if (bits > (int)(8 * sizeof(Key))) bits = 8 * sizeof(Key);
    const int passes = (bits + 7) / 8;
    const int ntiles = (int)((n + kSortTile - 1) / kSortTile);
    RIGC_TRY(tmp_keys.reserve(n * sizeof(Key)));
    RIGC_TRY(tmp_vals.reserve(n * sizeof(uint32_t)));
    if (ntiles == 1) {
        RIGC_COUNT_LAUNCH();
        k_sort_tile<Key><<<1, kSortThreads, 0, stream>>>(keys_in, vals_in, keys_out, vals_out,
                                                         tmp_keys.as<Key>(), tmp_vals.as<uint32_t>(),
                                                         (int)n, passes);
        RIGC_CUDA(cudaGetLastError());
        return RIGC_OK;
    }
    // digit-major histogram followed by the tile sums of its scan
    const int64_t m = (int64_t)256 * ntiles;
    RIGC_TRY(hist.reserve((size_t)(m + scan_tiles(m)) * sizeof(uint32_t)));
    int32_t* hist_i = reinterpret_cast<int32_t*>(hist.as<uint32_t>());
    // Pass p writes keys_out when (passes - 1 - p) is even, the temporaries
    // otherwise, so the last pass lands in keys_out and no pass writes the
    // buffer it reads (keys_in must not alias keys_out).
    const Key* src_k = keys_in;
    const uint32_t* src_v = vals_in;
    for (int p = 0; p < passes; p++) {
        bool to_out = ((passes - 1 - p) % 2) == 0;
        Key* dk = to_out ? keys_out : tmp_keys.as<Key>();
        uint32_t* dv = to_out ? vals_out : tmp_vals.as<uint32_t>();
        int shift = 8 * p;
        RIGC_COUNT_LAUNCH();
        k_digit_hist<Key><<<ntiles, kSortThreads, 0, stream>>>(src_k, n, shift, ntiles,
                                                               hist.as<uint32_t>());
        RIGC_TRY(scan_in_place(hist_i, m, hist_i + m, stream));
        RIGC_COUNT_LAUNCH();
        k_scatter<Key><<<ntiles, kSortThreads, 0, stream>>>(src_k, src_v, dk, dv, n, shift,
                                                            ntiles, hist.as<uint32_t>());
        src_k = dk;
        src_v = dv;
    }
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

template int radix_sort_pairs<uint32_t>(const uint32_t*, const uint32_t*, uint32_t*,
                                        uint32_t*, int64_t, int, DevBuf&, DevBuf&,
                                        DevBuf&, cudaStream_t);
template int radix_sort_pairs<uint64_t>(const uint64_t*, const uint32_t*, uint64_t*,
                                        uint32_t*, int64_t, int, DevBuf&, DevBuf&,
                                        DevBuf&, cudaStream_t);

// ---------------------------------------------------------------------------
// exclusive scan of int32: tile sums, single-block scan of tile sums, tile scan

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* total)
{
    __shared__ int32_t warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    int32_t before = warp ? warp_sums[warp - 1] : 0;
    *total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void k_tile_sums(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ sums)
{
    int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) s += in[base + k];
    int32_t tot;
    block_exclusive_scan(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int32_t* __restrict__ sums, int64_t m, int32_t* total_dev)
{
    // one block; loops over chunks of blockDim
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t b = 0; b < m; b += kScanThreads) {
        int64_t i = b + threadIdx.x;
        int32_t v = i < m ? sums[i] : 0;
        int32_t tot;
        int32_t ex = block_exclusive_scan(v, &tot);
        if (i < m) sums[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_dev) *total_dev = carry;
}

__global__ void k_tile_scan(const int32_t* in, int32_t* out, int64_t n,
                            const int32_t* __restrict__ sums)
{
    int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    int32_t tot;
    int32_t ex = block_exclusive_scan(s, &tot) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
}

// Short arrays (at most kSmallScan items, the histograms and flags of small
// scenes) are scanned by one block in one launch, tile after tile with a
// running carry: the same integer sums as the three-kernel scan, a third of
// the launches.
constexpr int64_t kSmallScan = 4 * kScanTile;

__global__ void k_scan_small(const int32_t* in, int32_t* out, int64_t n, int32_t* total_dev)
{
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t b = 0; b < n; b += kScanTile) {
        const int64_t base = b + threadIdx.x * kScanItems;
        int32_t v[kScanItems];
        int32_t s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            v[k] = base + k < n ? in[base + k] : 0;
            s += v[k];
        }
        int32_t tot;
        int32_t ex = block_exclusive_scan(s, &tot) + carry;  // reads precede the writes
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            if (base + k < n) out[base + k] = ex;
            ex += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_dev) *total_dev = carry;
}

int64_t scan_tiles(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

// exclusive scan of a[0..n) in place (each tile is read before it is written);
// sums holds scan_tiles(n) entries
int scan_in_place(int32_t* a, int64_t n, int32_t* sums, cudaStream_t stream)
{
    if (n <= kSmallScan) {
        RIGC_COUNT_LAUNCH();
        k_scan_small<<<1, kScanThreads, 0, stream>>>(a, a, n, nullptr);
        return RIGC_OK;
    }
    const int64_t tiles = scan_tiles(n);
    RIGC_COUNT_LAUNCH();
    k_tile_sums<<<(unsigned)tiles, kScanThreads, 0, stream>>>(a, n, sums);
    RIGC_COUNT_LAUNCH();
    k_scan_sums<<<1, kScanThreads, 0, stream>>>(sums, tiles, nullptr);
    RIGC_COUNT_LAUNCH();
    k_tile_scan<<<(unsigned)tiles, kScanThreads, 0, stream>>>(a, a, n, sums);
    return RIGC_OK;
}

} // namespace

int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, int32_t* total_dev,
                       DevBuf& tmp, cudaStream_t stream)
{
    if (n <= 0) {
        if (total_dev) RIGC_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(int32_t), stream));
        return RIGC_OK;
    }
    if (n <= kSmallScan) {
        RIGC_COUNT_LAUNCH();
        k_scan_small<<<1, kScanThreads, 0, stream>>>(in, out, n, total_dev);
        RIGC_CUDA(cudaGetLastError());
        return RIGC_OK;
    }
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    RIGC_TRY(tmp.reserve(tiles * sizeof(int32_t)));
    RIGC_COUNT_LAUNCH();
    k_tile_sums<<<(unsigned)tiles, kScanThreads, 0, stream>>>(in, n, tmp.as<int32_t>());
    RIGC_COUNT_LAUNCH();
    k_scan_sums<<<1, kScanThreads, 0, stream>>>(tmp.as<int32_t>(), tiles, total_dev);
    RIGC_COUNT_LAUNCH();
    k_tile_scan<<<(unsigned)tiles, kScanThreads, 0, stream>>>(in, out, n, tmp.as<int32_t>());
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

// ---------------------------------------------------------------------------
// deterministic double sum: fixed 1024 partials, then one block

namespace {
constexpr int kSumBlocks = 1024;

__global__ void k_sum_partials(const double* __restrict__ in, int64_t n, double* __restrict__ part)
{
    __shared__ double sh[256];
    double s = 0;
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256)
        s += in[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_sum_final(const double* __restrict__ part, int m, double* out)
{
    __shared__ double sh[1024];
    sh[threadIdx.x] = threadIdx.x < m ? part[threadIdx.x] : 0.0;
    __syncthreads();
    for (int o = 512; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}
} // namespace

int sum_f64(const double* in, int64_t n, double* out_dev, DevBuf& tmp, cudaStream_t stream)
{
    RIGC_TRY(tmp.reserve(kSumBlocks * sizeof(double)));
    RIGC_COUNT_LAUNCH();
    k_sum_partials<<<kSumBlocks, 256, 0, stream>>>(in, n, tmp.as<double>());
    RIGC_COUNT_LAUNCH();
    k_sum_final<<<1, 1024, 0, stream>>>(tmp.as<double>(), kSumBlocks, out_dev);
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

} // namespace rigc
