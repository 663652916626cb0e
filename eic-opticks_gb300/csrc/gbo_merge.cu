// gbo_merge.cu : hit merging by (sensor identity, time bucket), the reference's SPM::merge_partial_select
// (sysrap/SPM.cu) with sphoton::key_functor / reduce_op (sysrap/sphoton.h:277-304).
//
// key = identity << 48 | (unsigned)(time / tw); hits are stably sorted by key and each run of equal keys becomes one
// hit: the earliest-time member (the earlier in input order on a tie) with the run's flagmasks ORed and hitcounts
// (16 bits) summed.  The reference sorts with thrust and reduces with reduce_by_key; here:
//
//   k_merge_keys      key and input index per hit, OR of all keys (to skip radix passes over all-zero bytes)
//   k_radix_hist      per-tile histogram of one key byte (256 bins in shared memory), digit-major layout
//   k_scan_*          exclusive scan of the digit x tile counts (or of the run-head flags): tile sums, one-block
//                     scan of the tile sums, per-tile scan
//   k_radix_scatter   stable scatter: each warp owns a contiguous sub-tile, ranks equal digits with
//                     __match_any_sync and a per-warp running offset, so input order survives every pass
//   k_run_heads       1 where a key differs from its predecessor
//   k_run_reduce      one thread per run folds its members in sorted (= input) order
//
// Memory is stream-ordered (cudaMallocAsync / cudaFreeAsync) on the caller's stream.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbo_merge.h"

namespace {

constexpr int MB_THREADS = 256;                 // threads per block of the sort kernels
constexpr int MB_WARPS = MB_THREADS / 32;
constexpr int MB_TILE = 4096;                   // keys per block tile
constexpr int MB_WARP_TILE = MB_TILE / MB_WARPS;
constexpr int SCAN_THREADS = 1024;

__device__ __forceinline__ uint64_t merge_key(const gbo_sphoton& p, float tw)
{
    const unsigned id = p.identity & 0x00ffffffu;
    const unsigned bucket = (unsigned)(p.time / tw);
    return ((uint64_t)id << 48) | (uint64_t)bucket;
}

__global__ void k_merge_keys(const gbo_sphoton* in, long long n, float tw, uint64_t* keys, uint32_t* idx,
                             unsigned long long* key_or)
{
    __shared__ unsigned long long s_or;
    if (threadIdx.x == 0) s_or = 0ull;
    __syncthreads();
    unsigned long long acc = 0ull;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint64_t k = merge_key(in[i], tw);
        keys[i] = k;
        idx[i] = (uint32_t)i;
        acc |= k;
    }
    for (int o = 16; o > 0; o >>= 1) acc |= __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicOr(&s_or, acc);
    __syncthreads();
    if (threadIdx.x == 0) atomicOr(key_or, s_or);
}

__global__ void k_radix_hist(const uint64_t* keys, long long n, int shift, int ntiles, uint32_t* hist)
{
    __shared__ uint32_t h[256];
    for (int d = threadIdx.x; d < 256; d += blockDim.x) h[d] = 0u;
    __syncthreads();
    const long long base = (long long)blockIdx.x * MB_TILE;
    for (int j = threadIdx.x; j < MB_TILE; j += blockDim.x) {
        const long long i = base + j;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(size_t)d * ntiles + blockIdx.x] = h[d];
}

// Exclusive scan of n uint32 in place, in three launches: k_scan_tiles sums each SCAN_TILE-word tile, k_scan_partials
// scans the tile sums in one block (and writes the total), k_scan_down scans each tile from its tile's offset.  Each
// warp owns SCAN_WARP_TILE consecutive words and reads them 32 at a time (coalesced), carrying its running sum.
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_WARP_TILE = 32 * SCAN_ITEMS;
constexpr int SCAN_TILE = MB_WARPS * SCAN_WARP_TILE;

__global__ void __launch_bounds__(MB_THREADS) k_scan_tiles(const uint32_t* v, long long n, uint32_t* partial)
{
    __shared__ uint32_t wsum[MB_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)warp * SCAN_WARP_TILE;
    uint32_t s = 0u;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const long long i = base + k * 32 + lane;
        s += i < n ? v[i] : 0u;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) wsum[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0u;
        for (int w = 0; w < MB_WARPS; w++) t += wsum[w];
        partial[blockIdx.x] = t;
    }
}

// one block: exclusive scan of the m tile sums in place, each thread over a contiguous chunk; total in *total
__global__ void k_scan_partials(uint32_t* v, long long m, unsigned long long* total)
{
    __shared__ unsigned long long part[SCAN_THREADS];
    const long long per = (m + SCAN_THREADS - 1) / SCAN_THREADS;
    const long long lo = (long long)threadIdx.x * per;
    const long long hi = lo + per < m ? lo + per : m;
    unsigned long long s = 0ull;
    for (long long i = lo; i < hi; i++) s += v[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < SCAN_THREADS; off <<= 1) {          // Hillis-Steele over the chunk sums
        const unsigned long long x = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0ull;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    unsigned long long run = threadIdx.x ? part[threadIdx.x - 1] : 0ull;
    for (long long i = lo; i < hi; i++) {
        const uint32_t x = v[i];
        v[i] = (uint32_t)run;
        run += x;
    }
    if (threadIdx.x == SCAN_THREADS - 1 && total) *total = part[SCAN_THREADS - 1];
}

__global__ void __launch_bounds__(MB_THREADS) k_scan_down(uint32_t* v, long long n, const uint32_t* partial)
{
    __shared__ uint32_t wsum[MB_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)warp * SCAN_WARP_TILE;
    uint32_t x[SCAN_ITEMS];
    uint32_t s = 0u;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const long long i = base + k * 32 + lane;
        x[k] = i < n ? v[i] : 0u;
        s += x[k];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) wsum[warp] = s;
    __syncthreads();
    uint32_t run = partial[blockIdx.x];
    for (int w = 0; w < warp; w++) run += wsum[w];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        uint32_t inc = x[k];                                    // inclusive scan of this row of 32 words
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        const long long i = base + k * 32 + lane;
        if (i < n) v[i] = run + inc - x[k];
        run += __shfl_sync(0xffffffffu, inc, 31);
    }
}

// exclusive scan of v[0..n) in place; scratch holds ceil(n / SCAN_TILE) words; the total (if wanted) lands in *total
static void scan_exclusive(uint32_t* v, long long n, uint32_t* scratch, unsigned long long* total, cudaStream_t s)
{
    const long long tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_tiles<<<(unsigned)tiles, MB_THREADS, 0, s>>>(v, n, scratch);
    k_scan_partials<<<1, SCAN_THREADS, 0, s>>>(scratch, tiles, total);
    k_scan_down<<<(unsigned)tiles, MB_THREADS, 0, s>>>(v, n, scratch);
}

__global__ void __launch_bounds__(MB_THREADS) k_radix_scatter(const uint64_t* keys, const uint32_t* idx, long long n,
                                                              int shift, int ntiles, const uint32_t* offsets,
                                                              uint64_t* keys_out, uint32_t* idx_out)
{
    __shared__ uint32_t cnt[MB_WARPS][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (int d = threadIdx.x; d < MB_WARPS * 256; d += blockDim.x) (&cnt[0][0])[d] = 0u;
    __syncthreads();
    const long long wbase = (long long)blockIdx.x * MB_TILE + (long long)warp * MB_WARP_TILE;
    // 1. digit counts of each warp's sub-tile
    for (int c = 0; c < MB_WARP_TILE; c += 32) {
        const long long i = wbase + c + lane;
        const bool ok = i < n;
        const unsigned d = ok ? (unsigned)((keys[i] >> shift) & 0xffu) : 0u;
        const unsigned act = __ballot_sync(0xffffffffu, ok);
        if (ok) {
            const unsigned peers = __match_any_sync(act, d);
            if ((peers & lt) == 0u) cnt[warp][d] += __popc(peers);
        }
        __syncwarp();                                   // the next chunk's leader may be another lane
    }
    __syncthreads();
    // 2. running bases: the block's offset for the digit, then the earlier warps' counts
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        uint32_t run = offsets[(size_t)d * ntiles + blockIdx.x];
        for (int w = 0; w < MB_WARPS; w++) {
            const uint32_t c = cnt[w][d];
            cnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
    // 3. stable scatter in sub-tile order
    for (int c = 0; c < MB_WARP_TILE; c += 32) {
        const long long i = wbase + c + lane;
        const bool ok = i < n;
        const uint64_t k = ok ? keys[i] : 0ull;
        const unsigned d = (unsigned)((k >> shift) & 0xffu);
        const unsigned act = __ballot_sync(0xffffffffu, ok);
        unsigned peers = 0u, pos = 0u;
        if (ok) {
            peers = __match_any_sync(act, d);
            pos = cnt[warp][d] + __popc(peers & lt);
        }
        __syncwarp();
        if (ok) {
            keys_out[pos] = k;
            idx_out[pos] = idx[i];
            if ((peers & lt) == 0u) cnt[warp][d] += __popc(peers);
        }
        __syncwarp();
    }
}

__global__ void k_run_heads(const uint64_t* keys, long long n, uint32_t* head)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        head[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

__global__ void k_run_starts(const uint64_t* keys, long long n, const uint32_t* run_index, uint32_t* start)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (i == 0 || keys[i] != keys[i - 1]) start[run_index[i]] = (uint32_t)i;
}

// one hit as four 16-byte loads when the array is 16-byte aligned (cudaMalloc'd hit buffers are)
template <bool A16>
__device__ __forceinline__ gbo_sphoton load_hit(const gbo_sphoton* p)
{
    if (A16) {
        gbo_sphoton h;
        const uint4* q = reinterpret_cast<const uint4*>(p);
        uint4* o = reinterpret_cast<uint4*>(&h);
#pragma unroll
        for (int k = 0; k < 4; k++) o[k] = __ldg(q + k);
        return h;
    }
    return *p;
}

template <bool A16>
__global__ void k_run_reduce(const gbo_sphoton* in, const uint32_t* order, const uint32_t* start, long long runs,
                             long long n, gbo_sphoton* out)
{
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < runs; r += (long long)gridDim.x * blockDim.x) {
        const long long b = start[r];
        const long long e = r + 1 < runs ? (long long)start[r + 1] : n;
        gbo_sphoton acc = load_hit<A16>(in + order[b]);
        for (long long j = b + 1; j < e; j++) {
            const gbo_sphoton x = load_hit<A16>(in + order[j]);
            const bool a_first = fminf(acc.time, x.time) == acc.time;
            const unsigned fm = acc.flagmask | x.flagmask;
            const unsigned hc = ((acc.hitcount_iindex >> 16) + (x.hitcount_iindex >> 16)) & 0xffffu;
            if (!a_first) acc = x;
            acc.flagmask = fm;
            acc.hitcount_iindex = (acc.hitcount_iindex & 0x0000ffffu) | (hc << 16);
        }
        if (A16) {
            const uint4* q = reinterpret_cast<const uint4*>(&acc);
            uint4* o = reinterpret_cast<uint4*>(out + r);
#pragma unroll
            for (int k = 0; k < 4; k++) o[k] = q[k];
        } else {
            out[r] = acc;
        }
    }
}

#define MCU(x) do { cudaError_t err_ = (x); if (err_ != cudaSuccess) { rc = GBO_ERR_CUDA; goto done; } } while (0)

}  // namespace

namespace gbo {

// Grow-only device buffers of the hit merge, kept by an engine between events
struct MergeScratch {
    void* buf[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    size_t cap[7] = {0, 0, 0, 0, 0, 0, 0};
};

MergeScratch* merge_scratch_new() { return new MergeScratch(); }

void merge_scratch_free(MergeScratch* m)
{
    if (!m) return;
    for (void* b : m->buf)
        if (b) cudaFree(b);
    delete m;
}

// Merge n device hits into d_out (room for n); *num_out receives the merged count.  Synchronous on `stream`.  With
// `scratch` the work buffers come from (and grow) it; without, they are allocated and freed stream-ordered.
int merge_hits(const gbo_sphoton* d_in, int64_t n, float time_window, gbo_sphoton* d_out, int64_t* num_out,
               cudaStream_t s, MergeScratch* scratch)
{
    if (!num_out || n < 0 || (n > 0 && (!d_in || !d_out))) return GBO_ERR_ARG;
    if (n > 0xffffffffll) return GBO_ERR_CAPACITY;
    *num_out = 0;
    if (n == 0) return GBO_OK;
    if (time_window == 0.f) {                                   // NOMERGE_TIME_WINDOW: the hits as they are
        if (cudaMemcpyAsync(d_out, d_in, (size_t)n * sizeof(gbo_sphoton), cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return GBO_ERR_CUDA;
        *num_out = n;
        return GBO_OK;
    }
    int rc = GBO_OK;
    const int ntiles = (int)((n + MB_TILE - 1) / MB_TILE);
    const long long scan_n = n > 256ll * ntiles ? n : 256ll * ntiles;
    // k0, k1 (keys), i0, i1 (input indices), hist (digit x tile counts, later the run heads), scal ([0] key OR,
    // [1] run count), scan_tmp (tile sums of the scans)
    const size_t need[7] = {(size_t)n * 8, (size_t)n * 8, (size_t)n * 4, (size_t)n * 4, (size_t)scan_n * 4,
                            2 * sizeof(unsigned long long), (size_t)(scan_n / SCAN_TILE + 1) * 4};
    void* b[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    for (int k = 0; k < 7; k++) {
        if (scratch) {
            if (scratch->cap[k] < need[k]) {
                if (scratch->buf[k]) cudaFree(scratch->buf[k]);
                scratch->buf[k] = nullptr;
                scratch->cap[k] = 0;
                MCU(cudaMalloc(&scratch->buf[k], need[k]));
                scratch->cap[k] = need[k];
            }
            b[k] = scratch->buf[k];
        } else {
            MCU(cudaMallocAsync(&b[k], need[k], s));
        }
    }
    {
    uint64_t *k0 = (uint64_t*)b[0], *k1 = (uint64_t*)b[1];
    uint32_t *i0 = (uint32_t*)b[2], *i1 = (uint32_t*)b[3], *hist = (uint32_t*)b[4], *scan_tmp = (uint32_t*)b[6];
    unsigned long long* scal = (unsigned long long*)b[5];
    unsigned long long h_scal[2] = {0ull, 0ull};
    const int grid = (int)((n + MB_THREADS - 1) / MB_THREADS < 4096 ? (n + MB_THREADS - 1) / MB_THREADS : 4096);
    MCU(cudaMemsetAsync(scal, 0, 2 * sizeof(unsigned long long), s));
    k_merge_keys<<<grid, MB_THREADS, 0, s>>>(d_in, n, time_window, k0, i0, scal);
    MCU(cudaGetLastError());
    MCU(cudaMemcpyAsync(h_scal, scal, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    MCU(cudaStreamSynchronize(s));
    for (int byte = 0; byte < 8; byte++) {
        if (((h_scal[0] >> (8 * byte)) & 0xffull) == 0ull) continue;       // every key has a zero byte here
        k_radix_hist<<<ntiles, MB_THREADS, 0, s>>>(k0, n, 8 * byte, ntiles, hist);
        scan_exclusive(hist, (long long)256 * ntiles, scan_tmp, nullptr, s);
        k_radix_scatter<<<ntiles, MB_THREADS, 0, s>>>(k0, i0, n, 8 * byte, ntiles, hist, k1, i1);
        MCU(cudaGetLastError());
        uint64_t* tk = k0; k0 = k1; k1 = tk;
        uint32_t* ti = i0; i0 = i1; i1 = ti;
    }
    // runs of equal keys: heads -> exclusive scan (run index of each head) -> run starts -> fold
    uint32_t* head = hist;                                      // n words (hist was sized for max(n, 256 ntiles))
    k_run_heads<<<grid, MB_THREADS, 0, s>>>(k0, n, head);
    scan_exclusive(head, n, scan_tmp, scal + 1, s);
    MCU(cudaGetLastError());
    MCU(cudaMemcpyAsync(h_scal + 1, scal + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    MCU(cudaStreamSynchronize(s));
    const long long runs = (long long)h_scal[1];
    uint32_t* start = i1;                                       // free after the last pass
    k_run_starts<<<grid, MB_THREADS, 0, s>>>(k0, n, head, start);
    const int rgrid = (int)((runs + MB_THREADS - 1) / MB_THREADS < 4096 ? (runs + MB_THREADS - 1) / MB_THREADS : 4096);
    if ((((uintptr_t)d_in | (uintptr_t)d_out) & 15u) == 0u)
        k_run_reduce<true><<<rgrid > 0 ? rgrid : 1, MB_THREADS, 0, s>>>(d_in, i0, start, runs, n, d_out);
    else
        k_run_reduce<false><<<rgrid > 0 ? rgrid : 1, MB_THREADS, 0, s>>>(d_in, i0, start, runs, n, d_out);
    MCU(cudaGetLastError());
    MCU(cudaStreamSynchronize(s));
    *num_out = runs;
    }
done:
    if (!scratch)
        for (void* x : b)
            if (x) cudaFreeAsync(x, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && rc == GBO_OK) rc = GBO_ERR_CUDA;
    return rc;
}

}  // namespace gbo

// Merge n device hits into d_out (room for n) with stream-ordered temporary buffers.
extern "C" int gbo_merge_hits_device(const gbo_sphoton* d_in, int64_t n, float time_window, gbo_sphoton* d_out,
                                     int64_t* num_out, void* stream)
{
    return gbo::merge_hits(d_in, n, time_window, d_out, num_out, (cudaStream_t)stream, nullptr);
}
