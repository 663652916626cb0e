// gbo_engine.cu : engine lifecycle, event flow, hit compaction kernels and the C ABI of libgbopticks.so (the
// simulation kernels themselves are in gbo_sim.cuh, compiled per CSG form by gbo_sim_tree*.cu).
//
// One event = one pass of the photon program of CSGOptiX/CSGOptiX7.cu:405-503 over every photon its gensteps
// describe, then hit selection (sysrap/SU.cu:89-92,155-160 via qudarap/QEvt.cc:934-967,1113-1131).
//
// Device-side flow of an event:
//   k_genstep_prefix   inclusive prefix of genstep numphoton (replaces the seed array of QEvt.cu:181-237: a
//                      photon finds its genstep by binary search, so no per-photon seed buffer is written)
//   k_generate         kernel mode 2: every photon of the launch generated up front
//   k_simulate_pool    persistent photon pool (or k_simulate, one thread per photon): bounce loop of trace +
//                      propagate, final record; a warp ballot writes one 32-bit hit-bitmap word per 32 photons and
//                      hit photons are appended (warp-aggregated atomics) to an unordered buffer unless the full
//                      photon array is kept
//   k_word_prefix      per-word popcount prefix inside 256-word blocks + block totals
//   k_block_offsets    exclusive scan of the block totals (one block) -> number of hits
//   k_gather_*         hits written in photon order (the order thrust::copy_if gives the reference)
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gbopticks.h"
#include "gbo_accel.h"
#include "gbo_sim.cuh"
#include "gbo_merge.h"

namespace gbo {

constexpr int SCAN_WORDS = 256;     // words per block in k_word_prefix

// Every photon of the launch generated up front, converged, so that the pool kernel's refills are plain loads.  A
// warp generates GEN_PER_LANE x 32 consecutive photons, 32 at a time: the photons of a genstep are consecutive, so
// after one binary search a lane finds its next photon's genstep by stepping forward (usually not at all) instead of
// searching again (the search's chain of dependent loads had bound the kernel).
constexpr int GEN_PER_LANE = 8;

__global__ void __launch_bounds__(SIM_BLOCK) k_generate(const __grid_constant__ Params P)
{
    const unsigned lane = threadIdx.x & 31u;
    const long long first = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (32ll * GEN_PER_LANE);
    int gi = -1;
    for (int j = 0; j < GEN_PER_LANE; j++) {
        const long long idx = first + 32ll * j + lane;
        if (idx >= P.num_photon) return;
        if (gi < 0) gi = genstep_of(P, idx);
        else while (__ldg(P.gs_end + gi) <= (unsigned long long)idx) gi++;
        Photon p;
        RngT<false> rng;
        int hint;
        generate_at(P, idx, gi, p, rng, hint);
        store_photon(P.gen_photon + idx, p);
        P.gen_rng[idx] = make_ulonglong2(rng.pos, ((unsigned long long)rng.sub_hi << 32) | rng.sub_lo);
        P.gen_hint[idx] = hint;
    }
}

// Start instance of each genstep's photons: of the instances whose padded world box holds the genstep position
// (q1.xyz for every genstep type), the one with the smallest box, found by a point walk of the TLAS.  Only a
// traversal hint: trace finds the same closest hit with any hint or none, faster when the hint is right (the
// first step of a photon then skips the TLAS walk like every later step).
__global__ void k_genstep_hint(Accel a, const float4* gs, int num_gs, int* hint)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= num_gs) return;
    const float4 q1 = __ldg(gs + 6 * (size_t)g + 1);
    const float x = q1.x, y = q1.y, z = q1.z;
    int best = -1;
    float best_vol = INFINITY;
    int stack[TRAVERSAL_STACK];
    int sp = 0;
    int node = 0;
    for (;;) {
        const float4* nq = reinterpret_cast<const float4*>(a.tlas + node);
#pragma unroll
        for (int c = 0; c < 2; c++) {
            const float4 lo = __ldg(nq + 2 * c), hi = __ldg(nq + 2 * c + 1);
            const int count = __float_as_int(hi.w);
            if (count < 0 || !(x >= lo.x && x <= hi.x && y >= lo.y && y <= hi.y && z >= lo.z && z <= hi.z)) continue;
            if (count == 0) {
                if (sp < TRAVERSAL_STACK) stack[sp++] = __float_as_int(lo.w);
                continue;
            }
            const int first = __float_as_int(lo.w);
            for (int k = 0; k < count; k++) {
                const int ii = __ldg(a.tlas_index + first + k);
                const float4 blo = __ldg(a.inst_box + 2 * ii), bhi = __ldg(a.inst_box + 2 * ii + 1);
                if (!(x >= blo.x && x <= bhi.x && y >= blo.y && y <= bhi.y && z >= blo.z && z <= bhi.z)) continue;
                const float vol = (bhi.x - blo.x) * (bhi.y - blo.y) * (bhi.z - blo.z);
                if (vol < best_vol || (vol == best_vol && ii < best)) { best_vol = vol; best = ii; }
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    hint[g] = best;
}

// input_gs (may be null) receives 1 when any genstep is an INPUT_PHOTON genstep, else 0: the host then checks that
// input photons were given for every photon slot before any photon is generated
__global__ void k_genstep_prefix(const gbo_quad6* gs, int num_gs, unsigned long long* gs_end,
                                 unsigned long long* input_gs)
{
    // single block: chunked inclusive scan of numphoton
    __shared__ unsigned long long buf[1024];
    __shared__ unsigned long long carry;
    __shared__ int any_input;
    if (threadIdx.x == 0) { carry = 0ull; any_input = 0; }
    __syncthreads();
    for (int base = 0; base < num_gs; base += blockDim.x) {
        const int i = base + threadIdx.x;
        unsigned long long v = i < num_gs ? (unsigned long long)gs[i].q[0].u[3] : 0ull;
        if (i < num_gs && gs[i].q[0].i[0] == GBO_GS_INPUT_PHOTON) any_input = 1;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < (int)blockDim.x; off <<= 1) {
            unsigned long long add = threadIdx.x >= (unsigned)off ? buf[threadIdx.x - off] : 0ull;
            __syncthreads();
            buf[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < num_gs) gs_end[i] = carry + buf[threadIdx.x];
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += buf[threadIdx.x];
        __syncthreads();
    }
    if (input_gs && threadIdx.x == 0) *input_gs = any_input ? 1ull : 0ull;
}

__global__ void k_word_prefix(const uint32_t* bitmap, long long words, uint32_t* word_prefix, uint32_t* block_sum)
{
    __shared__ uint32_t buf[SCAN_WORDS];
    const long long w = (long long)blockIdx.x * SCAN_WORDS + threadIdx.x;
    const uint32_t c = w < words ? (uint32_t)__popc(bitmap[w]) : 0u;
    buf[threadIdx.x] = c;
    __syncthreads();
    for (int off = 1; off < SCAN_WORDS; off <<= 1) {
        uint32_t add = threadIdx.x >= (unsigned)off ? buf[threadIdx.x - off] : 0u;
        __syncthreads();
        buf[threadIdx.x] += add;
        __syncthreads();
    }
    if (w < words) word_prefix[w] = buf[threadIdx.x] - c;       // exclusive within block
    if (threadIdx.x == SCAN_WORDS - 1) block_sum[blockIdx.x] = buf[threadIdx.x];
}

__global__ void k_block_offsets(uint32_t* block_sum, long long nblocks, unsigned long long* block_offset,
                                unsigned long long* total)
{
    __shared__ unsigned long long buf[1024];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = 0ull;
    __syncthreads();
    for (long long base = 0; base < nblocks; base += blockDim.x) {
        const long long i = base + threadIdx.x;
        const unsigned long long v = i < nblocks ? (unsigned long long)block_sum[i] : 0ull;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < (int)blockDim.x; off <<= 1) {
            unsigned long long add = threadIdx.x >= (unsigned)off ? buf[threadIdx.x - off] : 0ull;
            __syncthreads();
            buf[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < nblocks) block_offset[i] = carry + buf[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += buf[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__device__ __forceinline__ void copy_photon(gbo_sphoton* dst, const gbo_sphoton* src)
{
    const float4* s = reinterpret_cast<const float4*>(src);
    float4* d = reinterpret_cast<float4*>(dst);
    const float4 a = __ldg(s), b = __ldg(s + 1), c = __ldg(s + 2), e = __ldg(s + 3);
    d[0] = a; d[1] = b; d[2] = c; d[3] = e;
}

// warp per bitmap word: lane j copies photon 32w+j when its bit is set
__global__ void k_gather_photons(const gbo_sphoton* photons, const uint32_t* bitmap, const uint32_t* word_prefix,
                                 const unsigned long long* block_offset, long long words, gbo_sphoton* hits)
{
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31u;
    if (w >= words) return;
    const uint32_t m = bitmap[w];
    if (!(m & (1u << lane))) return;
    const unsigned long long rank = block_offset[w / SCAN_WORDS] + word_prefix[w] + __popc(m & ((1u << lane) - 1u));
    copy_photon(hits + rank, photons + w * 32 + lane);
}

// thread per unordered hit: its photon index gives the bitmap rank, i.e. its place in photon order
__global__ void k_gather_unordered(const gbo_sphoton* unordered, const unsigned long long* count,
                                   unsigned long long photon_offset, const uint32_t* bitmap, const uint32_t* word_prefix,
                                   const unsigned long long* block_offset, gbo_sphoton* hits,
                                   const unsigned long long* gidx = nullptr)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((unsigned long long)i >= *count) return;
    const gbo_sphoton* src = unordered + i;
    const unsigned long long full = ((unsigned long long)(__ldg(&src->identity) >> 24) << 32) | __ldg(&src->index);
    const unsigned long long rel = gidx ? gidx[i] : full - photon_offset;
    const long long w = (long long)(rel >> 5);
    const unsigned j = (unsigned)(rel & 31u);
    const uint32_t m = bitmap[w];
    const unsigned long long rank = block_offset[w / SCAN_WORDS] + word_prefix[w] + __popc(m & ((1u << j) - 1u));
    copy_photon(hits + rank, src);
}

// hit rank of each event boundary photon: event e's hits are ordered hits [out[e], out[e+1])
__global__ void k_event_hit_ranges(const unsigned long long* ev_photon_begin, int n_ev, long long num_photon,
                                   const uint32_t* bitmap, const uint32_t* word_prefix,
                                   const unsigned long long* block_offset, const unsigned long long* total_hits,
                                   unsigned long long* out)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e > n_ev) return;
    const unsigned long long j = ev_photon_begin[e];
    if ((long long)j >= num_photon) { out[e] = *total_hits; return; }
    const long long w = (long long)(j >> 5);
    const unsigned b = (unsigned)(j & 31u);
    out[e] = block_offset[w / SCAN_WORDS] + word_prefix[w] + __popc(bitmap[w] & ((1u << b) - 1u));
}

// ---- known-answer kernels (the reference keeps equivalents in qudarap/QSim.cu for QSimTest) -----------------

__global__ void k_rng_sequence(uint64_t seed, uint64_t subsequence0, uint64_t position, int num_seq, int per_seq,
                               float* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num_seq) return;
    RngT<false> r;
    rng_init(r, seed, subsequence0 + (uint64_t)i, position);
    for (int k = 0; k < per_seq; k++) out[(size_t)i * per_seq + k] = uniform(r);
}

__global__ void k_tex_lookup(Tables t, const float2* xy, int n, int which, float4* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 c = xy[i];
    if (which == 0) out[i] = tex2D<float4>(t.bnd_tex, c.x, c.y);
    else out[i] = make_float4(tex2D<float>(t.icdf_tex, c.x, c.y), 0.f, 0.f, 0.f);
}

__global__ void k_scint_wavelength(Tables t, const float* u, int n, float* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = scint_wavelength(t, u[i]);
}

}  // namespace gbo

// ================================================================================================================
// host side

using namespace gbo;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CU(call)                                                                                           \
    do {                                                                                                   \
        cudaError_t err_ = (call);                                                                         \
        if (err_ != cudaSuccess) return fail(GBO_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(err_)); \
    } while (0)

template <typename T>
struct DBuf {
    T* ptr = nullptr;
    size_t cap = 0;     // elements
    int ensure(size_t n)
    {
        if (n <= cap && ptr) return 0;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        size_t want = n < 1 ? 1 : n;
        if (cudaMalloc(&ptr, want * sizeof(T)) != cudaSuccess) {
            ptr = nullptr;
            return fail(GBO_ERR_CUDA, "cudaMalloc of %zu bytes failed", want * sizeof(T));
        }
        cap = want;
        return 0;
    }
    void release() { if (ptr) cudaFree(ptr); ptr = nullptr; cap = 0; }
};

// Kernel mode 3's device state for n photons and max_bounce steps (hit records, the two step lists and the walk
// queue, the step counters), held in three buffers that grow as needed.
struct WavefrontBufs {
    DBuf<float4> hit;
    DBuf<int> list;
    DBuf<unsigned long long> count;
    DBuf<unsigned> bins;
    DBuf<Acc64> acc;
    void release() { hit.release(); list.release(); count.release(); bins.release(); acc.release(); }
    int ensure(long long n, int max_bounce, bool precise, Wavefront& w)
    {
        int rc;
        if ((rc = hit.ensure(2 * (size_t)n)) || (rc = list.ensure(5 * (size_t)n)) ||
            (rc = count.ensure(2 * (size_t)(max_bounce + 1))) ||
            (rc = bins.ensure((size_t)(max_bounce > 0 ? max_bounce : 1) * WF_CELLS)) ||
            (precise && (rc = acc.ensure((size_t)n))))
            return rc;
        w.acc = precise ? acc.ptr : nullptr;
        w.hit = hit.ptr;
        w.list[0] = list.ptr;
        w.list[1] = list.ptr + n;
        w.walk = list.ptr + 2 * n;
        w.walk_key = list.ptr + 3 * n;
        w.walk_sorted = list.ptr + 4 * n;
        w.count = count.ptr;
        w.bins = bins.ptr;
        return 0;
    }
};

template <typename T>
int upload(DBuf<T>& b, const void* src, size_t n, cudaStream_t s)
{
    int rc = b.ensure(n);
    if (rc) return rc;
    if (n) CU(cudaMemcpyAsync(b.ptr, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
    return 0;
}

bool env_float(const char* k, float& v) { const char* s = std::getenv(k); if (!s || !*s) return false; v = std::strtof(s, nullptr); return true; }
bool env_int(const char* k, long long& v) { const char* s = std::getenv(k); if (!s || !*s) return false; v = std::strtoll(s, nullptr, 10); return true; }

uint32_t parse_flag_mask(const char* spec)
{
    static const struct { const char* abbrev; uint32_t flag; } T[] = {
        {"CK", GBO_CERENKOV}, {"SI", GBO_SCINTILLATION}, {"TO", GBO_TORCH}, {"AB", GBO_BULK_ABSORB},
        {"RE", GBO_BULK_REEMIT}, {"SC", GBO_BULK_SCATTER}, {"SD", GBO_SURFACE_DETECT}, {"SA", GBO_SURFACE_ABSORB},
        {"DR", GBO_SURFACE_DREFLECT}, {"SR", GBO_SURFACE_SREFLECT}, {"BR", GBO_BOUNDARY_REFLECT},
        {"BT", GBO_BOUNDARY_TRANSMIT}, {"NA", GBO_NAN_ABORT}, {"EC", GBO_EFFICIENCY_COLLECT},
        {"EX", GBO_EFFICIENCY_CULL}, {"MI", GBO_MISS}};
    uint32_t m = 0;
    std::string s(spec);
    size_t pos = 0;
    while (pos <= s.size()) {
        size_t c = s.find(',', pos);
        std::string tok = s.substr(pos, c == std::string::npos ? std::string::npos : c - pos);
        for (auto& e : T) if (tok == e.abbrev) m |= e.flag;
        if (c == std::string::npos) break;
        pos = c + 1;
    }
    return m;
}

}  // namespace

struct gbo_engine {
    int device = 0;
    gbo_config cfg{};
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;     // hit downloads that overlap the next launch (gbo_simulate_to_host)
    // geometry
    DBuf<BvhNode2> tlas;
    DBuf<int32_t> tlas_index;
    DBuf<InstDev> inst;
    DBuf<double> inst64;                   // precision mode only
    DBuf<InstBox> inst_box;
    DBuf<InstBox> inner_box;
    DBuf<int32_t> overlap;
    DBuf<float> clear;
    DBuf<PrimDev> prim;
    DBuf<SolidDev> solid;
    DBuf<gbo_csgnode> node;
    DBuf<float4> plan;
    DBuf<gbo_qat4> itra;
    DBuf<uint4> optical;
    DBuf<float> bnd_y;
    cudaArray_t bnd_array = nullptr, icdf_array = nullptr;
    cudaTextureObject_t bnd_tex = 0, icdf_tex = 0;
    int bnd_nx = 0, bnd_ny = 0, hd_factor = 0;
    float nm0 = 60.f, nms = 1.f;
    int csg_form = 0;                       // 0: single-leaf prims, 1: boolean trees, 2: CSG list nodes too
    int sms = 0;                            // streaming multiprocessors of the device
    int pool_occ[7] = {0, 0, 0, 0, 0, 0, 0};    // most resident blocks of k_simulate_pool per SM, per kernel form
                                                // (kernel_form())
    // event
    DBuf<gbo_quad6> gs;
    DBuf<unsigned long long> gs_end;
    DBuf<gbo_sphoton> input;
    DBuf<gbo_sphoton> photon;
    DBuf<gbo_seq> seq;
    DBuf<gbo_sphoton> hits_unordered;
    DBuf<gbo_sphoton> hits;
    DBuf<gbo_sphoton> merged;               // hits merged by (identity, time bucket), gbo_merge_hits
    gbo::MergeScratch* merge_scratch = nullptr;     // the merge's work buffers, kept between events
    gbo_server* event_server = nullptr;             // started by the first gbo_event_submit
    std::mutex event_server_mu;
    DBuf<gbo_sphoton> gen_photon;           // kernel modes 2 and 3: pregenerated photons, their random-stream places
    DBuf<ulonglong2> gen_rng;               // and start instances (kernel mode 3: the live photons' state)
    DBuf<int> gen_hint;
    WavefrontBufs wf;                       // kernel mode 3
    DBuf<int> gs_hint;                      // start instance per genstep
    long long num_merged = -1;
    DBuf<uint32_t> bitmap, word_prefix, block_sum;
    DBuf<unsigned long long> block_offset;
    DBuf<unsigned long long> counters;      // [0] unordered hit count, [1] total hits, [2] photons
    unsigned long long* host_counters = nullptr;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};   // upload, simulate, compact, end; [4]
                                                                        // after the generation kernel (mode 2)
    long long num_photon = -1, num_hit = 0;
    int32_t event_id = -1;
    gbo_stats stats{};
};

// Simulation kernels one launch_simulate issues over n photons (the generation kernel counted by the caller): one,
// or in kernel mode 3 the wavefront's start pass and six kernels per step (three passes, the walk queue's sort).
static int simulate_kernels(const gbo_engine* e, long long n)
{
    if (e->cfg.kernel_mode == 3 && n < 0x7fffffffll) return 1 + 6 * e->cfg.max_bounce;
    return 1;
}

// Kernel form index: 2 x csg_form + precision, 6 for the single-leaf binary32 kernels with Philox blocks by call
// (the CSG-tree forms always call; gbo_config.rng_call chooses for the single-leaf binary32 form).
static int kernel_form(const gbo_engine* e)
{
    const bool precise = e->cfg.precision != 0;
    if (e->csg_form == 0 && !precise && e->cfg.rng_call == 1) return 6;
    return 2 * e->csg_form + (precise ? 1 : 0);
}

// One launch of the simulation kernel over n photons in the engine's kernel form (pool or one thread per photon,
// CSG trees or not, precision mode or not); `pool` is the photon-pool counter, zeroed by the caller.  With
// P.gen_photon set (kernel modes 2 and 3) the generation kernel runs first and the pool kernel (or the wavefront
// passes, over `wf`) reads its photons; `after_gen` (optional) is recorded between the two.
static void launch_simulate(const gbo_engine* e, const Params& P, long long n, unsigned long long* pool, cudaStream_t s,
                            cudaEvent_t after_gen = nullptr, const Wavefront* wf = nullptr)
{
    SimLaunch L{};
    L.n = n;
    L.pool = pool;
    L.stream = s;
    L.kernel_mode = e->cfg.kernel_mode;
    L.precise = e->cfg.precision != 0;
    L.rng_call = e->cfg.rng_call == 1;
    L.sms = e->sms;
    if (wf) L.wf = *wf;
    if (L.kernel_mode != 1) {
        if (P.gen_photon && n > 0) {
            const long long per_block = (long long)SIM_BLOCK * GEN_PER_LANE;
            k_generate<<<(unsigned)((n + per_block - 1) / per_block), SIM_BLOCK, 0, s>>>(P);
            if (after_gen) cudaEventRecord(after_gen, s);
        }
        const int form = kernel_form(e);
        const long long need = (n + SIM_BLOCK - 1) / SIM_BLOCK;
        const int want = e->cfg.blocks_per_sm, occ = e->pool_occ[form] > 0 ? e->pool_occ[form] : 1;
        const long long resident = (long long)e->sms * (want > 0 && want < occ ? want : occ);
        L.grid = need < resident ? need : resident;
        L.refill = e->cfg.refill_min < 1 ? 1 : (e->cfg.refill_min > 32 ? 32 : e->cfg.refill_min);
        L.period = e->cfg.refill_period < 1 ? 1 : e->cfg.refill_period;
    }
    switch (e->csg_form) {
        case 2:  sim_launch<2>(P, L); break;
        case 1:  sim_launch<1>(P, L); break;
        default: sim_launch<0>(P, L); break;
    }
}

extern "C" {

const char* gbo_last_error(void) { return g_last_error.c_str(); }

int gbo_config_default(gbo_config* c)
{
    if (!c) return fail(GBO_ERR_ARG, "gbo_config_default: null config");
    std::memset(c, 0, sizeof(*c));
    c->max_bounce = 31;
    c->max_time = 1.e27f;
    c->propagate_epsilon = 0.05f;
    c->propagate_epsilon0 = 0.05f;
    c->epsilon0_mask = GBO_TORCH | GBO_CERENKOV | GBO_SCINTILLATION | GBO_BULK_SCATTER | GBO_BULK_REEMIT;
    c->hit_mask = GBO_SURFACE_DETECT;
    c->rng_seed = 0;
    c->rng_offset = 0;
    c->event_skipahead = 100000;
    c->tmax = 1000000.f;
    c->debug_tag = 1;
    c->record_photon = 0;
    c->record_seq = 0;
    c->max_photon = 0;
    c->kernel_mode = 2;
    c->refill_min = 4;
    c->blocks_per_sm = 0;
    c->refill_period = 1;
    c->walk_min = 1;
    c->rng_call = 1;
    c->max_slot = 0;
    long long iv;
    float fv;
    if (env_int("OPTICKS_MAX_BOUNCE", iv)) c->max_bounce = (int32_t)iv;
    if (env_float("OPTICKS_MAX_TIME", fv)) c->max_time = fv;
    if (env_float("OPTICKS_PROPAGATE_EPSILON", fv)) c->propagate_epsilon = fv;
    if (env_float("OPTICKS_PROPAGATE_EPSILON0", fv)) c->propagate_epsilon0 = fv;
    if (const char* s = std::getenv("OPTICKS_PROPAGATE_EPSILON0_MASK")) c->epsilon0_mask = parse_flag_mask(s);
    if (const char* s = std::getenv("OPTICKS_HIT_MASK")) c->hit_mask = parse_flag_mask(s);
    if (env_int("OPTICKS_EVENT_SKIPAHEAD", iv)) c->event_skipahead = (uint64_t)iv;
    if (env_int("OPTICKS_MAX_SLOT", iv)) c->max_slot = iv;
    if (const char* s = std::getenv("QRng__SEED_OFFSET")) {
        char* end = nullptr;
        c->rng_seed = std::strtoull(s, &end, 10);
        if (end && *end == ':') c->rng_offset = std::strtoull(end + 1, nullptr, 10);
    }
    return GBO_OK;
}

static int make_texture(cudaArray_t* arr, cudaTextureObject_t* tex, const void* data, int nx, int ny, bool f4)
{
    cudaChannelFormatDesc ch = f4 ? cudaCreateChannelDesc<float4>() : cudaCreateChannelDesc<float>();
    CU(cudaMallocArray(arr, &ch, (size_t)nx, (size_t)ny));
    const size_t row = (size_t)nx * (f4 ? 16 : 4);
    CU(cudaMemcpy2DToArray(*arr, 0, 0, data, row, row, (size_t)ny, cudaMemcpyHostToDevice));
    cudaResourceDesc res;
    std::memset(&res, 0, sizeof(res));
    res.resType = cudaResourceTypeArray;
    res.res.array.array = *arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = cudaAddressModeWrap;
    td.addressMode[1] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    CU(cudaCreateTextureObject(tex, &res, &td, nullptr));
    return 0;
}

void gbo_engine_destroy(gbo_engine* e)
{
    if (!e) return;
    if (e->event_server) gbo_server_destroy(e->event_server);
    e->event_server = nullptr;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->bnd_tex) cudaDestroyTextureObject(e->bnd_tex);
    if (e->icdf_tex) cudaDestroyTextureObject(e->icdf_tex);
    if (e->bnd_array) cudaFreeArray(e->bnd_array);
    if (e->icdf_array) cudaFreeArray(e->icdf_array);
    e->tlas.release(); e->tlas_index.release(); e->inst.release(); e->inst64.release(); e->inst_box.release(); e->bnd_y.release(); e->inner_box.release(); e->overlap.release(); e->clear.release(); e->prim.release(); e->solid.release();
    e->node.release(); e->plan.release(); e->itra.release(); e->optical.release();
    e->gs.release(); e->gs_end.release(); e->input.release(); e->photon.release(); e->seq.release();
    e->hits_unordered.release(); e->hits.release(); e->merged.release(); gbo::merge_scratch_free(e->merge_scratch); e->merge_scratch = nullptr; e->gen_photon.release(); e->gen_rng.release(); e->gen_hint.release(); e->wf.release(); e->gs_hint.release(); e->bitmap.release(); e->word_prefix.release();
    e->block_sum.release(); e->block_offset.release(); e->counters.release();
    if (e->host_counters) cudaFreeHost(e->host_counters);
    for (auto& v : e->ev) if (v) cudaEventDestroy(v);
    if (e->stream) cudaStreamDestroy(e->stream);
    if (e->copy_stream) cudaStreamDestroy(e->copy_stream);
    delete e;
}

int gbo_engine_create(const gbo_geometry_desc* g, const gbo_config* cfg, int device, gbo_engine** out)
{
    if (!g || !out) return fail(GBO_ERR_ARG, "gbo_engine_create: null argument");
    *out = nullptr;
    if (!g->node || !g->prim || !g->solid || !g->inst || !g->bnd || !g->optical || !g->icdf)
        return fail(GBO_ERR_ARG, "gbo_engine_create: geometry array missing");
    if (g->num_bnd <= 0 || g->bnd_nx <= 1 || g->icdf_nx <= 1 || (g->icdf_ny != 1 && g->icdf_ny != 3))
        return fail(GBO_ERR_ARG, "gbo_engine_create: bad table shape (num_bnd %d bnd_nx %d icdf %dx%d)", g->num_bnd,
                    g->bnd_nx, g->icdf_ny, g->icdf_nx);
    if (g->hd_factor != 0 && g->hd_factor != 10 && g->hd_factor != 20)
        return fail(GBO_ERR_ARG, "gbo_engine_create: hd_factor %d not in {0,10,20}", g->hd_factor);
    if (g->bnd_domain_step <= 0.f) return fail(GBO_ERR_ARG, "gbo_engine_create: bnd_domain_step must be positive");
    int ndev = 0;
    CU(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(GBO_ERR_ARG, "gbo_engine_create: device %d of %d", device, ndev);
    CU(cudaSetDevice(device));

    AccelHost acc;
    char err[512] = {0};
    if (build_accel(g->node, g->num_node, g->prim, g->num_prim, g->solid, g->num_solid, g->inst, g->num_inst, acc, err,
                    sizeof(err)))
        return fail(GBO_ERR_ARG, "gbo_engine_create: %s", err);
    for (int n = 0; n < g->num_node; n++) {
        const unsigned tc = g->node[n].q3.u[2];
        const unsigned gt = g->node[n].q3.u[3] & 0x7fffffffu;
        if (tc >= GBO_CSG_UNION && tc <= GBO_CSG_DIFFERENCE) {}
        if (gt > (unsigned)g->num_itra) return fail(GBO_ERR_ARG, "node %d transform %u beyond %d itra", n, gt, g->num_itra);
    }
    // list nodes: every sub a leaf inside the prim that holds the list (the device code indexes subs from the root)
    for (int p = 0; p < g->num_prim; p++) {
        const int noff = g->prim[p].q0.i[1], nn = g->prim[p].q0.i[0];
        if (g->node[noff].q3.u[2] < GBO_CSG_NODE) {         // boolean tree: a complete binary tree inside the prim
            const unsigned tree_n = g->node[noff].q0.u[0];
            if (tree_n < 1 || tree_n > (unsigned)nn || tree_n > 255u || ((tree_n + 1) & tree_n) != 0)
                return fail(GBO_ERR_ARG, "prim %d: tree of %u nodes in a prim of %d nodes", p, tree_n, nn);
        }
        for (int k = 0; k < nn; k++) {
            const gbo_csgnode& nd = g->node[noff + k];
            const unsigned tc = nd.q3.u[2];
            if (tc < GBO_CSG_NODE || tc >= GBO_CSG_LEAF) continue;
            if (tc > GBO_CSG_OVERLAP) return fail(GBO_ERR_ARG, "prim %d node %d: typecode %u is not a CSG list", p, k, tc);
            const unsigned num_sub = nd.q0.u[0], off = nd.q0.u[1];
            if (off < 1 || (long long)off + num_sub > (long long)nn)
                return fail(GBO_ERR_ARG, "prim %d node %d: list subs [%u,+%u) outside the prim's %d nodes", p, k, off, num_sub, nn);
            for (unsigned j = 0; j < num_sub; j++)
                if (g->node[noff + off + j].q3.u[2] < GBO_CSG_LEAF)
                    return fail(GBO_ERR_ARG, "prim %d node %d: list sub %u is not a leaf", p, k, j);
        }
    }

    if (cfg && (cfg->kernel_mode < 0 || cfg->kernel_mode > 3))
        return fail(GBO_ERR_ARG, "kernel_mode %d not in 0..3", cfg->kernel_mode);
    gbo_engine* e = new gbo_engine();
    e->device = device;
    if (cfg) e->cfg = *cfg; else gbo_config_default(&e->cfg);
    int rc = 0;
#define TRY(x) do { rc = (x); if (rc) { gbo_engine_destroy(e); return rc; } } while (0)
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        gbo_engine_destroy(e);
        return fail(GBO_ERR_CUDA, "cudaStreamCreate failed");
    }
    for (auto& v : e->ev) if (cudaEventCreate(&v) != cudaSuccess) { gbo_engine_destroy(e); return fail(GBO_ERR_CUDA, "cudaEventCreate failed"); }
    if (cudaMallocHost(&e->host_counters, 4 * sizeof(unsigned long long)) != cudaSuccess) {
        gbo_engine_destroy(e);
        return fail(GBO_ERR_CUDA, "cudaMallocHost failed");
    }
    for (int p = 0; p < g->num_prim; p++) {
        const int noff = g->prim[p].q0.i[1], nn = g->prim[p].q0.i[0];
        for (int k = 0; k < nn; k++) {
            const unsigned tc = g->node[noff + k].q3.u[2];
            if (tc >= GBO_CSG_NODE && tc < GBO_CSG_LEAF) e->csg_form = 2;                  // a list node
            else if (tc < GBO_CSG_NODE && k == 0 && e->csg_form < 1) e->csg_form = 1;     // a boolean tree
        }
    }
    TRY(upload(e->tlas, acc.tlas2.data(), acc.tlas2.size(), e->stream));
    TRY(upload(e->tlas_index, acc.tlas_index.data(), acc.tlas_index.size(), e->stream));
    TRY(upload(e->inst, acc.inst.data(), acc.inst.size(), e->stream));
    if (e->cfg.precision) TRY(upload(e->inst64, acc.inst64.data(), acc.inst64.size(), e->stream));
    TRY(upload(e->inst_box, acc.inst_box.data(), acc.inst_box.size(), e->stream));
    TRY(upload(e->inner_box, acc.inner_box.data(), acc.inner_box.size(), e->stream));
    TRY(upload(e->overlap, acc.overlap.data(), acc.overlap.size(), e->stream));
    TRY(upload(e->clear, acc.clear.data(), acc.clear.size(), e->stream));
    TRY(upload(e->prim, acc.prim.data(), acc.prim.size(), e->stream));
    TRY(upload(e->solid, acc.solid.data(), acc.solid.size(), e->stream));
    TRY(upload(e->node, g->node, (size_t)g->num_node, e->stream));
    std::vector<float4> plan(g->num_plan > 0 ? g->num_plan : 1, make_float4(0, 0, 0, 0));
    if (g->num_plan > 0 && g->plan) std::memcpy(plan.data(), g->plan, sizeof(float4) * g->num_plan);
    TRY(upload(e->plan, plan.data(), plan.size(), e->stream));
    std::vector<gbo_qat4> itra(g->num_itra > 0 ? g->num_itra : 1);
    if (g->num_itra > 0 && g->itra) std::memcpy(itra.data(), g->itra, sizeof(gbo_qat4) * g->num_itra);
    TRY(upload(e->itra, itra.data(), itra.size(), e->stream));
    TRY(upload(e->optical, g->optical, (size_t)g->num_bnd * 4, e->stream));
    e->bnd_nx = g->bnd_nx;
    e->bnd_ny = g->num_bnd * 8;
    e->nm0 = g->bnd_domain_low;
    e->nms = g->bnd_domain_step;
    e->hd_factor = g->hd_factor;
    TRY(make_texture(&e->bnd_array, &e->bnd_tex, g->bnd, e->bnd_nx, e->bnd_ny, true));
    {
        // each boundary-texture row's normalized y, the binary32 quotient the lookups would otherwise divide out
        std::vector<float> y((size_t)e->bnd_ny);
        const float rows = (float)e->bnd_ny;
        for (int iy = 0; iy < e->bnd_ny; iy++) y[(size_t)iy] = ((float)iy + 0.5f) / rows;
        TRY(upload(e->bnd_y, y.data(), y.size(), e->stream));
    }
    TRY(make_texture(&e->icdf_array, &e->icdf_tex, g->icdf, g->icdf_nx, g->icdf_ny, false));
    TRY(e->counters.ensure(4));
    {
        int sms = 0, b[7] = {0, 0, 0, 0, 0, 0, 0};     // indexed by kernel_form()
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
            sim_pool_occupancy<0>(false, false, &b[0]) != cudaSuccess ||
            sim_pool_occupancy<0>(true, false, &b[1]) != cudaSuccess ||
            sim_pool_occupancy<1>(false, true, &b[2]) != cudaSuccess ||
            sim_pool_occupancy<1>(true, true, &b[3]) != cudaSuccess ||
            sim_pool_occupancy<2>(false, true, &b[4]) != cudaSuccess ||
            sim_pool_occupancy<2>(true, true, &b[5]) != cudaSuccess ||
            sim_pool_occupancy<0>(false, true, &b[6]) != cudaSuccess) {
            gbo_engine_destroy(e);
            return fail(GBO_ERR_CUDA, "occupancy query failed");
        }
        e->sms = sms;
        for (int f = 0; f < 7; f++) e->pool_occ[f] = b[f];
    }
    if (cudaStreamSynchronize(e->stream) != cudaSuccess) {
        gbo_engine_destroy(e);
        return fail(GBO_ERR_CUDA, "geometry upload failed");
    }
#undef TRY
    *out = e;
    return GBO_OK;
}

static Params make_params(gbo_engine* e)
{
    Params P;
    std::memset(&P, 0, sizeof(P));
    P.acc.tlas = e->tlas.ptr;
    P.acc.tlas_index = e->tlas_index.ptr;
    P.acc.inst = e->inst.ptr;
    P.acc.inst64 = e->inst64.ptr;
    P.acc.inst_box = reinterpret_cast<const float4*>(e->inst_box.ptr);
    P.acc.inner_box = reinterpret_cast<const float4*>(e->inner_box.ptr);
    P.acc.overlap = e->overlap.ptr;
    P.acc.clear = reinterpret_cast<const float4*>(e->clear.ptr);
    P.acc.prim = e->prim.ptr;
    P.acc.solid = e->solid.ptr;
    P.acc.node = e->node.ptr;
    P.acc.plan = e->plan.ptr;
    P.acc.itra = e->itra.ptr;
    P.tab.bnd_tex = e->bnd_tex;
    P.tab.bnd_y = e->bnd_y.ptr;
    P.tab.bnd_nx = (float)e->bnd_nx;
    P.tab.bnd_ny = (float)e->bnd_ny;
    P.tab.nm0 = e->nm0;
    P.tab.nms = e->nms;
    P.tab.optical = e->optical.ptr;
    P.tab.icdf_tex = e->icdf_tex;
    P.tab.hd_factor = e->hd_factor;
    P.tab.debug_tag = e->cfg.debug_tag;
    P.max_bounce = e->cfg.max_bounce;
    P.max_time = e->cfg.max_time;
    P.tmin = e->cfg.propagate_epsilon;
    P.tmin0 = e->cfg.propagate_epsilon0;
    P.tmax = e->cfg.tmax;
    P.eps0_mask = e->cfg.epsilon0_mask;
    P.hitmask = e->cfg.hit_mask;
    P.seed = e->cfg.rng_seed;
    P.walk_min = e->cfg.walk_min < 1 ? 1 : (e->cfg.walk_min > 32 ? 32 : e->cfg.walk_min);
    return P;
}

// Where one launch of an event goes: a launch covers event photons [photon_offset, photon_offset + n) and writes
// its photon/seq records from photon_base and its ordered hits from hit_base; `capacity` photons are reserved for
// the whole event so that later launches of a sliced event do not reallocate.
struct LaunchPlace {
    unsigned long long photon_offset = 0;
    long long photon_base = 0;
    long long hit_base = 0;
    long long capacity = 0;
};

// runs one launch whose gensteps (and input photons) are already on the device
// (d_gs_end: the launch's inclusive photon-count prefix of its gensteps)
static int run_event(gbo_engine* e, int32_t event_id, const gbo_quad6* d_gs, const unsigned long long* d_gs_end,
                     int64_t num_gs, const gbo_sphoton* d_input, int64_t num_input, long long num_photon,
                     cudaStream_t s, int prior_launches, LaunchPlace at = LaunchPlace())
{
    const bool keep_photon = e->cfg.record_photon != 0;
    const bool keep_seq = e->cfg.record_seq != 0;
    int rc;
    if (at.capacity < at.photon_base + num_photon) at.capacity = at.photon_base + num_photon;
    if (e->cfg.max_photon > 0 && at.capacity > e->cfg.max_photon)
        return fail(GBO_ERR_CAPACITY, "event of %lld photons above max_photon %lld", at.capacity, (long long)e->cfg.max_photon);
    if (num_input > 0 && num_input < num_photon)
        return fail(GBO_ERR_ARG, "%lld input photons for %lld photon slots", (long long)num_input, num_photon);
    const long long words = (num_photon + 31) / 32;
    const long long nblk = (words + SCAN_WORDS - 1) / SCAN_WORDS;
    if ((rc = e->bitmap.ensure(words))) return rc;
    if ((rc = e->word_prefix.ensure(words))) return rc;
    if ((rc = e->block_sum.ensure(nblk))) return rc;
    if ((rc = e->block_offset.ensure(nblk))) return rc;
    if (at.photon_base == 0 && (rc = e->hits.ensure(at.capacity))) return rc;
    if (keep_photon) { if (at.photon_base == 0 && (rc = e->photon.ensure(at.capacity))) return rc; }
    else { if ((rc = e->hits_unordered.ensure(num_photon))) return rc; }
    if (keep_seq && at.photon_base == 0) { if ((rc = e->seq.ensure(at.capacity))) return rc; }
    if (e->cfg.kernel_mode >= 2) {
        if ((rc = e->gen_photon.ensure(num_photon))) return rc;
        if ((rc = e->gen_rng.ensure(num_photon))) return rc;
        if ((rc = e->gen_hint.ensure(num_photon))) return rc;
    }
    Wavefront wf{};
    if (e->cfg.kernel_mode == 3 && (rc = e->wf.ensure(num_photon, e->cfg.max_bounce, e->cfg.precision != 0, wf)))
        return rc;
    if (num_gs > 0 && (rc = e->gs_hint.ensure(num_gs))) return rc;

    Params P = make_params(e);
    const uint64_t skip = e->cfg.event_skipahead * (uint64_t)(event_id < 0 ? 0 : event_id);
    P.position0 = e->cfg.rng_offset + skip;
    P.gs = reinterpret_cast<const float4*>(d_gs);
    P.gs_end = d_gs_end;
    P.num_gs = (int)num_gs;
    P.num_photon = num_photon;
    P.photon_offset = at.photon_offset;
    P.input_photon = d_input;
    P.photon_out = keep_photon ? e->photon.ptr + at.photon_base : nullptr;
    P.seq_out = keep_seq ? e->seq.ptr + at.photon_base : nullptr;
    P.hit_unordered = keep_photon ? nullptr : e->hits_unordered.ptr;
    P.hit_count = e->counters.ptr;
    P.bitmap = e->bitmap.ptr;

    CU(cudaMemsetAsync(e->counters.ptr, 0, 4 * sizeof(unsigned long long), s));
    int launches = prior_launches;
    const bool pool = e->cfg.kernel_mode != 1;
    if (pool && num_photon > 0) CU(cudaMemsetAsync(e->bitmap.ptr, 0, (size_t)words * sizeof(uint32_t), s));
    if (e->cfg.kernel_mode >= 2 && num_photon > 0) {
        P.gen_photon = e->gen_photon.ptr;
        P.gen_rng = e->gen_rng.ptr;
        P.gen_hint = e->gen_hint.ptr;
        launches++;
    }
    if (num_photon > 0) {
        k_genstep_hint<<<(unsigned)((num_gs + 127) / 128), 128, 0, s>>>(P.acc, P.gs, (int)num_gs, e->gs_hint.ptr);
        P.gs_hint = e->gs_hint.ptr;
        launches++;
    }
    CU(cudaEventRecord(e->ev[1], s));
    if (num_photon > 0) {
        launch_simulate(e, P, num_photon, e->counters.ptr + 2, s, P.gen_photon ? e->ev[4] : nullptr,
                        e->cfg.kernel_mode == 3 ? &wf : nullptr);
        CU(cudaGetLastError());
        launches += simulate_kernels(e, num_photon);
    }
    CU(cudaEventRecord(e->ev[2], s));
    if (num_photon > 0) {
        k_word_prefix<<<(unsigned)nblk, SCAN_WORDS, 0, s>>>(e->bitmap.ptr, words, e->word_prefix.ptr, e->block_sum.ptr);
        k_block_offsets<<<1, 1024, 0, s>>>(e->block_sum.ptr, nblk, e->block_offset.ptr, e->counters.ptr + 1);
        launches += 2;
        if (keep_photon) {
            const long long threads = words * 32;
            k_gather_photons<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
                e->photon.ptr + at.photon_base, e->bitmap.ptr, e->word_prefix.ptr, e->block_offset.ptr, words,
                e->hits.ptr + at.hit_base);
        } else {
            // the unordered count is only known on the device: launch for the worst case and let threads exit
            k_gather_unordered<<<(unsigned)((num_photon + 255) / 256), 256, 0, s>>>(
                e->hits_unordered.ptr, e->counters.ptr, at.photon_offset, e->bitmap.ptr, e->word_prefix.ptr,
                e->block_offset.ptr, e->hits.ptr + at.hit_base);
        }
        launches++;
        CU(cudaGetLastError());
    }
    CU(cudaEventRecord(e->ev[3], s));
    CU(cudaMemcpyAsync(e->host_counters, e->counters.ptr, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    e->num_photon = at.photon_base + num_photon;
    e->num_hit = at.hit_base + (long long)e->host_counters[1];
    e->num_merged = -1;
    e->event_id = event_id;
    e->stats.num_photon = e->num_photon;
    e->stats.num_hit = e->num_hit;
    e->stats.simulate_launches = num_photon > 0 ? 1 : 0;
    e->stats.kernel_launches = launches;
    cudaEventElapsedTime(&e->stats.ms_upload, e->ev[0], e->ev[1]);
    cudaEventElapsedTime(&e->stats.ms_simulate, e->ev[1], e->ev[2]);
    cudaEventElapsedTime(&e->stats.ms_compact, e->ev[2], e->ev[3]);
    e->stats.ms_generate = 0.f;
    if (P.gen_photon) cudaEventElapsedTime(&e->stats.ms_generate, e->ev[1], e->ev[4]);
    return GBO_OK;
}

// Where gbo_simulate_to_host puts an event's hits: the caller's host buffer of `capacity` hits.
struct HitSink {
    gbo_sphoton* host;
    int64_t capacity;
};

// Host-side checks shared by the host-genstep entry points; the event's photon count into *total.
static int check_host_event(const char* fn, const gbo_quad6* gs, int64_t num_gs, const gbo_sphoton* input_photon,
                            int64_t num_input_photon, unsigned long long* total)
{
    if (num_gs < 0 || (num_gs > 0 && !gs)) return fail(GBO_ERR_ARG, "%s: bad gensteps", fn);
    if (num_gs > 0x7fffffff) return fail(GBO_ERR_CAPACITY, "%s: %lld gensteps", fn, (long long)num_gs);
    if (num_input_photon < 0 || (num_input_photon > 0 && !input_photon)) return fail(GBO_ERR_ARG, "%s: bad input photons", fn);
    unsigned long long n = 0;
    bool has_input_gs = false;
    for (int64_t i = 0; i < num_gs; i++) {
        n += gs[i].q[0].u[3];
        if (gs[i].q[0].i[0] == GBO_GS_INPUT_PHOTON) has_input_gs = true;
    }
    if (has_input_gs && (long long)num_input_photon < (long long)n)
        return fail(GBO_ERR_ARG, "%s: INPUT_PHOTON gensteps need %llu photons, %lld given", fn, n, (long long)num_input_photon);
    *total = n;
    return GBO_OK;
}

// Genstep ranges [g0, g1) of the launches of one event: launches of at most max_slot photons at genstep
// granularity (SGenstep::GetGenstepSlices, qudarap/QSim.cc:481-529) when max_slot is set, else one launch.
static std::vector<std::pair<int64_t, int64_t>> launch_ranges(const gbo_quad6* gs, int64_t num_gs, long long max_slot)
{
    std::vector<std::pair<int64_t, int64_t>> r;
    if (max_slot > 0) {
        int64_t g0 = 0;
        while (g0 < num_gs) {
            int64_t g1 = g0;
            unsigned long long n = 0;
            while (g1 < num_gs && (g1 == g0 || (long long)(n + gs[g1].q[0].u[3]) <= max_slot)) n += gs[g1++].q[0].u[3];
            r.push_back({g0, g1});
            g0 = g1;
        }
        return r;
    }
    r.push_back({0, num_gs});
    return r;
}

// One event from host gensteps as the launches `ranges`.  Every photon keeps its event-level index
// (photon_slot_offset + idx, CSGOptiX7.cu:415), so the event's results do not depend on the launches.  With a
// sink, each launch's ordered hits go to the host buffer on the copy stream as soon as the launch ends, as the
// reference gathers each genstep slice's hits to the host in turn; the call returns when the last copy has landed.
// (On a GB300 with NVLink-C2C host memory, CUDA-event probes showed the next launch's first command on the
// simulation stream completing only when such a copy ended: the copies do not overlap the launches there.)
static int simulate_ranges(gbo_engine* e, int32_t event_id, const gbo_quad6* gs,
                           const std::vector<std::pair<int64_t, int64_t>>& ranges, const gbo_sphoton* input_photon,
                           int64_t num_input_photon, unsigned long long total, const HitSink* sink)
{
    cudaStream_t s = e->stream;
    const int64_t num_gs = ranges.empty() ? 0 : ranges.back().second;
    // every launch's gensteps and photon-count prefixes (from each launch's first genstep) go to the device before
    // the first launch: a host copy issued between launches queues behind the previous launch's hit download.  Input
    // photons still go up per launch, so that max_slot bounds their device memory too
    std::vector<unsigned long long> part((size_t)num_gs);
    for (const auto& gr : ranges) {
        unsigned long long c = 0;
        for (int64_t i = gr.first; i < gr.second; i++) { c += gs[i].q[0].u[3]; part[(size_t)i] = c; }
    }
    const bool inp = num_input_photon > 0;
    CU(cudaEventRecord(e->ev[0], s));
    int rc;
    if ((rc = upload(e->gs, gs, (size_t)num_gs, s))) return rc;
    if ((rc = upload(e->gs_end, part.data(), part.size(), s))) return rc;
    LaunchPlace at;
    at.capacity = (long long)total;
    gbo_stats acc{};
    for (const auto& gr : ranges) {
        const int64_t g0 = gr.first, g1 = gr.second;
        const unsigned long long n = g1 > g0 ? part[(size_t)(g1 - 1)] : 0ull;
        if (g0 > 0) CU(cudaEventRecord(e->ev[0], s));
        if (inp && n > 0 && (rc = upload(e->input, input_photon + at.photon_offset, (size_t)n, s))) break;
        if ((rc = run_event(e, event_id, e->gs.ptr + g0, e->gs_end.ptr + g0, g1 - g0, inp ? e->input.ptr : nullptr,
                            inp ? (int64_t)n : 0, (long long)n, s, 0, at)))
            break;
        if (sink) {
            // run_event returned after its stream finished: this launch's hits [hit_base, num_hit) are final and
            // the launches that follow write beyond them
            const long long lo = std::min<long long>(at.hit_base, sink->capacity);
            const long long hi = std::min<long long>(e->num_hit, sink->capacity);
            if (hi > lo) {
                const cudaError_t ce = cudaMemcpyAsync(sink->host + lo, e->hits.ptr + lo, (size_t)(hi - lo) * sizeof(gbo_sphoton),
                                                       cudaMemcpyDeviceToHost, e->copy_stream);
                if (ce != cudaSuccess) { rc = fail(GBO_ERR_CUDA, "hit download: %s", cudaGetErrorString(ce)); break; }
            }
        }
        acc.ms_upload += e->stats.ms_upload;
        acc.ms_simulate += e->stats.ms_simulate;
        acc.ms_compact += e->stats.ms_compact;
        acc.ms_generate += e->stats.ms_generate;
        acc.simulate_launches += e->stats.simulate_launches;
        acc.kernel_launches += e->stats.kernel_launches;
        at.photon_offset += n;
        at.photon_base += (long long)n;
        at.hit_base = e->num_hit;
    }
    if (sink) {
        const cudaError_t ce = cudaStreamSynchronize(e->copy_stream);
        if (rc == GBO_OK && ce != cudaSuccess) rc = fail(GBO_ERR_CUDA, "hit download: %s", cudaGetErrorString(ce));
    }
    if (rc) return rc;
    acc.num_photon = e->num_photon;
    acc.num_hit = e->num_hit;
    e->stats = acc;
    return GBO_OK;
}

int gbo_simulate(gbo_engine* e, int32_t event_id, const gbo_quad6* gs, int64_t num_gs, const gbo_sphoton* input_photon,
                 int64_t num_input_photon)
{
    if (!e) return fail(GBO_ERR_ARG, "gbo_simulate: null engine");
    unsigned long long total = 0;
    int rc;
    if ((rc = check_host_event("gbo_simulate", gs, num_gs, input_photon, num_input_photon, &total))) return rc;
    CU(cudaSetDevice(e->device));
    return simulate_ranges(e, event_id, gs, launch_ranges(gs, num_gs, e->cfg.max_slot), input_photon,
                           num_input_photon, total, nullptr);
}

int gbo_simulate_to_host(gbo_engine* e, int32_t event_id, const gbo_quad6* gs, int64_t num_gs,
                         const gbo_sphoton* input_photon, int64_t num_input_photon, gbo_sphoton* hits,
                         int64_t hit_capacity, int64_t* num_hit)
{
    if (!e || !num_hit) return fail(GBO_ERR_ARG, "gbo_simulate_to_host: null argument");
    if (hit_capacity < 0 || (hit_capacity > 0 && !hits)) return fail(GBO_ERR_ARG, "gbo_simulate_to_host: bad hit buffer");
    unsigned long long total = 0;
    int rc;
    if ((rc = check_host_event("gbo_simulate_to_host", gs, num_gs, input_photon, num_input_photon, &total))) return rc;
    CU(cudaSetDevice(e->device));
    const HitSink sink{hits, hit_capacity};
    if ((rc = simulate_ranges(e, event_id, gs, launch_ranges(gs, num_gs, e->cfg.max_slot), input_photon,
                              num_input_photon, total, &sink)))
        return rc;
    *num_hit = e->num_hit;
    if (e->num_hit > hit_capacity)
        return fail(GBO_ERR_CAPACITY, "gbo_simulate_to_host: %lld hits for a buffer of %lld", e->num_hit, (long long)hit_capacity);
    return GBO_OK;
}

int gbo_simulate_slice(gbo_engine* e, int32_t event_id, const gbo_quad6* gs, int64_t num_gs,
                       const gbo_sphoton* input_photon, int64_t num_input_photon, uint64_t photon_offset)
{
    if (!e) return fail(GBO_ERR_ARG, "gbo_simulate_slice: null engine");
    if (num_gs < 0 || (num_gs > 0 && !gs)) return fail(GBO_ERR_ARG, "gbo_simulate_slice: bad gensteps");
    if (num_gs > 0x7fffffff) return fail(GBO_ERR_CAPACITY, "gbo_simulate_slice: %lld gensteps", (long long)num_gs);
    if (num_input_photon < 0 || (num_input_photon > 0 && !input_photon)) return fail(GBO_ERR_ARG, "gbo_simulate_slice: bad input photons");
    CU(cudaSetDevice(e->device));
    std::vector<unsigned long long> end((size_t)num_gs);
    unsigned long long total = 0;
    bool has_input_gs = false;
    for (int64_t i = 0; i < num_gs; i++) {
        total += gs[i].q[0].u[3];
        end[(size_t)i] = total;
        if (gs[i].q[0].i[0] == GBO_GS_INPUT_PHOTON) has_input_gs = true;
    }
    if (has_input_gs && (long long)num_input_photon < (long long)total)
        return fail(GBO_ERR_ARG, "gbo_simulate_slice: INPUT_PHOTON gensteps need %llu photons, %lld given", total,
                    (long long)num_input_photon);
    cudaStream_t s = e->stream;
    CU(cudaEventRecord(e->ev[0], s));
    int rc;
    if ((rc = upload(e->gs, gs, (size_t)num_gs, s))) return rc;
    if ((rc = upload(e->gs_end, end.data(), end.size(), s))) return rc;
    if (num_input_photon > 0) { if ((rc = upload(e->input, input_photon, (size_t)num_input_photon, s))) return rc; }
    LaunchPlace at;
    at.photon_offset = photon_offset;
    return run_event(e, event_id, e->gs.ptr, e->gs_end.ptr, num_gs, num_input_photon > 0 ? e->input.ptr : nullptr, num_input_photon,
                     (long long)total, s, 0, at);
}

int gbo_simulate_device(gbo_engine* e, int32_t event_id, const void* d_gs, int64_t num_gs, const void* d_input,
                        int64_t num_input, void* stream)
{
    if (!e) return fail(GBO_ERR_ARG, "gbo_simulate_device: null engine");
    if (num_gs < 0 || (num_gs > 0 && !d_gs)) return fail(GBO_ERR_ARG, "gbo_simulate_device: bad gensteps");
    if (num_gs > 0x7fffffff) return fail(GBO_ERR_CAPACITY, "gbo_simulate_device: %lld gensteps", (long long)num_gs);
    if (num_input < 0 || (num_input > 0 && !d_input)) return fail(GBO_ERR_ARG, "gbo_simulate_device: bad input photons");
    CU(cudaSetDevice(e->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    int rc;
    // one slot past the prefix receives the INPUT_PHOTON flag
    if ((rc = e->gs_end.ensure((size_t)num_gs + 1))) return rc;
    CU(cudaEventRecord(e->ev[0], s));
    unsigned long long total = 0;
    if (num_gs > 0) {
        k_genstep_prefix<<<1, 1024, 0, s>>>((const gbo_quad6*)d_gs, (int)num_gs, e->gs_end.ptr, e->gs_end.ptr + num_gs);
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(e->host_counters + 2, e->gs_end.ptr + (num_gs - 1), 2 * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        total = e->host_counters[2];
        if (e->host_counters[3] && (long long)num_input < (long long)total)
            return fail(GBO_ERR_ARG, "gbo_simulate_device: INPUT_PHOTON gensteps need %llu photons, %lld given", total,
                        (long long)num_input);
    }
    return run_event(e, event_id, (const gbo_quad6*)d_gs, e->gs_end.ptr, num_gs, (const gbo_sphoton*)d_input, num_input,
                     (long long)total, s, num_gs > 0 ? 1 : 0);
}

int64_t gbo_num_hit(const gbo_engine* e) { return e && e->num_photon >= 0 ? e->num_hit : -1; }
int64_t gbo_num_photon(const gbo_engine* e) { return e ? e->num_photon : -1; }
const void* gbo_device_hits(const gbo_engine* e) { return e ? e->hits.ptr : nullptr; }

int gbo_copy_hits(gbo_engine* e, gbo_sphoton* dst, int64_t offset, int64_t count)
{
    if (!e || (!dst && count > 0)) return fail(GBO_ERR_ARG, "gbo_copy_hits: null argument");
    if (e->num_photon < 0) return fail(GBO_ERR_STATE, "gbo_copy_hits: no event simulated");
    if (offset < 0 || count < 0 || offset + count > e->num_hit)
        return fail(GBO_ERR_ARG, "gbo_copy_hits: range [%lld,+%lld) outside %lld hits", (long long)offset, (long long)count, e->num_hit);
    if (count == 0) return GBO_OK;
    CU(cudaSetDevice(e->device));
    CU(cudaMemcpyAsync(dst, e->hits.ptr + offset, (size_t)count * sizeof(gbo_sphoton), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    return GBO_OK;
}

int gbo_merge_hits(gbo_engine* e, float time_window, int64_t* num_merged)
{
    if (!e || !num_merged) return fail(GBO_ERR_ARG, "gbo_merge_hits: null argument");
    if (e->num_photon < 0) return fail(GBO_ERR_STATE, "gbo_merge_hits: no event simulated");
    if (!(time_window >= 0.f)) return fail(GBO_ERR_ARG, "gbo_merge_hits: time window %g", (double)time_window);
    CU(cudaSetDevice(e->device));
    int rc;
    if ((rc = e->merged.ensure(e->num_hit > 0 ? e->num_hit : 1))) return rc;
    int64_t n = 0;
    if (!e->merge_scratch) e->merge_scratch = gbo::merge_scratch_new();
    rc = gbo::merge_hits(e->hits.ptr, e->num_hit, time_window, e->merged.ptr, &n, e->stream, e->merge_scratch);
    if (rc) return fail(rc, "gbo_merge_hits: merge of %lld hits failed", e->num_hit);
    e->num_merged = n;
    *num_merged = n;
    return GBO_OK;
}

int gbo_copy_merged_hits(gbo_engine* e, gbo_sphoton* dst, int64_t offset, int64_t count)
{
    if (!e || (!dst && count > 0)) return fail(GBO_ERR_ARG, "gbo_copy_merged_hits: null argument");
    if (e->num_merged < 0) return fail(GBO_ERR_STATE, "gbo_copy_merged_hits: gbo_merge_hits not called");
    if (offset < 0 || count < 0 || offset + count > e->num_merged)
        return fail(GBO_ERR_ARG, "gbo_copy_merged_hits: range outside %lld merged hits", e->num_merged);
    if (count == 0) return GBO_OK;
    CU(cudaSetDevice(e->device));
    CU(cudaMemcpyAsync(dst, e->merged.ptr + offset, (size_t)count * sizeof(gbo_sphoton), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    return GBO_OK;
}

int gbo_copy_photons(gbo_engine* e, gbo_sphoton* dst, int64_t offset, int64_t count)
{
    if (!e || (!dst && count > 0)) return fail(GBO_ERR_ARG, "gbo_copy_photons: null argument");
    if (!e->cfg.record_photon) return fail(GBO_ERR_STATE, "gbo_copy_photons: record_photon is off");
    if (e->num_photon < 0) return fail(GBO_ERR_STATE, "gbo_copy_photons: no event simulated");
    if (offset < 0 || count < 0 || offset + count > e->num_photon) return fail(GBO_ERR_ARG, "gbo_copy_photons: range outside event");
    if (count == 0) return GBO_OK;
    CU(cudaSetDevice(e->device));
    CU(cudaMemcpyAsync(dst, e->photon.ptr + offset, (size_t)count * sizeof(gbo_sphoton), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    return GBO_OK;
}

int gbo_copy_seq(gbo_engine* e, gbo_seq* dst, int64_t offset, int64_t count)
{
    if (!e || (!dst && count > 0)) return fail(GBO_ERR_ARG, "gbo_copy_seq: null argument");
    if (!e->cfg.record_seq) return fail(GBO_ERR_STATE, "gbo_copy_seq: record_seq is off");
    if (e->num_photon < 0) return fail(GBO_ERR_STATE, "gbo_copy_seq: no event simulated");
    if (offset < 0 || count < 0 || offset + count > e->num_photon) return fail(GBO_ERR_ARG, "gbo_copy_seq: range outside event");
    if (count == 0) return GBO_OK;
    CU(cudaSetDevice(e->device));
    CU(cudaMemcpyAsync(dst, e->seq.ptr + offset, (size_t)count * sizeof(gbo_seq), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    return GBO_OK;
}

int gbo_reset(gbo_engine* e, int32_t event_id)
{
    if (!e) return fail(GBO_ERR_ARG, "gbo_reset: null engine");
    (void)event_id;
    e->num_photon = -1;
    e->num_hit = 0;
    e->num_merged = -1;
    e->event_id = -1;
    return GBO_OK;
}

int gbo_get_stats(const gbo_engine* e, gbo_stats* out)
{
    if (!e || !out) return fail(GBO_ERR_ARG, "gbo_get_stats: null argument");
    *out = e->stats;
    return GBO_OK;
}

int gbo_autotune(gbo_engine* e, int32_t event_id, const gbo_quad6* gs, int64_t num_gs, const gbo_sphoton* input_photon,
                 int64_t num_input_photon, int32_t trials, gbo_tune_result* out)
{
    if (!e || !out) return fail(GBO_ERR_ARG, "gbo_autotune: null argument");
    if (trials < 1) trials = 1;
    std::memset(out, 0, sizeof(*out));
    // candidates: (kernel mode, refill threshold, refill period, resident blocks per SM (0: the occupancy maximum),
    // lanes gathered per TLAS walk (1: none), Philox blocks by call in the single-leaf binary32 form)
    struct Cand { int mode, refill, period, blocks, walk, rcall; };
    std::vector<Cand> cands = {{1, 32, 1, 0, 1, 0}};
    for (int r : {1, 4, 16})
        for (int p : {1, 4}) cands.push_back({0, r, p, 0, 1, 0});
    for (int r : {1, 2, 4, 8, 16}) cands.push_back({2, r, 1, 0, 1, 0});
    for (int r : {2, 4})                                                     // refill (compaction) every 2 or 4 steps
        for (int p : {2, 4}) cands.push_back({2, r, p, 0, 1, 0});
    if (e->csg_form >= 1)                                                    // gathered walks: CSG-tree forms
        for (int w : {16, 24, 32}) cands.push_back({2, 4, 1, 0, w, 0});
    if (e->csg_form == 0 && !e->cfg.precision)
        for (const Cand& c : std::vector<Cand>{{1, 32, 1, 0, 1, 1}, {0, 4, 1, 0, 1, 1}, {0, 4, 4, 0, 1, 1},
                                               {2, 1, 1, 0, 1, 1}, {2, 4, 1, 0, 1, 1}, {2, 4, 2, 0, 1, 1},
                                               {2, 2, 4, 0, 1, 1}})
            cands.push_back(c);
    cands.push_back({3, 4, 1, 0, 1, 0});                                     // the wavefront form
    if (e->csg_form == 0 && !e->cfg.precision) cands.push_back({3, 4, 1, 0, 1, 1});
    const int form = 2 * e->csg_form + (e->cfg.precision ? 1 : 0);
    for (int b = 1; b < e->pool_occ[form] && cands.size() < 32; b++) {       // fewer resident blocks than fit
        cands.push_back({2, 4, 1, b, 1, 0});
        if (cands.size() < 32) cands.push_back({0, 4, 1, b, 1, 0});
    }
    const gbo_config saved = e->cfg;
    float best = 1e30f;
    Cand pick = cands[0];
    for (size_t c = 0; c < cands.size() && c < 32; c++) {
        e->cfg.kernel_mode = cands[c].mode;
        e->cfg.refill_min = cands[c].refill;
        e->cfg.refill_period = cands[c].period;
        e->cfg.blocks_per_sm = cands[c].blocks;
        e->cfg.walk_min = cands[c].walk;
        e->cfg.rng_call = cands[c].rcall;
        float ms = 1e30f;
        for (int t = 0; t <= trials; t++) {
            int rc = gbo_simulate(e, event_id, gs, num_gs, input_photon, num_input_photon);
            if (rc) { e->cfg = saved; return rc; }
            if (t > 0 && e->stats.ms_simulate < ms) ms = e->stats.ms_simulate;   // first run warms up
        }
        out->cand_mode[c] = cands[c].mode;
        out->cand_refill[c] = cands[c].refill;
        out->cand_period[c] = cands[c].period;
        out->cand_blocks[c] = cands[c].blocks;
        out->cand_walk[c] = cands[c].walk;
        out->cand_rng_call[c] = cands[c].rcall;
        out->cand_ms[c] = ms;
        out->num_candidates = (int32_t)(c + 1);
        if (ms < best) { best = ms; pick = cands[c]; }
    }
    e->cfg = saved;
    e->cfg.kernel_mode = pick.mode;
    e->cfg.refill_min = pick.refill;
    e->cfg.refill_period = pick.period;
    e->cfg.blocks_per_sm = pick.blocks;
    e->cfg.walk_min = pick.walk;
    e->cfg.rng_call = pick.rcall;
    out->kernel_mode = pick.mode;
    out->refill_min = pick.refill;
    out->refill_period = pick.period;
    out->blocks_per_sm = pick.blocks;
    out->walk_min = pick.walk;
    out->rng_call = pick.rcall;
    return GBO_OK;
}

}  // extern "C"

// ---- known-answer entry points ---------------------------------------------------------------------------------

namespace {
template <typename F>
int with_scratch(size_t in_bytes, const void* in, size_t out_bytes, void* out, F launch)
{
    void* d_in = nullptr;
    void* d_out = nullptr;
    if (in_bytes && cudaMalloc(&d_in, in_bytes) != cudaSuccess) return fail(GBO_ERR_CUDA, "cudaMalloc failed");
    if (cudaMalloc(&d_out, out_bytes) != cudaSuccess) { cudaFree(d_in); return fail(GBO_ERR_CUDA, "cudaMalloc failed"); }
    int rc = GBO_OK;
    if (in_bytes && cudaMemcpy(d_in, in, in_bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = fail(GBO_ERR_CUDA, "upload failed");
    if (!rc) {
        launch(d_in, d_out);
        cudaError_t err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaDeviceSynchronize();
        if (err != cudaSuccess) rc = fail(GBO_ERR_CUDA, "kernel failed: %s", cudaGetErrorString(err));
    }
    if (!rc && cudaMemcpy(out, d_out, out_bytes, cudaMemcpyDeviceToHost) != cudaSuccess) rc = fail(GBO_ERR_CUDA, "download failed");
    cudaFree(d_in);
    cudaFree(d_out);
    return rc;
}
}  // namespace

extern "C" {

int gbo_rng_sequence(int device, uint64_t seed, uint64_t subsequence0, uint64_t position, int32_t num_seq,
                     int32_t per_seq, float* out)
{
    if (!out || num_seq <= 0 || per_seq <= 0) return fail(GBO_ERR_ARG, "gbo_rng_sequence: bad arguments");
    CU(cudaSetDevice(device));
    return with_scratch(0, nullptr, (size_t)num_seq * per_seq * sizeof(float), out, [&](void*, void* d_out) {
        k_rng_sequence<<<(num_seq + 127) / 128, 128>>>(seed, subsequence0, position, num_seq, per_seq, (float*)d_out);
    });
}

int gbo_texture_lookup(gbo_engine* e, int32_t which, const float* xy, int32_t n, float* out)
{
    if (!e || !xy || !out || n <= 0 || (which != 0 && which != 1)) return fail(GBO_ERR_ARG, "gbo_texture_lookup: bad arguments");
    CU(cudaSetDevice(e->device));
    Params P = make_params(e);
    return with_scratch((size_t)n * sizeof(float2), xy, (size_t)n * sizeof(float4), out, [&](void* d_in, void* d_out) {
        k_tex_lookup<<<(n + 127) / 128, 128>>>(P.tab, (const float2*)d_in, n, which, (float4*)d_out);
    });
}

int gbo_trace_rays(gbo_engine* e, const float* pos, const float* dir, int32_t n, float tmin, float tmax, float* t_out,
                   uint32_t* boundary_out)
{
    if (!e || !pos || !dir || !t_out || !boundary_out || n <= 0) return fail(GBO_ERR_ARG, "gbo_trace_rays: bad arguments");
    CU(cudaSetDevice(e->device));
    Params P = make_params(e);
    std::vector<float> in((size_t)n * 6);
    std::memcpy(in.data(), pos, (size_t)n * 12);
    std::memcpy(in.data() + (size_t)n * 3, dir, (size_t)n * 12);
    std::vector<float> out((size_t)n * 2);
    const bool polish = e->cfg.precision != 0;
    int rc = with_scratch(in.size() * 4, in.data(), out.size() * 4, out.data(), [&](void* d_in, void* d_out) {
        const float3* dp = (const float3*)d_in;
        const float3* dd = (const float3*)((float*)d_in + (size_t)n * 3);
        float* dt = (float*)d_out;
        unsigned* db = (unsigned*)((float*)d_out + n);
        switch (e->csg_form) {
            case 2:  trace_rays_launch<2>(polish, P.acc, dp, dd, n, tmin, tmax, dt, db); break;
            case 1:  trace_rays_launch<1>(polish, P.acc, dp, dd, n, tmin, tmax, dt, db); break;
            default: trace_rays_launch<0>(polish, P.acc, dp, dd, n, tmin, tmax, dt, db); break;
        }
    });
    if (rc) return rc;
    std::memcpy(t_out, out.data(), (size_t)n * 4);
    std::memcpy(boundary_out, out.data() + n, (size_t)n * 4);
    return GBO_OK;
}

int gbo_scint_wavelength(gbo_engine* e, const float* u, int32_t n, float* out)
{
    if (!e || !u || !out || n <= 0) return fail(GBO_ERR_ARG, "gbo_scint_wavelength: bad arguments");
    CU(cudaSetDevice(e->device));
    Params P = make_params(e);
    return with_scratch((size_t)n * sizeof(float), u, (size_t)n * sizeof(float), out, [&](void* d_in, void* d_out) {
        k_scint_wavelength<<<(n + 127) / 128, 128>>>(P.tab, (const float*)d_in, n, (float*)d_out);
    });
}

}  // extern "C"

// ================================================================================================================
// Simulation without any allocation.
//
// Some callers cannot allocate device memory while events are processed: a trigger or DAQ process whose device
// memory is carved up once at start-up by another runtime, a host framework that forbids allocator calls on its
// event threads because cudaMalloc/cudaFree synchronise the device and stall every other stream, or code that
// must not grow its footprint after initialisation.  gbo_simulate_noalloc serves them: gensteps in and hits out
// are caller-owned device buffers, and all intermediate state (genstep prefix, hit bitmap and its scan, the
// unordered hit staging, counters) lives in one fixed file-scope device array.  The array is part of the
// loaded library image, so every GPU that loads libgbopticks.so holds its GBO_NOALLOC_SCRATCH_BYTES until the
// process exits.  The engine's geometry must have been created beforehand (gbo_engine_create allocates; this
// entry point never does).
// ================================================================================================================

namespace gbo {

constexpr long long NA_MAX_PHOTON = 1ll << 22;            // photons per call
constexpr long long NA_MAX_HIT = 1ll << 17;               // hits per call
constexpr long long NA_MAX_GENSTEP = 1ll << 15;           // gensteps per call
constexpr long long NA_WORDS = NA_MAX_PHOTON / 32;
constexpr long long NA_BLOCKS = NA_WORDS / SCAN_WORDS;
// byte offsets inside the scratch array (each a multiple of 256)
constexpr size_t NA_OFF_COUNTERS = 0;                                             // 4 x u64
constexpr size_t NA_OFF_GS_END = 256;                                             // NA_MAX_GENSTEP x u64
constexpr size_t NA_OFF_BITMAP = NA_OFF_GS_END + NA_MAX_GENSTEP * 8;              // NA_WORDS x u32
constexpr size_t NA_OFF_PREFIX = NA_OFF_BITMAP + NA_WORDS * 4;                    // NA_WORDS x u32
constexpr size_t NA_OFF_BLOCK_SUM = NA_OFF_PREFIX + NA_WORDS * 4;                 // NA_BLOCKS x u32
constexpr size_t NA_OFF_BLOCK_OFF = NA_OFF_BLOCK_SUM + NA_BLOCKS * 4;             // NA_BLOCKS x u64
constexpr size_t NA_OFF_STAGING = NA_OFF_BLOCK_OFF + NA_BLOCKS * 8;               // NA_MAX_HIT x sphoton
constexpr size_t NA_BYTES = NA_OFF_STAGING + NA_MAX_HIT * sizeof(gbo_sphoton);
static_assert(NA_OFF_BITMAP % 256 == 0 && NA_OFF_PREFIX % 256 == 0 && NA_OFF_BLOCK_SUM % 256 == 0 &&
              NA_OFF_BLOCK_OFF % 256 == 0 && NA_OFF_STAGING % 256 == 0, "scratch sections stay 256-byte aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

}  // namespace gbo

namespace {
constexpr int NA_MAX_DEVICES = 64;

// Restores the calling thread's current device when it goes out of scope.
struct DeviceGuard {
    int dev = -1;
    bool ok = false;
    DeviceGuard() { ok = cudaGetDevice(&dev) == cudaSuccess; }
    ~DeviceGuard() { if (ok) cudaSetDevice(dev); }
};

std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[NA_MAX_DEVICES] = {nullptr};

// Device address of the scratch array on the current device, looked up once per device.
int noalloc_scratch(int device, unsigned char** out)
{
    if (device < 0 || device >= NA_MAX_DEVICES) return fail(GBO_ERR_ARG, "gbo_simulate_noalloc: device %d out of range", device);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (err != cudaSuccess || !p)
            return fail(GBO_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(err));
        g_noalloc_ptr[device] = p;
    }
    *out = (unsigned char*)g_noalloc_ptr[device];
    return GBO_OK;
}
}  // namespace

extern "C" {

int64_t gbo_noalloc_scratch_bytes(void) { return (int64_t)NA_BYTES; }

int gbo_simulate_noalloc(gbo_engine* e, int32_t event_id, const void* d_gs, int64_t num_gs, const void* d_input_photon,
                         int64_t num_input_photon, gbo_sphoton* d_hits, int64_t hit_capacity, int64_t* num_hit,
                         void* cuda_stream)
{
    if (!e || !num_hit) return fail(GBO_ERR_ARG, "gbo_simulate_noalloc: null engine or num_hit");
    if (e->cfg.precision) return fail(GBO_ERR_ARG, "gbo_simulate_noalloc: the precision mode is not available here");
    *num_hit = 0;
    if (num_gs < 0 || (num_gs > 0 && !d_gs)) return fail(GBO_ERR_ARG, "gbo_simulate_noalloc: bad gensteps");
    if (num_gs > NA_MAX_GENSTEP)
        return fail(GBO_ERR_CAPACITY, "gbo_simulate_noalloc: %lld gensteps above the limit of %lld", (long long)num_gs,
                    NA_MAX_GENSTEP);
    if (hit_capacity < 0 || (hit_capacity > 0 && !d_hits)) return fail(GBO_ERR_ARG, "gbo_simulate_noalloc: bad hit buffer");
    if (num_input_photon < 0 || (num_input_photon > 0 && !d_input_photon))
        return fail(GBO_ERR_ARG, "gbo_simulate_noalloc: bad input photons");
    DeviceGuard keep_device;            // the caller's current device is restored on every return
    if (!keep_device.ok) return fail(GBO_ERR_CUDA, "gbo_simulate_noalloc: cudaGetDevice failed");
    CU(cudaSetDevice(e->device));
    unsigned char* s_base = nullptr;
    int rc = noalloc_scratch(e->device, &s_base);
    if (rc) return rc;
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : e->stream;
    unsigned long long* counters = (unsigned long long*)(s_base + NA_OFF_COUNTERS);
    unsigned long long* gs_end = (unsigned long long*)(s_base + NA_OFF_GS_END);
    uint32_t* bitmap = (uint32_t*)(s_base + NA_OFF_BITMAP);
    uint32_t* word_prefix = (uint32_t*)(s_base + NA_OFF_PREFIX);
    uint32_t* block_sum = (uint32_t*)(s_base + NA_OFF_BLOCK_SUM);
    unsigned long long* block_offset = (unsigned long long*)(s_base + NA_OFF_BLOCK_OFF);
    gbo_sphoton* staging = (gbo_sphoton*)(s_base + NA_OFF_STAGING);
    if (num_gs == 0) return GBO_OK;

    // counters left over from the previous call must start at zero
    CU(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), s));
    k_genstep_prefix<<<1, 1024, 0, s>>>((const gbo_quad6*)d_gs, (int)num_gs, gs_end, counters + 3);
    CU(cudaGetLastError());
    unsigned long long total = 0, input_gs = 0;
    CU(cudaMemcpyAsync(&total, gs_end + (num_gs - 1), sizeof(total), cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(&input_gs, counters + 3, sizeof(input_gs), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    if ((long long)total > NA_MAX_PHOTON)
        return fail(GBO_ERR_CAPACITY, "gbo_simulate_noalloc: %llu photons above the limit of %lld", total, NA_MAX_PHOTON);
    if ((input_gs || num_input_photon > 0) && (long long)num_input_photon < (long long)total)
        return fail(GBO_ERR_ARG, "gbo_simulate_noalloc: %lld input photons for %llu photon slots", (long long)num_input_photon, total);

    Params P = make_params(e);
    P.position0 = e->cfg.rng_offset + e->cfg.event_skipahead * (uint64_t)(event_id < 0 ? 0 : event_id);
    P.gs = (const float4*)d_gs;
    P.gs_end = gs_end;
    P.num_gs = (int)num_gs;
    P.num_photon = (long long)total;
    P.input_photon = (const gbo_sphoton*)d_input_photon;
    P.hit_unordered = staging;
    P.hit_count = counters;
    P.bitmap = bitmap;
    const long long words = ((long long)total + 31) / 32;
    const long long nblk = (words + SCAN_WORDS - 1) / SCAN_WORDS;
    if (total > 0) {
        const long long blocks = ((long long)total + SIM_BLOCK - 1) / SIM_BLOCK;
        if (e->csg_form == 2) sim_launch_bounded<2>(P, NA_MAX_HIT, (unsigned)blocks, s);
        else if (e->csg_form == 1) sim_launch_bounded<1>(P, NA_MAX_HIT, (unsigned)blocks, s);
        else sim_launch_bounded<0>(P, NA_MAX_HIT, (unsigned)blocks, s);
        CU(cudaGetLastError());
        k_word_prefix<<<(unsigned)nblk, SCAN_WORDS, 0, s>>>(bitmap, words, word_prefix, block_sum);
        k_block_offsets<<<1, 1024, 0, s>>>(block_sum, nblk, block_offset, counters + 1);
        CU(cudaGetLastError());
    }
    unsigned long long found = 0;
    CU(cudaMemcpyAsync(&found, counters + 1, sizeof(found), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    *num_hit = (int64_t)found;
    if ((long long)found > NA_MAX_HIT)
        return fail(GBO_ERR_CAPACITY, "gbo_simulate_noalloc: %llu hits above the staging limit of %lld", found, NA_MAX_HIT);
    if ((long long)found > hit_capacity)
        return fail(GBO_ERR_CAPACITY, "gbo_simulate_noalloc: %llu hits, hit buffer holds %lld", found, (long long)hit_capacity);
    if (found > 0) {
        k_gather_unordered<<<(unsigned)((found + 255) / 256), 256, 0, s>>>(staging, counters, 0ull, bitmap, word_prefix,
                                                                          block_offset, d_hits);
        CU(cudaGetLastError());
        CU(cudaStreamSynchronize(s));
    }
    return GBO_OK;
}

}  // extern "C"

#include "gbo_serve.inl"
