// gbo_sim.cuh : the photon program's kernels and their launch parameters, shared by the engine and the per-form
// translation units.
//
// The simulation kernels come in forms chosen by template arguments: TREE (0: single-leaf prims, 1: CSG boolean
// trees, 2: CSG list nodes as well), PRECISE (binary64 root polish and accumulators), PREGEN (the pool over photons
// generated up front) and RCALL (Philox blocks by an out-of-line call).  The kernels of each TREE value are
// instantiated in their own translation unit (gbo_sim_tree0.cu, gbo_sim_tree1.cu, gbo_sim_tree2.cu, all from
// gbo_sim_forms.inl), so the forms compile in parallel; the engine reaches them through the host launchers
// declared at the end of this header and never instantiates a simulation kernel itself.
#pragma once
#include <cuda_runtime.h>

#include "gbo_trace.cuh"

namespace gbo {

#ifndef GBO_SIM_MINB
#define GBO_SIM_MINB 5              // minimum resident blocks per SM asked of ptxas for the one-thread simulate kernel
                                    // (binary32, no CSG trees): 5 x 128 threads (96 registers) measured fastest
#endif
#ifndef GBO_SIM_MINB_WIDE
#define GBO_SIM_MINB_WIDE 1         // the same for its CSG-tree and precision forms, which need their registers
#endif
#ifndef GBO_POOL_MINB
#define GBO_POOL_MINB 4             // the same for the persistent photon-pool kernel: 4 x 128 threads per SM (128
                                    // registers) measured 12 % faster than ptxas' unbounded choice on the crystal event
#endif
#ifndef GBO_POOL_MINB_TREE
#define GBO_POOL_MINB_TREE 3        // the pool kernel's form for geometries with CSG trees: 3 x 128 threads per SM
                                    // (168 registers, no spills) measured 3 % faster than 4 (128 registers, 860 B of
                                    // spills) on the 20,000-sensor event
#endif
#ifdef GBO_POOL_MAXNREG                // register budget of the pool kernel instead of its launch bounds
#define GBO_POOL_BOUNDS __maxnreg__(GBO_POOL_MAXNREG)
#else
#define GBO_POOL_BOUNDS __launch_bounds__(SIM_BLOCK, TREE ? GBO_POOL_MINB_TREE : GBO_POOL_MINB)
#endif
#ifdef GBO_GENERATE_INLINE
#define GBO_GEN GBO_DEV
#else
#define GBO_GEN __device__ __noinline__   // photon generation runs once per photon: kept out of the bounce loop's code
#endif
constexpr int SIM_BLOCK = 128;

struct Params {
    Accel acc;
    Tables tab;
    int max_bounce;
    float max_time, tmin, tmin0, tmax;
    uint32_t eps0_mask, hitmask;
    uint64_t seed, position0;
    const float4* gs;
    const unsigned long long* gs_end;     // inclusive prefix of numphoton
    int num_gs;
    long long num_photon;
    unsigned long long photon_offset;
    const gbo_sphoton* input_photon;
    gbo_sphoton* photon_out;
    gbo_seq* seq_out;
    gbo_sphoton* hit_unordered;
    unsigned long long* hit_count;
    uint32_t* bitmap;
    // several events in one launch: event e owns gensteps [ev_gs_begin[e], ev_gs_begin[e+1]) and launch photons
    // [ev_photon_begin[e], ev_photon_begin[e+1]); its photons use stream position ev_pos0[e] and event-local indices
    int num_events;                         // 0: single event (photon_offset, position0 above)
    const int* ev_gs_begin;
    const unsigned long long* ev_photon_begin;
    const unsigned long long* ev_pos0;
    const unsigned long long* ev_photon_offset;     // event-local index of each entry's first photon (a piece of a
                                                    // sliced event starts past 0); nullptr: all 0
    unsigned long long* hit_gidx;           // launch index of each unordered hit (batched launches)
    // pregenerated photons (kernel mode 2): k_generate writes each photon as generated and its random-stream
    // place (draws consumed, subsequence); the pool kernel's refills read them instead of generating
    gbo_sphoton* gen_photon;
    ulonglong2* gen_rng;
    int* gen_hint;
    // start instance of each genstep's photons (k_genstep_hint), a traversal hint only; nullptr: none
    const int* gs_hint;
    int walk_min;                           // pool kernels: parked lanes that trigger the gathered TLAS walks
};

template <class R>
GBO_GEN void generate(const Params& P, long long idx, Photon& p, R& rng, int& hint);

// Kernel forms: TREE 1 when any prim is a CSG tree, 2 when CSG list nodes occur as well (their evaluation is
// compiled only into that form); PRECISE for the precision mode (binary64 root polish in the quadric leaves,
// binary64 position / time accumulators).  The default form compiles none of the latter.  RCALL: Philox blocks by
// an out-of-line call instead of inlined rounds (RngT).
template <int TREE, bool PRECISE, bool RCALL>
__global__ void __launch_bounds__(SIM_BLOCK, (TREE || PRECISE) ? GBO_SIM_MINB_WIDE : GBO_SIM_MINB)
k_simulate(const __grid_constant__ Params P)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = idx < P.num_photon;
    Photon p;
    bool is_hit = false;
    if (active) {
        RngT<RCALL> rng;
        Acc64 acc;
        int hint;
        generate(P, idx, p, rng, hint);
        if (PRECISE) acc_init(acc, p);

        int bounce = 0;
        if (P.seq_out) seq_start(P.seq_out + idx, flag_of(p), boundary_of(p));
        while (bounce < P.max_bounce && p.time < P.max_time) {
            const float tmin = (p.orient_boundary_flag & P.eps0_mask) ? P.tmin0 : P.tmin;
            Hit h;
            trace<TREE, PRECISE>(P.acc, p.pos, p.mom, tmin, P.tmax, hint, h);
            if ((h.prim_boundary & 0xffffu) == 0xffffu) break;
            hint = (int)(h.iindex_identity >> 16);
            h.normal = normalize(h.normal);
            const int command = propagate(P.tab, p, h, rng, PRECISE ? &acc : nullptr);
            bounce++;
            if (P.seq_out) seq_add(P.seq_out + idx, (unsigned)bounce, flag_of(p), boundary_of(p));
            if (command == CMD_BREAK) break;
        }
        is_hit = (p.flagmask & P.hitmask) == P.hitmask;
        if (P.photon_out) store_photon(P.photon_out + idx, p);
    }
    const unsigned lane = threadIdx.x & 31u;
    const unsigned mask = __ballot_sync(0xffffffffu, is_hit);
    const long long word = idx >> 5;
    if (lane == 0 && word * 32 < P.num_photon) P.bitmap[word] = mask;
    if (P.hit_unordered && mask) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(P.hit_count, (unsigned long long)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (is_hit) {
            store_photon(P.hit_unordered + base + __popc(mask & ((1u << lane) - 1u)), p);
            if (P.hit_gidx) P.hit_gidx[base + __popc(mask & ((1u << lane) - 1u))] = (unsigned long long)idx;
        }
    }
}

// ---- persistent form: lanes refill from a photon pool so a warp never idles behind its longest photon --------

// the genstep holding launch photon idx: the first whose inclusive numphoton prefix exceeds idx
GBO_DEV int genstep_of(const Params& P, long long idx)
{
    int lo = 0, hi = P.num_gs - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(P.gs_end + mid) > (unsigned long long)idx) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// Photon idx of genstep lo, as generate_photon makes it; `hint` receives the start instance found for the genstep
// (-1 when none was computed)
template <class R>
GBO_DEV void generate_in(const Params& P, long long idx, int lo, Photon& p, R& rng, int& hint)
{
    hint = P.gs_hint ? __ldg(P.gs_hint + lo) : -1;
    const float4* g = P.gs + 6 * (size_t)lo;
    float4 gq[6];
#pragma unroll
    for (int k = 0; k < 6; k++) gq[k] = __ldg(g + k);
    unsigned long long photon_idx = P.photon_offset + (unsigned long long)idx;
    uint64_t pos0 = P.position0;
    if (P.num_events > 0) {
        int a = 0, z = P.num_events - 1;          // event owning genstep lo
        while (a < z) {
            const int m = (a + z + 1) >> 1;
            if (__ldg(P.ev_gs_begin + m) <= lo) a = m; else z = m - 1;
        }
        photon_idx = (unsigned long long)idx - __ldg(P.ev_photon_begin + a);
        if (P.ev_photon_offset) photon_idx += __ldg(P.ev_photon_offset + a);
        pos0 = __ldg(P.ev_pos0 + a);
    }
    rng_init(rng, P.seed, photon_idx, pos0);
    p.pos = f3(0.f, 0.f, 0.f); p.time = 0.f; p.mom = f3(0.f, 0.f, 0.f); p.hitcount_iindex = 0u;
    p.pol = f3(0.f, 0.f, 0.f); p.wavelength = 0.f;
    p.orient_boundary_flag = 0u; p.identity = 0u; p.index = 0u; p.flagmask = 0u;
    const int gencode = __float_as_int(gq[0].x);
    switch (gencode) {
        case GBO_GS_TORCH: gen_torch(p, rng, gq, photon_idx); break;
        case GBO_GS_CERENKOV:
        case GBO_GS_G4Cerenkov_modified: gen_cerenkov(P.tab, p, rng, gq); break;
        case GBO_GS_SCINTILLATION:
        case GBO_GS_DsG4Scintillation_r4695: gen_scint(P.tab, p, rng, gq); break;
        case GBO_GS_INPUT_PHOTON:
            if (P.input_photon) { load_photon(p, P.input_photon + idx); set_flag(p, GBO_TORCH); }
            else { set_flag(p, GBO_NAN_ABORT); p.time = __int_as_float(0x7f800000); }   // hosts refuse this case
            break;
        default: break;
    }
    set_index(p, photon_idx);
}

template <class R>
GBO_GEN void generate(const Params& P, long long idx, Photon& p, R& rng, int& hint)
{
    generate_in(P, idx, genstep_of(P, idx), p, rng, hint);
}

// the same for a caller that knows the photon's genstep
template <class R>
GBO_GEN void generate_at(const Params& P, long long idx, int lo, Photon& p, R& rng, int& hint)
{
    generate_in(P, idx, lo, p, rng, hint);
}

constexpr int POOL_CHUNK = 32;      // pregenerated photons a warp claims at once (kernel mode 2)

// The end of a photon (lanes with `done`; every lane of the warp calls it): its bit in the hit bitmap, its record
// when the full photon array is kept, and, when it is a hit, its record appended to the unordered hits
// (warp-aggregated) with its launch index.
GBO_DEV void finish_photons(const Params& P, bool done, long long idx, const Photon& p)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    const bool is_hit = done && (p.flagmask & P.hitmask) == P.hitmask;
    if (done) {
        if (is_hit) atomicOr(P.bitmap + (idx >> 5), 1u << (idx & 31));
        if (P.photon_out) store_photon(P.photon_out + idx, p);
    }
    if (P.hit_unordered) {
        const unsigned hm = __ballot_sync(0xffffffffu, is_hit);
        if (hm) {
            const int leader = __ffs(hm) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(P.hit_count, (unsigned long long)__popc(hm));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (is_hit) {
                store_photon(P.hit_unordered + base + __popc(hm & lt), p);
                if (P.hit_gidx) P.hit_gidx[base + __popc(hm & lt)] = (unsigned long long)idx;
            }
        }
    }
}

// Kernel-mode-2 refill (warp-uniform chunk state cbase, cn, cused): idle lanes take the next pregenerated photons in
// lane order, the warp claiming POOL_CHUNK more with one atomic when its chunk runs short.
template <bool PRECISE, class R>
GBO_DEV void refill_pregenerated(const Params& P, unsigned long long* pool, unsigned idle, unsigned lane, unsigned lt,
                                 bool& live, long long& idx, Photon& p, R& rng, int& hint, Acc64& acc, int& bounce,
                                 long long& cbase, int& cn, int& cused, bool& pool_open)
{
    const int n_idle = __popc(idle), rank = __popc(idle & lt), avail = cn - cused;
    long long nb = 0;
    int nn = 0;
    if (avail < n_idle) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(pool, (unsigned long long)POOL_CHUNK);
        nb = (long long)__shfl_sync(0xffffffffu, b, 0);
        const long long left = P.num_photon - nb;
        nn = left <= 0 ? 0 : (left < POOL_CHUNK ? (int)left : POOL_CHUNK);
    }
    if (!live) {
        const long long j = rank < avail ? cbase + cused + rank : (rank - avail < nn ? nb + (rank - avail) : -1);
        if (j >= 0) {
            idx = j;
            load_photon_streamed(p, P.gen_photon + idx);
            const ulonglong2 r = __ldcg(P.gen_rng + idx);
            rng_init(rng, P.seed, r.y, r.x);
            hint = __ldcg(P.gen_hint + idx);
            if (PRECISE) acc_init(acc, p);
            bounce = 0;
            if (P.seq_out) seq_start(P.seq_out + idx, flag_of(p), boundary_of(p));
            live = true;
        }
    }
    if (avail < n_idle) {
        cbase = nb;
        cn = nn;
        cused = n_idle - avail < nn ? n_idle - avail : nn;
        if (nn == 0) pool_open = false;         // drained: every claimed photon has been handed out
    } else {
        cused += n_idle;
    }
}

// PREGEN: the kernel-mode-2 form without the generator.  Without a call to the out-of-line generator, its
// by-reference arguments no longer force the photon state through local memory (crystal event 751M -> 864M
// photons/s).
template <int TREE, bool PRECISE, bool PREGEN, bool RCALL>
__global__ void GBO_POOL_BOUNDS k_simulate_pool(const __grid_constant__ Params P,
                                                             unsigned long long* pool, int refill_min, int period)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    bool live = false;
    bool pool_open = true;
    long long idx = -1;
    int bounce = 0;
    int hint = -1;
    int phase = 0;                  // step count modulo `period`, kept by a counter (a modulo by it would divide)
    Photon p;
    RngT<RCALL> rng;
    Acc64 acc;
    // mode 2 (warp-uniform): the warp's claimed chunk of pregenerated photons [cbase, cbase + cn), cused taken
    long long cbase = 0;
    int cn = 0, cused = 0;
    bool parked = false;            // the photon's step waits for a gathered TLAS walk
    for (;; phase = phase + 1 == period ? 0 : phase + 1) {
        // refill every `period` steps (or when the warp is empty): idle lanes take the next photon indices in lane
        // order; mode 2 claims them POOL_CHUNK at a time (one atomic per chunk) and loads them as generated, the
        // other pool mode claims exactly the idle lanes' count and generates them
        const unsigned idle = __ballot_sync(0xffffffffu, !live);
        const bool refill = pool_open && (idle == 0xffffffffu || (phase == 0 && __popc(idle) >= refill_min));
        if (PREGEN || P.gen_photon) {
            if (refill)
                refill_pregenerated<PRECISE>(P, pool, idle, lane, lt, live, idx, p, rng, hint, acc, bounce, cbase, cn,
                                             cused, pool_open);
        } else if constexpr (!PREGEN) {
            if (refill) {
                unsigned long long base = 0;
                const int leader = __ffs(idle) - 1;
                if ((int)lane == leader) base = atomicAdd(pool, (unsigned long long)__popc(idle));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (base + __popc(idle) >= (unsigned long long)P.num_photon) pool_open = false;
                if (!live) {
                    const unsigned long long mine = base + __popc(idle & lt);
                    if (mine < (unsigned long long)P.num_photon) {
                        idx = (long long)mine;
                        generate(P, idx, p, rng, hint);
                        if (PRECISE) acc_init(acc, p);
                        bounce = 0;
                        if (P.seq_out) seq_start(P.seq_out + idx, flag_of(p), boundary_of(p));
                        live = true;
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, live)) {
            if (!pool_open) break;
            continue;
        }
        // gathered TLAS walks (CSG-tree forms): parked lanes walk once enough of them wait, or when no live lane is
        // left to step.  The single-leaf forms compile none of it: their walks are short, and the two ballots per
        // step cost 2 % on the crystal event.
        bool walk_now = false;
        if constexpr (TREE >= 1) {
            const unsigned parked_mask = __ballot_sync(0xffffffffu, parked);
            walk_now = parked_mask != 0u &&
                       (__popc(parked_mask) >= P.walk_min || parked_mask == __ballot_sync(0xffffffffu, live));
        }
        bool done = false;
        if (live) {
            if (parked || (bounce < P.max_bounce && p.time < P.max_time)) {
                const float tmin = (p.orient_boundary_flag & P.eps0_mask) ? P.tmin0 : P.tmin;
                // one call site: a query that may stop before its TLAS walk, or a parked lane's whole query (its
                // hint instance tested again, then the walk) once the warp gathers the walks
                Best b;
                trace_begin(b, P.tmax);
                int r = TRACE_WALK;
                if (!parked || walk_now)
                    r = trace_items<TREE, PRECISE>(P.acc, p.pos, p.mom, tmin, hint,
                                                   TREE >= 1 && !parked && P.walk_min > 1, b);
                parked = r == TRACE_WALK;
                if (!parked) {
                    Hit h;
                    trace_finish(P.acc, p.pos, p.mom, b, h);
                    if ((h.prim_boundary & 0xffffu) == 0xffffu) {
                        done = true;
                    } else {
                        hint = (int)(h.iindex_identity >> 16);
                        h.normal = normalize(h.normal);
                        const int command = propagate(P.tab, p, h, rng, PRECISE ? &acc : nullptr);
                        bounce++;
                        if (P.seq_out) seq_add(P.seq_out + idx, (unsigned)bounce, flag_of(p), boundary_of(p));
                        done = command == CMD_BREAK;
                    }
                }
            } else {
                done = true;
            }
        }
        finish_photons(P, done, idx, p);
        if (done) live = false;
    }
}

// The one-thread-per-photon program with a bounded hit append: hits beyond the staging capacity are counted
// but not stored, and the host reports the overflow.
template <int TREE>
__global__ void __launch_bounds__(SIM_BLOCK) k_simulate_bounded(const __grid_constant__ Params P, long long cap)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    Photon p;
    bool is_hit = false;
    if (idx < P.num_photon) {
        RngT<(TREE >= 1)> rng;
        int hint;
        generate(P, idx, p, rng, hint);
        int bounce = 0;
        while (bounce < P.max_bounce && p.time < P.max_time) {
            const float tmin = (p.orient_boundary_flag & P.eps0_mask) ? P.tmin0 : P.tmin;
            Hit h;
            trace<TREE>(P.acc, p.pos, p.mom, tmin, P.tmax, hint, h);
            if ((h.prim_boundary & 0xffffu) == 0xffffu) break;
            hint = (int)(h.iindex_identity >> 16);
            h.normal = normalize(h.normal);
            const int command = propagate(P.tab, p, h, rng);
            bounce++;
            if (command == CMD_BREAK) break;
        }
        is_hit = (p.flagmask & P.hitmask) == P.hitmask;
    }
    const unsigned lane = threadIdx.x & 31u;
    const unsigned mask = __ballot_sync(0xffffffffu, is_hit);
    const long long word = idx >> 5;
    if (lane == 0 && word * 32 < P.num_photon) P.bitmap[word] = mask;
    if (mask) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(P.hit_count, (unsigned long long)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, 0);
        const unsigned long long slot = base + __popc(mask & ((1u << lane) - 1u));
        if (is_hit && slot < (unsigned long long)cap) store_photon(P.hit_unordered + slot, p);
    }
}

// one thread per ray: the engine's closest-hit query (CSG/CSGScan.cu's _CSGScan_intersect plays this role for the
// reference); t = -1 on a miss
template <int TREE, bool POLISH>
__global__ void k_trace_rays(Accel acc, const float3* pos, const float3* dir, int n, float tmin, float tmax,
                             float* t_out, unsigned* boundary_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Hit h;
    trace<TREE, POLISH>(acc, pos[i], dir[i], tmin, tmax, -1, h);
    const bool miss = (h.prim_boundary & 0xffffu) == 0xffffu;
    t_out[i] = miss ? -1.f : h.t;
    boundary_out[i] = miss ? 0xffffffffu : (h.prim_boundary & 0xffffu);
}

// ---- per-form host launchers (defined in gbo_sim_forms.inl, one translation unit per TREE value) ---------------

// the wavefront form's device state (gbo_wavefront.cuh), besides the pregenerated-photon buffers
// the walk queue's sort grid (gbo_wavefront.cuh): 32 x 32 x 32 cells over the TLAS root box
constexpr int WF_CELL_BITS = 5;
constexpr int WF_CELLS = 1 << (3 * WF_CELL_BITS);
constexpr long long WF_SORT_MIN = 65536;        // walk queues shorter than this are walked unsorted

struct Wavefront {
    float4* hit;                    // 2 per photon: (normal, t), (lposz, iindex_identity, prim_boundary, 0)
    int* list[2];                   // live photons of even / odd steps
    int* walk;                      // photons of the current step whose query walks the instance tree
    int* walk_key;                  // their cells (the walk queue's sort key), at the same positions
    int* walk_sorted;               // the walk queue ordered by cell
    unsigned* bins;                 // per step, WF_CELLS cell counts turned into offsets (max_bounce x WF_CELLS)
    Acc64* acc;                     // precision mode: each photon's binary64 position / time accumulators
    unsigned long long* count;      // [2 s]: photons alive at step s; [2 s + 1]: of them queued for a walk;
                                    // 2 (max_bounce + 1) counters, zeroed by the launch
};

struct SimLaunch {
    long long n;                    // photons of the launch
    unsigned long long* pool;       // photon-pool counter, zeroed by the caller
    cudaStream_t stream;
    int kernel_mode;                // 0: pool generating its photons, 1: one thread per photon, 2: pool over
                                    // pregenerated photons (P.gen_photon set), 3: wavefront (P.gen_photon set)
    bool precise;                   // precision-mode kernels
    bool rng_call;                  // single-leaf binary32 kernels: Philox blocks by call (the CSG-tree forms
                                    // always call)
    long long grid;                 // pool kernels: blocks launched
    int refill, period;             // pool kernels: refill threshold and refill period
    int sms;                        // streaming multiprocessors (wavefront grids)
    Wavefront wf;                   // kernel mode 3
};

// the simulation kernel of form (TREE, L.precise, L.rng_call) over L.n photons
template <int TREE> void sim_launch(const Params& P, const SimLaunch& L);
// most resident blocks per SM of the pool kernel (pregenerated photons) of one form
template <int TREE> cudaError_t sim_pool_occupancy(bool precise, bool rng_call, int* blocks);
// the one-thread kernel with a bounded hit append (no-allocation entry point)
template <int TREE> void sim_launch_bounded(const Params& P, long long cap, unsigned grid, cudaStream_t s);
// closest hit of n arbitrary rays (default stream)
template <int TREE> void trace_rays_launch(bool polish, const Accel& acc, const float3* pos, const float3* dir, int n,
                                           float tmin, float tmax, float* t_out, unsigned* boundary_out);

#define GBO_SIM_FORM_INSTANCES(EXT, T)                                                                              \
    EXT template void sim_launch<T>(const Params&, const SimLaunch&);                                              \
    EXT template cudaError_t sim_pool_occupancy<T>(bool, bool, int*);                                              \
    EXT template void sim_launch_bounded<T>(const Params&, long long, unsigned, cudaStream_t);                     \
    EXT template void trace_rays_launch<T>(bool, const Accel&, const float3*, const float3*, int, float, float,    \
                                           float*, unsigned*);
GBO_SIM_FORM_INSTANCES(extern, 0)
GBO_SIM_FORM_INSTANCES(extern, 1)
GBO_SIM_FORM_INSTANCES(extern, 2)

}  // namespace gbo
