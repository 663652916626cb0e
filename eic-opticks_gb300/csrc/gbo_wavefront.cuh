// gbo_wavefront.cuh : the wavefront kernel form (kernel mode 3) of the photon program.
//
// The photon program of CSGOptiX/CSGOptiX7.cu:405-503 runs one photon per thread from generation to its last
// bounce.  The persistent pool forms keep that shape; this form cuts it at every step instead.  Step s of every live
// photon runs as kernels over the list of photons alive at step s: three passes, and a sort between the first two:
//
//   k_wf_trace<TREE, false>  the query's first part: the photon's previous instance, then that instance's overlap
//                            list or its clear ball (trace_items stopped before the instance-tree walk).  Queries
//                            that end there write their hit record; the others are queued for a walk.
//   k_wf_cells_*             a counting sort of the walk queue by the cell its segment runs through (long queues).
//   k_wf_trace<TREE, true>   the queued queries in full: the warps walk the instance tree together, every lane of a
//                            warp busy with a walk (the walks are a minority of the queries and the longest part).
//   k_wf_step                the physics of the step (qsim::propagate) from the hit record; photons that go on are
//                            appended to the list of step s + 1, the others finish (hit bitmap, hit record, photon
//                            record).
//
// Each kernel is a fraction of the whole photon program's code, so the instruction cache holds the kernel that is
// running, and every warp works on live photons only.  Between passes a photon lives in the pregenerated-photon
// buffers of kernel mode 2 (record, random-stream place, start instance) plus a 32-byte hit record and its list
// entries (in the precision mode also its binary64 position / time accumulators, 32 bytes); one step moves about
// 250 bytes per live photon through HBM.  Every live photon takes exactly one step per pass, so a photon of the
// list of step s has bounced s times.
//
// A photon's arithmetic is the same as in the other forms (same functions, same order), so photons, flag histories
// and hits are identical; only the order in which photons are appended to the lists differs, and no result depends
// on it.
#pragma once
#include "gbo_sim.cuh"

namespace gbo {

// Register budgets of the passes, measured on the 100M-photon, 20,000-sensor event: 128 for the query passes (4 blocks
// of 128 per SM, a few spills) beat 168 without spills by 10 %; a budget of 80 for the physics pass (ptxas then uses
// 72 without spills: 7 blocks per SM) beat ptxas' unbounded choice (72 with 20 B of spills) by 2 %.  A persistent walk pass (lanes whose walk ended taking the next
// queued query, one traversal round at a time) ran 17-23 % slower than these one-query-per-lane passes.
#ifndef GBO_WF_TRACE_BOUNDS
#define GBO_WF_TRACE_BOUNDS __maxnreg__(128)
#endif
#ifndef GBO_WF_STEP_BOUNDS
#define GBO_WF_STEP_BOUNDS __maxnreg__(80)
#endif

GBO_DEV void wf_store_hit(float4* q, const Hit& h)
{
    __stcg(q, make_float4(h.normal.x, h.normal.y, h.normal.z, h.t));
    __stcg(q + 1, make_float4(h.lposz, __uint_as_float(h.iindex_identity), __uint_as_float(h.prim_boundary), 0.f));
}

GBO_DEV void wf_load_hit(const float4* q, Hit& h)
{
    const float4 a = __ldcg(q), b = __ldcg(q + 1);
    h.normal = f3(a.x, a.y, a.z);
    h.t = a.w;
    h.lposz = b.x;
    h.iindex_identity = __float_as_uint(b.y);
    h.prim_boundary = __float_as_uint(b.z);
}

// warp-aggregated append of the lanes with `take` set (and their keys, when `keys` is given); every lane of the warp
// calls it
GBO_DEV void wf_append(int* list, unsigned long long* count, bool take, int idx, int* keys = nullptr, int key = 0)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    const int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if ((int)lane == leader) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take) {
        const unsigned long long at = base + __popc(m & ((1u << lane) - 1u));
        list[at] = idx;
        if (keys) keys[at] = key;
    }
}

// The walk queue is ordered by cell before the walk pass, so that the 32 walks of a warp run through the same part of
// the instance tree: the cell of a query is the midpoint of the segment it had reached when it stopped before the
// walk (its best hit so far, clamped to the scene), on the WF_CELLS grid over the TLAS root box, in Morton order.
// Measured on the 100M-photon, 20,000-sensor event: 505M -> 536M photons/s (the segment's start or end as the cell:
// 514M and 520M).  Short queues (a few warps per SM) are walked unsorted: there the sort's launches cost more than
// the coherence gains.
GBO_DEV unsigned wf_spread(unsigned v)          // 5 bits -> every third bit
{
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

GBO_DEV int wf_cell(const Accel& a, float3 pos, float3 dir, float t)
{
    const float4* root = reinterpret_cast<const float4*>(a.tlas);
    const float4 l0 = __ldg(root), h0 = __ldg(root + 1);
    float4 l1 = __ldg(root + 2), h1 = __ldg(root + 3);
    if (__float_as_int(h1.w) < 0) { l1 = l0; h1 = h0; }        // a root with one child
    const float3 lo = f3(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z));
    const float3 hi = f3(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z));
    const float3 ext = hi - lo;
    const float reach = fminf(t, ext.x + ext.y + ext.z);
    const float3 m = pos + (0.5f * reach) * dir;
    const float s = (float)(1 << WF_CELL_BITS);
    auto q = [&](float v, float l, float e) {
        const float c = e > 0.f ? (v - l) / e * s : 0.f;
        return (unsigned)fminf(fmaxf(c, 0.f), s - 1.f);
    };
    return (int)(wf_spread(q(m.x, lo.x, ext.x)) | (wf_spread(q(m.y, lo.y, ext.y)) << 1) |
                 (wf_spread(q(m.z, lo.z, ext.z)) << 2));
}

// Warp-uniform loops over [0, n): `base` is the same for the 32 lanes of a warp, so the ballots above see whole warps.
#define GBO_WF_FOR(base, n)                                                                                        \
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < (n);                    \
         base += (long long)gridDim.x * blockDim.x)

// Start: every photon of the launch as generated by k_generate; those that may step join the list of step 0.
template <int TREE, bool PRECISE>
__global__ void __launch_bounds__(SIM_BLOCK) k_wf_start(const __grid_constant__ Params P, Wavefront W)
{
    const unsigned lane = threadIdx.x & 31u;
    GBO_WF_FOR(base, P.num_photon) {
        const long long idx = base + lane;
        const bool valid = idx < P.num_photon;
        Photon p;
        bool go = false;
        if (valid) {
            load_photon_streamed(p, P.gen_photon + idx);
            if (P.seq_out) seq_start(P.seq_out + idx, flag_of(p), boundary_of(p));
            go = 0 < P.max_bounce && p.time < P.max_time;
            if (PRECISE && go) {
                Acc64 acc;
                acc_init(acc, p);
                W.acc[idx] = acc;
            }
        }
        wf_append(W.list[0], W.count, go, (int)idx);
        finish_photons(P, valid && !go, idx, p);
    }
}

// The query of each photon of step s up to the instance-tree walk (WALK false), or the queued queries in full.
template <int TREE, bool WALK, bool PRECISE>
__global__ void GBO_WF_TRACE_BOUNDS k_wf_trace(const __grid_constant__ Params P, Wavefront W, int s)
{
    const unsigned lane = threadIdx.x & 31u;
    const long long n = (long long)W.count[2 * s + (WALK ? 1 : 0)];
    const int* list = WALK ? (n >= WF_SORT_MIN ? W.walk_sorted : W.walk) : W.list[s & 1];
    GBO_WF_FOR(base, n) {
        const long long i = base + lane;
        int idx = 0, cell = 0;
        bool walk = false;
        if (i < n) {
            idx = __ldcg(list + i);
            const float4* q = reinterpret_cast<const float4*>(P.gen_photon + idx);
            const float4 a = __ldcg(q), b = __ldcg(q + 1);
            const unsigned obf = __float_as_uint(__ldcg(reinterpret_cast<const float*>(q + 3)));
            const float3 pos = f3(a.x, a.y, a.z), mom = f3(b.x, b.y, b.z);
            const float tmin = (obf & P.eps0_mask) ? P.tmin0 : P.tmin;
            Best bb;
            trace_begin(bb, P.tmax);
            walk = trace_items<TREE, PRECISE>(P.acc, pos, mom, tmin, __ldcg(P.gen_hint + idx), !WALK, bb) == TRACE_WALK;
            if (!walk) {
                Hit h;
                trace_finish(P.acc, pos, mom, bb, h);
                wf_store_hit(W.hit + 2 * (size_t)idx, h);
            } else if (!WALK) {
                cell = wf_cell(P.acc, pos, mom, bb.t);
            }
        }
        if (!WALK) wf_append(W.walk, W.count + 2 * s + 1, walk, idx, W.walk_key, cell);
    }
}

// Counting sort of step s's walk queue by cell: count, exclusive scan (one block), scatter.  The counts of each step
// have their own bins, zeroed with the launch's counters.  (TREE only gives each form's translation unit its own
// instance.)
template <int TREE>
__global__ void __launch_bounds__(SIM_BLOCK) k_wf_cells_count(Wavefront W, int s)
{
    const unsigned lane = threadIdx.x & 31u;
    const long long n = (long long)W.count[2 * s + 1];
    if (n < WF_SORT_MIN) return;
    unsigned* bins = W.bins + (size_t)s * WF_CELLS;
    GBO_WF_FOR(base, n) {
        const long long i = base + lane;
        const int key = i < n ? __ldcg(W.walk_key + i) : -1;
        const unsigned same = __match_any_sync(0xffffffffu, key);
        if (key >= 0 && (int)lane == __ffs(same) - 1) atomicAdd(bins + key, (unsigned)__popc(same));
    }
}

constexpr int WF_SCAN_THREADS = 1024;

template <int TREE>
__global__ void __launch_bounds__(WF_SCAN_THREADS) k_wf_cells_scan(Wavefront W, int s)
{
    if (W.count[2 * s + 1] < (unsigned long long)WF_SORT_MIN) return;
    constexpr int PER = WF_CELLS / WF_SCAN_THREADS;
    __shared__ unsigned warp_sum[WF_SCAN_THREADS / 32];
    unsigned* bins = W.bins + (size_t)s * WF_CELLS;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned v[PER], sum = 0;
#pragma unroll
    for (int k = 0; k < PER; k++) { v[k] = bins[t * PER + k]; sum += v[k]; }
    unsigned incl = sum;                        // inclusive scan of the thread sums over the block
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned o = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += o;
    }
    if (lane == 31) warp_sum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = warp_sum[lane];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned o = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += o;
        }
        warp_sum[lane] = w;
    }
    __syncthreads();
    unsigned run = incl - sum + (warp > 0 ? warp_sum[warp - 1] : 0u);
#pragma unroll
    for (int k = 0; k < PER; k++) { bins[t * PER + k] = run; run += v[k]; }
}

template <int TREE>
__global__ void __launch_bounds__(SIM_BLOCK) k_wf_cells_scatter(Wavefront W, int s)
{
    const unsigned lane = threadIdx.x & 31u;
    const long long n = (long long)W.count[2 * s + 1];
    if (n < WF_SORT_MIN) return;
    unsigned* bins = W.bins + (size_t)s * WF_CELLS;
    GBO_WF_FOR(base, n) {
        const long long i = base + lane;
        const int key = i < n ? __ldcg(W.walk_key + i) : -1;
        const unsigned same = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(same) - 1;
        unsigned first = 0;
        if (key >= 0 && (int)lane == leader) first = atomicAdd(bins + key, (unsigned)__popc(same));
        first = __shfl_sync(0xffffffffu, first, leader);
        if (key >= 0) W.walk_sorted[first + __popc(same & ((1u << lane) - 1u))] = __ldcg(W.walk + i);
    }
}

// The physics of step s: bounce s + 1 of every photon of the step's list.
template <int TREE, bool RCALL, bool PRECISE>
__global__ void GBO_WF_STEP_BOUNDS k_wf_step(const __grid_constant__ Params P, Wavefront W, int s)
{
    const unsigned lane = threadIdx.x & 31u;
    const long long n = (long long)W.count[2 * s];
    const int* list = W.list[s & 1];
    GBO_WF_FOR(base, n) {
        const long long i = base + lane;
        const bool valid = i < n;
        int idx = 0;
        Photon p;
        bool done = false;
        if (valid) {
            idx = __ldcg(list + i);
            load_photon_streamed(p, P.gen_photon + idx);
            Hit h;
            wf_load_hit(W.hit + 2 * (size_t)idx, h);
            if ((h.prim_boundary & 0xffffu) == 0xffffu) {
                done = true;
            } else {
                RngT<RCALL> rng;
                const ulonglong2 r = __ldcg(P.gen_rng + idx);
                rng_init(rng, P.seed, r.y, r.x);
                const int hint = (int)(h.iindex_identity >> 16);
                h.normal = normalize(h.normal);
                Acc64 acc;
                if (PRECISE) acc = W.acc[idx];
                const int command = propagate(P.tab, p, h, rng, PRECISE ? &acc : nullptr);
                const int bounce = s + 1;
                if (P.seq_out) seq_add(P.seq_out + idx, (unsigned)bounce, flag_of(p), boundary_of(p));
                done = command == CMD_BREAK || !(bounce < P.max_bounce && p.time < P.max_time);
                if (!done) {
                    store_photon(P.gen_photon + idx, p);
                    P.gen_rng[idx].x = rng.pos;
                    P.gen_hint[idx] = hint;
                    if (PRECISE) W.acc[idx] = acc;
                }
            }
        }
        wf_append(W.list[(s + 1) & 1], W.count + 2 * (s + 1), valid && !done, idx);
        finish_photons(P, valid && done, idx, p);
    }
}

#undef GBO_WF_FOR

}  // namespace gbo
