// gbo_wavefront.cuh : the wavefront kernel form (kernel mode 3) of the photon program.
//
// The photon program of CSGOptiX/CSGOptiX7.cu:405-503 runs one photon per thread from generation to its last
// bounce.  The persistent pool forms keep that shape; this form cuts it at every step instead.  Step s of every live
// photon runs as three passes over the list of photons alive at step s, each pass a kernel of its own:
//
//   k_wf_trace<TREE, false>  the query's first part: the photon's previous instance, then that instance's overlap
//                            list or its clear ball (trace_items stopped before the instance-tree walk).  Queries
//                            that end there write their hit record; the others are queued for a walk.
//   k_wf_trace<TREE, true>   the queued queries in full: the warps walk the instance tree together, every lane of a
//                            warp busy with a walk (the walks are a minority of the queries and the longest part).
//   k_wf_step                the physics of the step (qsim::propagate) from the hit record; photons that go on are
//                            appended to the list of step s + 1, the others finish (hit bitmap, hit record, photon
//                            record).
//
// Each kernel is a fraction of the whole photon program's code, so the instruction cache holds the kernel that is
// running, and every warp works on live photons only.  Between passes a photon lives in the pregenerated-photon
// buffers of kernel mode 2 (record, random-stream place, start instance) plus a 32-byte hit record; one step moves
// about 250 bytes per live photon through HBM.  Every live photon takes exactly one step per pass, so a photon of the
// list of step s has bounced s times.
//
// A photon's arithmetic is the same as in the other forms (same functions, same order), so photons, flag histories
// and hits are identical; only the order in which photons are appended to the lists differs, and no result depends
// on it.
#pragma once
#include "gbo_sim.cuh"

namespace gbo {

// Register budgets of the passes, measured on the 100M-photon, 20,000-sensor event: 128 for the query passes (4 blocks
// of 128 per SM, a few spills) beat 168 without spills by 10 %; 80 for the physics pass (6 blocks per SM) beat
// ptxas' own choice (72, 20 B of spills) by 2 %.  A persistent walk pass (lanes whose walk ended taking the next
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

// warp-aggregated append of the lanes with `take` set; every lane of the warp calls it
GBO_DEV void wf_append(int* list, unsigned long long* count, bool take, int idx)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    const int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if ((int)lane == leader) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take) list[base + __popc(m & ((1u << lane) - 1u))] = idx;
}

// Warp-uniform loops over [0, n): `base` is the same for the 32 lanes of a warp, so the ballots above see whole warps.
#define GBO_WF_FOR(base, n)                                                                                        \
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < (n);                    \
         base += (long long)gridDim.x * blockDim.x)

// Start: every photon of the launch as generated by k_generate; those that may step join the list of step 0.
template <int TREE>
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
        }
        wf_append(W.list[0], W.count, go, (int)idx);
        finish_photons(P, valid && !go, idx, p);
    }
}

// The query of each photon of step s up to the instance-tree walk (WALK false), or the queued queries in full.
template <int TREE, bool WALK>
__global__ void GBO_WF_TRACE_BOUNDS k_wf_trace(const __grid_constant__ Params P, Wavefront W, int s)
{
    const unsigned lane = threadIdx.x & 31u;
    const long long n = (long long)W.count[2 * s + (WALK ? 1 : 0)];
    const int* list = WALK ? W.walk : W.list[s & 1];
    GBO_WF_FOR(base, n) {
        const long long i = base + lane;
        int idx = 0;
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
            walk = trace_items<TREE, false>(P.acc, pos, mom, tmin, __ldcg(P.gen_hint + idx), !WALK, bb) == TRACE_WALK;
            if (!walk) {
                Hit h;
                trace_finish(P.acc, pos, mom, bb, h);
                wf_store_hit(W.hit + 2 * (size_t)idx, h);
            }
        }
        if (!WALK) wf_append(W.walk, W.count + 2 * s + 1, walk, idx);
    }
}

// The physics of step s: bounce s + 1 of every photon of the step's list.
template <int TREE, bool RCALL>
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
                const int command = propagate(P.tab, p, h, rng);
                const int bounce = s + 1;
                if (P.seq_out) seq_add(P.seq_out + idx, (unsigned)bounce, flag_of(p), boundary_of(p));
                done = command == CMD_BREAK || !(bounce < P.max_bounce && p.time < P.max_time);
                if (!done) {
                    store_photon(P.gen_photon + idx, p);
                    P.gen_rng[idx].x = rng.pos;
                    P.gen_hint[idx] = hint;
                }
            }
        }
        wf_append(W.list[(s + 1) & 1], W.count + 2 * (s + 1), valid && !done, idx);
        finish_photons(P, valid && done, idx, p);
    }
}

#undef GBO_WF_FOR

}  // namespace gbo
