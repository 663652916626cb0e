/*
 * ref_device.cu : the reference's own hot-path headers compiled by nvcc for the device (TEST INFRASTRUCTURE ONLY).
 *
 * Built by `make -C oracle ref-device` into oracle/_ref/ref_device.cubin (git-ignored) from the unmodified
 * reference headers: qudarap/qsim.h with qbnd.h, qscint.h, qcerenkov.h, sysrap/storch.h, and
 * CSG/csg_intersect_{leaf,node,tree}.h.  The switches are those of the reference's OptiX program build
 * (CSGOptiX/CMakeLists.txt:54-56): WITH_PRD, WITH_CONTIGUOUS, RNG_PHILOX, DEBUG_TAG and no PRODUCTION, so qsim
 * draws the same alignment "burn" randoms as the reference GPU path, with curand's own device Philox.  nvcc runs
 * with its default floating-point settings (contraction on, IEEE division and square root), as that build does.
 *
 * The kernel restates CSGOptiX/CSGOptiX7.cu:405-503 (simulate): one thread per photon, qrng<Philox>::init,
 * qsim::generate_photon, the bounce loop with the epsilon0 rule, ctx.point / ctx.trace / ctx.end for the flag
 * history, and the photon written at its launch index.  OptiX is replaced by a brute-force closest hit over every
 * instance and prim calling the reference's intersect_prim (CSG/csg_intersect_tree.h:683-719) in the instance
 * frame, with the closest-hit packing of CSGOptiX7.cu:749-847 (normal to world by the inverse transform,
 * iindex/identity, globalPrimIdx/boundary, lpos cos-theta/phi).  A padded world box per instance skips instances
 * the ray segment cannot reach: t is the same in world and instance frames, so the skip changes no result.
 * Ties in t keep the first (lowest instance, then prim), as the oracle does.
 *
 * Loaded by oracle/ref_device_run.cu through the CUDA driver API; never linked into the product.
 */
#include <cstdint>
#include <cstring>
#include <curand_kernel.h>

#include "srng.h"
#include "scuda.h"
#include "squad.h"
#include "srec.h"
#include "scerenkov.h"
#include "sscint.h"
#include "qsim.h"
#include "csg_intersect_leaf.h"
#include "csg_intersect_node.h"
#include "csg_intersect_tree.h"

#include "ref_device.h"
#include "../include/gbo_types.h"

static __device__ __forceinline__ bool ref_is_identity(const qat4& q)
{
    return q.q0.f.x == 1.f && q.q0.f.y == 0.f && q.q0.f.z == 0.f &&
           q.q1.f.x == 0.f && q.q1.f.y == 1.f && q.q1.f.z == 0.f &&
           q.q2.f.x == 0.f && q.q2.f.y == 0.f && q.q2.f.z == 1.f &&
           q.q3.f.x == 0.f && q.q3.f.y == 0.f && q.q3.f.z == 0.f;
}

/* slab test of the segment [t0, t1] against a padded world box; NaN slabs (0 * inf) are ignored */
static __device__ __forceinline__ bool ref_box_reached(const float* b, float3 o, float3 d, float t0, float t1)
{
    float ix = 1.f / d.x, iy = 1.f / d.y, iz = 1.f / d.z;
    float ax = (b[0] - o.x) * ix, bx = (b[3] - o.x) * ix;
    float ay = (b[1] - o.y) * iy, by = (b[4] - o.y) * iy;
    float az = (b[2] - o.z) * iz, bz = (b[5] - o.z) * iz;
    float lo = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fmaxf(fminf(az, bz), t0));
    float hi = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fminf(fmaxf(az, bz), t1));
    return lo <= hi;
}

/* optixTrace + __intersection__is + __closesthit__ch (WITH_PRD) by brute force */
static __device__ void ref_trace(const ref_dev_params& P, float3 pos, float3 dir, float tmin, float tmax, quad2* prd)
{
    const qat4* inst = (const qat4*)P.inst;
    const qat4* inst_inv = (const qat4*)P.inst_inv;
    const CSGPrim* prim = (const CSGPrim*)P.prim;
    const gbo_csgsolid* solid = (const gbo_csgsolid*)P.solid;
    const CSGNode* node = (const CSGNode*)P.node;
    float best_t = tmax;
    int best_inst = -1, best_prim = -1;
    float4 best = make_float4(0.f, 0.f, 0.f, 0.f);
    float3 best_lpos = make_float3(0.f, 0.f, 0.f);
    for (int ii = 0; ii < P.num_inst; ii++) {
        if (!ref_box_reached(P.inst_box + 6 * ii, pos, dir, tmin, best_t)) continue;
        const qat4& fwd = inst[ii];
        const qat4& inv = inst_inv[ii];
        int gas = fwd.q1.i.w;
        const gbo_csgsolid& so = solid[gas];
        bool ident = ref_is_identity(inv);
        float3 oo = ident ? pos : inv.right_multiply(pos, 1.f);
        float3 od = ident ? dir : inv.right_multiply(dir, 0.f);
        for (int k = 0; k < so.numPrim; k++) {
            int pi = so.primOffset + k;
            const CSGPrim& pr = prim[pi];
            const CSGNode* root = node + pr.nodeOffset();
            float4 isect = make_float4(0.f, 0.f, 0.f, 0.f);
            bool valid = intersect_prim(isect, root, (const float4*)P.plan, (const qat4*)P.itra, tmin, oo, od, false);
            // optixReportIntersection accepts a hit only inside the ray's [tmin, tmax] interval
            if (valid && isect.w >= tmin && isect.w < best_t) {
                best_t = isect.w; best_inst = ii; best_prim = pi; best = isect;
                best_lpos = oo + isect.w * od;
            }
        }
    }
    prd->zero();
    if (best_inst < 0) {
        prd->q0.f.w = 1.f;
        prd->set_iindex_identity_(0xffffffffu);
        prd->set_globalPrimIdx_boundary_(0xffffffffu);
        return;
    }
    const CSGPrim& pr = prim[best_prim];
    const CSGNode* root = node + pr.nodeOffset();
    unsigned boundary = root->boundary();
    unsigned gpi = pr.globalPrimIdx();
    const qat4& inv = inst_inv[best_inst];
    float4 n = best;
    if (!ref_is_identity(inv)) inv.left_multiply_inplace(n, 0.f);
    prd->q0.f = make_float4(n.x, n.y, n.z, best.w);
    prd->set_lpos(normalize_cost(best_lpos), normalize_fphi(best_lpos));
    unsigned identity = (unsigned)inst[best_inst].q2.i.w;
    prd->set_iindex_identity(unsigned(best_inst), identity);
    prd->set_globalPrimIdx_boundary(gpi, boundary);
}

extern "C" __global__ void ref_simulate_kernel(ref_dev_params P)
{
    unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
    if ((int64_t)idx >= P.num_photon) return;

    quad4 bnd_meta;
    memset(&bnd_meta, 0, sizeof(bnd_meta));
    bnd_meta.q0.u.x = P.bnd_nx;
    bnd_meta.q0.u.y = P.bnd_ny;
    bnd_meta.q1.f.x = P.bnd_nm0;
    bnd_meta.q1.f.z = P.bnd_nms;

    qbnd bnd;
    memset(&bnd, 0, sizeof(bnd));
    bnd.boundary_tex = (cudaTextureObject_t)P.bnd_tex;
    bnd.boundary_meta = &bnd_meta;
    bnd.optical = (quad*)P.optical;

    qscint scint;
    memset(&scint, 0, sizeof(scint));
    scint.scint_tex = (cudaTextureObject_t)P.icdf_tex;
    scint.hd_factor = (unsigned)P.hd_factor;

    qbase base;
    memset(&base, 0, sizeof(base));
    base.pidx = ~0ull;

    qcerenkov cerenkov;
    memset(&cerenkov, 0, sizeof(cerenkov));
    cerenkov.base = &base;
    cerenkov.bnd = &bnd;

    qrng<Philox> rngcfg;
    rngcfg.seed = P.seed;
    rngcfg.offset = P.offset;
    rngcfg.skipahead_event_offset = P.skipahead_event_offset;

    sevent evt;
    memset((void*)&evt, 0, sizeof(evt));
    evt.index = P.event_index;
    evt.max_bounce = P.max_bounce;
    evt.photon = (sphoton*)P.photon;
    evt.seq = (sseq*)P.seq;

    qsim sim;
    memset((void*)&sim, 0, sizeof(sim));
    sim.base = &base;
    sim.evt = &evt;
    sim.rng = &rngcfg;
    sim.bnd = &bnd;
    sim.cerenkov = &cerenkov;
    sim.scint = &scint;

    unsigned genstep_idx = (unsigned)P.seed_idx[idx];
    const quad6& gs = ((const quad6*)P.genstep)[genstep_idx];
    unsigned long long photon_idx = P.photon_offset + idx;

    RNG rng;
    sim.rng->init(rng, sim.evt->index, photon_idx);

    quad2 prd_;
    prd_.zero();
    quad2* prd = &prd_;

    sctx ctx = {};
    ctx.evt = &evt;
    ctx.prd = prd;
    ctx.idx = idx;
    ctx.pidx = photon_idx;

    sim.generate_photon(ctx.p, rng, gs, photon_idx, genstep_idx);

    int command = START;
    int bounce = 0;
    ctx.point(bounce);
    while (bounce < evt.max_bounce && ctx.p.time < P.max_time) {
        float tmin = (ctx.p.orient_boundary_flag & P.eps0_mask) ? P.tmin0 : P.tmin;
        ref_trace(P, ctx.p.pos, ctx.p.mom, tmin, P.tmax, prd);
        if (prd->boundary() == 0xffffu) break;
        float3* normal = prd->normal();
        *normal = normalize(*normal);
        ctx.trace(bounce);
        command = sim.propagate(bounce, rng, ctx);
        bounce++;
        ctx.point(bounce);
        if (command == BREAK) break;
    }
    ctx.end();
    evt.photon[idx] = ctx.p;
}
