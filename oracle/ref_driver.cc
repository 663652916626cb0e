/*
 * ref_driver.cc : drives the reference's own hot-path headers, compiled for the host, to pin the oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into oracle/_ref/libref.so from the unmodified
 * reference headers (qudarap/qsim.h and its includes, CSG/csg_intersect_*.h) when the reference source tree
 * is present; the output never enters the repository and never runs on the product path.
 *
 * Build switches mirror the reference's OptiX program build (CSGOptiX/CMakeLists.txt:54-56): DEBUG_TAG and
 * no PRODUCTION, so qsim consumes the same "burn" randoms as the reference GPU path, RNG_PHILOX so RNG is
 * curandStatePhilox4_32_10 (curand's own host-callable implementation from the CUDA toolkit headers), and
 * WITH_PRD.  __CUDABE__ selects the device branches of the headers.
 *
 * Project-written shims the headers need on the host: tex2D with CUDA linear filtering (the oracle's
 * orc_tex2d4/orc_tex2d1), erfcinvf (Newton iteration on erfc; only reached by smearing code that the hot
 * path never calls), __float2int_rn, __ffs.
 *
 * The driver restates the per-photon loop of CSGOptiX/CSGOptiX7.cu:405-503 around qsim::generate_photon and
 * qsim::propagate, with the OptiX traversal replaced by brute force over all instances and prims calling
 * the reference's intersect_prim (CSG/csg_intersect_tree.h:683-719).
 */
#include <cstdio>
#include <cmath>
#include <cstring>
#include <cstdint>
#include <strings.h>
#include <cuda_runtime.h>
#include <vector_types.h>
#include <vector_functions.h>

extern "C" {
#include "oracle.h"
}
#include "orc_internal.h"

static inline float erfcinvf(float y)
{
    double x = 0.0;
    for (int i = 0; i < 80; i++) {
        double f = erfc(x) - (double)y;
        double d = -2.0 / sqrt(M_PI) * exp(-x * x);
        x -= f / d;
    }
    return (float)x;
}
static inline int __float2int_rn(float f) { return (int)lrintf(f); }
static inline int __ffs(int x) { return ffs(x); }

template <typename T> T tex2D(cudaTextureObject_t tex, float x, float y);
template <> inline float4 tex2D<float4>(cudaTextureObject_t tex, float x, float y)
{
    v4 r = orc_tex2d4(reinterpret_cast<const orc_tex*>(tex), x, y);
    return make_float4(r.x, r.y, r.z, r.w);
}
template <> inline float tex2D<float>(cudaTextureObject_t tex, float x, float y)
{
    return orc_tex2d1(reinterpret_cast<const orc_tex*>(tex), x, y);
}

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

extern "C" {

void ref_curand_uniforms(uint64_t seed, uint64_t subsequence, uint64_t offset, uint64_t skip, int n, float* out)
{
    curandStatePhilox4_32_10 s;
    curand_init(seed, subsequence, offset, &s);
    if (skip) skipahead(skip, &s);
    for (int i = 0; i < n; i++) out[i] = curand_uniform(&s);
}

int ref_intersect_prim(const gbo_csgnode* node, const float* plan, const gbo_qat4* itra, float t_min,
                       const float* o, const float* d, float* out)
{
    float4 isect = make_float4(0.f, 0.f, 0.f, 0.f);
    float3 ro = make_float3(o[0], o[1], o[2]);
    float3 rd = make_float3(d[0], d[1], d[2]);
    bool valid = intersect_prim(isect, (const CSGNode*)node, (const float4*)plan, (const qat4*)itra, t_min, ro, rd, false);
    out[0] = isect.x; out[1] = isect.y; out[2] = isect.z; out[3] = isect.w;
    return valid ? 1 : 0;
}

}  // extern "C"

static bool is_identity(const qat4& q)
{
    return q.q0.f.x == 1.f && q.q0.f.y == 0.f && q.q0.f.z == 0.f &&
           q.q1.f.x == 0.f && q.q1.f.y == 1.f && q.q1.f.z == 0.f &&
           q.q2.f.x == 0.f && q.q2.f.y == 0.f && q.q2.f.z == 1.f &&
           q.q3.f.x == 0.f && q.q3.f.y == 0.f && q.q3.f.z == 0.f;
}

/* brute-force stand-in for optixTrace + __intersection__is + __closesthit__ch with WITH_PRD */
static void ref_trace(const orc_geom* g, float3 pos, float3 dir, float tmin, float tmax, quad2* prd)
{
    float best_t = tmax;
    int best_inst = -1, best_prim = -1;
    float4 best = make_float4(0.f, 0.f, 0.f, 0.f);
    float3 best_lpos = make_float3(0.f, 0.f, 0.f);
    for (int ii = 0; ii < g->num_inst; ii++) {
        const qat4& fwd = ((const qat4*)g->inst)[ii];
        const qat4& inv = ((const qat4*)g->inst_inv)[ii];
        int gas = fwd.q1.i.w;
        const gbo_csgsolid& so = g->solid[gas];
        bool ident = is_identity(inv);
        float3 oo = ident ? pos : inv.right_multiply(pos, 1.f);
        float3 od = ident ? dir : inv.right_multiply(dir, 0.f);
        for (int k = 0; k < so.numPrim; k++) {
            int pi = so.primOffset + k;
            const gbo_csgprim& pr = g->prim[pi];
            const CSGNode* root = (const CSGNode*)(g->node + pr.q0.i[1]);
            float4 isect = make_float4(0.f, 0.f, 0.f, 0.f);
            bool valid = intersect_prim(isect, root, (const float4*)g->plan, (const qat4*)g->itra, tmin, oo, od, false);
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
    const gbo_csgprim& pr = g->prim[best_prim];
    const CSGNode* root = (const CSGNode*)(g->node + pr.q0.i[1]);
    unsigned boundary = root->boundary();
    unsigned gpi = pr.q3.u[3];
    const qat4& inv = ((const qat4*)g->inst_inv)[best_inst];
    float4 n = best;
    if (!is_identity(inv)) inv.left_multiply_inplace(n, 0.f);
    prd->q0.f = make_float4(n.x, n.y, n.z, best.w);
    prd->set_lpos(normalize_cost(best_lpos), normalize_fphi(best_lpos));
    unsigned identity = (unsigned)((const qat4*)g->inst)[best_inst].q2.i.w;
    prd->set_iindex_identity(unsigned(best_inst), identity);
    prd->set_globalPrimIdx_boundary(gpi, boundary);
}

extern "C" void ref_simulate(const orc_sim* s, const gbo_quad6* gs, const int32_t* seed, const gbo_sphoton* input_photon,
                             uint64_t photon_offset, uint32_t event_index, int64_t num_photon,
                             gbo_sphoton* out, gbo_seq* seq_out)
{
    quad4 bnd_meta;
    memset(&bnd_meta, 0, sizeof(bnd_meta));
    bnd_meta.q0.u.x = (unsigned)s->bnd.nx;
    bnd_meta.q0.u.y = (unsigned)s->bnd.ny;
    bnd_meta.q1.f.x = s->bnd_nm0;
    bnd_meta.q1.f.z = s->bnd_nms;

    qbnd bnd;
    memset(&bnd, 0, sizeof(bnd));
    bnd.boundary_tex = (cudaTextureObject_t)(uintptr_t)&s->bnd;
    bnd.boundary_meta = &bnd_meta;
    bnd.optical = (quad*)s->optical;

    qscint scint;
    memset(&scint, 0, sizeof(scint));
    scint.scint_tex = (cudaTextureObject_t)(uintptr_t)&s->icdf;
    scint.hd_factor = (unsigned)s->hd_factor;

    qbase base;
    base.pidx = ~0ull;

    qcerenkov cerenkov;
    memset(&cerenkov, 0, sizeof(cerenkov));
    cerenkov.base = &base;
    cerenkov.bnd = &bnd;

    qrng<Philox> rngcfg;
    rngcfg.seed = s->seed;
    rngcfg.offset = s->offset;
    rngcfg.skipahead_event_offset = s->skipahead_event_offset;

    sevent evt;
    memset((void*)&evt, 0, sizeof(evt));
    evt.index = (int)event_index;
    evt.max_bounce = s->max_bounce;
    evt.photon = (sphoton*)input_photon;

    qsim sim;
    memset((void*)&sim, 0, sizeof(sim));
    sim.base = &base;
    sim.evt = &evt;
    sim.rng = &rngcfg;
    sim.bnd = &bnd;
    sim.cerenkov = &cerenkov;
    sim.scint = &scint;

    for (int64_t idx = 0; idx < num_photon; idx++) {
        unsigned genstep_idx = (unsigned)seed[idx];
        const quad6& g = ((const quad6*)gs)[genstep_idx];
        unsigned long long photon_idx = photon_offset + (unsigned long long)idx;
        RNG rng;
        curand_init(rngcfg.seed, photon_idx, rngcfg.offset, &rng);
        skipahead(rngcfg.skipahead_event_offset * (unsigned long long)event_index, &rng);

        quad2 prd;
        prd.zero();
        sctx ctx = {};
        ctx.evt = &evt;
        ctx.prd = &prd;
        ctx.idx = (unsigned)idx;
        ctx.pidx = photon_idx;

        sim.generate_photon(ctx.p, rng, g, photon_idx, genstep_idx);

        sseq sq;
        memset(&sq, 0, sizeof(sq));
        int bounce = 0;
        sq.add_nibble(bounce, ctx.p.flag(), ctx.p.boundary());
        while (bounce < s->max_bounce && ctx.p.time < s->max_time) {
            float tmin = (ctx.p.orient_boundary_flag & s->eps0_mask) ? s->tmin0 : s->tmin;
            ref_trace(&s->geom, ctx.p.pos, ctx.p.mom, tmin, s->tmax, &prd);
            if (prd.boundary() == 0xffffu) break;
            float3* normal = prd.normal();
            *normal = normalize(*normal);
            int command = sim.propagate(bounce, rng, ctx);
            bounce++;
            sq.add_nibble(bounce, ctx.p.flag(), ctx.p.boundary());
            if (command == BREAK) break;
        }
        memcpy(&out[idx], &ctx.p, sizeof(gbo_sphoton));
        if (seq_out) memcpy(&seq_out[idx], &sq, sizeof(gbo_seq));
    }
}
