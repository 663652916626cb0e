/*
 * oracle.h : CPU restatement of the reference's optical-photon hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this library, and only as the checker or the timed CPU baseline; the product path never calls it.
 *
 * It restates, in plain C, the per-photon program of CSGOptiX/CSGOptiX7.cu:405-503 (simulate) with the
 * qudarap/qsim.h physics, the sysrap/storch.h, qudarap/qscint.h and qudarap/qcerenkov.h generators, the
 * CSG/csg_intersect_{leaf,node,tree}.h intersection and the curand Philox4x32-10 stream set up as in
 * qudarap/qrng.h:131-137.  The OptiX acceleration structure is replaced by brute force over every
 * instance and prim with the OptiX closest-hit rule (smallest t, ties to the lowest instance then prim).
 */
#ifndef GBO_ORACLE_H
#define GBO_ORACLE_H

#include <stdint.h>
#include "../include/gbo_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* 2D float or float4 texture with cudaFilterModeLinear, normalized coordinates, cudaAddressModeWrap */
typedef struct orc_tex {
    int          nx, ny, ncomp;   /* ncomp 4 (bnd) or 1 (scint icdf) */
    const float* data;            /* row-major (ny, nx, ncomp) */
} orc_tex;

typedef struct orc_geom {
    const gbo_csgnode*  node;
    const gbo_csgprim*  prim;
    const gbo_csgsolid* solid;
    int                 num_solid;
    const gbo_qat4*     inst;       /* forward instance transforms, identity ints in the .w column */
    const gbo_qat4*     inst_inv;   /* inverse instance transforms (object <- world) */
    int                 num_inst;
    const gbo_qat4*     itra;       /* inverse node transforms, 1-based gtransformIdx */
    const float*        plan;       /* float4 planes */
} orc_geom;

typedef struct orc_sim {
    orc_geom        geom;
    orc_tex         bnd;            /* boundary texture (761, num_bnd*4*2) float4 */
    float           bnd_nm0, bnd_nms;
    const uint32_t* optical;        /* (num_bnd*4, 4) */
    orc_tex         icdf;           /* scintillation inverse-CDF texture (4096, 1|3) float */
    int             hd_factor;      /* 0, 10, 20 */
    int             max_bounce;     /* 31 */
    float           max_time;       /* 1e27 */
    float           tmin, tmin0, tmax;
    uint32_t        eps0_mask;      /* flags after which tmin0 is used */
    uint64_t        seed, offset, skipahead_event_offset;
    int             debug_tag;      /* 1: draw order of the reference GPU build (DEBUG_TAG burns), 0: PRODUCTION */
} orc_sim;

/* Simulate photons [0, num_photon) of one launch.  seed[i] = genstep index of photon i.
   input_photon is read for INPUT_PHOTON gensteps (indexed by launch photon index). seq may be NULL. */
void orc_simulate(const orc_sim* s, const gbo_quad6* gs, const int32_t* seed, const gbo_sphoton* input_photon,
                  uint64_t photon_offset, uint32_t event_index, int64_t num_photon,
                  gbo_sphoton* out, gbo_seq* seq, int nthreads);

/* seed[photon] = genstep index from numphoton prefix sums (QEvt.cu:181-237); returns total photons */
int64_t orc_fill_seed(const gbo_quad6* gs, int num_gs, int32_t* seed, int64_t max_seed);

/* hit selection : (flagmask & hitmask) == hitmask (sysrap/sphoton.h:1219-1225), order preserved */
int64_t orc_select_hits(const gbo_sphoton* p, int64_t n, uint32_t hitmask, gbo_sphoton* hits);
int64_t orc_merge_hits(const gbo_sphoton* in, int64_t n, float tw, gbo_sphoton* out);

/* unit pieces exposed for known-answer tests */
void  orc_philox_uniforms(uint64_t seed, uint64_t subsequence, uint64_t offset, uint64_t skip, int n, float* out);
void  orc_tex_lookup4(const orc_tex* t, const float* xy, int n, float* out);
void  orc_tex_lookup1(const orc_tex* t, const float* xy, int n, float* out);
int   orc_intersect_prim_c(const gbo_csgnode* node, const float* plan, const gbo_qat4* itra, float t_min,
                           const float* o, const float* d, float* isect);
void  orc_trace_c(const orc_geom* g, const float* pos, const float* dir, float tmin, float tmax, gbo_prd* prd);
void  orc_invert_transforms(const gbo_qat4* in, gbo_qat4* out, int n);

#ifdef __cplusplus
}
#endif
#endif
