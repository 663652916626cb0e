/*
 * ref_device.h : launch parameters of the reference-header device build (TEST INFRASTRUCTURE ONLY).
 *
 * oracle/ref_device.cu compiles the reference's unmodified qsim.h / csg_intersect_*.h headers with nvcc for
 * sm_103a into oracle/_ref/ref_device.cubin (recipe: oracle/Makefile, target ref-device, in a checkout that holds
 * the reference tree).  oracle/ref_device_run.cu, built wherever the GPU is, loads that cubin with the CUDA driver
 * API, creates the boundary and scintillation textures with the reference's descriptors and launches it.  The
 * resulting photons and flag histories are the reference's own device arithmetic on the same inputs, and become
 * fixtures under tests/golden/.  Nothing on the product path includes this header.
 *
 * Plain C: no reference types, no CUDA types beyond 64-bit texture handles.
 */
#ifndef GBO_REF_DEVICE_H
#define GBO_REF_DEVICE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ref_dev_params {
    /* geometry (device pointers, the CSGFoundry layouts of gbo_types.h) */
    const void*        node;        /* CSGNode     (64 B) */
    const void*        prim;        /* CSGPrim     (64 B) */
    const void*        solid;       /* CSGSolid    (48 B) */
    const void*        inst;        /* qat4 forward instance transforms, identity ints in .w */
    const void*        inst_inv;    /* qat4 inverse instance transforms */
    const float*       inst_box;    /* per instance: world box (x0,y0,z0,x1,y1,z1), padded; a prefilter only */
    const void*        itra;        /* qat4 inverse node transforms */
    const void*        plan;        /* float4 planes */
    int32_t            num_inst;
    int32_t            pad0;
    /* optical tables */
    uint64_t           bnd_tex;     /* cudaTextureObject_t: float4 (bnd_nx, bnd_ny), linear, normalized, wrap */
    uint32_t           bnd_nx, bnd_ny;
    float              bnd_nm0, bnd_nms;
    const uint32_t*    optical;     /* (num_bnd*4, 4) */
    uint64_t           icdf_tex;    /* cudaTextureObject_t: float (4096, 1|3), linear, normalized, wrap */
    int32_t            hd_factor;
    /* event configuration (SEventConfig defaults unless overridden) */
    int32_t            max_bounce;
    float              max_time, tmin, tmin0, tmax;
    uint32_t           eps0_mask;
    int32_t            pad1;
    uint64_t           seed, offset, skipahead_event_offset;
    /* launch */
    const void*        genstep;     /* quad6 */
    const int32_t*     seed_idx;    /* photon -> genstep index (QEvt seed array) */
    uint64_t           photon_offset;
    int32_t            event_index;
    int32_t            pad2;
    int64_t            num_photon;
    void*              photon;      /* sphoton out; holds the input photons on entry for INPUT_PHOTON gensteps */
    void*              seq;         /* sseq out (32 B per photon) */
} ref_dev_params;

#ifdef __cplusplus
}
#endif
#endif
