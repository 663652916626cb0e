/*
 * gbo_types.h : plain-old-data array layouts shared by the C ABI, the CUDA engine and the CPU oracle.
 *
 * Every struct here is a byte-for-byte stand-in for an array element that the reference passes between
 * host and device, so that a caller can hand the engine the same buffers it hands the reference:
 *
 *   gbo_quad      16 B  sysrap/squad.h  (union quad: float4 / uint4 / int4 views)
 *   gbo_quad6     96 B  sysrap/squad.h  quad6 : genstep (storch.h:43-69, scerenkov.h:29-58, sscint.h:34-62)
 *   gbo_sphoton   64 B  sysrap/sphoton.h:171-192 : photon and hit record, same bit packing
 *   gbo_prd       32 B  sysrap/squad.h:180-255 quad2 : per-ray intersect result (normal,t,lpos,iindex|identity,prim|boundary)
 *   gbo_csgnode   64 B  CSG/CSGNode.h:66-101,196 : CSG node (params, boundary, bbox, typecode, transform|complement)
 *   gbo_csgprim   64 B  CSG/CSGPrim.h:75-120 : prim (numNode, nodeOffset, tranOffset, planOffset, ...)
 *   gbo_csgsolid  48 B  CSG/CSGSolid.h:37-52 : solid (label, numPrim, primOffset, type, center_extent)
 *   gbo_qat4      64 B  sysrap/sqat4.h:22-120 : 4x4 float transform, row-vector convention, identity in .w column
 *
 * The header is C99 and C++ compatible and contains no CUDA types.
 */
#ifndef GBO_TYPES_H
#define GBO_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef union gbo_quad {
    float    f[4];
    uint32_t u[4];
    int32_t  i[4];
} gbo_quad;

typedef struct gbo_quad6 { gbo_quad q[6]; } gbo_quad6;

typedef struct gbo_sphoton {
    float    pos[3];
    float    time;
    float    mom[3];
    uint32_t hitcount_iindex;       /* hi16 hitcount, lo16 instance index */
    float    pol[3];
    float    wavelength;
    uint32_t orient_boundary_flag;  /* bit31 orient, bits 16-30 boundary, lo16 last flag */
    uint32_t identity;              /* hi8 extends index, lo24 sensor identity (sensor_identifier+1, 0: none) */
    uint32_t index;                 /* low 32 bits of the absolute photon index */
    uint32_t flagmask;              /* OR of every flag the photon collected */
} gbo_sphoton;

typedef struct gbo_prd { gbo_quad q0, q1; } gbo_prd;

typedef struct gbo_csgnode { gbo_quad q0, q1, q2, q3; } gbo_csgnode;
typedef struct gbo_csgprim { gbo_quad q0, q1, q2, q3; } gbo_csgprim;

typedef struct gbo_csgsolid {
    char    label[16];
    int32_t numPrim;
    int32_t primOffset;
    int32_t type;
    char    intent, pad0, pad1, pad2;
    float   center_extent[4];
} gbo_csgsolid;

typedef struct gbo_qat4 { gbo_quad q0, q1, q2, q3; } gbo_qat4;

/* photon history record (debug/parity output): sysrap/sseq.h NSEQ=2 x 64-bit, one 4-bit nibble per step point */
typedef struct gbo_seq { uint64_t seqhis[2]; uint64_t seqbnd[2]; } gbo_seq;

/* ---- enums restated from the reference ---------------------------------------------------------- */

/* photon flags : sysrap/OpticksPhoton.h:22-46 */
enum {
    GBO_CERENKOV           = 0x1 <<  0,
    GBO_SCINTILLATION      = 0x1 <<  1,
    GBO_TORCH              = 0x1 <<  2,
    GBO_BULK_ABSORB        = 0x1 <<  3,
    GBO_BULK_REEMIT        = 0x1 <<  4,
    GBO_BULK_SCATTER       = 0x1 <<  5,
    GBO_SURFACE_DETECT     = 0x1 <<  6,
    GBO_SURFACE_ABSORB     = 0x1 <<  7,
    GBO_SURFACE_DREFLECT   = 0x1 <<  8,
    GBO_SURFACE_SREFLECT   = 0x1 <<  9,
    GBO_BOUNDARY_REFLECT   = 0x1 << 10,
    GBO_BOUNDARY_TRANSMIT  = 0x1 << 11,
    GBO_NAN_ABORT          = 0x1 << 12,
    GBO_EFFICIENCY_COLLECT = 0x1 << 13,
    GBO_EFFICIENCY_CULL    = 0x1 << 14,
    GBO_MISS               = 0x1 << 15
};

/* genstep types : sysrap/OpticksGenstep.h:19-43 (only those the hot path generates from) */
enum {
    GBO_GS_DsG4Scintillation_r4695 = 5,
    GBO_GS_TORCH                   = 6,
    GBO_GS_CERENKOV                = 15,
    GBO_GS_SCINTILLATION           = 16,
    GBO_GS_G4Cerenkov_modified     = 18,
    GBO_GS_INPUT_PHOTON            = 19
};

/* torch sub-types : sysrap/storchtype.h:10-18 */
enum {
    GBO_T_UNDEF = 0, GBO_T_DISC, GBO_T_LINE, GBO_T_POINT, GBO_T_CIRCLE,
    GBO_T_RECTANGLE, GBO_T_SPHERE_MARSAGLIA, GBO_T_SPHERE
};

/* CSG node typecodes : sysrap/OpticksCSG.h */
enum {
    GBO_CSG_ZERO = 0,
    GBO_CSG_UNION = 1, GBO_CSG_INTERSECTION = 2, GBO_CSG_DIFFERENCE = 3,
    GBO_CSG_NODE = 11, GBO_CSG_CONTIGUOUS = 11, GBO_CSG_DISCONTIGUOUS = 12, GBO_CSG_OVERLAP = 13,
    GBO_CSG_LEAF = 101,
    GBO_CSG_SPHERE = 101, GBO_CSG_ZSPHERE = 103, GBO_CSG_CYLINDER = 105, GBO_CSG_CONE = 108,
    GBO_CSG_BOX3 = 110, GBO_CSG_CONVEXPOLYHEDRON = 112, GBO_CSG_HYPERBOLOID = 117,
    GBO_CSG_PHICUT = 121, GBO_CSG_HALFSPACE = 125
};

/* material/surface type "ems" in optical[line].y : sysrap/smatsur.h:8-15 */
enum {
    GBO_EMS_MATERIAL = 0, GBO_EMS_NOSURFACE = 1, GBO_EMS_SURFACE = 2,
    GBO_EMS_ZPLUS_SENSOR_A = 3, GBO_EMS_ZPLUS_SENSOR_CUSTOMART = 4, GBO_EMS_ZMINUS = 5
};

/* boundary texture lines : qudarap/qbnd.h:12-17 */
enum { GBO_OMAT = 0, GBO_OSUR = 1, GBO_ISUR = 2, GBO_IMAT = 3 };

#ifdef __cplusplus
}  /* extern "C" */
static_assert(sizeof(gbo_quad) == 16, "quad is 16 bytes");
static_assert(sizeof(gbo_quad6) == 96, "genstep quad6 is 96 bytes");
static_assert(sizeof(gbo_sphoton) == 64, "sphoton is 64 bytes");
static_assert(sizeof(gbo_prd) == 32, "prd quad2 is 32 bytes");
static_assert(sizeof(gbo_csgnode) == 64, "CSGNode is 64 bytes");
static_assert(sizeof(gbo_csgprim) == 64, "CSGPrim is 64 bytes");
static_assert(sizeof(gbo_csgsolid) == 48, "CSGSolid is 48 bytes");
static_assert(sizeof(gbo_qat4) == 64, "qat4 is 64 bytes");
static_assert(sizeof(gbo_seq) == 32, "seq is 32 bytes");
#else
_Static_assert(sizeof(gbo_quad6) == 96, "genstep quad6 is 96 bytes");
_Static_assert(sizeof(gbo_sphoton) == 64, "sphoton is 64 bytes");
_Static_assert(sizeof(gbo_csgsolid) == 48, "CSGSolid is 48 bytes");
#endif

#endif /* GBO_TYPES_H */
