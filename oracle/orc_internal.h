/*
 * orc_internal.h : float3 helpers and internal declarations of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the CUDA engine; it is never linked into,
 * called by, or used as a fallback of the product library.
 *
 * All arithmetic is IEEE binary32 in the same operation order as the reference device code.  The build
 * uses -ffp-contract=off so results are identical on x86-64 and aarch64 hosts.
 */
#ifndef ORC_INTERNAL_H
#define ORC_INTERNAL_H

#include <math.h>
#include <stdint.h>
#include "oracle.h"

typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } v4;

static inline v3 V3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v4 V4(float x, float y, float z, float w) { v4 r = {x, y, z, w}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vscale(float s, v3 a) { return V3(s * a.x, s * a.y, s * a.z); }
static inline v3 vneg(v3 a) { return V3(-a.x, -a.y, -a.z); }
/* dot/cross/length/normalize follow the CUDA sample helper_math expression order used by sysrap/scuda.h */
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) { return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline float vlength(v3 a) { return sqrtf(vdot(a, a)); }
static inline v3 vnormalize(v3 a) { float inv = 1.0f / sqrtf(vdot(a, a)); return vscale(inv, a); }
static inline v3 v3of(const float* p) { return V3(p[0], p[1], p[2]); }
static inline void v3to(float* p, v3 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }

#define ORC_PI_F 3.14159265358979323846f   /* M_PIf */

#ifdef __cplusplus
extern "C" {
#endif

/* ---- rng (orc_rng.c) ---- */
typedef struct {
    uint32_t ctr[4];
    uint32_t key[2];
    uint32_t out[4];
    int      lane;
} orc_rng;
void  orc_rng_init(orc_rng* r, uint64_t seed, uint64_t subsequence, uint64_t offset);
void  orc_rng_skipahead(orc_rng* r, uint64_t n);
float orc_uniform(orc_rng* r);

/* ---- texture emulation (orc_rng.c) ---- */
v4    orc_tex2d4(const orc_tex* t, float x, float y);
float orc_tex2d1(const orc_tex* t, float x, float y);

/* ---- CSG (orc_csg.c) ---- */
int   orc_intersect_prim(v4* isect, const gbo_csgnode* node, const float* plan, const gbo_qat4* itra,
                         float t_min, v3 o, v3 d);
void  orc_trace(const orc_geom* g, v3 pos, v3 dir, float tmin, float tmax, gbo_prd* prd);

/* ---- physics helpers (orc_qsim.c) ---- */
void  orc_rotateUz(v3* d, v3 u);

#ifdef __cplusplus
}
#endif
#endif
