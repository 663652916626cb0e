// gbo_trace.cuh : closest-hit ray query over the two-level acceleration structure.
//
// Replaces optixTrace + __intersection__is + __closesthit__ch of the reference (CSGOptiX/CSGOptiX7.cu:110-216,
// :749-940) with the same results:
//   * intersections with t in (tmin, tmax) via intersect_prim on the object-frame ray (the instance's inverse
//     transform applied to the world ray; t is shared between frames);
//   * the closest t wins; equal t resolve to the lowest (instance, prim) so that the result does not depend on
//     traversal order;
//   * the object-frame normal goes to the world frame through the inverse-transpose
//     (optixTransformNormalFromObjectToWorldSpace); identity instances skip both transforms;
//   * iindex|identity and globalPrimIdx|boundary packed in 16-bit halves (CSGOptiX7.cu:753, :929);
//   * a miss returns boundary 0xffff (__miss__ms).
#pragma once
#include "gbo_csg.cuh"
#include "gbo_physics.cuh"
#include "gbo_accel.h"

namespace gbo {

struct Accel {
    const BvhNode* tlas;
    const int32_t* tlas_index;
    const InstDev* inst;
    const PrimDev* prim;
    const SolidDev* solid;
    const gbo_csgnode* node;
    const float4* plan;
    const gbo_qat4* itra;
};

GBO_DEV bool slab(float4 bmin, float4 bmax, float3 o, float3 inv, float tmin, float tmax, float& tnear)
{
    const float tx0 = (bmin.x - o.x) * inv.x, tx1 = (bmax.x - o.x) * inv.x;
    const float ty0 = (bmin.y - o.y) * inv.y, ty1 = (bmax.y - o.y) * inv.y;
    const float tz0 = (bmin.z - o.z) * inv.z, tz1 = (bmax.z - o.z) * inv.z;
    tnear = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
    const float tfar = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    return tnear <= tfar && tfar >= tmin && tnear <= tmax;
}

GBO_DEV float3 safe_inv(float3 d) { return f3(1.f / d.x, 1.f / d.y, 1.f / d.z); }

GBO_DEV float3 inst_point(const InstDev& d, float3 v)
{
    const float4 c0 = *reinterpret_cast<const float4*>(d.c0);
    const float4 c1 = *reinterpret_cast<const float4*>(d.c1);
    const float4 c2 = *reinterpret_cast<const float4*>(d.c2);
    return f3(c0.x * v.x + c0.y * v.y + c0.z * v.z + c0.w * 1.f,
              c1.x * v.x + c1.y * v.y + c1.z * v.z + c1.w * 1.f,
              c2.x * v.x + c2.y * v.y + c2.z * v.z + c2.w * 1.f);
}
GBO_DEV float3 inst_vector(const InstDev& d, float3 v)
{
    const float4 c0 = *reinterpret_cast<const float4*>(d.c0);
    const float4 c1 = *reinterpret_cast<const float4*>(d.c1);
    const float4 c2 = *reinterpret_cast<const float4*>(d.c2);
    return f3(c0.x * v.x + c0.y * v.y + c0.z * v.z + c0.w * 0.f,
              c1.x * v.x + c1.y * v.y + c1.z * v.z + c1.w * 0.f,
              c2.x * v.x + c2.y * v.y + c2.z * v.z + c2.w * 0.f);
}
GBO_DEV float3 inst_normal(const InstDev& d, float3 n)    // transpose of the inverse 3x3
{
    return f3(d.c0[0] * n.x + d.c1[0] * n.y + d.c2[0] * n.z,
              d.c0[1] * n.x + d.c1[1] * n.y + d.c2[1] * n.z,
              d.c0[2] * n.x + d.c1[2] * n.y + d.c2[2] * n.z);
}

GBO_DEV InstDev load_inst(const InstDev* p)
{
    const float4* q = reinterpret_cast<const float4*>(p);
    InstDev d;
    float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    int4 e = __ldg(reinterpret_cast<const int4*>(q + 3));
    d.c0[0] = a.x; d.c0[1] = a.y; d.c0[2] = a.z; d.c0[3] = a.w;
    d.c1[0] = b.x; d.c1[1] = b.y; d.c1[2] = b.z; d.c1[3] = b.w;
    d.c2[0] = c.x; d.c2[1] = c.y; d.c2[2] = c.z; d.c2[3] = c.w;
    d.solid = e.x; d.identity = (uint32_t)e.y; d.is_identity = e.z; d.iindex = (uint32_t)e.w;
    return d;
}

template <bool TREE>
GBO_DEV bool prim_hit(float4& is, const Accel& a, int node_offset, float t_min, float3 o, float3 d)
{
    const gbo_csgnode* root = a.node + node_offset;
    if (TREE) return intersect_prim(is, root, a.plan, a.itra, t_min, o, d);
    if (node_typecode(root) >= GBO_CSG_LEAF) return intersect_leaf(is, root, a.plan, a.itra, t_min, o, d);
    is = make_float4(0.f, 0.f, 0.f, 0.f);
    return false;
}

constexpr int TRAVERSAL_STACK = 64;

template <bool TREE>
GBO_DEV void trace(const Accel& a, float3 pos, float3 dir, float tmin, float tmax, Hit& h)
{
    float best_t = tmax;
    unsigned best_key = 0xffffffffu;
    float4 best_is = make_float4(0.f, 0.f, 0.f, 0.f);
    int best_inst = -1;
    unsigned best_pb = 0u;
    const float3 inv = safe_inv(dir);

    int stack[TRAVERSAL_STACK];
    int sp = 0;
    int ni = 0;
    for (;;) {
        const float4* nq = reinterpret_cast<const float4*>(a.tlas + ni);
        const float4 nb0 = __ldg(nq), nb1 = __ldg(nq + 1);
        const int count = __float_as_int(nb1.w);
        float tn;
        bool visit = slab(nb0, nb1, pos, inv, tmin, best_t, tn);
        if (visit && count > 0) {
            const int first = __float_as_int(nb0.w);
            for (int k = 0; k < count; k++) {
                const int ii = __ldg(a.tlas_index + first + k);
                const InstDev d = load_inst(a.inst + ii);
                const float3 oo = d.is_identity ? pos : inst_point(d, pos);
                const float3 od = d.is_identity ? dir : inst_vector(d, dir);
                const float3 oinv = safe_inv(od);
                const int2 so = __ldg(reinterpret_cast<const int2*>(a.solid + d.solid));
                for (int k2 = 0; k2 < so.y; k2++) {
                    const float4* pq = reinterpret_cast<const float4*>(a.prim + so.x + k2);
                    const float4 pb0 = __ldg(pq), pb1 = __ldg(pq + 1);
                    float ptn;
                    if (!slab(pb0, pb1, oo, oinv, tmin, best_t, ptn)) continue;
                    float4 is;
                    if (!prim_hit<TREE>(is, a, __float_as_int(pb0.w), tmin, oo, od)) continue;
                    const unsigned key = ((unsigned)ii << 16) | (unsigned)k2;
                    if (is.w < best_t || (is.w == best_t && best_key != 0xffffffffu && key < best_key)) {
                        best_t = is.w; best_key = key; best_is = is; best_inst = ii;
                        best_pb = __float_as_uint(pb1.w);
                    }
                }
            }
        } else if (visit) {
            const int left = ni + 1, right = __float_as_int(nb0.w);
            if (sp < TRAVERSAL_STACK) stack[sp++] = right;
            ni = left;
            continue;
        }
        if (sp == 0) break;
        ni = stack[--sp];
    }

    if (best_inst < 0) {
        h.normal = f3(0.f, 0.f, 0.f);
        h.t = 1.f;
        h.lposcost = 0.f;
        h.lposfphi = 0.f;
        h.iindex_identity = 0xffffffffu;
        h.prim_boundary = 0xffffffffu;
        return;
    }
    const InstDev d = load_inst(a.inst + best_inst);
    float3 n = f3(best_is.x, best_is.y, best_is.z);
    float3 lpos;
    if (d.is_identity) {
        lpos = pos + best_is.w * dir;
    } else {
        n = inst_normal(d, n);
        lpos = inst_point(d, pos) + best_is.w * inst_vector(d, dir);
    }
    h.normal = n;
    h.t = best_is.w;
    h.lposcost = lpos.z / sqrtf(dot(lpos, lpos));
    h.lposfphi = 0.f;
    h.iindex_identity = ((d.iindex & 0xffffu) << 16) | (d.identity & 0xffffu);
    h.prim_boundary = best_pb;
}

}  // namespace gbo
