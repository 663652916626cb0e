// gbo_trace.cuh : closest-hit ray query over the two-level acceleration structure.
//
// Replaces optixTrace + __intersection__is + __closesthit__ch of the reference (CSGOptiX/CSGOptiX7.cu:110-216,
// :749-940) with the same results:
//   * intersections with t in (tmin, tmax) via intersect_prim on the object-frame ray (the instance's inverse
//     transform applied to the world ray; t is shared between frames);
//   * the closest t wins; equal t resolve to the lowest (instance, prim) so that the result does not depend on
//     traversal order or on the instance hint;
//   * the object-frame normal goes to the world frame through the inverse-transpose
//     (optixTransformNormalFromObjectToWorldSpace); identity instances skip both transforms, and in the single-leaf
//     forms translated instances take the ray by one addition when that gives the transform's result bit for bit;
//   * iindex|identity and globalPrimIdx|boundary packed in 16-bit halves (CSGOptiX7.cu:753, :929);
//   * a miss returns boundary 0xffff (__miss__ms).
// Traversal: the instance the photon last hit (the hint) is intersected first, since photons mostly stay inside
// one solid.  If that hit keeps the whole segment inside the hint's box, only the instances whose boxes overlap
// that box can hold a closer hit, and their short precomputed list replaces the TLAS.  For a container whose list
// is too long, a segment inside its clear ball (entered by no other instance's box) meets no other instance at all.
// Otherwise the TLAS is walked front to back (while-while: descend inner nodes, then process leaves), with nodes
// that carry both child boxes, pruning boxes beyond the current best.  Every path tests every instance that could
// hold a hit at t <= the best, so the result is the same whichever path runs.
#pragma once
#include "gbo_csg.cuh"
#include "gbo_physics.cuh"
#include "gbo_accel.h"

namespace gbo {

struct Accel {
    const BvhNode2* tlas;
    const int32_t* tlas_index;
    const InstDev* inst;
    const PrimDev* prim;
    const SolidDev* solid;
    const gbo_csgnode* node;
    const float4* plan;
    const gbo_qat4* itra;
    const double* inst64;       // binary64 inverse columns, 12 per instance (precision mode only)
    const float4* inst_box;     // InstBox per instance (2 x float4): world box, overlap list range
    const float4* inner_box;    // InstBox per instance: the world box shrunk by the inside test's margin
    const int* overlap;         // overlap lists
    const float4* clear;        // per instance: ball (centre, r^2) that no other instance's box enters
};

// p inside the ball (c, r^2) by a relative margin far above the rounding of p
GBO_DEV bool inside_ball(float4 c, float3 p)
{
    const float dx = p.x - c.x, dy = p.y - c.y, dz = p.z - c.z;
    return dx * dx + dy * dy + dz * dz < c.w * 0.9999f;
}

// p inside an instance's box by a margin of ~30 binary32 ulp of the coordinates involved: far above the rounding of
// p and of pos + t dir, far below the boxes' padding (1e-5 x extent + 1e-3 mm), so photons sitting on a face of
// their instance's solid still pass.  The margin is folded into the instance's inner box on the host (its largest
// value over the box), so the test is six compares.
GBO_DEV bool inside_box(float4 lo, float4 hi, float3 p)
{
    return p.x > lo.x && p.x < hi.x && p.y > lo.y && p.y < hi.y && p.z > lo.z && p.z < hi.z;
}

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
    return f3(d.c0[0] * v.x + d.c0[1] * v.y + d.c0[2] * v.z + d.c0[3] * 1.f,
              d.c1[0] * v.x + d.c1[1] * v.y + d.c1[2] * v.z + d.c1[3] * 1.f,
              d.c2[0] * v.x + d.c2[1] * v.y + d.c2[2] * v.z + d.c2[3] * 1.f);
}
GBO_DEV float3 inst_vector(const InstDev& d, float3 v)
{
    return f3(d.c0[0] * v.x + d.c0[1] * v.y + d.c0[2] * v.z + d.c0[3] * 0.f,
              d.c1[0] * v.x + d.c1[1] * v.y + d.c1[2] * v.z + d.c1[3] * 0.f,
              d.c2[0] * v.x + d.c2[1] * v.y + d.c2[2] * v.z + d.c2[3] * 0.f);
}
GBO_DEV float3 inst_normal(const InstDev& d, float3 n)    // transpose of the inverse 3x3
{
    return f3(d.c0[0] * n.x + d.c1[0] * n.y + d.c2[0] * n.z,
              d.c0[1] * n.x + d.c1[1] * n.y + d.c2[1] * n.z,
              d.c0[2] * n.x + d.c1[2] * n.y + d.c2[2] * n.z);
}

// precision mode: the world -> object transform of the ray in binary64, rounded once to binary32
GBO_DEV void inst_ray64(const double* c, float3 p, float3 v, float3& op, float3& ov)
{
    const double2* q = reinterpret_cast<const double2*>(c);
    double r[12];
#pragma unroll
    for (int k = 0; k < 6; k++) { const double2 x = __ldg(q + k); r[2 * k] = x.x; r[2 * k + 1] = x.y; }
    const double px = p.x, py = p.y, pz = p.z, vx = v.x, vy = v.y, vz = v.z;
    op = f3((float)(r[0] * px + r[1] * py + r[2] * pz + r[3]), (float)(r[4] * px + r[5] * py + r[6] * pz + r[7]),
            (float)(r[8] * px + r[9] * py + r[10] * pz + r[11]));
    ov = f3((float)(r[0] * vx + r[1] * vy + r[2] * vz), (float)(r[4] * vx + r[5] * vy + r[6] * vz),
            (float)(r[8] * vx + r[9] * vy + r[10] * vz));
}

GBO_DEV InstDev load_inst(const InstDev* p)
{
    const float4* q = reinterpret_cast<const float4*>(p);
    InstDev d;
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    const int4 e = __ldg(reinterpret_cast<const int4*>(q + 3));
    d.c0[0] = a.x; d.c0[1] = a.y; d.c0[2] = a.z; d.c0[3] = a.w;
    d.c1[0] = b.x; d.c1[1] = b.y; d.c1[2] = b.z; d.c1[3] = b.w;
    d.c2[0] = c.x; d.c2[1] = c.y; d.c2[2] = c.z; d.c2[3] = c.w;
    d.solid = e.x; d.identity = (uint32_t)e.y; d.is_identity = e.z; d.iindex = (uint32_t)e.w;
    return d;
}

// TREE: 0 when every prim is a single leaf, 1 with boolean trees, 2 with CSG list nodes as well
// POLISH (precision mode): binary64 Newton polish of the quadric roots of sphere, zsphere and cylinder leaves
// d_inv (optional): the correctly rounded reciprocals of d's components, for a single box3 leaf to reuse
template <int TREE, bool POLISH>
GBO_DEV bool prim_hit(float4& is, const Accel& a, int node_word, float t_min, float3 o, float3 d,
                      const float3* d_inv = nullptr)
{
    const gbo_csgnode* root = a.node + (node_word & 0x3fffffff);
    if (TREE) {
        if (node_word & (1 << 30)) {                        // pure union tree: try the all-entering fast path
            const int r = intersect_union_enter(is, root, a.plan, a.itra, t_min, o, d, POLISH);
            if (r >= 0) return r == 1;
        }
        return intersect_prim<(TREE >= 2)>(is, root, a.plan, a.itra, t_min, o, d, POLISH);
    }
    if (node_typecode(root) >= GBO_CSG_LEAF)
        return intersect_leaf(is, root, a.plan, a.itra, t_min, o, d, POLISH, d_inv, true);
    is = make_float4(0.f, 0.f, 0.f, 0.f);
    return false;
}

struct Best {
    float t;
    unsigned key;
    float4 is;
    int inst;
    unsigned pb;
};

GBO_DEV bool no_zero(float3 v) { return v.x != 0.f && v.y != 0.f && v.z != 0.f; }

// Single-leaf forms share the world-frame reciprocal direction between the instance tests and the box tests of a
// query, and take translated instances by the shortcut below.  In the CSG-tree forms both cost more registers than
// they save (the wavefront walk pass ran 4 % slower on the 20,000-sensor sphere, whose sensors are rotated).
template <int TREE> struct InvShare { static constexpr bool on = TREE == 0; };

// the world-frame reciprocal direction `inv`, computed once per query by the first test that needs it
template <int TREE>
GBO_DEV void need_inv(float3& inv, bool& inv_ok, float3 dir)
{
    if (!InvShare<TREE>::on || !inv_ok) { inv = safe_inv(dir); inv_ok = true; }
}

template <int TREE, bool POLISH>
GBO_DEV void test_instance(const Accel& a, int ii, float3 pos, float3 dir, float tmin, Best& b, float3& inv,
                           bool& inv_ok)
{
    const InstDev d = load_inst(a.inst + ii);
    // an inverse that is a pure translation (rotation block 1 on the diagonal, +0 elsewhere; is_identity 2) maps a
    // ray with no zero coordinate to exactly pos + t and dir: the general transform's products by 1 and +0 are exact
    // and its sums of them add nothing, so this local ray and its reciprocal direction equal the general ones bit
    // for bit
    const bool shift = InvShare<TREE>::on && !POLISH && d.is_identity == 2 && no_zero(pos) && no_zero(dir);
    float3 oo, od, oinv;
    if (d.is_identity == 1 || shift) {
        oo = shift ? f3(pos.x + d.c0[3], pos.y + d.c1[3], pos.z + d.c2[3]) : pos;
        od = dir;
        if (InvShare<TREE>::on) {
            need_inv<TREE>(inv, inv_ok, dir);
            oinv = inv;
        } else {
            oinv = safe_inv(od);
        }
    } else {
        oo = inst_point(d, pos);
        od = inst_vector(d, dir);
        oinv = safe_inv(od);
    }
    // precision mode: the ray handed to the prims is transformed in binary64, once per instance and only when a
    // prim box is hit (the box test keeps the binary32 ray: boxes are padded far beyond its error)
    float3 po = oo, pd = od;
    bool have64 = !POLISH || d.is_identity == 1;
    const int2 so = __ldg(reinterpret_cast<const int2*>(a.solid + d.solid));
    for (int k2 = 0; k2 < so.y; k2++) {
        const float4* pq = reinterpret_cast<const float4*>(a.prim + so.x + k2);
        const float4 pb0 = __ldg(pq), pb1 = __ldg(pq + 1);
        float ptn;
        if (!slab(pb0, pb1, oo, oinv, tmin, b.t, ptn)) continue;
        float4 is;
        if (!have64) { inst_ray64(a.inst64 + 12 * (size_t)ii, pos, dir, po, pd); have64 = true; }
        // the prim-box reciprocals are those of the ray the leaf sees unless the precision mode re-transformed it
        if (!prim_hit<TREE, POLISH>(is, a, __float_as_int(pb0.w), tmin, po, pd, POLISH ? nullptr : &oinv)) continue;
        // OptiX accepts a reported hit only inside the ray's [tmin, tmax] interval: a convex polyhedron behind the
        // ray reports a valid t of 0 (csg_intersect_leaf_convexpolyhedron.h:87-104 writes no t when both planes
        // lie at or below t_min), also inside a tree or list (single-leaf prims check it in intersect_leaf)
        if (TREE && !(is.w >= tmin)) continue;
        const unsigned key = ((unsigned)ii << 16) | (unsigned)k2;
        if (is.w < b.t || (is.w == b.t && b.key != 0xffffffffu && key < b.key)) {
            b.t = is.w; b.key = key; b.is = is; b.inst = ii; b.pb = __float_as_uint(pb1.w);
        }
    }
}

constexpr int TRAVERSAL_STACK = TLAS_STACK_DEPTH;

constexpr int HINT_FIRST = 0x7fffff;     // leaf item standing for the photon's previous instance
constexpr int OVERLAP_FIRST = 0x7ffffe;  // leaf item standing for that instance's overlap list

// work items: an inner node index (>= 0), a leaf range encoded as -(1 + (first << 8 | count)), or ITEM_NONE
GBO_DEV int leaf_item(int first, int count) { return -(1 + ((first << 8) | count)); }
constexpr int ITEM_NONE = -0x7fffffff;

// next work item: the top of the stack, else the TLAS root when it is still pending, else none
GBO_DEV int pop_item(const int* stack, int& sp, bool& root_next)
{
    if (sp) return stack[--sp];
    const int item = root_next ? 0 : ITEM_NONE;
    root_next = false;
    return item;
}

enum { TRACE_DONE = 0, TRACE_WALK = 1 };

// The query's item loop, from the hint instance (or from the TLAS root when there is none), the best hit kept in
// `b` (set by trace_begin).  With stop_at_root the loop returns TRACE_WALK instead of entering the TLAS: the caller
// defers the query (the photon-pool kernel gathers the walks of several lanes of a warp so that they run together)
// and runs it again later without the stop; the result is that of one uninterrupted query.
template <int TREE, bool POLISH>
GBO_DEV int trace_items(const Accel& a, float3 pos, float3 dir, float tmin, int hint, bool stop_at_root, Best& b)
{
    // the world-frame reciprocal direction serves the TLAS and list-neighbour box tests, which a step that stays
    // inside its hint instance never reaches: computed on the way out of the hint item
    float3 inv = f3(0.f, 0.f, 0.f);
    int stack[TRAVERSAL_STACK];
    int sp = 0;
    constexpr int NONE = ITEM_NONE;
    int item = 0;
    int ov_first = 0;
    bool root_next = false;         // the TLAS root waits under the hint item (kept out of the local-memory stack)
    bool inv_ok = false;
    if (hint >= 0) {
        root_next = true;
        item = leaf_item(HINT_FIRST, 1);
    } else {
        if (stop_at_root) return TRACE_WALK;
        inv = safe_inv(dir);
        inv_ok = true;
    }
    // while-while traversal (Aila & Laine 2009): every lane first descends inner nodes until it holds a leaf, then
    // the lanes process their leaves together, so the expensive instance / CSG work runs with the warp converged;
    // each lane still visits its items in the same order as a one-item-per-iteration loop.  Leaf items are TLAS
    // leaves, the photon's previous instance (HINT_FIRST) or that instance's overlap list (OVERLAP_FIRST), all
    // tested at the single test_instance call site.
    while (item != NONE) {
        while (item >= 0) {
            const float4* nq = reinterpret_cast<const float4*>(a.tlas + item);
            const float4 l0 = __ldg(nq), h0 = __ldg(nq + 1), l1 = __ldg(nq + 2), h1 = __ldg(nq + 3);
            float t0, t1;
            const int c0 = __float_as_int(h0.w), c1 = __float_as_int(h1.w);
            const bool v0 = c0 >= 0 && slab(l0, h0, pos, inv, tmin, b.t, t0);
            const bool v1 = c1 >= 0 && slab(l1, h1, pos, inv, tmin, b.t, t1);
            const int it0 = c0 > 0 ? leaf_item(__float_as_int(l0.w), c0) : __float_as_int(l0.w);
            const int it1 = c1 > 0 ? leaf_item(__float_as_int(l1.w), c1) : __float_as_int(l1.w);
            if (v0 && v1) {                         // nearer child next, the other on the stack
                const bool near0 = t0 <= t1;
                item = near0 ? it0 : it1;
                if (sp < TRAVERSAL_STACK) stack[sp++] = near0 ? it1 : it0;
            } else if (v0) {
                item = it0;
            } else if (v1) {
                item = it1;
            } else {
                item = pop_item(stack, sp, root_next);
            }
        }
        while (item < 0 && item != NONE) {
            const int code = -item - 1;
            const int first = code >> 8, count = code & 0xff;
#pragma unroll 1
            for (int k = 0; k < count; k++) {
                const int ii = first == HINT_FIRST ? hint
                             : first == OVERLAP_FIRST ? __ldg(a.overlap + ov_first + k) : __ldg(a.tlas_index + first + k);
                if (first < OVERLAP_FIRST && ii == hint) continue;
                if (first == OVERLAP_FIRST || count > 1) {
                    // the instance's padded world box first: a list neighbour or a leaf sibling whose box the
                    // segment (tmin, best] misses holds no closer hit, and skips the transform and prim tests
                    const float4 wlo = __ldg(a.inst_box + 2 * ii), whi = __ldg(a.inst_box + 2 * ii + 1);
                    float tn;
                    if (!slab(wlo, whi, pos, inv, tmin, b.t, tn)) continue;
                }
                test_instance<TREE, POLISH>(a, ii, pos, dir, tmin, b, inv, inv_ok);
            }
            if (first == HINT_FIRST) {
                // when the previous instance's closest hit keeps the whole segment inside its box, only the instances
                // whose boxes overlap that box can hold a closer hit: their short list replaces the TLAS
                const float4 blo = __ldg(a.inner_box + 2 * hint), bhi = __ldg(a.inner_box + 2 * hint + 1);
                const int ocount = __float_as_int(bhi.w);
                const float3 e = pos + b.t * dir;
                if (ocount >= 0 && inside_box(blo, bhi, pos) && inside_box(blo, bhi, e)) {
                    ov_first = __float_as_int(blo.w);
                    sp = 0;
                    root_next = false;
                    item = NONE;
                    if (ocount > 0) {
                        item = leaf_item(OVERLAP_FIRST, ocount);
                        need_inv<TREE>(inv, inv_ok, dir);
                    }
                    continue;
                }
                // a container (long overlap list): a segment inside its clear ball meets no other instance
                if (ocount < 0) {
                    const float4 cb = __ldg(a.clear + hint);
                    if (cb.w > 0.f && inside_ball(cb, pos) && inside_ball(cb, e)) {
                        sp = 0;
                        root_next = false;
                        item = NONE;
                        continue;
                    }
                }
                if (stop_at_root) return TRACE_WALK;      // the TLAS walk, deferred by the caller
                need_inv<TREE>(inv, inv_ok, dir);     // the TLAS walk follows
            }
            item = pop_item(stack, sp, root_next);
        }
    }
    return TRACE_DONE;
}

GBO_DEV void trace_begin(Best& b, float tmax)
{
    b.t = tmax; b.key = 0xffffffffu; b.is = make_float4(0.f, 0.f, 0.f, 0.f); b.inst = -1; b.pb = 0u;
}

// The hit record of a finished query: closest-hit packing of CSGOptiX7.cu:749-847 (normal to the world frame,
// instance-frame z for the lpos sign, iindex|identity, globalPrimIdx|boundary) or the miss record.
GBO_DEV void trace_finish(const Accel& a, float3 pos, float3 dir, const Best& b, Hit& h)
{
    if (b.inst < 0) {
        h.normal = f3(0.f, 0.f, 0.f);
        h.t = 1.f;
        h.lposz = 0.f;
        h.iindex_identity = 0xffffffffu;
        h.prim_boundary = 0xffffffffu;
        return;
    }
    const InstDev d = load_inst(a.inst + b.inst);
    float3 n = f3(b.is.x, b.is.y, b.is.z);
    float lz;
    if (d.is_identity == 1) {
        lz = pos.z + b.is.w * dir.z;
    } else {
        n = inst_normal(d, n);
        lz = (d.c2[0] * pos.x + d.c2[1] * pos.y + d.c2[2] * pos.z + d.c2[3]) +
             b.is.w * (d.c2[0] * dir.x + d.c2[1] * dir.y + d.c2[2] * dir.z);
    }
    h.normal = n;
    h.t = b.is.w;
    h.lposz = lz;
    h.iindex_identity = ((d.iindex & 0xffffu) << 16) | (d.identity & 0xffffu);
    h.prim_boundary = b.pb;
}

template <int TREE, bool POLISH = false>
GBO_DEV void trace(const Accel& a, float3 pos, float3 dir, float tmin, float tmax, int hint, Hit& h)
{
    Best b;
    b.t = tmax; b.key = 0xffffffffu; b.is = make_float4(0.f, 0.f, 0.f, 0.f); b.inst = -1; b.pb = 0u;
    // the world-frame reciprocal direction serves the TLAS and list-neighbour box tests, which a step that stays
    // inside its hint instance never reaches: computed on the way out of the hint item
    float3 inv = f3(0.f, 0.f, 0.f);
    int stack[TRAVERSAL_STACK];
    int sp = 0;
    constexpr int NONE = ITEM_NONE;
    int item = 0;
    int ov_first = 0;
    bool root_next = false;         // the TLAS root waits under the hint item (kept out of the local-memory stack)
    bool inv_ok = hint < 0;
    if (hint >= 0) { root_next = true; item = leaf_item(HINT_FIRST, 1); }
    else inv = safe_inv(dir);
    // while-while traversal (Aila & Laine 2009): every lane first descends inner nodes until it holds a leaf, then
    // the lanes process their leaves together, so the expensive instance / CSG work runs with the warp converged;
    // each lane still visits its items in the same order as a one-item-per-iteration loop.  Leaf items are TLAS
    // leaves, the photon's previous instance (HINT_FIRST) or that instance's overlap list (OVERLAP_FIRST), all
    // tested at the single test_instance call site.
    while (item != NONE) {
        while (item >= 0) {
            const float4* nq = reinterpret_cast<const float4*>(a.tlas + item);
            const float4 l0 = __ldg(nq), h0 = __ldg(nq + 1), l1 = __ldg(nq + 2), h1 = __ldg(nq + 3);
            float t0, t1;
            const int c0 = __float_as_int(h0.w), c1 = __float_as_int(h1.w);
            const bool v0 = c0 >= 0 && slab(l0, h0, pos, inv, tmin, b.t, t0);
            const bool v1 = c1 >= 0 && slab(l1, h1, pos, inv, tmin, b.t, t1);
            const int it0 = c0 > 0 ? leaf_item(__float_as_int(l0.w), c0) : __float_as_int(l0.w);
            const int it1 = c1 > 0 ? leaf_item(__float_as_int(l1.w), c1) : __float_as_int(l1.w);
            if (v0 && v1) {                         // nearer child next, the other on the stack
                const bool near0 = t0 <= t1;
                item = near0 ? it0 : it1;
                if (sp < TRAVERSAL_STACK) stack[sp++] = near0 ? it1 : it0;
            } else if (v0) {
                item = it0;
            } else if (v1) {
                item = it1;
            } else {
                item = pop_item(stack, sp, root_next);
            }
        }
        while (item < 0 && item != NONE) {
            const int code = -item - 1;
            const int first = code >> 8, count = code & 0xff;
#pragma unroll 1
            for (int k = 0; k < count; k++) {
                const int ii = first == HINT_FIRST ? hint
                             : first == OVERLAP_FIRST ? __ldg(a.overlap + ov_first + k) : __ldg(a.tlas_index + first + k);
                if (first < OVERLAP_FIRST && ii == hint) continue;
                if (first == OVERLAP_FIRST || count > 1) {
                    // the instance's padded world box first: a list neighbour or a leaf sibling whose box the
                    // segment (tmin, best] misses holds no closer hit, and skips the transform and prim tests
                    const float4 wlo = __ldg(a.inst_box + 2 * ii), whi = __ldg(a.inst_box + 2 * ii + 1);
                    float tn;
                    if (!slab(wlo, whi, pos, inv, tmin, b.t, tn)) continue;
                }
                test_instance<TREE, POLISH>(a, ii, pos, dir, tmin, b, inv, inv_ok);
            }
            if (first == HINT_FIRST) {
                // when the previous instance's closest hit keeps the whole segment inside its box, only the instances
                // whose boxes overlap that box can hold a closer hit: their short list replaces the TLAS
                const float4 blo = __ldg(a.inner_box + 2 * hint), bhi = __ldg(a.inner_box + 2 * hint + 1);
                const int ocount = __float_as_int(bhi.w);
                const float3 e = pos + b.t * dir;
                if (ocount >= 0 && inside_box(blo, bhi, pos) && inside_box(blo, bhi, e)) {
                    ov_first = __float_as_int(blo.w);
                    sp = 0;
                    root_next = false;
                    item = NONE;
                    if (ocount > 0) {
                        item = leaf_item(OVERLAP_FIRST, ocount);
                        need_inv<TREE>(inv, inv_ok, dir);
                    }
                    continue;
                }
                // a container (long overlap list): a segment inside its clear ball meets no other instance
                if (ocount < 0) {
                    const float4 cb = __ldg(a.clear + hint);
                    if (cb.w > 0.f && inside_ball(cb, pos) && inside_ball(cb, e)) {
                        sp = 0;
                        root_next = false;
                        item = NONE;
                        continue;
                    }
                }
                need_inv<TREE>(inv, inv_ok, dir);     // the TLAS walk follows
            }
            item = pop_item(stack, sp, root_next);
        }
    }

    if (b.inst < 0) {
        h.normal = f3(0.f, 0.f, 0.f);
        h.t = 1.f;
        h.lposz = 0.f;
        h.iindex_identity = 0xffffffffu;
        h.prim_boundary = 0xffffffffu;
        return;
    }
    const InstDev d = load_inst(a.inst + b.inst);
    float3 n = f3(b.is.x, b.is.y, b.is.z);
    float lz;
    if (d.is_identity == 1) {
        lz = pos.z + b.is.w * dir.z;
    } else {
        n = inst_normal(d, n);
        lz = (d.c2[0] * pos.x + d.c2[1] * pos.y + d.c2[2] * pos.z + d.c2[3]) +
             b.is.w * (d.c2[0] * dir.x + d.c2[1] * dir.y + d.c2[2] * dir.z);
    }
    h.normal = n;
    h.t = b.is.w;
    h.lposz = lz;
    h.iindex_identity = ((d.iindex & 0xffffu) << 16) | (d.identity & 0xffffu);
    h.prim_boundary = b.pb;
}

}  // namespace gbo
