/*
 * orc_csg.c : CSG leaf and boolean-tree intersection, and the brute-force closest-hit trace of the oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Leaf functions restate CSG/csg_intersect_leaf_*.h operation by operation (binary32, same order):
 *   sphere          csg_intersect_leaf_sphere.h:14-55
 *   zsphere         csg_intersect_leaf_zsphere.h:44-151
 *   cylinder        csg_intersect_leaf_cylinder.h:33-82
 *   box3            csg_intersect_leaf_box3.h:63-155
 *   cone (newcone)  csg_intersect_leaf_newcone.h:38-121
 *   convexpolyhedron csg_intersect_leaf_convexpolyhedron.h:40-106
 *   hyperboloid     csg_intersect_leaf_hyperboloid.h:36-106
 *   halfspace       csg_intersect_leaf_halfspace.h
 *   phicut          csg_intersect_leaf_phicut.h:580-640 (intersect_leaf_phicut_simple)
 * with the node transform and complement handling of intersect_leaf (csg_intersect_leaf.h:174-325), the
 * robust quadratic roots of csg_robust_quadratic_roots.h:151-191, and the single-hit boolean tree of
 * intersect_tree (csg_intersect_tree.h:276-672) using the classification table of csg_classify.h:55-101.
 *
 * orc_trace replaces the OptiX IAS/GAS traversal (CSGOptiX/CSGOptiX7.cu:110-216, :749-940) by testing every
 * prim of every instance: the world ray is taken to the instance frame with the inverse instance
 * transform, the prim is intersected, the closest t wins (ties: lowest instance, then lowest prim), and the
 * object-frame normal is returned to the world frame with the inverse-transpose (what
 * optixTransformNormalFromObjectToWorldSpace does).
 */
#include <string.h>
#include "orc_internal.h"

#define RT_DEFAULT_MAX 1.e27f

/* ---- node accessors : CSG/CSGNode.h:324-341 ---- */
static inline unsigned nd_typecode(const gbo_csgnode* n) { return n->q3.u[2]; }
static inline unsigned nd_gtransform(const gbo_csgnode* n) { return n->q3.u[3] & 0x7fffffffu; }
static inline int nd_complement(const gbo_csgnode* n) { return (n->q3.u[3] & 0x80000000u) != 0; }
static inline unsigned nd_subnum(const gbo_csgnode* n) { return n->q0.u[0]; }

/* qat4 products : sysrap/sqat4.h:45-104 */
static inline v3 qat_right(const gbo_qat4* q, v3 v, float w)
{
    return V3(q->q0.f[0] * v.x + q->q1.f[0] * v.y + q->q2.f[0] * v.z + q->q3.f[0] * w,
              q->q0.f[1] * v.x + q->q1.f[1] * v.y + q->q2.f[1] * v.z + q->q3.f[1] * w,
              q->q0.f[2] * v.x + q->q1.f[2] * v.y + q->q2.f[2] * v.z + q->q3.f[2] * w);
}
static inline int qat_is_identity(const gbo_qat4* q)
{
    return q->q0.f[0] == 1.f && q->q0.f[1] == 0.f && q->q0.f[2] == 0.f &&
           q->q1.f[0] == 0.f && q->q1.f[1] == 1.f && q->q1.f[2] == 0.f &&
           q->q2.f[0] == 0.f && q->q2.f[1] == 0.f && q->q2.f[2] == 1.f &&
           q->q3.f[0] == 0.f && q->q3.f[1] == 0.f && q->q3.f[2] == 0.f;
}
static inline v3 qat_left(const gbo_qat4* q, v3 v, float w)
{
    return V3(q->q0.f[0] * v.x + q->q0.f[1] * v.y + q->q0.f[2] * v.z + q->q0.f[3] * w,
              q->q1.f[0] * v.x + q->q1.f[1] * v.y + q->q1.f[2] * v.z + q->q1.f[3] * w,
              q->q2.f[0] * v.x + q->q2.f[1] * v.y + q->q2.f[2] * v.z + q->q2.f[3] * w);
}

static void robust_roots(float* t1, float* t2, float* disc, float* sdisc, float d, float b, float c)
{
    *disc = b * b - d * c;
    *sdisc = *disc > 0.f ? sqrtf(*disc) : 0.f;
    float q = b > 0.f ? -(b + *sdisc) : -(b - *sdisc);
    float root1 = q / d;
    float root2 = c / q;
    *t1 = fminf(root1, root2);
    *t2 = fmaxf(root1, root2);
}

static void robust_roots_disq(float t_min, float* t1, float* t2, float* disc, float* sdisc, float d, float b, float c)
{
    *disc = b * b - d * c;
    *sdisc = *disc > 0.f ? sqrtf(*disc) : 0.f;
    float q = b > 0.f ? -(b + *sdisc) : -(b - *sdisc);
    float root1 = *sdisc > 0.f ? q / d : t_min;
    float root2 = *sdisc > 0.f ? c / q : t_min;
    *t1 = fminf(root1, root2);
    *t2 = fmaxf(root1, root2);
}

static int leaf_sphere(v4* is, const gbo_quad* q0, float t_min, v3 ro, v3 rd)
{
    v3 center = V3(q0->f[0], q0->f[1], q0->f[2]);
    float radius = q0->f[3];
    v3 O = vsub(ro, center);
    v3 D = rd;
    float b = vdot(O, D);
    float c = vdot(O, O) - radius * radius;
    float d = vdot(D, D);
    float root1, root2, disc, sdisc;
    robust_roots(&root1, &root2, &disc, &sdisc, d, b, c);
    float t_cand = sdisc > 0.f ? (root1 > t_min ? root1 : root2) : t_min;
    int valid = t_cand > t_min;
    if (valid) {
        is->x = (O.x + t_cand * D.x) / radius;
        is->y = (O.y + t_cand * D.y) / radius;
        is->z = (O.z + t_cand * D.z) / radius;
        is->w = t_cand;
    }
    return valid;
}

static int leaf_zsphere(v4* is, const gbo_quad* q0, const gbo_quad* q1, float t_min, v3 ro, v3 rd)
{
    v3 center = V3(q0->f[0], q0->f[1], q0->f[2]);
    v3 O = vsub(ro, center);
    v3 D = rd;
    float radius = q0->f[3];
    float b = vdot(O, D);
    float c = vdot(O, O) - radius * radius;
    if (c > 0.f && b > 0.f) return 0;
    float zmax = center.z + q1->f[1];
    float zmin = center.z + q1->f[0];
    float d = vdot(D, D);
    float t1sph, t2sph, disc, sdisc;
    robust_roots(&t1sph, &t2sph, &disc, &sdisc, d, b, c);
    float z1sph = ro.z + t1sph * rd.z;
    float z2sph = ro.z + t2sph * rd.z;
    float idz = 1.f / rd.z;
    float t_QCAP = (zmax - ro.z) * idz;
    float t_PCAP = (zmin - ro.z) * idz;
    float t1cap = fminf(t_QCAP, t_PCAP);
    float t2cap = fmaxf(t_QCAP, t_PCAP);
    if (t1cap < t1sph || t1cap > t2sph) t1cap = t_min;
    if (t2cap < t1sph || t2cap > t2sph) t2cap = t_min;
    float t_cand = t_min;
    if (sdisc > 0.f) {
        if (t1sph > t_min && z1sph > zmin && z1sph <= zmax) t_cand = t1sph;
        else if (t1cap > t_min) t_cand = t1cap;
        else if (t2cap > t_min) t_cand = t2cap;
        else if (t2sph > t_min && z2sph > zmin && z2sph <= zmax) t_cand = t2sph;
    }
    int valid = t_cand > t_min;
    if (valid) {
        is->w = t_cand;
        if (t_cand == t1sph || t_cand == t2sph) {
            is->x = (O.x + t_cand * D.x) / radius;
            is->y = (O.y + t_cand * D.y) / radius;
            is->z = (O.z + t_cand * D.z) / radius;
        } else {
            is->x = 0.f;
            is->y = 0.f;
            is->z = t_cand == t_PCAP ? -1.f : 1.f;
        }
    }
    return valid;
}

static int leaf_cylinder(v4* is, const gbo_quad* q0, const gbo_quad* q1, float t_min, v3 ro, v3 rd)
{
    const float r = q0->f[3];
    const float z1 = q1->f[0];
    const float z2 = q1->f[1];
    const float ox = ro.x, oy = ro.y, oz = ro.z;
    const float vx = rd.x, vy = rd.y, vz = rd.z;
    const float r2 = r * r;
    const float a = vx * vx + vy * vy;
    const float b = ox * vx + oy * vy;
    const float c = ox * ox + oy * oy - r2;
    float t_near, t_far, disc, sdisc;
    robust_roots_disq(t_min, &t_near, &t_far, &disc, &sdisc, a, b, c);
    float z_near = oz + t_near * vz;
    float z_far = oz + t_far * vz;
    const float t_z1cap = (z1 - oz) / vz;
    const float r2_z1cap = (ox + t_z1cap * vx) * (ox + t_z1cap * vx) + (oy + t_z1cap * vy) * (oy + t_z1cap * vy);
    const float t_z2cap = (z2 - oz) / vz;
    const float r2_z2cap = (ox + t_z2cap * vx) * (ox + t_z2cap * vx) + (oy + t_z2cap * vy) * (oy + t_z2cap * vy);
    float t_cand = INFINITY;
    if (t_near > t_min && z_near > z1 && z_near < z2 && t_near < t_cand) t_cand = t_near;
    if (t_far > t_min && z_far > z1 && z_far < z2 && t_far < t_cand) t_cand = t_far;
    if (t_z1cap > t_min && r2_z1cap <= r2 && t_z1cap < t_cand) t_cand = t_z1cap;
    if (t_z2cap > t_min && r2_z2cap <= r2 && t_z2cap < t_cand) t_cand = t_z2cap;
    int valid = t_cand > t_min && t_cand < INFINITY;
    if (valid) {
        int sheet = (t_cand == t_near || t_cand == t_far);
        is->x = sheet ? (ox + t_cand * vx) / r : 0.f;
        is->y = sheet ? (oy + t_cand * vy) / r : 0.f;
        is->z = sheet ? 0.f : (t_cand == t_z1cap ? -1.f : 1.f);
        is->w = t_cand;
    }
    return valid;
}

static int leaf_box3(v4* is, const gbo_quad* q0, float t_min, v3 ro, v3 rd)
{
    const v3 bmin = V3(-q0->f[0] / 2.f, -q0->f[1] / 2.f, -q0->f[2] / 2.f);
    const v3 bmax = V3(q0->f[0] / 2.f, q0->f[1] / 2.f, q0->f[2] / 2.f);
    v3 idir = V3(1.f / rd.x, 1.f / rd.y, 1.f / rd.z);
    v3 t0 = vmul(vsub(bmin, ro), idir);
    v3 t1 = vmul(vsub(bmax, ro), idir);
    v3 nr = V3(fminf(t0.x, t1.x), fminf(t0.y, t1.y), fminf(t0.z, t1.z));
    v3 fr = V3(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y), fmaxf(t0.z, t1.z));
    float t_near = fmaxf(fmaxf(nr.x, nr.y), nr.z);
    float t_far = fminf(fminf(fr.x, fr.y), fr.z);
    int along_x = rd.x != 0.f && rd.y == 0.f && rd.z == 0.f;
    int along_y = rd.x == 0.f && rd.y != 0.f && rd.z == 0.f;
    int along_z = rd.x == 0.f && rd.y == 0.f && rd.z != 0.f;
    int in_x = ro.x > bmin.x && ro.x < bmax.x;
    int in_y = ro.y > bmin.y && ro.y < bmax.y;
    int in_z = ro.z > bmin.z && ro.z < bmax.z;
    int has = 0;
    if (along_x) has = in_y && in_z;
    else if (along_y) has = in_x && in_z;
    else if (along_z) has = in_x && in_y;
    else has = (t_far > t_near && t_far > 0.f);
    int valid = 0;
    if (has) {
        float t_cand = t_min < t_near ? t_near : (t_min < t_far ? t_far : t_min);
        v3 p = vadd(ro, vscale(t_cand, rd));          /* bcen is the origin */
        v3 pa = V3(fabsf(p.x) / (bmax.x - bmin.x), fabsf(p.y) / (bmax.y - bmin.y), fabsf(p.z) / (bmax.z - bmin.z));
        v3 n = V3(0.f, 0.f, 0.f);
        if (pa.x >= pa.y && pa.x >= pa.z) n.x = copysignf(1.f, p.x);
        else if (pa.y >= pa.x && pa.y >= pa.z) n.y = copysignf(1.f, p.y);
        else if (pa.z >= pa.x && pa.z >= pa.y) n.z = copysignf(1.f, p.z);
        if (t_cand > t_min) {
            valid = 1;
            is->x = n.x; is->y = n.y; is->z = n.z; is->w = t_cand;
        }
    }
    return valid;
}

static inline float fmin4(float a, float b, float c, float d) { return fminf(fminf(a, b), fminf(c, d)); }

static int leaf_cone(v4* is, const gbo_quad* q0, float t_min, v3 o, v3 d)
{
    const float r1 = q0->f[0], z1 = q0->f[1], r2 = q0->f[2], z2 = q0->f[3];
    const float r1r1 = r1 * r1, r2r2 = r2 * r2;
    const float tth = (r2 - r1) / (z2 - z1);
    const float tth2 = tth * tth;
    const float z0 = (z2 * r1 - z1 * r2) / (r1 - r2);
    const float idz = 1.f / d.z;
    float t_cap1 = d.z == 0.f ? RT_DEFAULT_MAX : (z1 - o.z) * idz;
    float t_cap2 = d.z == 0.f ? RT_DEFAULT_MAX : (z2 - o.z) * idz;
    const float rr_cap1 = (o.x + t_cap1 * d.x) * (o.x + t_cap1 * d.x) + (o.y + t_cap1 * d.y) * (o.y + t_cap1 * d.y);
    const float rr_cap2 = (o.x + t_cap2 * d.x) * (o.x + t_cap2 * d.x) + (o.y + t_cap2 * d.y) * (o.y + t_cap2 * d.y);
    t_cap1 = rr_cap1 < r1r1 && t_cap1 > t_min ? t_cap1 : RT_DEFAULT_MAX;
    t_cap2 = rr_cap2 < r2r2 && t_cap2 > t_min ? t_cap2 : RT_DEFAULT_MAX;
    const float c2 = d.x * d.x + d.y * d.y - d.z * d.z * tth2;
    const float c1 = o.x * d.x + o.y * d.y - (o.z - z0) * d.z * tth2;
    const float c0 = o.x * o.x + o.y * o.y - (o.z - z0) * (o.z - z0) * tth2;
    float t_near, t_far, disc, sdisc;
    robust_roots_disq(RT_DEFAULT_MAX, &t_near, &t_far, &disc, &sdisc, c2, c1, c0);
    const float z_near = o.z + t_near * d.z;
    const float z_far = o.z + t_far * d.z;
    t_near = z_near > z1 && z_near < z2 && t_near > t_min ? t_near : RT_DEFAULT_MAX;
    t_far = z_far > z1 && z_far < z2 && t_far > t_min ? t_far : RT_DEFAULT_MAX;
    const float t_cand = fmin4(t_near, t_far, t_cap1, t_cap2);
    int valid = t_cand > t_min && t_cand < RT_DEFAULT_MAX;
    if (valid) {
        if (t_cand == t_cap1 || t_cand == t_cap2) {
            is->x = 0.f; is->y = 0.f; is->z = t_cand == t_cap2 ? 1.f : -1.f;
        } else {
            v3 n = vnormalize(V3(o.x + t_cand * d.x, o.y + t_cand * d.y, (z0 - (o.z + t_cand * d.z)) * tth2));
            is->x = n.x; is->y = n.y; is->z = n.z;
        }
        is->w = t_cand;
    }
    return valid;
}

static int leaf_convexpolyhedron(v4* is, const gbo_csgnode* node, const float* plan, float t_min, v3 ro, v3 rd)
{
    float t0 = -INFINITY, t1 = INFINITY;
    v3 t0n = V3(0.f, 0.f, 0.f), t1n = V3(0.f, 0.f, 0.f);
    unsigned planeIdx = node->q0.u[0], planeNum = node->q0.u[1];
    for (unsigned i = 0; i < planeNum; i++) {
        const float* pl = plan + 4 * (size_t)(planeIdx + i);
        v3 n = V3(pl[0], pl[1], pl[2]);
        float dplane = pl[3];
        float nd = vdot(n, rd);
        float no = vdot(n, ro);
        float dist = no - dplane;
        float t_cand = -dist / nd;
        int parallel_inside = nd == 0.f && dist < 0.f;
        int parallel_outside = nd == 0.f && dist > 0.f;
        if (parallel_inside) continue;
        if (parallel_outside) return 0;
        if (nd < 0.f) { if (t_cand > t0) { t0 = t_cand; t0n = n; } }
        else { if (t_cand < t1) { t1 = t_cand; t1n = n; } }
    }
    int valid = t0 < t1;
    if (valid) {
        if (t0 > t_min) { is->x = t0n.x; is->y = t0n.y; is->z = t0n.z; is->w = t0; }
        else if (t1 > t_min) { is->x = t1n.x; is->y = t1n.y; is->z = t1n.z; is->w = t1; }
    }
    return valid;
}

static int leaf_hyperboloid(v4* is, const gbo_quad* q0, float t_min, v3 ro, v3 rd)
{
    const float zero = 0.f, one = 1.f;
    const float r0 = q0->f[0], zf = q0->f[1], z1 = q0->f[2], z2 = q0->f[3];
    const float rr0 = r0 * r0;
    const float z1s = z1 / zf, z2s = z2 / zf;
    const float rr1 = rr0 * (z1s * z1s + one);
    const float rr2 = rr0 * (z2s * z2s + one);
    const float A = -rr0 / (zf * zf);
    const float B = -rr0;
    const float sx = rd.x, sy = rd.y, sz = rd.z, ox = ro.x, oy = ro.y, oz = ro.z;
    const float d = sx * sx + sy * sy + A * sz * sz;
    const float b = ox * sx + oy * sy + A * oz * sz;
    const float c = ox * ox + oy * oy + A * oz * oz + B;
    float t1hyp, t2hyp, disc, sdisc;
    robust_roots(&t1hyp, &t2hyp, &disc, &sdisc, d, b, c);
    const float h1z = oz + t1hyp * sz;
    const float h2z = oz + t2hyp * sz;
    float osz = one / sz;
    float t2cap = (z2 - oz) * osz;
    float t1cap = (z1 - oz) * osz;
    const v3 c1 = vadd(ro, vscale(t1cap, rd));
    const v3 c2 = vadd(ro, vscale(t2cap, rd));
    float crr1 = c1.x * c1.x + c1.y * c1.y;
    float crr2 = c2.x * c2.x + c2.y * c2.y;
    float ca = t1hyp > t_min && disc > zero && h1z > z1 && h1z < z2 ? t1hyp : RT_DEFAULT_MAX;
    float cb = t2hyp > t_min && disc > zero && h2z > z1 && h2z < z2 ? t2hyp : RT_DEFAULT_MAX;
    float cc = t2cap > t_min && crr2 < rr2 ? t2cap : RT_DEFAULT_MAX;
    float cd = t1cap > t_min && crr1 < rr1 ? t1cap : RT_DEFAULT_MAX;
    float t_cand = fmin4(ca, cb, cc, cd);
    int valid = t_cand > t_min && t_cand < RT_DEFAULT_MAX;
    if (valid) {
        is->w = t_cand;
        if (t_cand == t1hyp || t_cand == t2hyp) {
            const v3 p = vadd(ro, vscale(t_cand, rd));
            v3 n = vnormalize(V3(p.x, p.y, A * p.z));
            is->x = n.x; is->y = n.y; is->z = n.z;
        } else {
            is->x = zero; is->y = zero; is->z = t_cand == t1cap ? -one : one;
        }
    }
    return valid;
}

static int leaf_halfspace(v4* is, const gbo_quad* q0, float t_min, v3 o, v3 d)
{
    v3 n = V3(q0->f[0], q0->f[1], q0->f[2]);
    float w = q0->f[3];
    float on = vdot(o, n), dn = vdot(d, n);
    float on_w = on - w;
    float adn = fabsf(dn);
    int inside = on_w < -1e-9f;
    float t = adn > 0.f ? -on_w / dn : t_min;
    int valid = t > t_min;
    if (valid) { is->x = n.x; is->y = n.y; is->z = n.z; is->w = t; }
    else if (inside) is->y = -0.f;
    return valid;
}

static int leaf_phicut(v4* is, const gbo_quad* q0, float t_min, v3 o, v3 d)
{
    const float cosPhi0 = q0->f[0], sinPhi0 = q0->f[1], cosPhi1 = q0->f[2], sinPhi1 = q0->f[3];
    float d_n0 = d.x * sinPhi0 + d.y * (-cosPhi0);
    float d_n1 = d.x * (-sinPhi1) + d.y * (cosPhi1);
    float o_n0 = o.x * sinPhi0 + o.y * (-cosPhi0);
    float o_n1 = o.x * (-sinPhi1) + o.y * (cosPhi1);
    float t0 = d_n0 == 0.f ? t_min : -o_n0 / d_n0;
    float t1 = d_n1 == 0.f ? t_min : -o_n1 / d_n1;
    const float PR = d_n0 == 0.f ? -o_n0 : -d_n0;
    const float QR = d_n1 == 0.f ? -o_n1 : -d_n1;
    const float PQ = cosPhi0 * sinPhi1 - cosPhi1 * sinPhi0;
    int unbounded_exit = PQ >= 0.f ? (PR >= 0.f && QR <= 0.f) : (PR >= 0.f || QR <= 0.f);
    float side0 = o.x * cosPhi0 + o.y * sinPhi0 + (d.x * cosPhi0 + d.y * sinPhi0) * t0;
    float side1 = o.x * cosPhi1 + o.y * sinPhi1 + (d.x * cosPhi1 + d.y * sinPhi1) * t1;
    if (side0 < 0.f) t0 = t_min;
    if (side1 < 0.f) t1 = t_min;
    float t_near = fminf(t0, t1), t_far = fmaxf(t0, t1);
    float t_cand = t_near > t_min ? t_near : (t_far > t_min ? t_far : t_min);
    int valid = t_cand > t_min;
    if (valid) {
        is->x = t_cand == t1 ? -sinPhi1 : sinPhi0;
        is->y = t_cand == t1 ? cosPhi1 : -cosPhi0;
        is->z = 0.f;
        is->w = t_cand;
    } else if (unbounded_exit) {
        is->y = -is->y;
    }
    return valid;
}

/* intersect_leaf : csg_intersect_leaf.h:174-325 (non-HEISENBUG branch) */
static int intersect_leaf(v4* is, const gbo_csgnode* node, const float* plan, const gbo_qat4* itra,
                          float t_min, v3 ro, v3 rd)
{
    *is = V4(0.f, 0.f, 0.f, 0.f);
    unsigned typecode = nd_typecode(node);
    unsigned gt = nd_gtransform(node);
    int complement = nd_complement(node);
    const gbo_qat4* q = gt > 0 ? itra + gt - 1 : 0;
    v3 origin = q ? qat_right(q, ro, 1.f) : ro;
    v3 direction = q ? qat_right(q, rd, 0.f) : rd;
    int valid = 0;
    switch (typecode) {
        case GBO_CSG_SPHERE:   valid = leaf_sphere(is, &node->q0, t_min, origin, direction); break;
        case GBO_CSG_ZSPHERE:  valid = leaf_zsphere(is, &node->q0, &node->q1, t_min, origin, direction); break;
        case GBO_CSG_CYLINDER: valid = leaf_cylinder(is, &node->q0, &node->q1, t_min, origin, direction); break;
        case GBO_CSG_BOX3:     valid = leaf_box3(is, &node->q0, t_min, origin, direction); break;
        case GBO_CSG_CONE:     valid = leaf_cone(is, &node->q0, t_min, origin, direction); break;
        case GBO_CSG_CONVEXPOLYHEDRON: valid = leaf_convexpolyhedron(is, node, plan, t_min, origin, direction); break;
        case GBO_CSG_HYPERBOLOID: valid = leaf_hyperboloid(is, &node->q0, t_min, origin, direction); break;
        case GBO_CSG_PHICUT:   valid = leaf_phicut(is, &node->q0, t_min, origin, direction); break;
        case GBO_CSG_HALFSPACE: valid = leaf_halfspace(is, &node->q0, t_min, origin, direction); break;
        default: break;
    }
    if (valid && q) {
        v3 n = qat_left(q, V3(is->x, is->y, is->z), 0.f);
        is->x = n.x; is->y = n.y; is->z = n.z;
    }
    if (complement) {
        is->x = valid ? -is->x : -0.f;
        is->y = valid ? -is->y : is->y;
        is->z = valid ? -is->z : is->z;
    }
    return valid;
}

/* ---- boolean tree : csg_intersect_tree.h:276-672 ---- */

enum { CTRL_RETURN_MISS = 0, CTRL_RETURN_A = 1, CTRL_RETURN_B = 2, CTRL_RETURN_FLIP_B = 3, CTRL_LOOP_A = 4, CTRL_LOOP_B = 5 };
enum { ST_ENTER = 0, ST_EXIT = 1, ST_MISS = 2 };

/* packed boolean lookup tables : csg_classify.h:86-101 (4-bit actions indexed by 3*stateA+stateB, per op) */
static const unsigned LUT_ACLOSER[4] = { 0x22121141u, 0x00014014u, 0x00141141u, 0x00000000u };
static const unsigned LUT_BCLOSER[4] = { 0x22115122u, 0x00022055u, 0x00133155u, 0x00000000u };

static int lut_lookup(unsigned op, int sa, int sb, int acloser)
{
    const unsigned* lut = acloser ? LUT_ACLOSER : LUT_BCLOSER;
    unsigned offset = 3u * (unsigned)sa + (unsigned)sb;
    unsigned index = op - GBO_CSG_UNION;
    return offset < 8 ? (int)((lut[index] >> (offset * 4)) & 0xfu) : CTRL_RETURN_MISS;
}

static inline int classify(v4 ise, v3 dir, float tmin)
{
    return fabsf(ise.w) > tmin ? (ise.x * dir.x + ise.y * dir.y + ise.z * dir.z < 0.f ? ST_ENTER : ST_EXIT) : ST_MISS;
}

/* ---- list nodes : csg_intersect_node.h (compiled WITH_CONTIGUOUS in the reference's OptiX build) ----
 * A header node lists subNum (q0.u[0]) leaves at root + subOffset (q0.u[1]). */
#define LIST_EPSILON 0.0001f
#define LIST_MAX_ENTER 8      /* enter slots of intersect_node_contiguous */

/* intersect_node_contiguous : csg_intersect_node.h:390-626 */
static int list_contiguous(v4* isect, const gbo_csgnode* node, const gbo_csgnode* root, const float* plan,
                           const gbo_qat4* itra, float t_min, v3 ro, v3 rd)
{
    const int num_sub = (int)node->q0.u[0];
    const int offset_sub = (int)node->q0.u[1];
    v4 nearest_enter = V4(0.f, 0.f, 0.f, RT_DEFAULT_MAX);
    v4 farthest_exit = V4(0.f, 0.f, 0.f, t_min);
    v4 sub;
    int exit_count = 0;
    for (int i = 0; i < num_sub; i++) {                       /* zeroth pass: nearest enter, count exits */
        if (!intersect_leaf(&sub, root + offset_sub + i, plan, itra, t_min, ro, rd)) continue;
        int st = classify(sub, rd, t_min);
        if (st == ST_ENTER) { if (sub.w < nearest_enter.w) nearest_enter = sub; }
        else if (st == ST_EXIT) exit_count += 1;
    }
    if (exit_count == 0) {                                    /* outside the compound */
        int valid = nearest_enter.w > t_min && nearest_enter.w < RT_DEFAULT_MAX;
        if (valid) *isect = nearest_enter;
        return valid;
    }
    int enter_count = 0;
    float enter[LIST_MAX_ENTER];
    int which[LIST_MAX_ENTER], order[LIST_MAX_ENTER];
    for (int i = 0; i < num_sub; i++) {                       /* first pass: enters, farthest first exit */
        if (!intersect_leaf(&sub, root + offset_sub + i, plan, itra, t_min, ro, rd)) continue;
        int st = classify(sub, rd, t_min);
        if (st == ST_ENTER) {
            if (enter_count < LIST_MAX_ENTER) {
                which[enter_count] = i;
                order[enter_count] = enter_count;
                enter[enter_count] = sub.w;
                enter_count += 1;
            }
        } else if (st == ST_EXIT) {
            exit_count += 1;
            if (sub.w > farthest_exit.w) farthest_exit = sub;
        }
    }
    for (int i = 1; i < enter_count; i++) {                  /* enter slots by ascending distance */
        int key = order[i];
        int j = i - 1;
        while (j >= 0 && enter[order[j]] > enter[key]) { order[j + 1] = order[j]; j -= 1; }
        order[j + 1] = key;
    }
    for (int i = 0; i < enter_count; i++) {                   /* second pass: exits of contiguous enters */
        float t_adv = enter[order[i]] + LIST_EPSILON;
        if (!(t_adv < farthest_exit.w)) continue;
        if (!intersect_leaf(&sub, root + offset_sub + which[order[i]], plan, itra, t_adv, ro, rd)) continue;
        if (classify(sub, rd, t_adv) == ST_EXIT) {
            exit_count += 1;
            if (sub.w > farthest_exit.w) farthest_exit = sub;
        }
    }
    int valid = exit_count > 0 && farthest_exit.w > t_min;
    if (valid) *isect = farthest_exit;
    return valid;
}

/* intersect_node_discontiguous : csg_intersect_node.h:654-686 */
static int list_discontiguous(v4* isect, const gbo_csgnode* node, const gbo_csgnode* root, const float* plan,
                              const gbo_qat4* itra, float t_min, v3 ro, v3 rd)
{
    const int num_sub = (int)node->q0.u[0];
    const int offset_sub = (int)node->q0.u[1];
    v4 closest = V4(0.f, 0.f, 0.f, RT_DEFAULT_MAX);
    v4 sub;
    for (int i = 0; i < num_sub; i++)
        if (intersect_leaf(&sub, root + offset_sub + i, plan, itra, t_min, ro, rd) && sub.w < closest.w) closest = sub;
    int valid = closest.w < RT_DEFAULT_MAX;
    if (valid) *isect = closest;
    return valid;
}

/* intersect_node_overlap : csg_intersect_node.h:819-895 */
static int list_overlap(v4* isect, const gbo_csgnode* node, const gbo_csgnode* root, const float* plan,
                        const gbo_qat4* itra, float t_min, v3 ro, v3 rd)
{
    const unsigned num_sub = node->q0.u[0];
    const unsigned offset_sub = node->q0.u[1];
    v4 farthest_enter = V4(0.f, 0.f, 0.f, t_min);
    v4 nearest_exit = V4(0.f, 0.f, 0.f, RT_DEFAULT_MAX);
    v4 sub;
    unsigned enter_count = 0, exit_count = 0;
    for (unsigned i = 0; i < num_sub; i++) {
        const gbo_csgnode* leaf = root + offset_sub + i;
        if (!intersect_leaf(&sub, leaf, plan, itra, t_min, ro, rd)) continue;
        int st = classify(sub, rd, t_min);
        if (st == ST_ENTER) {
            enter_count += 1;
            if (sub.w > farthest_enter.w) farthest_enter = sub;
            float t_adv = sub.w + LIST_EPSILON;
            if (intersect_leaf(&sub, leaf, plan, itra, t_adv, ro, rd) && classify(sub, rd, t_adv) == ST_EXIT) {
                exit_count += 1;
                if (sub.w < nearest_exit.w) nearest_exit = sub;
            }
        } else if (st == ST_EXIT) {
            exit_count += 1;
            if (sub.w < nearest_exit.w) nearest_exit = sub;
        }
    }
    unsigned most = enter_count > exit_count ? enter_count : exit_count;
    if (!(farthest_enter.w < nearest_exit.w && most == num_sub)) return 0;
    if (farthest_enter.w > t_min && farthest_enter.w < RT_DEFAULT_MAX) { *isect = farthest_enter; return 1; }
    if (nearest_exit.w > t_min && nearest_exit.w < RT_DEFAULT_MAX) { *isect = nearest_exit; return 1; }
    return 0;
}

/* intersect_node : csg_intersect_node.h:913-938 */
static int intersect_node(v4* isect, const gbo_csgnode* node, const gbo_csgnode* root, const float* plan,
                          const gbo_qat4* itra, float t_min, v3 ro, v3 rd)
{
    switch (nd_typecode(node)) {
        case GBO_CSG_CONTIGUOUS:    return list_contiguous(isect, node, root, plan, itra, t_min, ro, rd);
        case GBO_CSG_OVERLAP:       return list_overlap(isect, node, root, plan, itra, t_min, ro, rd);
        case GBO_CSG_DISCONTIGUOUS: return list_discontiguous(isect, node, root, plan, itra, t_min, ro, rd);
        default:                    return intersect_leaf(isect, node, plan, itra, t_min, ro, rd);
    }
}

#define PACK4(a, b, c, d) ((((a) & 0xffu) << 0) | (((b) & 0xffu) << 8) | (((c) & 0xffu) << 16) | (((d) & 0xffu) << 24))
#define UNPACK4_2(p) (((p) >> 16) & 0xffu)
#define UNPACK4_3(p) (((p) >> 24) & 0xffu)
#define CSG_STACK_SIZE 15
#define TRANCHE_STACK_SIZE 4

static inline unsigned tree_depth(unsigned idx) { return 32u - (unsigned)__builtin_clz(idx) - 1u; }
static inline unsigned postorder_next(unsigned i, unsigned elev) { return (i & 1u) ? i >> 1 : (i << elev) + (1u << elev); }

static int intersect_tree(v4* isect, const gbo_csgnode* node, const float* plan, const gbo_qat4* itra,
                          float t_min, v3 ro, v3 rd)
{
    const int numNode = (int)nd_subnum(node);
    unsigned height = (unsigned)(__builtin_ffs(numNode + 1) - 2);
    const float propagate_epsilon = 0.0001f;
    int ierr = 0;

    float tr_tmin[TRANCHE_STACK_SIZE];
    unsigned tr_slice[TRANCHE_STACK_SIZE];
    int tr_curr = -1;

    v4 cdata[CSG_STACK_SIZE];
    int ccurr = -1;

#define TR_PUSH(sl, tm) do { if (tr_curr >= TRANCHE_STACK_SIZE - 1) { ierr = 1; } else { tr_curr++; tr_slice[tr_curr] = (sl); tr_tmin[tr_curr] = (tm); } } while (0)
#define CSG_PUSH(v, i) do { if (ccurr >= CSG_STACK_SIZE - 1) { ierr = 1; } else { ccurr++; cdata[ccurr] = (v); (void)(i); } } while (0)
#define CSG_POP0() do { if (ccurr < 0) { ierr = 1; } else { ccurr--; } } while (0)

    unsigned fullTree = PACK4(0u, 0u, 1u << height, 0u);
    TR_PUSH(fullTree, t_min);

    while (tr_curr > -1) {
        unsigned slice = tr_slice[tr_curr];
        float tmin = tr_tmin[tr_curr];
        tr_curr--;
        unsigned beginIdx = UNPACK4_2(slice);
        unsigned endIdx = UNPACK4_3(slice);
        unsigned nodeIdx = beginIdx;
        while (nodeIdx != endIdx) {
            unsigned depth = tree_depth(nodeIdx);
            unsigned elevation = height - depth;
            const gbo_csgnode* nd = node + nodeIdx - 1;
            unsigned typecode = nd_typecode(nd);
            if (typecode == GBO_CSG_ZERO) { nodeIdx = postorder_next(nodeIdx, elevation); continue; }
            int node_or_leaf = typecode >= GBO_CSG_NODE;
            if (node_or_leaf) {
                v4 nd_isect = V4(0.f, 0.f, 0.f, 0.f);
                intersect_node(&nd_isect, nd, node, plan, itra, tmin, ro, rd);
                nd_isect.w = copysignf(nd_isect.w, nodeIdx % 2 == 0 ? -1.f : 1.f);
                CSG_PUSH(nd_isect, nodeIdx);
                if (ierr) break;
            } else {
                if (ccurr < 1) { ierr = 1; break; }
                int firstLeft = signbit(cdata[ccurr].w) != 0;
                int secondLeft = signbit(cdata[ccurr - 1].w) != 0;
                if (!(firstLeft ^ secondLeft)) { ierr = 1; break; }
                int left = firstLeft ? ccurr : ccurr - 1;
                int right = firstLeft ? ccurr - 1 : ccurr;
                int l_state = classify(cdata[left], rd, tmin);
                int r_state = classify(cdata[right], rd, tmin);
                float t_left = fabsf(cdata[left].w);
                float t_right = fabsf(cdata[right].w);
                int leftIsCloser = t_left <= t_right;
                int l_complement = signbit(cdata[left].x) != 0;
                int r_complement = signbit(cdata[right].x) != 0;
                int l_unbounded = signbit(cdata[left].y) != 0;
                int r_unbounded = signbit(cdata[right].y) != 0;
                int l_promote_miss = l_state == ST_MISS && (l_complement || l_unbounded);
                int r_promote_miss = r_state == ST_MISS && (r_complement || r_unbounded);
                if (r_promote_miss) { r_state = ST_EXIT; leftIsCloser = 1; }
                if (l_promote_miss) { l_state = ST_EXIT; leftIsCloser = 0; }
                int ctrl = lut_lookup(typecode, l_state, r_state, leftIsCloser);
                int act_break = 0;
                if (ctrl < CTRL_LOOP_A) {
                    v4 result = ctrl == CTRL_RETURN_MISS ? V4(0.f, 0.f, 0.f, 0.f) : cdata[ctrl == CTRL_RETURN_A ? left : right];
                    if (ctrl == CTRL_RETURN_FLIP_B) { result.x = -result.x; result.y = -result.y; result.z = -result.z; }
                    result.w = copysignf(result.w, nodeIdx % 2 == 0 ? -1.f : 1.f);
                    CSG_POP0(); if (ierr) break;
                    CSG_POP0(); if (ierr) break;
                    CSG_PUSH(result, nodeIdx); if (ierr) break;
                } else {
                    int loopside = ctrl == CTRL_LOOP_A ? left : right;
                    int otherside = ctrl == CTRL_LOOP_A ? right : left;
                    unsigned leftIdx = 2u * nodeIdx;
                    unsigned rightIdx = leftIdx + 1u;
                    unsigned otherIdx = ctrl == CTRL_LOOP_A ? rightIdx : leftIdx;
                    float tminAdvanced = fabsf(cdata[loopside].w) + propagate_epsilon;
                    v4 other = cdata[otherside];
                    CSG_POP0(); if (ierr) break;
                    CSG_POP0(); if (ierr) break;
                    CSG_PUSH(other, otherIdx); if (ierr) break;
                    unsigned endTree = PACK4(0u, 0u, nodeIdx, endIdx);
                    unsigned leftTree = PACK4(0u, 0u, leftIdx << (elevation - 1), rightIdx << (elevation - 1));
                    unsigned rightTree = PACK4(0u, 0u, rightIdx << (elevation - 1), nodeIdx);
                    unsigned loopTree = ctrl == CTRL_LOOP_A ? leftTree : rightTree;
                    TR_PUSH(endTree, tmin); if (ierr) break;
                    TR_PUSH(loopTree, tminAdvanced); if (ierr) break;
                    act_break = 1;
                }
                if (act_break) break;
            }
            nodeIdx = postorder_next(nodeIdx, elevation);
        }
        if (ierr) break;
    }
    if (ccurr == 0) *isect = cdata[0];
    return isect->w > 0.f;
#undef TR_PUSH
#undef CSG_PUSH
#undef CSG_POP0
}

/* intersect_prim : csg_intersect_tree.h:683-719 (a list prim's header node is its own root) */
int orc_intersect_prim(v4* isect, const gbo_csgnode* node, const float* plan, const gbo_qat4* itra,
                       float t_min, v3 o, v3 d)
{
    unsigned typecode = nd_typecode(node);
    if (typecode >= GBO_CSG_LEAF) return intersect_leaf(isect, node, plan, itra, t_min, o, d);
    if (typecode < GBO_CSG_NODE) return intersect_tree(isect, node, plan, itra, t_min, o, d);
    return intersect_node(isect, node, node, plan, itra, t_min, o, d);
}

int orc_intersect_prim_c(const gbo_csgnode* node, const float* plan, const gbo_qat4* itra, float t_min,
                         const float* o, const float* d, float* isect)
{
    v4 is = V4(0.f, 0.f, 0.f, 0.f);
    int valid = orc_intersect_prim(&is, node, plan, itra, t_min, v3of(o), v3of(d));
    isect[0] = is.x; isect[1] = is.y; isect[2] = is.z; isect[3] = is.w;
    return valid;
}

/* ---- closest hit over all instances ---- */

static inline float normalize_cost(v3 v) { return v.z / sqrtf(vdot(v, v)); }
static inline float normalize_fphi(v3 v)
{
    /* sysrap/scuda.h normalize_fphi : phi/(2 pi) folded into [0,1) */
    float fphi = atan2f(v.y, v.x) / (2.f * ORC_PI_F);
    return fphi < 0.f ? fphi + 1.f : fphi;
}

void orc_trace(const orc_geom* g, v3 pos, v3 dir, float tmin, float tmax, gbo_prd* prd)
{
    float best_t = tmax;
    int best_inst = -1, best_prim = -1;
    v4 best_isect = V4(0.f, 0.f, 0.f, 0.f);
    v3 best_lpos = V3(0.f, 0.f, 0.f);
    for (int ii = 0; ii < g->num_inst; ii++) {
        const gbo_qat4* fwd = &g->inst[ii];
        const gbo_qat4* inv = &g->inst_inv[ii];
        int gas = fwd->q1.i[3];
        const gbo_csgsolid* so = &g->solid[gas];
        int ident = qat_is_identity(inv);
        v3 oo = ident ? pos : qat_right(inv, pos, 1.f);
        v3 od = ident ? dir : qat_right(inv, dir, 0.f);
        for (int k = 0; k < so->numPrim; k++) {
            int pi = so->primOffset + k;
            const gbo_csgprim* pr = &g->prim[pi];
            const gbo_csgnode* root = g->node + pr->q0.i[1];
            v4 is = V4(0.f, 0.f, 0.f, 0.f);
            int valid = orc_intersect_prim(&is, root, g->plan, g->itra, tmin, oo, od);
            /* OptiX accepts a reported hit only inside the ray's [tmin, tmax] interval (a convex polyhedron can
               report a valid t of 0 for a ray leaving it); strict: ties keep the lower (instance, prim) */
            if (valid && is.w >= tmin && is.w < best_t) {
                best_t = is.w; best_inst = ii; best_prim = pi; best_isect = is;
                best_lpos = vadd(oo, vscale(is.w, od));
            }
        }
    }
    memset(prd, 0, sizeof(*prd));
    if (best_inst < 0) {
        prd->q1.u[2] = 0xffffffffu;     /* __miss__ms */
        prd->q1.u[3] = 0xffffffffu;
        prd->q0.f[3] = 1.f;
        return;
    }
    const gbo_csgprim* pr = &g->prim[best_prim];
    const gbo_csgnode* root = g->node + pr->q0.i[1];
    unsigned boundary = root->q1.u[2];
    unsigned gpi = pr->q3.u[3];
    /* object -> world normal : transpose of the inverse instance transform */
    const gbo_qat4* inv = &g->inst_inv[best_inst];
    v3 n = V3(best_isect.x, best_isect.y, best_isect.z);
    if (!qat_is_identity(inv)) n = qat_left(inv, n, 0.f);
    prd->q0.f[0] = n.x; prd->q0.f[1] = n.y; prd->q0.f[2] = n.z; prd->q0.f[3] = best_isect.w;
    prd->q1.f[0] = normalize_cost(best_lpos);
    prd->q1.f[1] = normalize_fphi(best_lpos);
    unsigned identity = (unsigned)g->inst[best_inst].q2.i[3];   /* sensor_identifier+1, sqat4.h:367-372 */
    prd->q1.u[2] = (((unsigned)best_inst & 0xffffu) << 16) | (identity & 0xffffu);
    prd->q1.u[3] = ((gpi & 0xffffu) << 16) | (boundary & 0xffffu);
}

void orc_trace_c(const orc_geom* g, const float* pos, const float* dir, float tmin, float tmax, gbo_prd* prd)
{
    orc_trace(g, v3of(pos), v3of(dir), tmin, tmax, prd);
}

void orc_invert_transforms(const gbo_qat4* in, gbo_qat4* out, int n)
{
    /* affine inverse in double: rows q0..q2 hold the 3x3 (row-vector convention), q3 the translation */
    for (int k = 0; k < n; k++) {
        const gbo_qat4* q = &in[k];
        double m[3][3], t[3];
        m[0][0] = q->q0.f[0]; m[0][1] = q->q0.f[1]; m[0][2] = q->q0.f[2];
        m[1][0] = q->q1.f[0]; m[1][1] = q->q1.f[1]; m[1][2] = q->q1.f[2];
        m[2][0] = q->q2.f[0]; m[2][1] = q->q2.f[1]; m[2][2] = q->q2.f[2];
        t[0] = q->q3.f[0]; t[1] = q->q3.f[1]; t[2] = q->q3.f[2];
        double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1])
                   - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0])
                   + m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        double r[3][3];
        r[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / det;
        r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
        r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
        r[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / det;
        r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
        r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
        r[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / det;
        r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
        r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
        double it[3];
        for (int j = 0; j < 3; j++) it[j] = -(t[0] * r[0][j] + t[1] * r[1][j] + t[2] * r[2][j]);
        gbo_qat4* o = &out[k];
        memset(o, 0, sizeof(*o));
        for (int j = 0; j < 3; j++) {
            o->q0.f[j] = (float)r[0][j];
            o->q1.f[j] = (float)r[1][j];
            o->q2.f[j] = (float)r[2][j];
            o->q3.f[j] = (float)it[j];
        }
        o->q3.f[3] = 1.f;
    }
}
