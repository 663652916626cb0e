// gbo_csg.cuh : CSG leaf and boolean-tree intersection on the device.
//
// The leaf functions and the single-hit boolean tree restate the reference's CSG code operation by operation,
// because a different but equally valid formula would move intersections by ulps and flip photon histories:
//   robust quadratic roots     CSG/csg_robust_quadratic_roots.h:151-191
//   sphere / zsphere / cylinder / box3 / cone / convexpolyhedron / hyperboloid / halfspace / phicut
//                              CSG/csg_intersect_leaf_*.h (see each function)
//   intersect_leaf             CSG/csg_intersect_leaf.h:174-325 (node transform, complement flags)
//   intersect_tree             CSG/csg_intersect_tree.h:276-672 (postorder tranches, LOOP_A/LOOP_B)
//   classification table       CSG/csg_classify.h:55-101
// Node records are read as float4 through the read-only path (CSGNode is 4 x float4 = 64 B).
#pragma once
#include "gbo_device.cuh"

namespace gbo {

// Leaf types the benchmark and test geometries use rarely stay out of line, to keep the traversal loop's code (and
// the instruction cache it needs) small; the common ones (sphere, zsphere, cylinder, box3) are inlined.
#define GBO_COLD static __device__ __noinline__

constexpr float RT_DEFAULT_MAX = 1.e27f;

struct NodeView {            // the parts of a CSGNode the intersectors read
    float4 q0;
    float2 q1;
    unsigned typecode, gtransform_complement;
};

GBO_DEV unsigned node_typecode(const gbo_csgnode* n) { return __ldg(&n->q3.u[2]); }
GBO_DEV NodeView load_node(const gbo_csgnode* n)
{
    const float4* q = reinterpret_cast<const float4*>(n);
    NodeView v;
    v.q0 = __ldg(q);
    float4 q1 = __ldg(q + 1);
    v.q1 = make_float2(q1.x, q1.y);
    uint4 q3 = __ldg(reinterpret_cast<const uint4*>(q + 3));
    v.typecode = q3.z;
    v.gtransform_complement = q3.w;
    return v;
}

struct Qat3x4 { float4 r0, r1, r2, r3; };   // qat4 rows (sysrap/sqat4.h)
GBO_DEV Qat3x4 load_qat(const gbo_qat4* q)
{
    const float4* p = reinterpret_cast<const float4*>(q);
    Qat3x4 m;
    m.r0 = __ldg(p); m.r1 = __ldg(p + 1); m.r2 = __ldg(p + 2); m.r3 = __ldg(p + 3);
    return m;
}
GBO_DEV float3 right_multiply(const Qat3x4& q, float3 v, float w)   // sqat4.h:45-52
{
    return f3(q.r0.x * v.x + q.r1.x * v.y + q.r2.x * v.z + q.r3.x * w,
              q.r0.y * v.x + q.r1.y * v.y + q.r2.y * v.z + q.r3.y * w,
              q.r0.z * v.x + q.r1.z * v.y + q.r2.z * v.z + q.r3.z * w);
}
GBO_DEV float3 left_multiply(const Qat3x4& q, float3 v, float w)    // sqat4.h:88-104
{
    return f3(q.r0.x * v.x + q.r0.y * v.y + q.r0.z * v.z + q.r0.w * w,
              q.r1.x * v.x + q.r1.y * v.y + q.r1.z * v.z + q.r1.w * w,
              q.r2.x * v.x + q.r2.y * v.y + q.r2.z * v.z + q.r2.w * w);
}

GBO_DEV void robust_roots(float& t1, float& t2, float& disc, float& sdisc, float d, float b, float c)
{
    disc = b * b - d * c;
    sdisc = disc > 0.f ? sqrtf(disc) : 0.f;
    const float q = b > 0.f ? -(b + sdisc) : -(b - sdisc);
    const float root1 = q / d;
    const float root2 = c / q;
    t1 = fminf(root1, root2);
    t2 = fmaxf(root1, root2);
}

// Precision mode: Newton polish in binary64 of a binary32 root of a t^2 + 2 b t + c = 0, the coefficients formed
// in binary64 from the binary32 ray.  The binary32 root loses accuracy both to the resolution of t and to the
// cancellation in c = |O|^2 - r^2 when the ray starts far from the quadric, so every accepted quadric root is
// polished.  Each Newton step evaluates the residual in binary64 and divides in binary32: the correction is a few
// ulp of t, so its own relative error of 2^-24 is immaterial, and binary64 division is slow on this part.  Two
// steps from the binary32 root.  The polished root replaces the binary32 one only when it is still above t_min:
// every root a leaf returns stays strictly above the t_min it was given, which is what makes the CSG tree's loop
// tranches advance and end.
GBO_DEV float polish_root(float t, float t_min, double a, double b, double c)
{
    double x = (double)t;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const double f = fma(fma(a, x, 2.0 * b), x, c);
        const float df = (float)(2.0 * fma(a, x, b));
        if (df != 0.f) x -= (double)((float)f / df);
    }
    const float r = (float)x;
    return r > t_min && r < __int_as_float(0x7f800000) ? r : t;
}

GBO_DEV void robust_roots_disq(float t_min, float& t1, float& t2, float& disc, float& sdisc, float d, float b, float c)
{
    disc = b * b - d * c;
    sdisc = disc > 0.f ? sqrtf(disc) : 0.f;
    const float q = b > 0.f ? -(b + sdisc) : -(b - sdisc);
    const float root1 = sdisc > 0.f ? q / d : t_min;
    const float root2 = sdisc > 0.f ? c / q : t_min;
    t1 = fminf(root1, root2);
    t2 = fmaxf(root1, root2);
}

// csg_intersect_leaf_sphere.h:14-55
GBO_DEV bool leaf_sphere(float4& is, float4 q0, float t_min, float3 ro, float3 rd, bool polish = false)
{
    const float3 center = f3(q0.x, q0.y, q0.z);
    const float radius = q0.w;
    const float3 O = ro - center;
    const float3 D = rd;
    const float b = dot(O, D);
    const float c = dot(O, O) - radius * radius;
    const float d = dot(D, D);
    float root1, root2, disc, sdisc;
    robust_roots(root1, root2, disc, sdisc, d, b, c);
    float t_cand = sdisc > 0.f ? (root1 > t_min ? root1 : root2) : t_min;
    if (polish && t_cand > t_min) {
        const double ox = (double)ro.x - q0.x, oy = (double)ro.y - q0.y, oz = (double)ro.z - q0.z;
        const double a2 = (double)rd.x * rd.x + (double)rd.y * rd.y + (double)rd.z * rd.z;
        const double b2 = ox * rd.x + oy * rd.y + oz * rd.z;
        const double c2 = ox * ox + oy * oy + oz * oz - (double)radius * radius;
        t_cand = polish_root(t_cand, t_min, a2, b2, c2);
    }
    const bool valid = t_cand > t_min;
    if (valid) {
        is.x = (O.x + t_cand * D.x) / radius;
        is.y = (O.y + t_cand * D.y) / radius;
        is.z = (O.z + t_cand * D.z) / radius;
        is.w = t_cand;
    }
    return valid;
}

// csg_intersect_leaf_zsphere.h:44-151
GBO_DEV bool leaf_zsphere(float4& is, float4 q0, float2 q1, float t_min, float3 ro, float3 rd, bool polish = false)
{
    const float3 center = f3(q0.x, q0.y, q0.z);
    const float3 O = ro - center;
    const float3 D = rd;
    const float radius = q0.w;
    const float b = dot(O, D);
    const float c = dot(O, O) - radius * radius;
    if (c > 0.f && b > 0.f) return false;
    const float zmax = center.z + q1.y;
    const float zmin = center.z + q1.x;
    const float d = dot(D, D);
    float t1sph, t2sph, disc, sdisc;
    robust_roots(t1sph, t2sph, disc, sdisc, d, b, c);
    const float z1sph = ro.z + t1sph * rd.z;
    const float z2sph = ro.z + t2sph * rd.z;
    const float idz = 1.f / rd.z;
    const float t_QCAP = (zmax - ro.z) * idz;
    const float t_PCAP = (zmin - ro.z) * idz;
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
    const bool valid = t_cand > t_min;
    if (valid) {
        is.w = t_cand;
        if (t_cand == t1sph || t_cand == t2sph) {
            if (polish) {
                const double ox = (double)ro.x - center.x, oy = (double)ro.y - center.y, oz = (double)ro.z - center.z;
                const double a2 = (double)rd.x * rd.x + (double)rd.y * rd.y + (double)rd.z * rd.z;
                const double b2 = ox * rd.x + oy * rd.y + oz * rd.z;
                const double c2 = ox * ox + oy * oy + oz * oz - (double)radius * radius;
                t_cand = polish_root(t_cand, t_min, a2, b2, c2);
                is.w = t_cand;
            }
            is.x = (O.x + t_cand * D.x) / radius;
            is.y = (O.y + t_cand * D.y) / radius;
            is.z = (O.z + t_cand * D.z) / radius;
        } else {
            is.x = 0.f;
            is.y = 0.f;
            is.z = t_cand == t_PCAP ? -1.f : 1.f;
        }
    }
    return valid;
}

// csg_intersect_leaf_cylinder.h:33-82
GBO_DEV bool leaf_cylinder(float4& is, float4 q0, float2 q1, float t_min, float3 ro, float3 rd, bool polish = false)
{
    const float r = q0.w, z1 = q1.x, z2 = q1.y;
    const float ox = ro.x, oy = ro.y, oz = ro.z;
    const float vx = rd.x, vy = rd.y, vz = rd.z;
    const float r2 = r * r;
    const float a = vx * vx + vy * vy;
    const float b = ox * vx + oy * vy;
    const float c = ox * ox + oy * oy - r2;
    float t_near, t_far, disc, sdisc;
    robust_roots_disq(t_min, t_near, t_far, disc, sdisc, a, b, c);
    const float z_near = oz + t_near * vz;
    const float z_far = oz + t_far * vz;
    const float t_z1cap = (z1 - oz) / vz;
    const float r2_z1cap = (ox + t_z1cap * vx) * (ox + t_z1cap * vx) + (oy + t_z1cap * vy) * (oy + t_z1cap * vy);
    const float t_z2cap = (z2 - oz) / vz;
    const float r2_z2cap = (ox + t_z2cap * vx) * (ox + t_z2cap * vx) + (oy + t_z2cap * vy) * (oy + t_z2cap * vy);
    float t_cand = __int_as_float(0x7f800000);
    if (t_near > t_min && z_near > z1 && z_near < z2 && t_near < t_cand) t_cand = t_near;
    if (t_far > t_min && z_far > z1 && z_far < z2 && t_far < t_cand) t_cand = t_far;
    if (t_z1cap > t_min && r2_z1cap <= r2 && t_z1cap < t_cand) t_cand = t_z1cap;
    if (t_z2cap > t_min && r2_z2cap <= r2 && t_z2cap < t_cand) t_cand = t_z2cap;
    const bool valid = t_cand > t_min && t_cand < __int_as_float(0x7f800000);
    if (valid) {
        const bool sheet = (t_cand == t_near || t_cand == t_far);
        if (sheet && polish) {
            const double a2 = (double)vx * vx + (double)vy * vy;
            const double b2 = (double)ox * vx + (double)oy * vy;
            const double c2 = (double)ox * ox + (double)oy * oy - (double)r * r;
            t_cand = polish_root(t_cand, t_min, a2, b2, c2);
        }
        is.x = sheet ? (ox + t_cand * vx) / r : 0.f;
        is.y = sheet ? (oy + t_cand * vy) / r : 0.f;
        is.z = sheet ? 0.f : (t_cand == t_z1cap ? -1.f : 1.f);
        is.w = t_cand;
    }
    return valid;
}

// csg_intersect_leaf_box3.h:63-155
// idir = (1/rd.x, 1/rd.y, 1/rd.z), correctly rounded; the caller may pass the reciprocals it already holds
GBO_DEV bool leaf_box3(float4& is, float4 q0, float t_min, float3 ro, float3 rd, float3 idir)
{
    const float3 bmin = f3(-q0.x / 2.f, -q0.y / 2.f, -q0.z / 2.f);
    const float3 bmax = f3(q0.x / 2.f, q0.y / 2.f, q0.z / 2.f);
    const float3 t0 = (bmin - ro) * idir;
    const float3 t1 = (bmax - ro) * idir;
    const float3 nr = fminf3(t0, t1);
    const float3 fr = fmaxf3(t0, t1);
    const float t_near = fmaxf(fmaxf(nr.x, nr.y), nr.z);
    const float t_far = fminf(fminf(fr.x, fr.y), fr.z);
    const bool along_x = rd.x != 0.f && rd.y == 0.f && rd.z == 0.f;
    const bool along_y = rd.x == 0.f && rd.y != 0.f && rd.z == 0.f;
    const bool along_z = rd.x == 0.f && rd.y == 0.f && rd.z != 0.f;
    const bool in_x = ro.x > bmin.x && ro.x < bmax.x;
    const bool in_y = ro.y > bmin.y && ro.y < bmax.y;
    const bool in_z = ro.z > bmin.z && ro.z < bmax.z;
    bool has;
    if (along_x) has = in_y && in_z;
    else if (along_y) has = in_x && in_z;
    else if (along_z) has = in_x && in_y;
    else has = (t_far > t_near && t_far > 0.f);
    bool valid = false;
    if (has) {
        const float t_cand = t_min < t_near ? t_near : (t_min < t_far ? t_far : t_min);
        const float3 p = ro + t_cand * rd;
        const float3 pa = f3(fabsf(p.x) / (bmax.x - bmin.x), fabsf(p.y) / (bmax.y - bmin.y), fabsf(p.z) / (bmax.z - bmin.z));
        float3 n = f3(0.f, 0.f, 0.f);
        if (pa.x >= pa.y && pa.x >= pa.z) n.x = copysignf(1.f, p.x);
        else if (pa.y >= pa.x && pa.y >= pa.z) n.y = copysignf(1.f, p.y);
        else if (pa.z >= pa.x && pa.z >= pa.y) n.z = copysignf(1.f, p.z);
        if (t_cand > t_min) {
            valid = true;
            is = make_float4(n.x, n.y, n.z, t_cand);
        }
    }
    return valid;
}

GBO_DEV float fmin4(float a, float b, float c, float d) { return fminf(fminf(a, b), fminf(c, d)); }

// csg_intersect_leaf_newcone.h:38-121
GBO_COLD bool leaf_cone(float4& is, float4 q0, float t_min, float3 o, float3 d)
{
    const float r1 = q0.x, z1 = q0.y, r2 = q0.z, z2 = q0.w;
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
    robust_roots_disq(RT_DEFAULT_MAX, t_near, t_far, disc, sdisc, c2, c1, c0);
    const float z_near = o.z + t_near * d.z;
    const float z_far = o.z + t_far * d.z;
    t_near = z_near > z1 && z_near < z2 && t_near > t_min ? t_near : RT_DEFAULT_MAX;
    t_far = z_far > z1 && z_far < z2 && t_far > t_min ? t_far : RT_DEFAULT_MAX;
    const float t_cand = fmin4(t_near, t_far, t_cap1, t_cap2);
    const bool valid = t_cand > t_min && t_cand < RT_DEFAULT_MAX;
    if (valid) {
        if (t_cand == t_cap1 || t_cand == t_cap2) {
            is.x = 0.f; is.y = 0.f; is.z = t_cand == t_cap2 ? 1.f : -1.f;
        } else {
            const float3 n = normalize(f3(o.x + t_cand * d.x, o.y + t_cand * d.y, (z0 - (o.z + t_cand * d.z)) * tth2));
            is.x = n.x; is.y = n.y; is.z = n.z;
        }
        is.w = t_cand;
    }
    return valid;
}

// csg_intersect_leaf_convexpolyhedron.h:40-106
GBO_COLD bool leaf_convexpolyhedron(float4& is, float4 q0, const float4* plan, float t_min, float3 ro, float3 rd)
{
    float t0 = -__int_as_float(0x7f800000), t1 = __int_as_float(0x7f800000);
    float3 t0n = f3(0.f, 0.f, 0.f), t1n = f3(0.f, 0.f, 0.f);
    const unsigned planeIdx = __float_as_uint(q0.x), planeNum = __float_as_uint(q0.y);
    for (unsigned i = 0; i < planeNum; i++) {
        const float4 pl = __ldg(plan + planeIdx + i);
        const float3 n = f3(pl.x, pl.y, pl.z);
        const float nd = dot(n, rd);
        const float no = dot(n, ro);
        const float dist = no - pl.w;
        const float t_cand = -dist / nd;
        const bool parallel_inside = nd == 0.f && dist < 0.f;
        const bool parallel_outside = nd == 0.f && dist > 0.f;
        if (parallel_inside) continue;
        if (parallel_outside) return false;
        if (nd < 0.f) { if (t_cand > t0) { t0 = t_cand; t0n = n; } }
        else { if (t_cand < t1) { t1 = t_cand; t1n = n; } }
    }
    const bool valid = t0 < t1;
    if (valid) {
        if (t0 > t_min) is = make_float4(t0n.x, t0n.y, t0n.z, t0);
        else if (t1 > t_min) is = make_float4(t1n.x, t1n.y, t1n.z, t1);
    }
    return valid;
}

// csg_intersect_leaf_hyperboloid.h:36-106
GBO_COLD bool leaf_hyperboloid(float4& is, float4 q0, float t_min, float3 ro, float3 rd)
{
    const float zero = 0.f, one = 1.f;
    const float r0 = q0.x, zf = q0.y, z1 = q0.z, z2 = q0.w;
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
    robust_roots(t1hyp, t2hyp, disc, sdisc, d, b, c);
    const float h1z = oz + t1hyp * sz;
    const float h2z = oz + t2hyp * sz;
    const float osz = one / sz;
    const float t2cap = (z2 - oz) * osz;
    const float t1cap = (z1 - oz) * osz;
    const float3 c1 = ro + t1cap * rd;
    const float3 c2 = ro + t2cap * rd;
    const float crr1 = c1.x * c1.x + c1.y * c1.y;
    const float crr2 = c2.x * c2.x + c2.y * c2.y;
    const float ca = t1hyp > t_min && disc > zero && h1z > z1 && h1z < z2 ? t1hyp : RT_DEFAULT_MAX;
    const float cb = t2hyp > t_min && disc > zero && h2z > z1 && h2z < z2 ? t2hyp : RT_DEFAULT_MAX;
    const float cc = t2cap > t_min && crr2 < rr2 ? t2cap : RT_DEFAULT_MAX;
    const float cd = t1cap > t_min && crr1 < rr1 ? t1cap : RT_DEFAULT_MAX;
    const float t_cand = fmin4(ca, cb, cc, cd);
    const bool valid = t_cand > t_min && t_cand < RT_DEFAULT_MAX;
    if (valid) {
        is.w = t_cand;
        if (t_cand == t1hyp || t_cand == t2hyp) {
            const float3 p = ro + t_cand * rd;
            const float3 n = normalize(f3(p.x, p.y, A * p.z));
            is.x = n.x; is.y = n.y; is.z = n.z;
        } else {
            is.x = zero; is.y = zero; is.z = t_cand == t1cap ? -one : one;
        }
    }
    return valid;
}

// csg_intersect_leaf_halfspace.h
GBO_COLD bool leaf_halfspace(float4& is, float4 q0, float t_min, float3 o, float3 d)
{
    const float3 n = f3(q0.x, q0.y, q0.z);
    const float on = dot(o, n), dn = dot(d, n);
    const float on_w = on - q0.w;
    const float adn = fabsf(dn);
    const bool inside = on_w < -1e-9f;
    const float t = adn > 0.f ? -on_w / dn : t_min;
    const bool valid = t > t_min;
    if (valid) is = make_float4(n.x, n.y, n.z, t);
    else if (inside) is.y = -0.f;
    return valid;
}

// csg_intersect_leaf_phicut.h:580-640
GBO_COLD bool leaf_phicut(float4& is, float4 q0, float t_min, float3 o, float3 d)
{
    const float cosPhi0 = q0.x, sinPhi0 = q0.y, cosPhi1 = q0.z, sinPhi1 = q0.w;
    const float d_n0 = d.x * sinPhi0 + d.y * (-cosPhi0);
    const float d_n1 = d.x * (-sinPhi1) + d.y * (cosPhi1);
    const float o_n0 = o.x * sinPhi0 + o.y * (-cosPhi0);
    const float o_n1 = o.x * (-sinPhi1) + o.y * (cosPhi1);
    float t0 = d_n0 == 0.f ? t_min : -o_n0 / d_n0;
    float t1 = d_n1 == 0.f ? t_min : -o_n1 / d_n1;
    const float PR = d_n0 == 0.f ? -o_n0 : -d_n0;
    const float QR = d_n1 == 0.f ? -o_n1 : -d_n1;
    const float PQ = cosPhi0 * sinPhi1 - cosPhi1 * sinPhi0;
    const bool unbounded_exit = PQ >= 0.f ? (PR >= 0.f && QR <= 0.f) : (PR >= 0.f || QR <= 0.f);
    const float side0 = o.x * cosPhi0 + o.y * sinPhi0 + (d.x * cosPhi0 + d.y * sinPhi0) * t0;
    const float side1 = o.x * cosPhi1 + o.y * sinPhi1 + (d.x * cosPhi1 + d.y * sinPhi1) * t1;
    if (side0 < 0.f) t0 = t_min;
    if (side1 < 0.f) t1 = t_min;
    const float t_near = fminf(t0, t1), t_far = fmaxf(t0, t1);
    const float t_cand = t_near > t_min ? t_near : (t_far > t_min ? t_far : t_min);
    const bool valid = t_cand > t_min;
    if (valid) {
        is.x = t_cand == t1 ? -sinPhi1 : sinPhi0;
        is.y = t_cand == t1 ? cosPhi1 : -cosPhi0;
        is.z = 0.f;
        is.w = t_cand;
    } else if (unbounded_exit) {
        is.y = -is.y;
    }
    return valid;
}

// csg_intersect_leaf.h:174-325
// rd_inv (optional): the correctly rounded reciprocals of rd's components, reused by an untransformed box3
// whole_prim: the leaf is a prim by itself, whose hit OptiX accepts only inside the ray's [tmin, tmax] interval.  Of
// the leaves only a convex polyhedron reports a valid hit below t_min (t = 0 when both its planes lie at or below
// t_min: csg_intersect_leaf_convexpolyhedron.h:87-104 writes no t), so the check sits on its out-of-line path.
GBO_DEV bool intersect_leaf(float4& is, const gbo_csgnode* node, const float4* plan, const gbo_qat4* itra,
                            float t_min, float3 ro, float3 rd, bool polish = false, const float3* rd_inv = nullptr,
                            bool whole_prim = false)
{
    is = make_float4(0.f, 0.f, 0.f, 0.f);
    const NodeView nd = load_node(node);
    const unsigned gt = nd.gtransform_complement & 0x7fffffffu;
    const bool complement = (nd.gtransform_complement & 0x80000000u) != 0u;
    Qat3x4 q;
    float3 origin = ro, direction = rd;
    if (gt > 0) {
        q = load_qat(itra + gt - 1);
        origin = right_multiply(q, ro, 1.f);
        direction = right_multiply(q, rd, 0.f);
    }
    bool valid = false;
    switch (nd.typecode) {
        case GBO_CSG_SPHERE:           valid = leaf_sphere(is, nd.q0, t_min, origin, direction, polish); break;
        case GBO_CSG_ZSPHERE:          valid = leaf_zsphere(is, nd.q0, nd.q1, t_min, origin, direction, polish); break;
        case GBO_CSG_CYLINDER:         valid = leaf_cylinder(is, nd.q0, nd.q1, t_min, origin, direction, polish); break;
        case GBO_CSG_BOX3:
            valid = leaf_box3(is, nd.q0, t_min, origin, direction,
                              gt == 0 && rd_inv ? *rd_inv
                                                : f3(1.f / direction.x, 1.f / direction.y, 1.f / direction.z));
            break;
        // the out-of-line leaves write a copy: `is` itself never has its address taken, so it stays in registers
        // on the other paths
        case GBO_CSG_CONE:             { float4 c = is; valid = leaf_cone(c, nd.q0, t_min, origin, direction); is = c; } break;
        case GBO_CSG_CONVEXPOLYHEDRON: {
            float4 c = is;
            valid = leaf_convexpolyhedron(c, nd.q0, plan, t_min, origin, direction) && (!whole_prim || c.w >= t_min);
            is = c;
        } break;
        case GBO_CSG_HYPERBOLOID:      { float4 c = is; valid = leaf_hyperboloid(c, nd.q0, t_min, origin, direction); is = c; } break;
        case GBO_CSG_PHICUT:           { float4 c = is; valid = leaf_phicut(c, nd.q0, t_min, origin, direction); is = c; } break;
        case GBO_CSG_HALFSPACE:        { float4 c = is; valid = leaf_halfspace(c, nd.q0, t_min, origin, direction); is = c; } break;
        default: break;
    }
    if (valid && gt > 0) {
        const float3 n = left_multiply(q, f3(is.x, is.y, is.z), 0.f);
        is.x = n.x; is.y = n.y; is.z = n.z;
    }
    if (complement) {
        is.x = valid ? -is.x : -0.f;
        is.y = valid ? -is.y : is.y;
        is.z = valid ? -is.z : is.z;
    }
    return valid;
}

// ---- boolean tree : csg_intersect_tree.h:276-672 -------------------------------------------------------------
enum { CTRL_RETURN_MISS = 0, CTRL_RETURN_A = 1, CTRL_RETURN_B = 2, CTRL_RETURN_FLIP_B = 3, CTRL_LOOP_A = 4, CTRL_LOOP_B = 5 };
enum { ST_ENTER = 0, ST_EXIT = 1, ST_MISS = 2 };

// CSG_CLASSIFY, csg_classify.h:55: enter, exit or miss of a hit at |t| against the ray direction
GBO_DEV int classify(float4 ise, float3 dir, float tmin)
{
    return fabsf(ise.w) > tmin ? (ise.x * dir.x + ise.y * dir.y + ise.z * dir.z < 0.f ? ST_ENTER : ST_EXIT) : ST_MISS;
}

// ---- list nodes : csg_intersect_node.h (the reference's OptiX build defines WITH_CONTIGUOUS) --------------------
// A list header node holds subNum (q0.u.x) leaves starting subOffset (q0.u.y) nodes after the prim's root; the
// leaves carry their own transforms.  Geometry creation checks that every sub is a leaf inside its prim.
constexpr float LIST_EPSILON = 0.0001f;      // propagate_epsilon of csg_intersect_node.h
constexpr int LIST_MAX_ENTER = 8;            // enter slots of intersect_node_contiguous (its arrays hold 8)

// CSG_CONTIGUOUS, csg_intersect_node.h:390-626: a multi-union whose leaves overlap into one connected shape.  A
// ray whose first hits all enter starts outside: the nearest enter is the answer.  Otherwise it starts inside:
// the exit is the farthest first-exit, extended by the exits of the leaves it enters before reaching that exit,
// taken in order of their enter distances (a leaf entered beyond the current exit is disjoint and skipped).
GBO_DEV bool list_contiguous(float4& isect, const gbo_csgnode* node, const gbo_csgnode* root, const float4* plan,
                              const gbo_qat4* itra, float t_min, float3 ro, float3 rd)
{
    const int num_sub = (int)__ldg(&node->q0.u[0]);
    const int offset_sub = (int)__ldg(&node->q0.u[1]);
    float4 nearest_enter = make_float4(0.f, 0.f, 0.f, RT_DEFAULT_MAX);
    float4 farthest_exit = make_float4(0.f, 0.f, 0.f, t_min);
    float4 sub;
    int exit_count = 0;
    for (int i = 0; i < num_sub; i++) {
        if (!intersect_leaf(sub, root + offset_sub + i, plan, itra, t_min, ro, rd)) continue;
        const int st = classify(sub, rd, t_min);
        if (st == ST_ENTER) { if (sub.w < nearest_enter.w) nearest_enter = sub; }
        else if (st == ST_EXIT) exit_count += 1;
    }
    if (exit_count == 0) {
        const bool valid = nearest_enter.w > t_min && nearest_enter.w < RT_DEFAULT_MAX;
        if (valid) isect = nearest_enter;
        return valid;
    }
    int enter_count = 0;
    float enter[LIST_MAX_ENTER];
    int which[LIST_MAX_ENTER], order[LIST_MAX_ENTER];
    for (int i = 0; i < num_sub; i++) {
        if (!intersect_leaf(sub, root + offset_sub + i, plan, itra, t_min, ro, rd)) continue;
        const int st = classify(sub, rd, t_min);
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
    // enter slots in ascending enter distance (a stable insertion sort of the slot indices)
    for (int i = 1; i < enter_count; i++) {
        const int key = order[i];
        int j = i - 1;
        while (j >= 0 && enter[order[j]] > enter[key]) { order[j + 1] = order[j]; j -= 1; }
        order[j + 1] = key;
    }
    for (int i = 0; i < enter_count; i++) {
        const float t_adv = enter[order[i]] + LIST_EPSILON;
        if (!(t_adv < farthest_exit.w)) continue;
        if (!intersect_leaf(sub, root + offset_sub + which[order[i]], plan, itra, t_adv, ro, rd)) continue;
        if (classify(sub, rd, t_adv) == ST_EXIT) {
            exit_count += 1;
            if (sub.w > farthest_exit.w) farthest_exit = sub;
        }
    }
    const bool valid = exit_count > 0 && farthest_exit.w > t_min;
    if (valid) isect = farthest_exit;
    return valid;
}

// CSG_DISCONTIGUOUS, csg_intersect_node.h:654-686: leaves that never overlap; the nearest leaf hit is the answer.
GBO_DEV bool list_discontiguous(float4& isect, const gbo_csgnode* node, const gbo_csgnode* root, const float4* plan,
                                 const gbo_qat4* itra, float t_min, float3 ro, float3 rd)
{
    const int num_sub = (int)__ldg(&node->q0.u[0]);
    const int offset_sub = (int)__ldg(&node->q0.u[1]);
    float4 closest = make_float4(0.f, 0.f, 0.f, RT_DEFAULT_MAX);
    float4 sub;
    for (int i = 0; i < num_sub; i++)
        if (intersect_leaf(sub, root + offset_sub + i, plan, itra, t_min, ro, rd) && sub.w < closest.w) closest = sub;
    const bool valid = closest.w < RT_DEFAULT_MAX;
    if (valid) isect = closest;
    return valid;
}

// CSG_OVERLAP, csg_intersect_node.h:819-895: a multi-intersection shaped like a ball.  Each leaf contributes its
// enter (and the exit after it) or its exit; the shape is hit when every leaf was met and the farthest enter lies
// before the nearest exit: that enter from outside, else the exit from inside.
GBO_DEV bool list_overlap(float4& isect, const gbo_csgnode* node, const gbo_csgnode* root, const float4* plan,
                           const gbo_qat4* itra, float t_min, float3 ro, float3 rd)
{
    const unsigned num_sub = __ldg(&node->q0.u[0]);
    const unsigned offset_sub = __ldg(&node->q0.u[1]);
    float4 farthest_enter = make_float4(0.f, 0.f, 0.f, t_min);
    float4 nearest_exit = make_float4(0.f, 0.f, 0.f, RT_DEFAULT_MAX);
    float4 sub;
    unsigned enter_count = 0, exit_count = 0;
    for (unsigned i = 0; i < num_sub; i++) {
        const gbo_csgnode* leaf = root + offset_sub + i;
        if (!intersect_leaf(sub, leaf, plan, itra, t_min, ro, rd)) continue;
        const int st = classify(sub, rd, t_min);
        if (st == ST_ENTER) {
            enter_count += 1;
            if (sub.w > farthest_enter.w) farthest_enter = sub;
            const float t_adv = sub.w + LIST_EPSILON;
            if (intersect_leaf(sub, leaf, plan, itra, t_adv, ro, rd) && classify(sub, rd, t_adv) == ST_EXIT) {
                exit_count += 1;
                if (sub.w < nearest_exit.w) nearest_exit = sub;
            }
        } else if (st == ST_EXIT) {
            exit_count += 1;
            if (sub.w < nearest_exit.w) nearest_exit = sub;
        }
    }
    const bool overlap_all = farthest_enter.w < nearest_exit.w && max(enter_count, exit_count) == num_sub;
    if (!overlap_all) return false;
    if (farthest_enter.w > t_min && farthest_enter.w < RT_DEFAULT_MAX) { isect = farthest_enter; return true; }
    if (nearest_exit.w > t_min && nearest_exit.w < RT_DEFAULT_MAX) { isect = nearest_exit; return true; }
    return false;
}

// The three list kinds behind one out-of-line entry, so that the boolean tree and the prim dispatch each hold a
// single call site (lists are rare; the call keeps their code and registers out of the common paths).  The result
// is written through a copy, so that the caller's `isect` stays in registers.
GBO_COLD bool intersect_list(float4& isect, const gbo_csgnode* node, const gbo_csgnode* root, const float4* plan,
                             const gbo_qat4* itra, float t_min, float3 ro, float3 rd)
{
    switch (node_typecode(node)) {
        case GBO_CSG_CONTIGUOUS:    return list_contiguous(isect, node, root, plan, itra, t_min, ro, rd);
        case GBO_CSG_OVERLAP:       return list_overlap(isect, node, root, plan, itra, t_min, ro, rd);
        case GBO_CSG_DISCONTIGUOUS: return list_discontiguous(isect, node, root, plan, itra, t_min, ro, rd);
        default:                    return false;
    }
}

// intersect_node, csg_intersect_node.h:913-938: a list header or a plain leaf
GBO_DEV bool intersect_node(float4& isect, const gbo_csgnode* node, const gbo_csgnode* root, const float4* plan,
                            const gbo_qat4* itra, float t_min, float3 ro, float3 rd, bool polish)
{
    if (node_typecode(node) >= GBO_CSG_LEAF) return intersect_leaf(isect, node, plan, itra, t_min, ro, rd, polish);
    float4 c = isect;
    const bool valid = intersect_list(c, node, root, plan, itra, t_min, ro, rd);
    isect = c;
    return valid;
}

GBO_DEV int lut_lookup(unsigned op, int sa, int sb, bool acloser)
{
    // packed 4-bit actions indexed by 3*stateA+stateB, one word per boolean operation (csg_classify.h:86-101)
    const unsigned idx = op - GBO_CSG_UNION;
    unsigned word;
    if (acloser) word = idx == 0 ? 0x22121141u : (idx == 1 ? 0x00014014u : (idx == 2 ? 0x00141141u : 0u));
    else         word = idx == 0 ? 0x22115122u : (idx == 1 ? 0x00022055u : (idx == 2 ? 0x00133155u : 0u));
    const unsigned offset = 3u * (unsigned)sa + (unsigned)sb;
    return offset < 8 ? (int)((word >> (offset * 4)) & 0xfu) : CTRL_RETURN_MISS;
}


GBO_DEV unsigned pack_slice(unsigned begin, unsigned end) { return ((begin & 0xffu) << 16) | ((end & 0xffu) << 24); }
GBO_DEV unsigned postorder_next(unsigned i, unsigned elev) { return (i & 1u) ? i >> 1 : (i << elev) + (1u << elev); }

constexpr int CSG_STACK = 15;
constexpr int TRANCHE_STACK = 4;
// Guard on tranches evaluated per tree: every loop tranche restarts above the last root, so an evaluation ends after
// a few tranches per leaf root; this bound, far above that, turns any arithmetic corner that failed to advance into
// a miss instead of an unbounded loop.
constexpr int MAX_TRANCHES = 256;

// LISTS: the geometry holds CSG list nodes (their evaluation is compiled only into the kernel forms that need it)
template <bool LISTS>
GBO_DEV bool intersect_tree(float4& isect, const gbo_csgnode* node, const float4* plan, const gbo_qat4* itra,
                            float t_min, float3 ro, float3 rd, bool polish = false)
{
    const int numNode = (int)__ldg(&node->q0.u[0]);
    const unsigned height = (unsigned)(__ffs(numNode + 1) - 2);
    const float propagate_epsilon = 0.0001f;
    bool err = false;

    float tr_tmin[TRANCHE_STACK];
    unsigned tr_slice[TRANCHE_STACK];
    int tr_curr = 0;
    tr_slice[0] = pack_slice(1u << height, 0u);
    tr_tmin[0] = t_min;

    float4 cdata[CSG_STACK];
    int ccurr = -1;
    int tranches = 0;

    while (tr_curr > -1 && !err) {
        if (++tranches > MAX_TRANCHES) { err = true; break; }
        const unsigned slice = tr_slice[tr_curr];
        const float tmin = tr_tmin[tr_curr];
        tr_curr--;
        const unsigned endIdx = (slice >> 24) & 0xffu;
        unsigned nodeIdx = (slice >> 16) & 0xffu;
        while (nodeIdx != endIdx) {
            const unsigned depth = 31u - (unsigned)__clz(nodeIdx);
            const unsigned elevation = height - depth;
            const gbo_csgnode* nd = node + nodeIdx - 1;
            const unsigned typecode = node_typecode(nd);
            if (typecode == GBO_CSG_ZERO) { nodeIdx = postorder_next(nodeIdx, elevation); continue; }
            if (typecode >= GBO_CSG_NODE) {
                float4 nd_isect = make_float4(0.f, 0.f, 0.f, 0.f);
                if constexpr (LISTS) intersect_node(nd_isect, nd, node, plan, itra, tmin, ro, rd, polish);
                else intersect_leaf(nd_isect, nd, plan, itra, tmin, ro, rd, polish);
                nd_isect.w = copysignf(nd_isect.w, nodeIdx % 2 == 0 ? -1.f : 1.f);
                if (ccurr >= CSG_STACK - 1) { err = true; break; }
                cdata[++ccurr] = nd_isect;
            } else {
                if (ccurr < 1) { err = true; break; }
                const bool firstLeft = signbit(cdata[ccurr].w);
                const bool secondLeft = signbit(cdata[ccurr - 1].w);
                if (!(firstLeft ^ secondLeft)) { err = true; break; }
                const int left = firstLeft ? ccurr : ccurr - 1;
                const int right = firstLeft ? ccurr - 1 : ccurr;
                const float4 L = cdata[left], R = cdata[right];
                int l_state = classify(L, rd, tmin);
                int r_state = classify(R, rd, tmin);
                const float t_left = fabsf(L.w), t_right = fabsf(R.w);
                bool leftIsCloser = t_left <= t_right;
                const bool l_promote_miss = l_state == ST_MISS && (signbit(L.x) || signbit(L.y));
                const bool r_promote_miss = r_state == ST_MISS && (signbit(R.x) || signbit(R.y));
                if (r_promote_miss) { r_state = ST_EXIT; leftIsCloser = true; }
                if (l_promote_miss) { l_state = ST_EXIT; leftIsCloser = false; }
                const int ctrl = lut_lookup(typecode, l_state, r_state, leftIsCloser);
                if (ctrl < CTRL_LOOP_A) {
                    float4 result = ctrl == CTRL_RETURN_MISS ? make_float4(0.f, 0.f, 0.f, 0.f) : (ctrl == CTRL_RETURN_A ? L : R);
                    if (ctrl == CTRL_RETURN_FLIP_B) { result.x = -result.x; result.y = -result.y; result.z = -result.z; }
                    result.w = copysignf(result.w, nodeIdx % 2 == 0 ? -1.f : 1.f);
                    ccurr -= 2;
                    cdata[++ccurr] = result;
                } else {
                    const float4 loopv = ctrl == CTRL_LOOP_A ? L : R;
                    const float4 other = ctrl == CTRL_LOOP_A ? R : L;
                    const unsigned leftIdx = 2u * nodeIdx;
                    const unsigned rightIdx = leftIdx + 1u;
                    const float tminAdvanced = fabsf(loopv.w) + propagate_epsilon;
                    ccurr -= 2;
                    cdata[++ccurr] = other;
                    const unsigned endTree = pack_slice(nodeIdx, endIdx);
                    const unsigned leftTree = pack_slice(leftIdx << (elevation - 1), rightIdx << (elevation - 1));
                    const unsigned rightTree = pack_slice(rightIdx << (elevation - 1), nodeIdx);
                    const unsigned loopTree = ctrl == CTRL_LOOP_A ? leftTree : rightTree;
                    if (tr_curr >= TRANCHE_STACK - 1) { err = true; break; }
                    tr_curr++; tr_slice[tr_curr] = endTree; tr_tmin[tr_curr] = tmin;
                    if (tr_curr >= TRANCHE_STACK - 1) { err = true; break; }
                    tr_curr++; tr_slice[tr_curr] = loopTree; tr_tmin[tr_curr] = tminAdvanced;
                    break;
                }
            }
            nodeIdx = postorder_next(nodeIdx, elevation);
        }
    }
    isect = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ccurr == 0) isect = cdata[0];
    return isect.w > 0.f;
}

// Union fast path for trees whose internal nodes are all unions and whose leaves are plain: evaluate every leaf
// once at t_min, in postorder (left to right).  While every leaf's first hit enters it (the ray starts outside all
// of them), Kensler's union table returns the nearest entering hit, the left one on a tie (ReturnAIfCloser with
// leftIsCloser = tA <= tB), which is what the loop below keeps.  A leaf hit that exits (the ray starts inside that
// leaf) needs the table's loop cases: the function then returns -1 and the caller runs intersect_tree.
GBO_DEV int intersect_union_enter(float4& isect, const gbo_csgnode* node, const float4* plan, const gbo_qat4* itra,
                                  float t_min, float3 ro, float3 rd, bool polish)
{
    const int numNode = (int)__ldg(&node->q0.u[0]);
    const unsigned height = (unsigned)(__ffs(numNode + 1) - 2);
    float4 best = make_float4(0.f, 0.f, 0.f, 0.f);
    bool found = false;
    unsigned nodeIdx = 1u << height;
    while (nodeIdx != 0u) {
        const unsigned depth = 31u - (unsigned)__clz(nodeIdx);
        const unsigned elevation = height - depth;
        const gbo_csgnode* nd = node + nodeIdx - 1;
        if (node_typecode(nd) >= GBO_CSG_LEAF) {
            float4 is;
            intersect_leaf(is, nd, plan, itra, t_min, ro, rd, polish);
            if (fabsf(is.w) > t_min) {
                if (!(is.x * rd.x + is.y * rd.y + is.z * rd.z < 0.f)) return -1;     // exits: full algorithm
                if (!found || is.w < best.w) { best = is; found = true; }
            }
        }
        nodeIdx = postorder_next(nodeIdx, elevation);
    }
    isect = best;
    return found ? 1 : 0;
}

// csg_intersect_tree.h:683-719: a leaf, a boolean tree or (LISTS) a list prim (the list's own node is the root)
template <bool LISTS>
GBO_DEV bool intersect_prim(float4& isect, const gbo_csgnode* node, const float4* plan, const gbo_qat4* itra,
                            float t_min, float3 o, float3 d, bool polish = false)
{
    const unsigned typecode = node_typecode(node);
    if (typecode >= GBO_CSG_LEAF) return intersect_leaf(isect, node, plan, itra, t_min, o, d, polish);
    if (typecode < GBO_CSG_NODE) return intersect_tree<LISTS>(isect, node, plan, itra, t_min, o, d, polish);
    isect = make_float4(0.f, 0.f, 0.f, 0.f);
    if constexpr (LISTS) return intersect_node(isect, node, node, plan, itra, t_min, o, d, polish);
    return false;
}

}  // namespace gbo
