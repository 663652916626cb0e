/*
 * orc_csg64.c : double-precision CSG intersection, the FP64 reference for intersection distances.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * The reference has no FP64 intersector (only distance_leaf_sphere is templated,
 * CSG/csg_intersect_leaf_templated.h:64; CSGQuery, CSG/CSGQuery.cc:231-278, calls the float intersect_prim).
 * This file restates the leaf functions (sphere, zsphere, cylinder, box3, cone), the node transform and complement
 * handling and the single-hit boolean tree of orc_csg.c in binary64, with the node and instance transforms
 * inverted in binary64 from the float forward transforms, so that the engine's binary32 intersection distances
 * (with or without its FP64 root polish) can be measured against an independent binary64 result.
 */
#include <math.h>
#include <string.h>
#include "orc_internal.h"

typedef struct { double x, y, z; } d3;
typedef struct { double x, y, z, w; } d4;
static inline d3 D3(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline d3 dadd(d3 a, d3 b) { return D3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline d3 dsub(d3 a, d3 b) { return D3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 dscale(double s, d3 a) { return D3(s * a.x, s * a.y, s * a.z); }
static inline double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

#define RT_MAX64 1.e300

typedef struct { double m[3][3]; double t[3]; } xf64;     /* row-vector affine: p' = p m + t */

static void xf_from_qat(const gbo_qat4* q, xf64* x)
{
    for (int j = 0; j < 3; j++) {
        x->m[0][j] = q->q0.f[j];
        x->m[1][j] = q->q1.f[j];
        x->m[2][j] = q->q2.f[j];
        x->t[j] = q->q3.f[j];
    }
}

static void xf_invert(const xf64* a, xf64* r)
{
    const double (*m)[3] = a->m;
    double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                 m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    r->m[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / det;
    r->m[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
    r->m[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
    r->m[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / det;
    r->m[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
    r->m[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
    r->m[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / det;
    r->m[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
    r->m[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
    for (int j = 0; j < 3; j++) r->t[j] = -(a->t[0] * r->m[0][j] + a->t[1] * r->m[1][j] + a->t[2] * r->m[2][j]);
}

static d3 xf_point(const xf64* x, d3 v)
{
    return D3(v.x * x->m[0][0] + v.y * x->m[1][0] + v.z * x->m[2][0] + x->t[0],
              v.x * x->m[0][1] + v.y * x->m[1][1] + v.z * x->m[2][1] + x->t[1],
              v.x * x->m[0][2] + v.y * x->m[1][2] + v.z * x->m[2][2] + x->t[2]);
}
static d3 xf_vector(const xf64* x, d3 v)
{
    return D3(v.x * x->m[0][0] + v.y * x->m[1][0] + v.z * x->m[2][0],
              v.x * x->m[0][1] + v.y * x->m[1][1] + v.z * x->m[2][1],
              v.x * x->m[0][2] + v.y * x->m[1][2] + v.z * x->m[2][2]);
}
static d3 xf_normal(const xf64* inv, d3 n)      /* transpose of the inverse */
{
    return D3(inv->m[0][0] * n.x + inv->m[0][1] * n.y + inv->m[0][2] * n.z,
              inv->m[1][0] * n.x + inv->m[1][1] * n.y + inv->m[1][2] * n.z,
              inv->m[2][0] * n.x + inv->m[2][1] * n.y + inv->m[2][2] * n.z);
}

static void roots(double* t1, double* t2, double* sdisc, double d, double b, double c)
{
    double disc = b * b - d * c;
    *sdisc = disc > 0.0 ? sqrt(disc) : 0.0;
    double q = b > 0.0 ? -(b + *sdisc) : -(b - *sdisc);
    double r1 = q / d, r2 = c / q;
    *t1 = fmin(r1, r2);
    *t2 = fmax(r1, r2);
}

static int leaf_sphere64(d4* is, const gbo_quad* q0, double t_min, d3 ro, d3 rd)
{
    d3 center = D3(q0->f[0], q0->f[1], q0->f[2]);
    double radius = q0->f[3];
    d3 O = dsub(ro, center);
    double b = ddot(O, rd), c = ddot(O, O) - radius * radius, d = ddot(rd, rd);
    double r1, r2, sdisc;
    roots(&r1, &r2, &sdisc, d, b, c);
    double t = sdisc > 0.0 ? (r1 > t_min ? r1 : r2) : t_min;
    if (!(t > t_min)) return 0;
    is->x = (O.x + t * rd.x) / radius; is->y = (O.y + t * rd.y) / radius; is->z = (O.z + t * rd.z) / radius; is->w = t;
    return 1;
}

static int leaf_zsphere64(d4* is, const gbo_quad* q0, const gbo_quad* q1, double t_min, d3 ro, d3 rd)
{
    d3 center = D3(q0->f[0], q0->f[1], q0->f[2]);
    d3 O = dsub(ro, center);
    double radius = q0->f[3];
    double b = ddot(O, rd), c = ddot(O, O) - radius * radius;
    if (c > 0.0 && b > 0.0) return 0;
    double zmax = center.z + q1->f[1], zmin = center.z + q1->f[0];
    double d = ddot(rd, rd);
    double t1s, t2s, sdisc;
    roots(&t1s, &t2s, &sdisc, d, b, c);
    double z1s = ro.z + t1s * rd.z, z2s = ro.z + t2s * rd.z;
    double tq = (zmax - ro.z) / rd.z, tp = (zmin - ro.z) / rd.z;
    double t1c = fmin(tq, tp), t2c = fmax(tq, tp);
    if (t1c < t1s || t1c > t2s) t1c = t_min;
    if (t2c < t1s || t2c > t2s) t2c = t_min;
    double t = t_min;
    if (sdisc > 0.0) {
        if (t1s > t_min && z1s > zmin && z1s <= zmax) t = t1s;
        else if (t1c > t_min) t = t1c;
        else if (t2c > t_min) t = t2c;
        else if (t2s > t_min && z2s > zmin && z2s <= zmax) t = t2s;
    }
    if (!(t > t_min)) return 0;
    is->w = t;
    if (t == t1s || t == t2s) { is->x = (O.x + t * rd.x) / radius; is->y = (O.y + t * rd.y) / radius; is->z = (O.z + t * rd.z) / radius; }
    else { is->x = 0.0; is->y = 0.0; is->z = t == tp ? -1.0 : 1.0; }
    return 1;
}

static int leaf_cylinder64(d4* is, const gbo_quad* q0, const gbo_quad* q1, double t_min, d3 o, d3 v)
{
    double r = q0->f[3], z1 = q1->f[0], z2 = q1->f[1];
    double r2 = r * r;
    double a = v.x * v.x + v.y * v.y, b = o.x * v.x + o.y * v.y, c = o.x * o.x + o.y * o.y - r2;
    double disc = b * b - a * c;
    double sdisc = disc > 0.0 ? sqrt(disc) : 0.0;
    double q = b > 0.0 ? -(b + sdisc) : -(b - sdisc);
    double tn = sdisc > 0.0 ? fmin(q / a, c / q) : t_min, tf = sdisc > 0.0 ? fmax(q / a, c / q) : t_min;
    double zn = o.z + tn * v.z, zf = o.z + tf * v.z;
    double tc1 = (z1 - o.z) / v.z, tc2 = (z2 - o.z) / v.z;
    double rc1 = (o.x + tc1 * v.x) * (o.x + tc1 * v.x) + (o.y + tc1 * v.y) * (o.y + tc1 * v.y);
    double rc2 = (o.x + tc2 * v.x) * (o.x + tc2 * v.x) + (o.y + tc2 * v.y) * (o.y + tc2 * v.y);
    double t = INFINITY;
    if (tn > t_min && zn > z1 && zn < z2 && tn < t) t = tn;
    if (tf > t_min && zf > z1 && zf < z2 && tf < t) t = tf;
    if (tc1 > t_min && rc1 <= r2 && tc1 < t) t = tc1;
    if (tc2 > t_min && rc2 <= r2 && tc2 < t) t = tc2;
    if (!(t > t_min && t < INFINITY)) return 0;
    int sheet = (t == tn || t == tf);
    is->x = sheet ? (o.x + t * v.x) / r : 0.0;
    is->y = sheet ? (o.y + t * v.y) / r : 0.0;
    is->z = sheet ? 0.0 : (t == tc1 ? -1.0 : 1.0);
    is->w = t;
    return 1;
}

static int leaf_box3_64(d4* is, const gbo_quad* q0, double t_min, d3 o, d3 d)
{
    d3 bmin = D3(-q0->f[0] / 2.0, -q0->f[1] / 2.0, -q0->f[2] / 2.0), bmax = D3(q0->f[0] / 2.0, q0->f[1] / 2.0, q0->f[2] / 2.0);
    double tx0 = (bmin.x - o.x) / d.x, tx1 = (bmax.x - o.x) / d.x;
    double ty0 = (bmin.y - o.y) / d.y, ty1 = (bmax.y - o.y) / d.y;
    double tz0 = (bmin.z - o.z) / d.z, tz1 = (bmax.z - o.z) / d.z;
    double tn = fmax(fmax(fmin(tx0, tx1), fmin(ty0, ty1)), fmin(tz0, tz1));
    double tf = fmin(fmin(fmax(tx0, tx1), fmax(ty0, ty1)), fmax(tz0, tz1));
    if (!(tf > tn && tf > 0.0)) return 0;
    double t = t_min < tn ? tn : (t_min < tf ? tf : t_min);
    if (!(t > t_min)) return 0;
    d3 p = dadd(o, dscale(t, d));
    double ax = fabs(p.x) / (bmax.x - bmin.x), ay = fabs(p.y) / (bmax.y - bmin.y), az = fabs(p.z) / (bmax.z - bmin.z);
    is->x = is->y = is->z = 0.0;
    if (ax >= ay && ax >= az) is->x = copysign(1.0, p.x);
    else if (ay >= ax && ay >= az) is->y = copysign(1.0, p.y);
    else is->z = copysign(1.0, p.z);
    is->w = t;
    return 1;
}

static int leaf64(d4* is, const gbo_csgnode* node, const gbo_qat4* itra, double t_min, d3 ro, d3 rd)
{
    memset(is, 0, sizeof(*is));
    unsigned tc = node->q3.u[2];
    unsigned gt = node->q3.u[3] & 0x7fffffffu;
    int complement = (node->q3.u[3] & 0x80000000u) != 0;
    xf64 inv;
    d3 o = ro, d = rd;
    if (gt > 0) {
        xf_from_qat(itra + gt - 1, &inv);      /* the node transform is defined by its stored inverse */
        o = xf_point(&inv, ro);
        d = xf_vector(&inv, rd);
    }
    int valid = 0;
    switch (tc) {
        case GBO_CSG_SPHERE: valid = leaf_sphere64(is, &node->q0, t_min, o, d); break;
        case GBO_CSG_ZSPHERE: valid = leaf_zsphere64(is, &node->q0, &node->q1, t_min, o, d); break;
        case GBO_CSG_CYLINDER: valid = leaf_cylinder64(is, &node->q0, &node->q1, t_min, o, d); break;
        case GBO_CSG_BOX3: valid = leaf_box3_64(is, &node->q0, t_min, o, d); break;
        default: break;
    }
    if (valid && gt > 0) {
        d3 n = xf_normal(&inv, D3(is->x, is->y, is->z));
        is->x = n.x; is->y = n.y; is->z = n.z;
    }
    if (complement) {
        is->x = valid ? -is->x : -0.0;
        is->y = valid ? -is->y : is->y;
        is->z = valid ? -is->z : is->z;
    }
    return valid;
}

/* single-hit boolean tree, as intersect_tree in orc_csg.c, in binary64 */
static int tree64(d4* isect, const gbo_csgnode* node, const gbo_qat4* itra, double t_min, d3 ro, d3 rd)
{
    static const unsigned LA[4] = { 0x22121141u, 0x00014014u, 0x00141141u, 0u };
    static const unsigned LB[4] = { 0x22115122u, 0x00022055u, 0x00133155u, 0u };
    const int numNode = (int)node->q0.u[0];
    unsigned height = (unsigned)(__builtin_ffs(numNode + 1) - 2);
    double trm[4];
    unsigned trs[4];
    int tc = 0;
    trs[0] = ((1u << height) & 0xffu) << 16;
    trm[0] = t_min;
    d4 cd[15];
    int cc = -1;
    int err = 0;
    while (tc > -1 && !err) {
        unsigned slice = trs[tc];
        double tmin = trm[tc];
        tc--;
        unsigned endIdx = (slice >> 24) & 0xffu;
        unsigned ni = (slice >> 16) & 0xffu;
        while (ni != endIdx) {
            unsigned depth = 31u - (unsigned)__builtin_clz(ni);
            unsigned elev = height - depth;
            const gbo_csgnode* nd = node + ni - 1;
            unsigned t = nd->q3.u[2];
            if (t == GBO_CSG_ZERO) { ni = (ni & 1u) ? ni >> 1 : (ni << elev) + (1u << elev); continue; }
            if (t >= GBO_CSG_NODE) {
                d4 v;
                leaf64(&v, nd, itra, tmin, ro, rd);
                v.w = copysign(v.w, ni % 2 == 0 ? -1.0 : 1.0);
                if (cc >= 14) { err = 1; break; }
                cd[++cc] = v;
            } else {
                if (cc < 1) { err = 1; break; }
                int fl = signbit(cd[cc].w) != 0, sl = signbit(cd[cc - 1].w) != 0;
                if (!(fl ^ sl)) { err = 1; break; }
                int l = fl ? cc : cc - 1, r = fl ? cc - 1 : cc;
                d4 L = cd[l], R = cd[r];
                int ls = fabs(L.w) > tmin ? (L.x * rd.x + L.y * rd.y + L.z * rd.z < 0.0 ? 0 : 1) : 2;
                int rs = fabs(R.w) > tmin ? (R.x * rd.x + R.y * rd.y + R.z * rd.z < 0.0 ? 0 : 1) : 2;
                int lc = fabs(L.w) <= fabs(R.w);
                if (rs == 2 && (signbit(R.x) || signbit(R.y))) { rs = 1; lc = 1; }
                if (ls == 2 && (signbit(L.x) || signbit(L.y))) { ls = 1; lc = 0; }
                unsigned off = 3u * (unsigned)ls + (unsigned)rs;
                unsigned word = (lc ? LA : LB)[t - GBO_CSG_UNION];
                int ctrl = off < 8 ? (int)((word >> (off * 4)) & 0xfu) : 0;
                if (ctrl < 4) {
                    d4 res = ctrl == 0 ? (d4){0, 0, 0, 0} : (ctrl == 1 ? L : R);
                    if (ctrl == 3) { res.x = -res.x; res.y = -res.y; res.z = -res.z; }
                    res.w = copysign(res.w, ni % 2 == 0 ? -1.0 : 1.0);
                    cc -= 2;
                    cd[++cc] = res;
                } else {
                    d4 loop = ctrl == 4 ? L : R, other = ctrl == 4 ? R : L;
                    unsigned li = 2u * ni, rix = li + 1u;
                    double adv = fabs(loop.w) + 0.0001;
                    cc -= 2;
                    cd[++cc] = other;
                    unsigned endTree = ((ni & 0xffu) << 16) | ((endIdx & 0xffu) << 24);
                    unsigned lt = (((li << (elev - 1)) & 0xffu) << 16) | (((rix << (elev - 1)) & 0xffu) << 24);
                    unsigned rt = (((rix << (elev - 1)) & 0xffu) << 16) | ((ni & 0xffu) << 24);
                    if (tc >= 3) { err = 1; break; }
                    trs[++tc] = endTree; trm[tc] = tmin;
                    if (tc >= 3) { err = 1; break; }
                    trs[++tc] = ctrl == 4 ? lt : rt; trm[tc] = adv;
                    break;
                }
            }
            ni = (ni & 1u) ? ni >> 1 : (ni << elev) + (1u << elev);
        }
    }
    memset(isect, 0, sizeof(*isect));
    if (cc == 0) *isect = cd[0];
    return isect->w > 0.0;
}

static int prim64(d4* is, const gbo_csgnode* root, const gbo_qat4* itra, double t_min, d3 o, d3 d)
{
    unsigned t = root->q3.u[2];
    if (t >= GBO_CSG_LEAF) return leaf64(is, root, itra, t_min, o, d);
    if (t < GBO_CSG_NODE) return tree64(is, root, itra, t_min, o, d);
    return 0;
}

/* per-instance binary64 data: inverse transform and a world bounding sphere of its solid */
typedef struct { xf64 inv; d3 center; double radius; int solid; } inst64;

static void make_inst64(const orc_geom* g, inst64* out)
{
    for (int ii = 0; ii < g->num_inst; ii++) {
        const gbo_qat4* q = &g->inst[ii];
        xf64 fwd;
        xf_from_qat(q, &fwd);
        xf_invert(&fwd, &out[ii].inv);
        const int s = q->q1.i[3];
        out[ii].solid = s;
        const gbo_csgsolid* so = &g->solid[s];
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int k = 0; k < so->numPrim; k++) {
            const gbo_csgprim* pr = &g->prim[so->primOffset + k];
            double a[3] = {pr->q2.f[0], pr->q2.f[1], pr->q2.f[2]}, b[3] = {pr->q2.f[3], pr->q3.f[0], pr->q3.f[1]};
            for (int j = 0; j < 3; j++) { lo[j] = fmin(lo[j], a[j]); hi[j] = fmax(hi[j], b[j]); }
        }
        d3 c = D3(0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2]));
        d3 h = D3(0.5 * (hi[0] - lo[0]), 0.5 * (hi[1] - lo[1]), 0.5 * (hi[2] - lo[2]));
        /* the solid's box corner distance, scaled by the largest stretch of the transform */
        double smax = 0.0;
        for (int j = 0; j < 3; j++)
            smax = fmax(smax, sqrt(fwd.m[j][0] * fwd.m[j][0] + fwd.m[j][1] * fwd.m[j][1] + fwd.m[j][2] * fwd.m[j][2]));
        out[ii].center = xf_point(&fwd, c);
        out[ii].radius = sqrt(ddot(h, h)) * smax * (1.0 + 1e-9) + 1e-6;
    }
}

static double trace64(const orc_geom* g, const inst64* I, d3 P, d3 Dv, double tmin, double tmax, unsigned* boundary)
{
    double best = tmax;
    int found = 0;
    const double dd = ddot(Dv, Dv);
    for (int ii = 0; ii < g->num_inst; ii++) {
        /* cull: the ray misses the instance's bounding sphere, or meets it only beyond the best hit */
        d3 oc = dsub(I[ii].center, P);
        double tc = ddot(oc, Dv) / dd;
        d3 perp = dsub(oc, dscale(tc, Dv));
        double r = I[ii].radius;
        if (ddot(perp, perp) > r * r) continue;
        if (tc - r / sqrt(dd) > best) continue;
        const gbo_csgsolid* so = &g->solid[I[ii].solid];
        d3 o = xf_point(&I[ii].inv, P), d = xf_vector(&I[ii].inv, Dv);
        for (int k = 0; k < so->numPrim; k++) {
            const gbo_csgprim* pr = &g->prim[so->primOffset + k];
            const gbo_csgnode* root = g->node + pr->q0.i[1];
            d4 is;
            if (prim64(&is, root, g->itra, tmin, o, d) && is.w >= tmin && is.w < best) {
                best = is.w;
                found = 1;
                if (boundary) *boundary = root->q1.u[2];
            }
        }
    }
    return found ? best : -1.0;
}

typedef struct {
    const orc_geom* g; const inst64* I; const float* pos; const float* dir;
    int64_t begin, end; double tmin, tmax; double* t; uint32_t* b;
} job64;

#include <pthread.h>
#include <stdlib.h>

static void* run64(void* arg)
{
    job64* j = (job64*)arg;
    for (int64_t i = j->begin; i < j->end; i++) {
        d3 p = D3(j->pos[3 * i], j->pos[3 * i + 1], j->pos[3 * i + 2]);
        d3 d = D3(j->dir[3 * i], j->dir[3 * i + 1], j->dir[3 * i + 2]);
        unsigned b = 0xffffffffu;
        j->t[i] = trace64(j->g, j->I, p, d, j->tmin, j->tmax, &b);
        j->b[i] = b;
    }
    return 0;
}

/* closest-hit distance in binary64 for each ray (t = -1 on a miss), with the boundary of the prim hit */
void orc_trace64_batch(const orc_geom* g, const float* pos, const float* dir, int64_t n, double tmin, double tmax,
                       double* t_out, uint32_t* boundary_out, int nthreads)
{
    inst64* I = (inst64*)malloc(sizeof(inst64) * (size_t)g->num_inst);
    make_inst64(g, I);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    job64 jobs[256];
    int64_t per = (n + nthreads - 1) / nthreads;
    for (int k = 0; k < nthreads; k++) {
        jobs[k] = (job64){g, I, pos, dir, k * per, (k + 1) * per < n ? (k + 1) * per : n, tmin, tmax, t_out, boundary_out};
        if (jobs[k].begin > jobs[k].end) jobs[k].begin = jobs[k].end;
        pthread_create(&th[k], 0, run64, &jobs[k]);
    }
    for (int k = 0; k < nthreads; k++) pthread_join(th[k], 0);
    free(I);
}
