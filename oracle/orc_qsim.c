/*
 * orc_qsim.c : photon generation, bulk/boundary/surface physics and the per-photon simulate loop.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Each function restates the named reference function in binary32 with its draw order:
 *   simulate                    CSGOptiX/CSGOptiX7.cu:405-503
 *   qsim::generate_photon       qudarap/qsim.h:2521-2541
 *   storch::generate            sysrap/storch.h:189-516
 *   qscint::generate            qudarap/qscint.h:55-75, mom_pol_wavelength :117-145, wavelength_hd* :165-228
 *   qcerenkov::generate         qudarap/qcerenkov.h:56-119, fraction_sampled :139-163,
 *                               wavelength_sampled_bndtex :285-327
 *   qsim::propagate             qudarap/qsim.h:2218-2327
 *   qbnd::fill_state            qudarap/qbnd.h:184-214, boundary_lookup :103-125
 *   qsim::propagate_to_boundary qudarap/qsim.h:718-863 (DEBUG_TAG burns :730-735)
 *   qsim::rayleigh_scatter      qudarap/qsim.h:601-689
 *   qsim::propagate_at_boundary qudarap/qsim.h:998-1205 (burns :1088-1091, :1188-1201)
 *   qsim::propagate_at_surface  qudarap/qsim.h:1677-1747 (burn :1685-1691)
 *   qsim::reflect_diffuse       qudarap/qsim.h:1977-2012, lambertian_direction :430-483,
 *                               random_direction_marsaglia :551-572
 *   qsim::reflect_specular      qudarap/qsim.h:2030-2082
 *   qsim::uniform_sphere        qudarap/qsim.h:177-183
 *   smath::rotateUz             sysrap/smath.h:77-95
 *   sphoton setters             sysrap/sphoton.h:171-231, set_prd :482-488
 *   sseq::add_nibble            sysrap/sseq.h:174-184
 * Loops that the reference leaves unbounded (Marsaglia, Rayleigh, Cerenkov fraction) are capped at
 * 100000 turns, which a uniform stream exceeds with negligible probability.
 */
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include "orc_internal.h"

enum { F_UNDEFINED = 0, F_BREAK = 1, F_CONTINUE = 2, F_BOUNDARY = 3 };
#define LOOP_CAP 100000

typedef struct {
    v4 material1, m1group2, material2, surface;
    uint32_t optical[4];
} orc_state;

typedef struct {
    v3 pos; float time;
    v3 mom; uint32_t hitcount_iindex;
    v3 pol; float wavelength;
    uint32_t orient_boundary_flag, identity, index, flagmask;
} orc_photon;

/* ---- sphoton bit packing ---- */
static inline unsigned ph_flag(const orc_photon* p) { return p->orient_boundary_flag & 0xffffu; }
static inline unsigned ph_boundary(const orc_photon* p) { return (p->orient_boundary_flag & 0x7fff0000u) >> 16; }
static inline void ph_set_flag(orc_photon* p, unsigned f)
{
    p->orient_boundary_flag = (p->orient_boundary_flag & 0xffff0000u) | (f & 0xffffu);
    p->flagmask |= f;
}
static inline void ph_zero_flags(orc_photon* p)
{
    p->orient_boundary_flag = 0u; p->identity = 0u; p->index = 0u; p->flagmask = 0u; p->hitcount_iindex = 0u;
}
static inline void ph_set_prd(orc_photon* p, unsigned boundary, unsigned identity, float orient, unsigned iindex)
{
    p->orient_boundary_flag = (p->orient_boundary_flag & 0x8000ffffu) | ((boundary & 0x7fffu) << 16);
    p->identity = (p->identity & 0xff000000u) | (identity & 0x00ffffffu);
    p->orient_boundary_flag = (p->orient_boundary_flag & 0x7fffffffu) | ((orient < 0.f ? 0x1u : 0x0u) << 31);
    p->hitcount_iindex = 0x00010000u | (0x0000ffffu & iindex);
}
static inline void ph_set_index(orc_photon* p, uint64_t full)
{
    p->index = (uint32_t)(full & 0xffffffffu);
    p->identity = ((uint32_t)((full >> 32) & 0xffu) << 24) | (p->identity & 0xffffffu);
}

static void ph_from(orc_photon* p, const gbo_sphoton* s)
{
    p->pos = v3of(s->pos); p->time = s->time;
    p->mom = v3of(s->mom); p->hitcount_iindex = s->hitcount_iindex;
    p->pol = v3of(s->pol); p->wavelength = s->wavelength;
    p->orient_boundary_flag = s->orient_boundary_flag; p->identity = s->identity;
    p->index = s->index; p->flagmask = s->flagmask;
}
static void ph_to(gbo_sphoton* s, const orc_photon* p)
{
    v3to(s->pos, p->pos); s->time = p->time;
    v3to(s->mom, p->mom); s->hitcount_iindex = p->hitcount_iindex;
    v3to(s->pol, p->pol); s->wavelength = p->wavelength;
    s->orient_boundary_flag = p->orient_boundary_flag; s->identity = p->identity;
    s->index = p->index; s->flagmask = p->flagmask;
}

/* float3 / float in the reference helpers multiplies by the reciprocal (sysrap/scuda.h:544-548) */
static inline v3 vdivs(v3 a, float s) { float inv = 1.0f / s; return V3(a.x * inv, a.y * inv, a.z * inv); }

void orc_rotateUz(v3* d, v3 u)
{
    float up = u.x * u.x + u.y * u.y;
    if (up > 0.f) {
        up = sqrtf(up);
        float px = d->x, py = d->y, pz = d->z;
        d->x = (u.x * u.z * px - u.y * py) / up + u.x * pz;
        d->y = (u.y * u.z * px + u.x * py) / up + u.y * pz;
        d->z = -up * px + u.z * pz;
    } else if (u.z < 0.f) {
        d->x = -d->x;
        d->z = -d->z;
    }
}

/* ---- material/surface lookup ---- */
static v4 boundary_lookup(const orc_sim* s, float nm, unsigned line, unsigned k)
{
    const unsigned nx = (unsigned)s->bnd.nx, ny = (unsigned)s->bnd.ny;
    float fx = (nm - s->bnd_nm0) / s->bnd_nms;
    float x = (fx + 0.5f) / (float)nx;
    unsigned iy = 2u * line + k;
    float y = ((float)iy + 0.5f) / (float)ny;
    return orc_tex2d4(&s->bnd, x, y);
}

static void fill_state(const orc_sim* s, orc_state* st, unsigned boundary, float wavelength, float cosTheta)
{
    const int line = (int)boundary * 4;
    const int m1_line = cosTheta > 0.f ? line + GBO_IMAT : line + GBO_OMAT;
    const int m2_line = cosTheta > 0.f ? line + GBO_OMAT : line + GBO_IMAT;
    const int su_line = cosTheta > 0.f ? line + GBO_ISUR : line + GBO_OSUR;
    st->material1 = boundary_lookup(s, wavelength, (unsigned)m1_line, 0);
    st->m1group2 = boundary_lookup(s, wavelength, (unsigned)m1_line, 1);
    st->material2 = boundary_lookup(s, wavelength, (unsigned)m2_line, 0);
    st->surface = boundary_lookup(s, wavelength, (unsigned)su_line, 0);
    memcpy(st->optical, s->optical + 4 * (size_t)su_line, sizeof(st->optical));
}

static float scint_wavelength(const orc_sim* s, float u0)
{
    const float y0 = 0.5f / 3.f, y1 = 1.5f / 3.f, y2 = 2.5f / 3.f;
    switch (s->hd_factor) {
        case 0: return orc_tex2d1(&s->icdf, u0, y0);
        case 10:
            if (u0 < 0.1f) return orc_tex2d1(&s->icdf, u0 * 10.f, y1);
            if (u0 > 0.9f) return orc_tex2d1(&s->icdf, (u0 - 0.9f) * 10.f, y2);
            return orc_tex2d1(&s->icdf, u0, y0);
        case 20:
            if (u0 < 0.05f) return orc_tex2d1(&s->icdf, u0 * 20.f, y1);
            if (u0 > 0.95f) return orc_tex2d1(&s->icdf, (u0 - 0.95f) * 20.f, y2);
            return orc_tex2d1(&s->icdf, u0, y0);
        default: return 0.f;
    }
}

static v3 uniform_sphere(float u0, float u1)
{
    float phi = u0 * 2.f * ORC_PI_F;
    float cosTheta = 2.f * u1 - 1.f;
    float sinTheta = sqrtf(1.f - cosTheta * cosTheta);
    return V3(cosf(phi) * sinTheta, sinf(phi) * sinTheta, cosTheta);
}

/* ---- generators ---- */

static void gen_torch(orc_photon* p, orc_rng* rng, const gbo_quad6* g, uint64_t photon_id)
{
    const v3 gpos = V3(g->q[1].f[0], g->q[1].f[1], g->q[1].f[2]);
    const float gtime = g->q[1].f[3];
    const v3 gmom = V3(g->q[2].f[0], g->q[2].f[1], g->q[2].f[2]);
    const v3 gpol = V3(g->q[3].f[0], g->q[3].f[1], g->q[3].f[2]);
    const float gwl = g->q[3].f[3];
    const float zx = g->q[4].f[0], zy = g->q[4].f[1], ax = g->q[4].f[2], ay = g->q[4].f[3];
    const float radius = g->q[5].f[0], distance = g->q[5].f[1];
    const unsigned numphoton = g->q[0].u[3];
    const unsigned type = g->q[5].u[3];
    (void)gpol;
    if (type == GBO_T_DISC) {
        p->wavelength = gwl; p->time = gtime; p->mom = gmom;
        float u_zenith = zx + orc_uniform(rng) * (zy - zx);
        float u_azimuth = ax + orc_uniform(rng) * (ay - ax);
        float r = radius * u_zenith;
        float phi = 2.f * ORC_PI_F * u_azimuth;
        float sinPhi = sinf(phi), cosPhi = cosf(phi);
        p->pos = V3(r * cosPhi, r * sinPhi, 0.f);
        orc_rotateUz(&p->pos, p->mom);
        p->pos = vadd(p->pos, gpos);
        p->pol = V3(sinPhi, -cosPhi, 0.f);
        orc_rotateUz(&p->pol, p->mom);
    } else if (type == GBO_T_SPHERE) {
        p->wavelength = gwl; p->time = gtime;
        float u_zenith = zx + orc_uniform(rng) * (zy - zx);
        float u_azimuth = ax + orc_uniform(rng) * (ay - ax);
        float phi = 2.f * ORC_PI_F * u_azimuth;
        float sinPhi = sinf(phi), cosPhi = cosf(phi);
        float cosTheta = 1.f - 2.0f * u_zenith;
        float sinTheta = sqrtf(1.0f - cosTheta * cosTheta);
        float flip = copysignf(1.f, radius);
        p->mom = V3(flip * sinTheta * cosPhi, flip * sinTheta * sinPhi, flip * cosTheta);
        float rad = fabsf(radius);
        p->pos = V3(sinTheta * cosPhi * rad, sinTheta * sinPhi * rad, cosTheta * rad);
        float phase = 2.f * ORC_PI_F * distance;
        p->pol = V3(cosf(phase), sinf(phase), 0.f);
        orc_rotateUz(&p->pol, p->mom);
    } else if (type == GBO_T_SPHERE_MARSAGLIA) {
        p->wavelength = gwl; p->time = gtime;
        float u = 0.f, v = 0.f, b = 2.f;
        for (int k = 0; k < LOOP_CAP && b > 1.f; k++) {
            float u0 = zx + orc_uniform(rng) * (zy - zx);
            float u1 = ax + orc_uniform(rng) * (ay - ax);
            u = 2.f * u0 - 1.f; v = 2.f * u1 - 1.f; b = u * u + v * v;
        }
        float a = 2.f * sqrtf(1.f - b);
        float rad = fabsf(radius);
        float flip = copysignf(1.f, radius);
        p->mom = V3(flip * a * u, flip * a * v, flip * (2.f * b - 1.f));
        p->pos = V3(a * u * rad, a * v * rad, (2.f * b - 1.f) * rad);
        float phase = 2.f * ORC_PI_F * distance;
        p->pol = V3(cosf(phase), sinf(phase), 0.f);
        orc_rotateUz(&p->pol, p->mom);
    } else if (type == GBO_T_LINE) {
        p->wavelength = gwl; p->time = gtime; p->mom = gmom;
        float frac = (float)photon_id / (float)numphoton;
        float sfrac = 2.f * (frac - 0.5f);
        float r = radius * sfrac;
        p->pos = V3(r, 0.f, 0.f);
        orc_rotateUz(&p->pos, p->mom);
        p->pos = vadd(p->pos, gpos);
        p->pol = V3(0.f, -1.f, 0.f);
        orc_rotateUz(&p->pol, p->mom);
    } else if (type == GBO_T_POINT) {
        p->wavelength = gwl; p->time = gtime; p->mom = gmom;
        p->pos = V3(0.f, 0.f, 0.f);
        orc_rotateUz(&p->pos, p->mom);
        p->pos = vadd(p->pos, gpos);
        p->pol = V3(0.f, -1.f, 0.f);
        orc_rotateUz(&p->pol, p->mom);
    } else if (type == GBO_T_CIRCLE) {
        p->wavelength = gwl; p->time = gtime;
        float f = (float)photon_id / (float)numphoton;
        float frac = ax * (1.f - f) + ay * (f);
        float phi = 2.f * ORC_PI_F * frac;
        float sinPhi = sinf(phi), cosPhi = cosf(phi);
        float r = radius < 0.f ? -radius : radius;
        p->mom = V3(radius < 0.f ? -cosPhi : cosPhi, 0.f, radius < 0.f ? -sinPhi : sinPhi);
        p->pos = V3(r * cosPhi, 0.f, r * sinPhi);
        p->pos = vadd(p->pos, gpos);
        p->pol = V3(0.f, -1.f, 0.f);
        orc_rotateUz(&p->pol, p->mom);
    } else if (type == GBO_T_RECTANGLE) {
        p->wavelength = gwl; p->time = gtime;
        int side_size = (int)(numphoton / 4u);
        int side = (int)(photon_id / (uint64_t)(int64_t)side_size);
        int side_offset = side * side_size;
        int side_index = (int)photon_id - side_offset;
        float frac = (float)side_index / (float)side_size;
        if (side == 0 || side == 1) {
            p->pos = V3(side == 0 ? ax : ay, 0.f, (1.f - frac) * zx + frac * zy);
            p->mom = V3(side == 0 ? 1.f : -1.f, 0.f, 0.f);
        } else if (side == 2 || side == 3) {
            p->pos = V3((1.f - frac) * ax + frac * ay, 0.f, side == 2 ? zx : zy);
            p->mom = V3(0.f, 0.f, side == 2 ? 1.f : -1.f);
        }
        p->pos = vadd(p->pos, gpos);
        p->pol = V3(0.f, -1.f, 0.f);
        orc_rotateUz(&p->pol, p->mom);
    }
    ph_zero_flags(p);
    ph_set_flag(p, GBO_TORCH);
}

static void mom_pol_wavelength(const orc_sim* s, orc_photon* p, orc_rng* rng)
{
    float u0 = orc_uniform(rng), u1 = orc_uniform(rng), u2 = orc_uniform(rng), u3 = orc_uniform(rng);
    float cost = 1.f - 2.f * u0;
    float sint = sqrtf((1.f - cost) * (1.f + cost));
    float phi = 2.f * ORC_PI_F * u1;
    float sinp = sinf(phi), cosp = cosf(phi);
    p->mom = V3(sint * cosp, sint * sinp, cost);
    p->pol = V3(cost * cosp, cost * sinp, -sint);
    phi = 2.f * ORC_PI_F * u2;
    sinp = sinf(phi); cosp = cosf(phi);
    v3 c = vcross(p->mom, p->pol);
    p->pol = vnormalize(V3(cosp * p->pol.x + sinp * c.x, cosp * p->pol.y + sinp * c.y, cosp * p->pol.z + sinp * c.z));
    p->wavelength = scint_wavelength(s, u3);
}

static void gen_scint(const orc_sim* s, orc_photon* p, orc_rng* rng, const gbo_quad6* g)
{
    mom_pol_wavelength(s, p, rng);
    const v3 gpos = V3(g->q[1].f[0], g->q[1].f[1], g->q[1].f[2]);
    const float gtime = g->q[1].f[3];
    const v3 dpos = V3(g->q[2].f[0], g->q[2].f[1], g->q[2].f[2]);
    const float step_length = g->q[2].f[3];
    const float charge = g->q[3].f[1];
    const float meanVelocity = g->q[3].f[3];
    const float ScintillationTime = g->q[5].f[0];
    float fraction = charge == 0.f ? 1.f : orc_uniform(rng);
    p->pos = vadd(gpos, vscale(fraction, dpos));
    float u4 = orc_uniform(rng);
    float deltaTime = fraction * step_length / meanVelocity - ScintillationTime * logf(u4);
    p->time = gtime + deltaTime;
    ph_zero_flags(p);
    ph_set_flag(p, GBO_SCINTILLATION);
}

static void gen_cerenkov(const orc_sim* s, orc_photon* p, orc_rng* rng, const gbo_quad6* g)
{
    const unsigned matline = g->q[0].u[2];
    const v3 gpos = V3(g->q[1].f[0], g->q[1].f[1], g->q[1].f[2]);
    const float gtime = g->q[1].f[3];
    const v3 dpos = V3(g->q[2].f[0], g->q[2].f[1], g->q[2].f[2]);
    const float step_length = g->q[2].f[3];
    const float preVelocity = g->q[3].f[3];
    const float BetaInverse = g->q[4].f[0], Wmin = g->q[4].f[1], Wmax = g->q[4].f[2];
    const float maxSin2 = g->q[5].f[0], M1 = g->q[5].f[1], M2 = g->q[5].f[2], postVelocity = g->q[5].f[3];

    const v3 p0 = vnormalize(dpos);
    float wavelength = 0.f, cosTheta = 0.f, sin2Theta = 0.f;
    unsigned count = 0;
    float u_maxSin2;
    do {
        float u0 = orc_uniform(rng);
        float w = Wmin + u0 * (Wmax - Wmin);
        wavelength = Wmin * Wmax / w;
        v4 props = boundary_lookup(s, wavelength, matline, 0u);
        float sampledRI = props.x;
        cosTheta = BetaInverse / sampledRI;
        sin2Theta = fmaxf(0.f, (1.f - cosTheta) * (1.f + cosTheta));
        float u1 = orc_uniform(rng);
        u_maxSin2 = u1 * maxSin2;
        count += 1;
    } while (u_maxSin2 > sin2Theta && count < 100);

    float sinTheta = sqrtf(sin2Theta);
    float u0 = orc_uniform(rng);
    float phi = 2.f * ORC_PI_F * u0;
    float sinPhi = sinf(phi), cosPhi = cosf(phi);
    p->mom = V3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
    orc_rotateUz(&p->mom, p0);
    p->pol = V3(cosTheta * cosPhi, cosTheta * sinPhi, -sinTheta);
    orc_rotateUz(&p->pol, p0);
    p->wavelength = wavelength;

    float MeanNumberOfPhotonsMax = fmaxf(M1, M2);
    float DeltaN = (M1 - M2);
    float fraction = 0.f, delta = 0.f, NumberOfPhotons, N;
    int k = 0;
    do {
        fraction = orc_uniform(rng);
        delta = fraction * step_length;
        NumberOfPhotons = M1 - fraction * DeltaN;
        float u = orc_uniform(rng);
        N = u * MeanNumberOfPhotonsMax;
        k++;
    } while (N > NumberOfPhotons && k < LOOP_CAP);

    float midVelocity = preVelocity + fraction * (postVelocity - preVelocity) * 0.5f;
    p->time = gtime + delta / midVelocity;
    p->pos = vadd(gpos, vscale(fraction, dpos));
    ph_zero_flags(p);
    ph_set_flag(p, GBO_CERENKOV);
}

/* ---- bulk, boundary and surface physics ---- */

static void rayleigh_scatter(orc_photon* p, orc_rng* rng)
{
    v3 direction = V3(0.f, 0.f, 0.f), polarization = V3(0.f, 0.f, 0.f);
    int looping = 1;
    for (int k = 0; k < LOOP_CAP && looping; k++) {
        float u0 = orc_uniform(rng), u1 = orc_uniform(rng), u2 = orc_uniform(rng),
              u3 = orc_uniform(rng), u4 = orc_uniform(rng);
        float cosTheta = u0;
        float sinTheta = sqrtf(1.0f - u0 * u0);
        if (u1 < 0.5f) cosTheta = -cosTheta;
        float phi = 2.f * ORC_PI_F * u2;
        float sinPhi = sinf(phi), cosPhi = cosf(phi);
        direction = V3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
        orc_rotateUz(&direction, p->mom);
        float constant = -vdot(direction, p->pol);
        polarization = V3(p->pol.x + constant * direction.x, p->pol.y + constant * direction.y,
                          p->pol.z + constant * direction.z);
        if (vdot(polarization, polarization) == 0.f) {
            phi = 2.f * ORC_PI_F * u3;
            sinPhi = sinf(phi); cosPhi = cosf(phi);
            polarization = V3(cosPhi, sinPhi, 0.f);
            orc_rotateUz(&polarization, direction);
        } else {
            if (u3 < 0.5f) polarization = vneg(polarization);
        }
        polarization = vnormalize(polarization);
        float doCosTheta = vdot(polarization, p->pol);
        float doCosTheta2 = doCosTheta * doCosTheta;
        looping = doCosTheta2 < u4;
    }
    p->mom = direction;
    p->pol = polarization;
}

static int propagate_to_boundary(const orc_sim* s, orc_photon* p, const orc_state* st, const gbo_prd* prd,
                                 orc_rng* rng, unsigned* flag)
{
    const float absorption_length = st->material1.y;
    const float scattering_length = st->material1.z;
    const float reemission_prob = st->material1.w;
    const float group_velocity = st->m1group2.x;
    const float distance_to_boundary = prd->q0.f[3];
    if (s->debug_tag) { (void)orc_uniform(rng); (void)orc_uniform(rng); }
    float u_scattering = orc_uniform(rng);
    float u_absorption = orc_uniform(rng);
    float scattering_distance = -scattering_length * logf(u_scattering);
    float absorption_distance = -absorption_length * logf(u_absorption);

    if (absorption_distance <= scattering_distance) {
        if (absorption_distance <= distance_to_boundary) {
            p->time += absorption_distance / group_velocity;
            p->pos = vadd(p->pos, vscale(absorption_distance, p->mom));
            float u_reemit = reemission_prob == 0.f ? 2.f : orc_uniform(rng);
            if (u_reemit < reemission_prob) {
                float u_re_wavelength = orc_uniform(rng);
                float u_re_mom_ph = orc_uniform(rng);
                float u_re_mom_ct = orc_uniform(rng);
                float u_re_pol_ph = orc_uniform(rng);
                float u_re_pol_ct = orc_uniform(rng);
                p->wavelength = scint_wavelength(s, u_re_wavelength);
                p->mom = uniform_sphere(u_re_mom_ph, u_re_mom_ct);
                p->pol = vnormalize(vcross(uniform_sphere(u_re_pol_ph, u_re_pol_ct), p->mom));
                *flag = GBO_BULK_REEMIT;
                return F_CONTINUE;
            }
            *flag = GBO_BULK_ABSORB;
            return F_BREAK;
        }
    } else {
        if (scattering_distance <= distance_to_boundary) {
            p->time += scattering_distance / group_velocity;
            p->pos = vadd(p->pos, vscale(scattering_distance, p->mom));
            rayleigh_scatter(p, rng);
            *flag = GBO_BULK_SCATTER;
            return F_CONTINUE;
        }
    }
    p->pos = vadd(p->pos, vscale(distance_to_boundary, p->mom));
    p->time += distance_to_boundary / group_velocity;
    return F_BOUNDARY;
}

static int propagate_at_boundary(const orc_sim* s, orc_photon* p, const orc_state* st, const gbo_prd* prd,
                                 orc_rng* rng, unsigned* flag)
{
    const float n1 = st->material1.x;
    const float n2 = st->material2.x;
    const float eta = n1 / n2;
    const v3 normal = V3(prd->q0.f[0], prd->q0.f[1], prd->q0.f[2]);
    const float _c1 = -vdot(p->mom, normal);
    const v3 oriented_normal = _c1 < 0.f ? vneg(normal) : normal;
    const v3 trans = vcross(p->mom, oriented_normal);
    const float trans_length = vlength(trans);
    const int normal_incidence = trans_length < 1e-6f;
    const v3 A_trans = normal_incidence ? p->pol : vdivs(trans, trans_length);
    const float E1_perp = vdot(p->pol, A_trans);
    const float c1 = fabsf(_c1);
    const float c2c2 = 1.f - eta * eta * (1.f - c1 * c1);
    const int tir = c2c2 < 0.f;
    const float EdotN = vdot(p->pol, oriented_normal);
    const float c2 = tir ? 0.f : sqrtf(c2c2);
    const float n1c1 = n1 * c1, n2c2 = n2 * c2, n2c1 = n2 * c1, n1c2 = n1 * c2;
    float E1x, E1y;
    if (normal_incidence) { E1x = 0.f; E1y = 1.f; }
    else {
        E1x = E1_perp;
        E1y = vlength(vsub(p->pol, vscale(E1_perp, A_trans)));
    }
    const float E2_tx = 2.f * n1c1 * E1x / (n1c1 + n2c2);
    const float E2_ty = 2.f * n1c1 * E1y / (n2c1 + n1c2);
    const float E2_rx = E2_tx - E1x;
    const float E2_ry = (n2 * E2_ty / n1) - E1y;
    const float rinv = 1.0f / sqrtf(E2_rx * E2_rx + E2_ry * E2_ry);
    const float RRx = E2_rx * rinv, RRy = E2_ry * rinv;
    const float tinv = 1.0f / sqrtf(E2_tx * E2_tx + E2_ty * E2_ty);
    const float TTx = E2_tx * tinv, TTy = E2_ty * tinv;
    const float TransCoeff = (tir || n1c1 == 0.f) ? 0.f : n2c2 * (E2_tx * E2_tx + E2_ty * E2_ty) / n1c1;

    if (s->debug_tag) (void)orc_uniform(rng);
    const float u_reflect = orc_uniform(rng);
    const int reflect = u_reflect > TransCoeff;

    if (reflect) p->mom = vadd(p->mom, vscale(2.0f * c1, oriented_normal));
    else p->mom = vadd(vscale(eta, p->mom), vscale(eta * c1 - c2, oriented_normal));

    const v3 A_paral = vnormalize(vcross(p->mom, A_trans));
    if (normal_incidence) {
        if (reflect) p->pol = vscale(n2 > n1 ? -1.f : 1.f, p->pol);
    } else if (reflect) {
        if (tir) p->pol = vadd(vneg(p->pol), vscale(2.f * EdotN, oriented_normal));
        else p->pol = vadd(vscale(RRx, A_trans), vscale(RRy, A_paral));
    } else {
        p->pol = vadd(vscale(TTx, A_trans), vscale(TTy, A_paral));
    }
    *flag = reflect ? GBO_BOUNDARY_REFLECT : GBO_BOUNDARY_TRANSMIT;
    if (s->debug_tag && reflect) {
        (void)orc_uniform(rng); (void)orc_uniform(rng); (void)orc_uniform(rng); (void)orc_uniform(rng);
    }
    return F_CONTINUE;
}

static v3 random_direction_marsaglia(orc_rng* rng)
{
    float u = 0.f, v = 0.f, b = 2.f;
    for (int k = 0; k < LOOP_CAP && b > 1.f; k++) {
        float u0 = orc_uniform(rng), u1 = orc_uniform(rng);
        u = 2.f * u0 - 1.f;
        v = 2.f * u1 - 1.f;
        b = u * u + v * v;
    }
    float a = 2.f * sqrtf(1.f - b);
    return V3(a * u, a * v, 2.f * b - 1.f);
}

static v3 lambertian_direction(v3 normal, float orient, orc_rng* rng)
{
    v3 dir;
    float ndotv, u;
    int count = 0;
    do {
        count++;
        dir = random_direction_marsaglia(rng);
        ndotv = vdot(dir, normal) * orient;
        if (ndotv < 0.f) { dir = vscale(-1.f, dir); ndotv = -1.f * ndotv; }
        u = orc_uniform(rng);
    } while (!(u < ndotv) && (count < 1024));
    return dir;
}

static void reflect_diffuse(orc_photon* p, const gbo_prd* prd, orc_rng* rng)
{
    v3 old_mom = p->mom;
    const v3 normal = V3(prd->q0.f[0], prd->q0.f[1], prd->q0.f[2]);
    const float orient = vdot(old_mom, normal) > 0.f ? -1.f : 1.f;
    p->mom = lambertian_direction(normal, orient, rng);
    v3 facet_normal = vnormalize(vsub(p->mom, old_mom));
    const float EdotN = vdot(p->pol, facet_normal);
    p->pol = vadd(vscale(-1.f, p->pol), vscale(2.f * EdotN, facet_normal));
}

static void reflect_specular(orc_photon* p, const gbo_prd* prd)
{
    const v3 normal = V3(prd->q0.f[0], prd->q0.f[1], prd->q0.f[2]);
    const float PdotN = vdot(p->mom, normal);
    p->mom = vsub(p->mom, vscale(2.f * PdotN, normal));
    const float EdotN = vdot(p->pol, normal);
    p->pol = vadd(vscale(-1.f, p->pol), vscale(2.f * EdotN, normal));
}

static int propagate_at_surface(const orc_sim* s, orc_photon* p, const orc_state* st, const gbo_prd* prd,
                                orc_rng* rng, unsigned* flag)
{
    const float detect = st->surface.x;
    const float absorb = st->surface.y;
    const float reflect_diffuse_ = st->surface.w;
    float u_surface = orc_uniform(rng);
    if (s->debug_tag) (void)orc_uniform(rng);
    int action = u_surface < absorb + detect ? F_BREAK : F_CONTINUE;
    if (action == F_BREAK) {
        *flag = u_surface < absorb ? GBO_SURFACE_ABSORB : GBO_SURFACE_DETECT;
    } else {
        *flag = u_surface < absorb + detect + reflect_diffuse_ ? GBO_SURFACE_DREFLECT : GBO_SURFACE_SREFLECT;
        if (*flag == GBO_SURFACE_DREFLECT) reflect_diffuse(p, prd, rng);
        else reflect_specular(p, prd);
    }
    return action;
}

static int propagate(const orc_sim* s, orc_photon* p, const gbo_prd* prd, orc_rng* rng)
{
    const unsigned boundary = prd->q1.u[3] & 0xffffu;
    const unsigned identity = prd->q1.u[2] & 0xffffu;
    const unsigned iindex = prd->q1.u[2] >> 16;
    const float lposcost = prd->q1.f[0];
    const v3 normal = V3(prd->q0.f[0], prd->q0.f[1], prd->q0.f[2]);
    float cosTheta = vdot(p->mom, normal);
    ph_set_prd(p, boundary, identity, cosTheta, iindex);
    orc_state st;
    fill_state(s, &st, boundary, p->wavelength, cosTheta);
    unsigned flag = 0;
    int command = propagate_to_boundary(s, p, &st, prd, rng, &flag);
    if (command == F_BOUNDARY) {
        const int ems = (int)st.optical[1];
        if (ems == GBO_EMS_NOSURFACE) command = propagate_at_boundary(s, p, &st, prd, rng, &flag);
        else if (ems == GBO_EMS_SURFACE) command = propagate_at_surface(s, p, &st, prd, rng, &flag);
        else if (lposcost < 0.f) command = propagate_at_surface(s, p, &st, prd, rng, &flag);
        else if (ems == GBO_EMS_ZPLUS_SENSOR_A) {
            (void)orc_uniform(rng);
            flag = GBO_SURFACE_DETECT;
            command = F_BREAK;
        }
    }
    ph_set_flag(p, flag);
    return command;
}

static inline void seq_add(gbo_seq* q, unsigned slot, unsigned flag, unsigned boundary)
{
    unsigned iseq = slot / 16u;
    unsigned shift = 4u * (slot - iseq * 16u);
    if (iseq < 2u) {
        q->seqhis[iseq] |= ((uint64_t)(__builtin_ffs((int)flag) & 0xf) << shift);
        q->seqbnd[iseq] |= ((uint64_t)(boundary & 0xfu) << shift);
    }
}

static void simulate_one(const orc_sim* s, const gbo_quad6* gsarr, const int32_t* seed,
                         const gbo_sphoton* input_photon, uint64_t photon_offset, uint32_t event_index,
                         int64_t idx, gbo_sphoton* out, gbo_seq* seqout)
{
    const int32_t genstep_idx = seed[idx];
    const gbo_quad6* g = &gsarr[genstep_idx];
    const uint64_t photon_idx = photon_offset + (uint64_t)idx;
    orc_rng rng;
    orc_rng_init(&rng, s->seed, photon_idx, s->offset);
    orc_rng_skipahead(&rng, s->skipahead_event_offset * (uint64_t)event_index);

    orc_photon p;
    memset(&p, 0, sizeof(p));
    const int gencode = g->q[0].i[0];
    switch (gencode) {
        case GBO_GS_TORCH: gen_torch(&p, &rng, g, photon_idx); break;
        case GBO_GS_G4Cerenkov_modified:
        case GBO_GS_CERENKOV: gen_cerenkov(s, &p, &rng, g); break;
        case GBO_GS_DsG4Scintillation_r4695:
        case GBO_GS_SCINTILLATION: gen_scint(s, &p, &rng, g); break;
        case GBO_GS_INPUT_PHOTON: ph_from(&p, &input_photon[photon_idx - photon_offset]); ph_set_flag(&p, GBO_TORCH); break;
        default: break;
    }
    ph_set_index(&p, photon_idx);

    gbo_seq sq;
    memset(&sq, 0, sizeof(sq));
    int bounce = 0;
    seq_add(&sq, (unsigned)bounce, ph_flag(&p), ph_boundary(&p));
    gbo_prd prd;
    memset(&prd, 0, sizeof(prd));
    while (bounce < s->max_bounce && p.time < s->max_time) {
        float tmin = (p.orient_boundary_flag & s->eps0_mask) ? s->tmin0 : s->tmin;
        orc_trace(&s->geom, p.pos, p.mom, tmin, s->tmax, &prd);
        if ((prd.q1.u[3] & 0xffffu) == 0xffffu) break;
        v3 n = vnormalize(V3(prd.q0.f[0], prd.q0.f[1], prd.q0.f[2]));
        prd.q0.f[0] = n.x; prd.q0.f[1] = n.y; prd.q0.f[2] = n.z;
        int command = propagate(s, &p, &prd, &rng);
        bounce++;
        seq_add(&sq, (unsigned)bounce, ph_flag(&p), ph_boundary(&p));
        if (command == F_BREAK) break;
    }
    ph_to(&out[idx], &p);
    if (seqout) seqout[idx] = sq;
}

typedef struct {
    const orc_sim* s; const gbo_quad6* gs; const int32_t* seed; const gbo_sphoton* input;
    uint64_t photon_offset; uint32_t event_index; int64_t begin, end;
    gbo_sphoton* out; gbo_seq* seq;
} orc_job;

static void* run_job(void* arg)
{
    orc_job* j = (orc_job*)arg;
    for (int64_t i = j->begin; i < j->end; i++)
        simulate_one(j->s, j->gs, j->seed, j->input, j->photon_offset, j->event_index, i, j->out, j->seq);
    return 0;
}

void orc_simulate(const orc_sim* s, const gbo_quad6* gs, const int32_t* seed, const gbo_sphoton* input_photon,
                  uint64_t photon_offset, uint32_t event_index, int64_t num_photon,
                  gbo_sphoton* out, gbo_seq* seq, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (num_photon < (int64_t)nthreads) nthreads = 1;
    pthread_t th[256];
    orc_job jobs[256];
    int64_t per = (num_photon + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        orc_job* j = &jobs[t];
        j->s = s; j->gs = gs; j->seed = seed; j->input = input_photon;
        j->photon_offset = photon_offset; j->event_index = event_index;
        j->begin = (int64_t)t * per;
        j->end = j->begin + per < num_photon ? j->begin + per : num_photon;
        if (j->begin > j->end) j->begin = j->end;
        j->out = out; j->seq = seq;
    }
    if (nthreads == 1) { run_job(&jobs[0]); return; }
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], 0, run_job, &jobs[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], 0);
}

int64_t orc_fill_seed(const gbo_quad6* gs, int num_gs, int32_t* seed, int64_t max_seed)
{
    int64_t n = 0;
    for (int i = 0; i < num_gs; i++) {
        int64_t np = (int64_t)gs[i].q[0].u[3];
        for (int64_t k = 0; k < np; k++) {
            if (seed && n < max_seed) seed[n] = i;
            n++;
        }
    }
    return n;
}

int64_t orc_select_hits(const gbo_sphoton* p, int64_t n, uint32_t hitmask, gbo_sphoton* hits)
{
    int64_t h = 0;
    for (int64_t i = 0; i < n; i++) {
        if ((p[i].flagmask & hitmask) == hitmask) {
            if (hits) hits[h] = p[i];
            h++;
        }
    }
    return h;
}

/* ---- hit merge (sysrap/sphoton.h:277-304 key_functor / reduce_op, sysrap/SPM.cu merge_partial_select) ----------
 * key = identity << 48 | (unsigned)(time / tw), stable sort by key, then each run of equal keys becomes the hit
 * with the earliest time (the earlier one in photon order on a tie), flagmasks ORed, hitcounts (16 bits) summed.
 * tw = 0 returns the hits unmerged (NOMERGE_TIME_WINDOW). */
typedef struct { uint64_t key; int64_t idx; } orc_keyidx;

static int cmp_keyidx(const void* a, const void* b)
{
    const orc_keyidx* x = (const orc_keyidx*)a;
    const orc_keyidx* y = (const orc_keyidx*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx ? 1 : 0);
}

static uint64_t merge_key(const gbo_sphoton* p, float tw)
{
    const unsigned id = p->identity & 0x00ffffffu;
    const unsigned bucket = (unsigned)(p->time / tw);
    return ((uint64_t)id << 48) | (uint64_t)bucket;
}

int64_t orc_merge_hits(const gbo_sphoton* in, int64_t n, float tw, gbo_sphoton* out)
{
    if (n <= 0) return 0;
    if (tw == 0.f) {
        for (int64_t i = 0; i < n; i++) out[i] = in[i];
        return n;
    }
    orc_keyidx* k = (orc_keyidx*)malloc(sizeof(orc_keyidx) * (size_t)n);
    for (int64_t i = 0; i < n; i++) { k[i].key = merge_key(&in[i], tw); k[i].idx = i; }
    qsort(k, (size_t)n, sizeof(orc_keyidx), cmp_keyidx);
    int64_t m = 0;
    for (int64_t i = 0; i < n;) {
        gbo_sphoton r = in[k[i].idx];
        int64_t j = i + 1;
        for (; j < n && k[j].key == k[i].key; j++) {
            const gbo_sphoton* b = &in[k[j].idx];
            const int a_first = fminf(r.time, b->time) == r.time;
            const unsigned fm = r.flagmask | b->flagmask;
            const unsigned hc = ((r.hitcount_iindex >> 16) + (b->hitcount_iindex >> 16)) & 0xffffu;
            if (!a_first) r = *b;
            r.flagmask = fm;
            r.hitcount_iindex = (r.hitcount_iindex & 0x0000ffffu) | (hc << 16);
        }
        out[m++] = r;
        i = j;
    }
    free(k);
    return m;
}
