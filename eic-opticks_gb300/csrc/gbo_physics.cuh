// gbo_physics.cuh : photon generation and the bulk / boundary / surface physics of one step.
//
// Each function keeps the reference's draw order and binary32 operation order (see the citation on each), so
// the engine consumes the same Philox stream as the reference GPU path and reaches the same decisions:
//   qsim::generate_photon qudarap/qsim.h:2521-2541      storch::generate sysrap/storch.h:189-516
//   qscint::generate      qudarap/qscint.h:55-145       qcerenkov::generate qudarap/qcerenkov.h:56-327
//   qsim::propagate       qudarap/qsim.h:2218-2327      qbnd::fill_state qudarap/qbnd.h:103-214
//   propagate_to_boundary qudarap/qsim.h:718-863        rayleigh_scatter qudarap/qsim.h:601-689
//   propagate_at_boundary qudarap/qsim.h:998-1205       propagate_at_surface qudarap/qsim.h:1677-1747
//   reflect_diffuse       qudarap/qsim.h:1977-2012      reflect_specular qudarap/qsim.h:2030-2082
//   lambertian_direction  qudarap/qsim.h:430-483        random_direction_marsaglia qudarap/qsim.h:551-572
// The "DEBUG_TAG" alignment draws of the reference's OptiX build (qsim.h:730-735, :1088-1091, :1188-1201,
// :1685-1691) are consumed when Params::debug_tag is set, which is the default.
// Loops the reference leaves unbounded are capped at LOOP_CAP turns (never reached with a uniform stream).
#pragma once
#include "gbo_device.cuh"

namespace gbo {

enum { CMD_BREAK = 1, CMD_CONTINUE = 2, CMD_BOUNDARY = 3 };
constexpr int LOOP_CAP = 100000;

struct Tables {
    cudaTextureObject_t bnd_tex;     // float4 (761, num_bnd*8), linear, normalized, wrap
    float bnd_nx, bnd_ny, nm0, nms;
    const float* bnd_y;              // per texture row iy: (iy + 0.5f) / bnd_ny, the row's normalized y, in binary32
    const uint4* optical;            // (num_bnd*4)
    cudaTextureObject_t icdf_tex;    // float (4096, 3)
    int hd_factor;
    int debug_tag;
};

// Precision mode keeps each photon's global position and time in binary64 and rounds them to the binary32
// record after every advance, so metre-scale paths do not accumulate binary32 rounding step by step.
struct Acc64 { double x, y, z, t; };
GBO_DEV void acc_init(Acc64& a, const Photon& p) { a.x = p.pos.x; a.y = p.pos.y; a.z = p.pos.z; a.t = p.time; }

GBO_DEV void advance(Photon& p, float d, float group_velocity, Acc64* acc)
{
    if (acc) {
        acc->t += (double)(d / group_velocity);         // the increment in binary32, its sum in binary64
        acc->x += (double)d * (double)p.mom.x;
        acc->y += (double)d * (double)p.mom.y;
        acc->z += (double)d * (double)p.mom.z;
        p.time = (float)acc->t;
        p.pos = f3((float)acc->x, (float)acc->y, (float)acc->z);
    } else {
        p.time += d / group_velocity;
        p.pos = p.pos + d * p.mom;
    }
}

struct State {
    float4 material1, m1group2, material2, surface;
    uint4 optical;
};

struct Hit {                 // per-ray intersect result, sysrap/squad.h:180-255 quad2 fields
    float3 normal;
    float t;
    // z of the intersect in the instance frame.  The reference carries lposcost = lpos.z / |lpos| and the photon
    // path reads only its sign (qsim.h:2293, `lposcost < 0.f`), which is the sign of lpos.z; the cosine itself
    // feeds the JUNO PMT surface models and the photonlite output, neither of which is on this path.
    float lposz;
    unsigned iindex_identity;
    unsigned prim_boundary;
};

GBO_DEV void rotateUz(float3& d, float3 u)     // sysrap/smath.h:77-95
{
    float up = u.x * u.x + u.y * u.y;
    if (up > 0.f) {
        up = sqrtf(up);
        const float px = d.x, py = d.y, pz = d.z;
        d.x = (u.x * u.z * px - u.y * py) / up + u.x * pz;
        d.y = (u.y * u.z * px + u.x * py) / up + u.y * pz;
        d.z = -up * px + u.z * pz;
    } else if (u.z < 0.f) {
        d.x = -d.x;
        d.z = -d.z;
    }
}

GBO_DEV float4 boundary_lookup(const Tables& t, float nm, unsigned line, unsigned k)
{
    const float fx = (nm - t.nm0) / t.nms;
    const float x = (fx + 0.5f) / t.bnd_nx;
    const unsigned iy = 2u * line + k;
    const float y = __ldg(t.bnd_y + iy);              // ((float)iy + 0.5f) / t.bnd_ny, divided once on the host
    return tex2D<float4>(t.bnd_tex, x, y);
}

GBO_DEV void fill_state(const Tables& t, State& s, unsigned boundary, float wavelength, float cosTheta)
{
    const int line = (int)boundary * 4;
    const int m1_line = cosTheta > 0.f ? line + GBO_IMAT : line + GBO_OMAT;
    const int m2_line = cosTheta > 0.f ? line + GBO_OMAT : line + GBO_IMAT;
    const int su_line = cosTheta > 0.f ? line + GBO_ISUR : line + GBO_OSUR;
    s.material1 = boundary_lookup(t, wavelength, (unsigned)m1_line, 0);
    s.m1group2 = boundary_lookup(t, wavelength, (unsigned)m1_line, 1);
    s.material2 = boundary_lookup(t, wavelength, (unsigned)m2_line, 0);
    s.surface = boundary_lookup(t, wavelength, (unsigned)su_line, 0);
    s.optical = __ldg(t.optical + su_line);
}

GBO_DEV float scint_wavelength(const Tables& t, float u0)
{
    constexpr float y0 = 0.5f / 3.f, y1 = 1.5f / 3.f, y2 = 2.5f / 3.f;
    switch (t.hd_factor) {
        case 0: return tex2D<float>(t.icdf_tex, u0, y0);
        case 10:
            if (u0 < 0.1f) return tex2D<float>(t.icdf_tex, u0 * 10.f, y1);
            if (u0 > 0.9f) return tex2D<float>(t.icdf_tex, (u0 - 0.9f) * 10.f, y2);
            return tex2D<float>(t.icdf_tex, u0, y0);
        case 20:
            if (u0 < 0.05f) return tex2D<float>(t.icdf_tex, u0 * 20.f, y1);
            if (u0 > 0.95f) return tex2D<float>(t.icdf_tex, (u0 - 0.95f) * 20.f, y2);
            return tex2D<float>(t.icdf_tex, u0, y0);
        default: return 0.f;
    }
}

GBO_DEV float3 uniform_sphere(float u0, float u1)   // qsim.h:177-183
{
    const float phi = u0 * 2.f * PI_F;
    const float cosTheta = 2.f * u1 - 1.f;
    const float sinTheta = sqrtf(1.f - cosTheta * cosTheta);
    return f3(cosf(phi) * sinTheta, sinf(phi) * sinTheta, cosTheta);
}

// ---- generators ----------------------------------------------------------------------------------------------

template <class R>
GBO_DEV void gen_torch(Photon& p, R& rng, const float4* g, uint64_t photon_id)
{
    const float4 q0 = g[0], q1 = g[1], q2 = g[2], q3 = g[3], q4 = g[4], q5 = g[5];
    const float3 gpos = f3(q1.x, q1.y, q1.z);
    const float gtime = q1.w;
    const float3 gmom = f3(q2.x, q2.y, q2.z);
    const float gwl = q3.w;
    const float zx = q4.x, zy = q4.y, ax = q4.z, ay = q4.w;
    const float radius = q5.x, distance = q5.y;
    const unsigned numphoton = __float_as_uint(q0.w);
    const unsigned type = __float_as_uint(q5.w);
    if (type == GBO_T_DISC) {
        p.wavelength = gwl; p.time = gtime; p.mom = gmom;
        const float u_zenith = zx + uniform(rng) * (zy - zx);
        const float u_azimuth = ax + uniform(rng) * (ay - ax);
        const float r = radius * u_zenith;
        const float phi = 2.f * PI_F * u_azimuth;
        const float sinPhi = sinf(phi), cosPhi = cosf(phi);
        p.pos = f3(r * cosPhi, r * sinPhi, 0.f);
        rotateUz(p.pos, p.mom);
        p.pos = p.pos + gpos;
        p.pol = f3(sinPhi, -cosPhi, 0.f);
        rotateUz(p.pol, p.mom);
    } else if (type == GBO_T_SPHERE) {
        p.wavelength = gwl; p.time = gtime;
        const float u_zenith = zx + uniform(rng) * (zy - zx);
        const float u_azimuth = ax + uniform(rng) * (ay - ax);
        const float phi = 2.f * PI_F * u_azimuth;
        const float sinPhi = sinf(phi), cosPhi = cosf(phi);
        const float cosTheta = 1.f - 2.0f * u_zenith;
        const float sinTheta = sqrtf(1.0f - cosTheta * cosTheta);
        const float flip = copysignf(1.f, radius);
        p.mom = f3(flip * sinTheta * cosPhi, flip * sinTheta * sinPhi, flip * cosTheta);
        const float rad = fabsf(radius);
        p.pos = f3(sinTheta * cosPhi * rad, sinTheta * sinPhi * rad, cosTheta * rad);
        const float phase = 2.f * PI_F * distance;
        p.pol = f3(cosf(phase), sinf(phase), 0.f);
        rotateUz(p.pol, p.mom);
    } else if (type == GBO_T_SPHERE_MARSAGLIA) {
        p.wavelength = gwl; p.time = gtime;
        float u = 0.f, v = 0.f, b = 2.f;
        for (int k = 0; k < LOOP_CAP && b > 1.f; k++) {
            const float u0 = zx + uniform(rng) * (zy - zx);
            const float u1 = ax + uniform(rng) * (ay - ax);
            u = 2.f * u0 - 1.f; v = 2.f * u1 - 1.f; b = u * u + v * v;
        }
        const float a = 2.f * sqrtf(1.f - b);
        const float rad = fabsf(radius);
        const float flip = copysignf(1.f, radius);
        p.mom = f3(flip * a * u, flip * a * v, flip * (2.f * b - 1.f));
        p.pos = f3(a * u * rad, a * v * rad, (2.f * b - 1.f) * rad);
        const float phase = 2.f * PI_F * distance;
        p.pol = f3(cosf(phase), sinf(phase), 0.f);
        rotateUz(p.pol, p.mom);
    } else if (type == GBO_T_LINE) {
        p.wavelength = gwl; p.time = gtime; p.mom = gmom;
        const float frac = (float)photon_id / (float)numphoton;
        const float sfrac = 2.f * (frac - 0.5f);
        const float r = radius * sfrac;
        p.pos = f3(r, 0.f, 0.f);
        rotateUz(p.pos, p.mom);
        p.pos = p.pos + gpos;
        p.pol = f3(0.f, -1.f, 0.f);
        rotateUz(p.pol, p.mom);
    } else if (type == GBO_T_POINT) {
        p.wavelength = gwl; p.time = gtime; p.mom = gmom;
        p.pos = f3(0.f, 0.f, 0.f);
        rotateUz(p.pos, p.mom);
        p.pos = p.pos + gpos;
        p.pol = f3(0.f, -1.f, 0.f);
        rotateUz(p.pol, p.mom);
    } else if (type == GBO_T_CIRCLE) {
        p.wavelength = gwl; p.time = gtime;
        const float f = (float)photon_id / (float)numphoton;
        const float frac = ax * (1.f - f) + ay * (f);
        const float phi = 2.f * PI_F * frac;
        const float sinPhi = sinf(phi), cosPhi = cosf(phi);
        const float r = radius < 0.f ? -radius : radius;
        p.mom = f3(radius < 0.f ? -cosPhi : cosPhi, 0.f, radius < 0.f ? -sinPhi : sinPhi);
        p.pos = f3(r * cosPhi, 0.f, r * sinPhi);
        p.pos = p.pos + gpos;
        p.pol = f3(0.f, -1.f, 0.f);
        rotateUz(p.pol, p.mom);
    } else if (type == GBO_T_RECTANGLE) {
        p.wavelength = gwl; p.time = gtime;
        const int side_size = (int)(numphoton / 4u);
        const int side = (int)(photon_id / (uint64_t)(int64_t)side_size);
        const int side_offset = side * side_size;
        const int side_index = (int)photon_id - side_offset;
        const float frac = (float)side_index / (float)side_size;
        if (side == 0 || side == 1) {
            p.pos = f3(side == 0 ? ax : ay, 0.f, (1.f - frac) * zx + frac * zy);
            p.mom = f3(side == 0 ? 1.f : -1.f, 0.f, 0.f);
        } else if (side == 2 || side == 3) {
            p.pos = f3((1.f - frac) * ax + frac * ay, 0.f, side == 2 ? zx : zy);
            p.mom = f3(0.f, 0.f, side == 2 ? 1.f : -1.f);
        }
        p.pos = p.pos + gpos;
        p.pol = f3(0.f, -1.f, 0.f);
        rotateUz(p.pol, p.mom);
    }
    zero_flags(p);
    set_flag(p, GBO_TORCH);
}

template <class R>
GBO_DEV void gen_scint(const Tables& t, Photon& p, R& rng, const float4* g)
{
    const float u0 = uniform(rng), u1 = uniform(rng), u2 = uniform(rng), u3 = uniform(rng);
    const float cost = 1.f - 2.f * u0;
    const float sint = sqrtf((1.f - cost) * (1.f + cost));
    float phi = 2.f * PI_F * u1;
    float sinp = sinf(phi), cosp = cosf(phi);
    p.mom = f3(sint * cosp, sint * sinp, cost);
    p.pol = f3(cost * cosp, cost * sinp, -sint);
    phi = 2.f * PI_F * u2;
    sinp = sinf(phi); cosp = cosf(phi);
    p.pol = normalize(cosp * p.pol + sinp * cross(p.mom, p.pol));
    p.wavelength = scint_wavelength(t, u3);

    const float4 q1 = g[1], q2 = g[2], q3 = g[3], q5 = g[5];
    const float fraction = q3.y == 0.f ? 1.f : uniform(rng);     // charge
    p.pos = f3(q1.x, q1.y, q1.z) + fraction * f3(q2.x, q2.y, q2.z);
    const float u4 = uniform(rng);
    const float deltaTime = fraction * q2.w / q3.w - q5.x * logf(u4);
    p.time = q1.w + deltaTime;
    zero_flags(p);
    set_flag(p, GBO_SCINTILLATION);
}

template <class R>
GBO_DEV void gen_cerenkov(const Tables& t, Photon& p, R& rng, const float4* g)
{
    const float4 q0 = g[0], q1 = g[1], q2 = g[2], q3 = g[3], q4 = g[4], q5 = g[5];
    const unsigned matline = __float_as_uint(q0.z);
    const float3 dpos = f3(q2.x, q2.y, q2.z);
    const float step_length = q2.w;
    const float preVelocity = q3.w;
    const float BetaInverse = q4.x, Wmin = q4.y, Wmax = q4.z;
    const float maxSin2 = q5.x, M1 = q5.y, M2 = q5.z, postVelocity = q5.w;

    const float3 p0 = normalize(dpos);
    float wavelength, cosTheta, sin2Theta, u_maxSin2;
    unsigned count = 0;
    do {
        const float u0 = uniform(rng);
        const float w = Wmin + u0 * (Wmax - Wmin);
        wavelength = Wmin * Wmax / w;
        const float4 props = boundary_lookup(t, wavelength, matline, 0u);
        cosTheta = BetaInverse / props.x;
        sin2Theta = fmaxf(0.f, (1.f - cosTheta) * (1.f + cosTheta));
        const float u1 = uniform(rng);
        u_maxSin2 = u1 * maxSin2;
        count += 1;
    } while (u_maxSin2 > sin2Theta && count < 100);

    const float sinTheta = sqrtf(sin2Theta);
    const float u0 = uniform(rng);
    const float phi = 2.f * PI_F * u0;
    const float sinPhi = sinf(phi), cosPhi = cosf(phi);
    p.mom = f3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
    rotateUz(p.mom, p0);
    p.pol = f3(cosTheta * cosPhi, cosTheta * sinPhi, -sinTheta);
    rotateUz(p.pol, p0);
    p.wavelength = wavelength;

    const float MeanNumberOfPhotonsMax = fmaxf(M1, M2);
    const float DeltaN = (M1 - M2);
    float fraction, delta, NumberOfPhotons, N;
    int k = 0;
    do {
        fraction = uniform(rng);
        delta = fraction * step_length;
        NumberOfPhotons = M1 - fraction * DeltaN;
        const float u = uniform(rng);
        N = u * MeanNumberOfPhotonsMax;
        k++;
    } while (N > NumberOfPhotons && k < LOOP_CAP);

    const float midVelocity = preVelocity + fraction * (postVelocity - preVelocity) * 0.5f;
    p.time = q1.w + delta / midVelocity;
    p.pos = f3(q1.x, q1.y, q1.z) + fraction * dpos;
    zero_flags(p);
    set_flag(p, GBO_CERENKOV);
}

// ---- physics of one step -------------------------------------------------------------------------------------

template <class R>
GBO_DEV void rayleigh_scatter(Photon& p, R& rng)
{
    float3 direction = f3(0.f, 0.f, 0.f), polarization = f3(0.f, 0.f, 0.f);
    bool looping = true;
    for (int k = 0; k < LOOP_CAP && looping; k++) {
        const float u0 = uniform(rng), u1 = uniform(rng), u2 = uniform(rng), u3 = uniform(rng), u4 = uniform(rng);
        float cosTheta = u0;
        const float sinTheta = sqrtf(1.0f - u0 * u0);
        if (u1 < 0.5f) cosTheta = -cosTheta;
        float sinPhi, cosPhi;
        sincosf(2.f * PI_F * u2, &sinPhi, &cosPhi);
        direction = f3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
        rotateUz(direction, p.mom);
        const float constant = -dot(direction, p.pol);
        polarization = f3(p.pol.x + constant * direction.x, p.pol.y + constant * direction.y,
                          p.pol.z + constant * direction.z);
        if (dot(polarization, polarization) == 0.f) {
            sincosf(2.f * PI_F * u3, &sinPhi, &cosPhi);
            polarization = f3(cosPhi, sinPhi, 0.f);
            rotateUz(polarization, direction);
        } else if (u3 < 0.5f) {
            polarization = -polarization;
        }
        polarization = normalize(polarization);
        const float doCosTheta = dot(polarization, p.pol);
        looping = doCosTheta * doCosTheta < u4;
    }
    p.mom = direction;
    p.pol = polarization;
}

template <class R>
GBO_DEV int propagate_to_boundary(const Tables& t, Photon& p, const State& s, float distance_to_boundary, R& rng,
                                  unsigned& flag, Acc64* acc = nullptr)
{
    const float absorption_length = s.material1.y;
    const float scattering_length = s.material1.z;
    const float reemission_prob = s.material1.w;
    const float group_velocity = s.m1group2.x;
    if (t.debug_tag) skip(rng, 2);
    const float u_scattering = uniform(rng);
    const float u_absorption = uniform(rng);
    const float scattering_distance = -scattering_length * logf(u_scattering);
    const float absorption_distance = -absorption_length * logf(u_absorption);

    if (absorption_distance <= scattering_distance) {
        if (absorption_distance <= distance_to_boundary) {
            advance(p, absorption_distance, group_velocity, acc);
            const float u_reemit = reemission_prob == 0.f ? 2.f : uniform(rng);
            if (GBO_UNLIKELY(u_reemit < reemission_prob)) {
                const float u_re_wavelength = uniform(rng);
                const float u_re_mom_ph = uniform(rng);
                const float u_re_mom_ct = uniform(rng);
                const float u_re_pol_ph = uniform(rng);
                const float u_re_pol_ct = uniform(rng);
                p.wavelength = scint_wavelength(t, u_re_wavelength);
                p.mom = uniform_sphere(u_re_mom_ph, u_re_mom_ct);
                p.pol = normalize(cross(uniform_sphere(u_re_pol_ph, u_re_pol_ct), p.mom));
                flag = GBO_BULK_REEMIT;
                return CMD_CONTINUE;
            }
            flag = GBO_BULK_ABSORB;
            return CMD_BREAK;
        }
    } else if (GBO_UNLIKELY(scattering_distance <= distance_to_boundary)) {
        advance(p, scattering_distance, group_velocity, acc);
        rayleigh_scatter(p, rng);
        flag = GBO_BULK_SCATTER;
        return CMD_CONTINUE;
    }
    advance(p, distance_to_boundary, group_velocity, acc);
    return CMD_BOUNDARY;
}

template <class R>
GBO_DEV int propagate_at_boundary(const Tables& t, Photon& p, const State& s, float3 normal, R& rng, unsigned& flag)
{
    const float n1 = s.material1.x;
    const float n2 = s.material2.x;
    const float eta = n1 / n2;
    const float _c1 = -dot(p.mom, normal);
    const float3 oriented_normal = _c1 < 0.f ? -normal : normal;
    const float3 trans = cross(p.mom, oriented_normal);
    const float trans_length = length(trans);
    const bool normal_incidence = trans_length < 1e-6f;
    const float3 A_trans = normal_incidence ? p.pol : divs(trans, trans_length);
    const float E1_perp = dot(p.pol, A_trans);
    const float c1 = fabsf(_c1);
    const float c2c2 = 1.f - eta * eta * (1.f - c1 * c1);
    const bool tir = c2c2 < 0.f;
    const float EdotN = dot(p.pol, oriented_normal);
    const float c2 = tir ? 0.f : sqrtf(c2c2);
    const float n1c1 = n1 * c1, n2c2 = n2 * c2, n2c1 = n2 * c1, n1c2 = n1 * c2;
    const float E1x = normal_incidence ? 0.f : E1_perp;
    const float E1y = normal_incidence ? 1.f : length(p.pol - (E1_perp * A_trans));
    const float E2_tx = 2.f * n1c1 * E1x / (n1c1 + n2c2);
    const float E2_ty = 2.f * n1c1 * E1y / (n2c1 + n1c2);
    const float E2_rx = E2_tx - E1x;
    const float E2_ry = (n2 * E2_ty / n1) - E1y;
    const float rinv = 1.0f / sqrtf(E2_rx * E2_rx + E2_ry * E2_ry);
    const float tinv = 1.0f / sqrtf(E2_tx * E2_tx + E2_ty * E2_ty);
    const float RRx = E2_rx * rinv, RRy = E2_ry * rinv;
    const float TTx = E2_tx * tinv, TTy = E2_ty * tinv;
    const float TransCoeff = (tir || n1c1 == 0.f) ? 0.f : n2c2 * (E2_tx * E2_tx + E2_ty * E2_ty) / n1c1;

    if (t.debug_tag) skip(rng, 1);
    const float u_reflect = uniform(rng);
    const bool reflect = u_reflect > TransCoeff;

    p.mom = reflect ? p.mom + (2.0f * c1) * oriented_normal
                    : eta * p.mom + (eta * c1 - c2) * oriented_normal;
    const float3 A_paral = normalize(cross(p.mom, A_trans));
    if (normal_incidence) {
        if (reflect) p.pol = p.pol * (n2 > n1 ? -1.f : 1.f);
    } else if (reflect) {
        p.pol = tir ? -p.pol + (2.f * EdotN) * oriented_normal : RRx * A_trans + RRy * A_paral;
    } else {
        p.pol = TTx * A_trans + TTy * A_paral;
    }
    flag = reflect ? GBO_BOUNDARY_REFLECT : GBO_BOUNDARY_TRANSMIT;
    if (t.debug_tag && reflect) skip(rng, 4);
    return CMD_CONTINUE;
}

template <class R>
GBO_DEV float3 random_direction_marsaglia(R& rng)
{
    float u = 0.f, v = 0.f, b = 2.f;
    for (int k = 0; k < LOOP_CAP && b > 1.f; k++) {
        const float u0 = uniform(rng), u1 = uniform(rng);
        u = 2.f * u0 - 1.f;
        v = 2.f * u1 - 1.f;
        b = u * u + v * v;
    }
    const float a = 2.f * sqrtf(1.f - b);
    return f3(a * u, a * v, 2.f * b - 1.f);
}

template <class R>
GBO_DEV int propagate_at_surface(const Tables& t, Photon& p, const State& s, float3 normal, R& rng, unsigned& flag)
{
    const float detect = s.surface.x;
    const float absorb = s.surface.y;
    const float reflect_diffuse_ = s.surface.w;
    const float u_surface = uniform(rng);
    if (t.debug_tag) skip(rng, 1);
    const int action = u_surface < absorb + detect ? CMD_BREAK : CMD_CONTINUE;
    if (action == CMD_BREAK) {
        flag = u_surface < absorb ? GBO_SURFACE_ABSORB : GBO_SURFACE_DETECT;
    } else if (GBO_UNLIKELY(u_surface < absorb + detect + reflect_diffuse_)) {
        flag = GBO_SURFACE_DREFLECT;
        const float3 old_mom = p.mom;
        const float orient = dot(old_mom, normal) > 0.f ? -1.f : 1.f;
        float3 dir;
        float ndotv, u;
        int count = 0;
        do {
            count++;
            dir = random_direction_marsaglia(rng);
            ndotv = dot(dir, normal) * orient;
            if (ndotv < 0.f) { dir = -1.f * dir; ndotv = -1.f * ndotv; }
            u = uniform(rng);
        } while (!(u < ndotv) && (count < 1024));
        p.mom = dir;
        const float3 facet_normal = normalize(p.mom - old_mom);
        const float EdotN = dot(p.pol, facet_normal);
        p.pol = -1.f * p.pol + (2.f * EdotN) * facet_normal;
    } else {
        flag = GBO_SURFACE_SREFLECT;
        const float PdotN = dot(p.mom, normal);
        p.mom = p.mom - (2.f * PdotN) * normal;
        const float EdotN = dot(p.pol, normal);
        p.pol = -1.f * p.pol + (2.f * EdotN) * normal;
    }
    return action;
}

// qsim::propagate : one step given the normalized intersect
template <class R>
GBO_DEV int propagate(const Tables& t, Photon& p, const Hit& h, R& rng, Acc64* acc = nullptr)
{
    const unsigned boundary = h.prim_boundary & 0xffffu;
    const unsigned identity = h.iindex_identity & 0xffffu;
    const unsigned iindex = h.iindex_identity >> 16;
    const float cosTheta = dot(p.mom, h.normal);
    set_prd(p, boundary, identity, cosTheta, iindex);
    State s;
    fill_state(t, s, boundary, p.wavelength, cosTheta);
    unsigned flag = 0;
    int command = propagate_to_boundary(t, p, s, h.t, rng, flag, acc);
    if (command == CMD_BOUNDARY) {
        const int ems = (int)s.optical.y;
        // qsim.h:2284-2305: a surface, or the back (lpos z < 0) of a z-plus sensor, takes propagate_at_surface (one
        // call site, so its code is inlined once)
        if (ems == GBO_EMS_NOSURFACE) command = propagate_at_boundary(t, p, s, h.normal, rng, flag);
        else if (ems == GBO_EMS_SURFACE || h.lposz < 0.f) command = propagate_at_surface(t, p, s, h.normal, rng, flag);
        else if (GBO_UNLIKELY(ems == GBO_EMS_ZPLUS_SENSOR_A)) {
            skip(rng, 1);
            flag = GBO_SURFACE_DETECT;
            command = CMD_BREAK;
        }
    }
    set_flag(p, flag);
    return command;
}

}  // namespace gbo
