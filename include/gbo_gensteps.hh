// gbo_gensteps.hh : header-only C++ genstep producers for a Geant4 application's stepping actions, without Geant4
// types in the signatures.
//
// The reference fills its gensteps from G4Track / G4Step inside U4::CollectGenstep_DsG4Scintillation_r4695 and
// U4::CollectGenstep_G4Cerenkov_modified (u4/U4.cc:82-305) and appends them with SEvt::AddGenstep.  The same
// quad6 payloads (sysrap/sscint.h:34-62, sysrap/scerenkov.h:29-58) are produced here from plain values a stepping
// action reads off its G4Step:
//
//     gbo::StepPoints sp;                      // pre/post position (mm), global time (ns), velocity (mm/ns)
//     sp.pre = {{x0.x(), x0.y(), x0.z()}, pre->GetGlobalTime(), pre->GetVelocity()};  ...
//     gbo::SEvt::AddGenstep(gbo::MakeGenstep_DsG4Scintillation_r4695(track, sp, matline, n, scnt, tau));
//
// `matline` is the boundary-texture line of the step's material (4 * boundary + 3 for a boundary whose inner
// material it is); the reference maps Geant4 material indices to those lines in SEvt::setGenstep.
// CerenkovMeanPhotonsPerMM restates the Cerenkov yield of u4/Local_G4Cerenkov_modified.cc
// (GetAverageNumberOfPhotons): 369.81 photons / (eV cm) x charge^2 x the integral over photon energy of
// (1 - 1/(beta n)^2) where beta n > 1, with n(E) linear between the table points and the threshold crossings
// solved on each segment (n need not be monotonic).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gbopticks.h"

namespace gbo {

struct StepPoint {
    double pos[3];      // mm
    double time;        // global time, ns
    double velocity;    // mm/ns
};

struct StepPoints {
    StepPoint pre, post;
    double step_length = -1.0;  // G4Step::GetStepLength (mm): the true path length, which exceeds the chord |post - pre|
                                // for steps bent by a field or by multiple scattering; < 0 takes the chord
};

struct TrackInfo {
    int32_t trackid = 0;
    int32_t pdg_code = 0;
    double charge = 0.0;    // units of the positron charge
    double weight = 1.0;
};

constexpr double HC_EVNM = 1239.8418754200;       // h c in eV nm (sysrap/smath.h)

// Geant4's internal units and the two constants u4/U4.cc uses for Wmin / Wmax (h_Planck * c_light / p / nm, p in MeV):
// the SI 2019 definitions in CLHEP's units (mm, ns, MeV), each built in the order CLHEP's headers build it.
namespace clhep {
constexpr double MeV = 1.0, eV = 1.e-6 * MeV, e_SI = 1.602176634e-19, joule = eV / e_SI;
constexpr double ns = 1.0, s = 1.e+9 * ns, mm = 1.0, m = 1000. * mm, nm = 1.e-9 * m;
constexpr double h_Planck = 6.62607015e-34 * joule * s;
constexpr double c_light = 2.99792458e+8 * m / s;
}  // namespace clhep

namespace detail {
inline void put_f(gbo_quad6& g, int q, int c, double v) { g.q[q].f[c] = (float)v; }
inline void put_u(gbo_quad6& g, int q, int c, uint32_t v) { g.q[q].u[c] = v; }
inline void put_i(gbo_quad6& g, int q, int c, int32_t v) { g.q[q].i[c] = v; }

inline void common(gbo_quad6& g, uint32_t gentype, const TrackInfo& t, const StepPoints& s, uint32_t matline,
                   int32_t numphoton)
{
    std::memset(&g, 0, sizeof(g));
    put_u(g, 0, 0, gentype);
    put_u(g, 0, 1, (uint32_t)t.trackid);
    put_u(g, 0, 2, matline);
    put_u(g, 0, 3, (uint32_t)numphoton);
    for (int k = 0; k < 3; k++) put_f(g, 1, k, s.pre.pos[k]);
    put_f(g, 1, 3, s.pre.time);
    double len2 = 0.0;
    for (int k = 0; k < 3; k++) {
        const double d = s.post.pos[k] - s.pre.pos[k];       // G4Step::GetDeltaPosition, not normalized
        put_f(g, 2, k, d);
        len2 += d * d;
    }
    put_f(g, 2, 3, s.step_length >= 0.0 ? s.step_length : std::sqrt(len2));      // G4Step::GetStepLength
    put_i(g, 3, 0, t.pdg_code);
    put_f(g, 3, 1, t.charge);
    put_f(g, 3, 2, t.weight);
}
}  // namespace detail

// sscint layout: q3.w meanVelocity, q4.x scnt, q5.x ScintillationTime (u4/U4.cc:82-140)
inline gbo_quad6 MakeGenstep_DsG4Scintillation_r4695(const TrackInfo& t, const StepPoints& s, uint32_t matline,
                                                      int32_t numPhotons, int32_t scnt, double ScintillationTime)
{
    gbo_quad6 g;
    detail::common(g, GBO_GS_DsG4Scintillation_r4695, t, s, matline, numPhotons);
    detail::put_f(g, 3, 3, 0.5 * (s.pre.velocity + s.post.velocity));
    detail::put_i(g, 4, 0, scnt);
    detail::put_f(g, 5, 0, ScintillationTime);
    return g;
}

// scerenkov layout: q3.w preVelocity, q4 (BetaInverse, Wmin, Wmax, maxCos), q5 (maxSin2, MeanNumberOfPhotons1,
// MeanNumberOfPhotons2, postVelocity); Wmin/Wmax in nm from the photon energy range pmin/pmax in eV, converted as
// u4/U4.cc:200-260 converts Geant4's MeV values (h_Planck * c_light / p / nm)
inline gbo_quad6 MakeGenstep_G4Cerenkov_modified(const TrackInfo& t, const StepPoints& s, uint32_t matline,
                                                  int32_t numPhotons, double betaInverse, double pmin_eV,
                                                  double pmax_eV, double maxCos, double maxSin2,
                                                  double meanNumberOfPhotons1, double meanNumberOfPhotons2)
{
    gbo_quad6 g;
    detail::common(g, GBO_GS_G4Cerenkov_modified, t, s, matline, numPhotons);
    detail::put_f(g, 3, 3, s.pre.velocity);
    detail::put_f(g, 4, 0, betaInverse);
    detail::put_f(g, 4, 1, clhep::h_Planck * clhep::c_light / (pmax_eV * clhep::eV) / clhep::nm);
    detail::put_f(g, 4, 2, clhep::h_Planck * clhep::c_light / (pmin_eV * clhep::eV) / clhep::nm);
    detail::put_f(g, 4, 3, maxCos);
    detail::put_f(g, 5, 0, maxSin2);
    detail::put_f(g, 5, 1, meanNumberOfPhotons1);
    detail::put_f(g, 5, 2, meanNumberOfPhotons2);
    detail::put_f(g, 5, 3, s.post.velocity);
    return g;
}

// Mean Cerenkov photons per mm for a particle of `charge` and `beta` in a medium with refractive index n(E) given at
// increasing photon energies (eV).
inline double CerenkovMeanPhotonsPerMM(double charge, double beta, const double* energy_eV, const double* rindex,
                                       int n)
{
    if (beta <= 0.0 || n < 2) return 0.0;
    const double bi2 = 1.0 / (beta * beta);
    double integral = 0.0;
    for (int i = 0; i + 1 < n; i++) {
        const double e0 = energy_eV[i], e1 = energy_eV[i + 1];
        const double n0 = rindex[i], n1 = rindex[i + 1];
        if (e1 <= e0) continue;
        // f(E) = 1 - bi2 / n(E)^2 over the part of [e0, e1] where n(E) > 1/beta (n linear in E)
        const double thr = 1.0 / beta;
        double a = e0, b = e1;
        const bool in0 = n0 > thr, in1 = n1 > thr;
        if (!in0 && !in1) continue;
        if (in0 != in1) {
            const double ec = e0 + (thr - n0) * (e1 - e0) / (n1 - n0);      // crossing of n = 1/beta
            if (in0) b = ec; else a = ec;
        }
        // exact integral of 1 - bi2 / (p + q E)^2 with n = p + q E on [a, b]
        const double q = (n1 - n0) / (e1 - e0);
        const double p = n0 - q * e0;
        const double na = p + q * a, nb = p + q * b;
        const double inv = std::fabs(q) > 0.0 ? (1.0 / na - 1.0 / nb) / q : (b - a) / (na * na);
        integral += (b - a) - bi2 * inv;
    }
    return 36.981 * charge * charge * integral;            // 369.81 / (eV cm) = 36.981 / (eV mm)
}

// Cerenkov step quantities from the medium's n(E) and the pre/post velocities, as G4Cerenkov_modified prepares them:
// BetaInverse at the pre point, maxCos = BetaInverse / nMax, maxSin2 = (1 - maxCos)(1 + maxCos), the mean photon
// numbers at the pre and post betas for the step length, energy range of the table.
inline gbo_quad6 MakeGenstep_Cerenkov_FromTable(const TrackInfo& t, const StepPoints& s, uint32_t matline,
                                                int32_t numPhotons, const double* energy_eV, const double* rindex,
                                                int n)
{
    const double c = 299.792458;
    const double beta_pre = s.pre.velocity / c, beta_post = s.post.velocity / c;
    double nmax = rindex[0];
    for (int i = 1; i < n; i++) nmax = rindex[i] > nmax ? rindex[i] : nmax;
    const double bi = 1.0 / beta_pre;
    const double maxCos = bi / nmax;
    double len2 = 0.0;
    for (int k = 0; k < 3; k++) len2 += (s.post.pos[k] - s.pre.pos[k]) * (s.post.pos[k] - s.pre.pos[k]);
    const double step = s.step_length >= 0.0 ? s.step_length : std::sqrt(len2);
    const double m1 = CerenkovMeanPhotonsPerMM(t.charge, beta_pre, energy_eV, rindex, n) * step;
    const double m2 = CerenkovMeanPhotonsPerMM(t.charge, beta_post, energy_eV, rindex, n) * step;
    return MakeGenstep_G4Cerenkov_modified(t, s, matline, numPhotons, bi, energy_eV[0], energy_eV[n - 1], maxCos,
                                           (1.0 - maxCos) * (1.0 + maxCos), m1, m2);
}

// ---- torch gensteps : storch::FillGenstep (sysrap/storch.h:104-146) ----------------------------------------------
// The reference's test and demo gensteps: every field from an environment key with the same default
// (storch_FillGenstep_pos "0,0,-90", _time "0.0", _mom "0,0,1" then normalized in binary32, _wavelength "420",
// _distance "0", _weight "0", _zenith "0,1", _azimuth "0,1", _radius "50", _type "disc"; mode 255).  Type names
// as sysrap/storchtype.h: undef disc line point circle rectangle sphere_marsaglia sphere.

struct TorchParams {
    float pos[3] = {0.f, 0.f, -90.f};
    float time = 0.f;
    float mom[3] = {0.f, 0.f, 1.f};
    float weight = 0.f;
    float wavelength = 420.f;
    float zenith[2] = {0.f, 1.f};
    float azimuth[2] = {0.f, 1.f};
    float radius = 50.f;
    float distance = 0.f;
    uint32_t type = GBO_T_DISC;
};

inline uint32_t TorchType(const char* name)
{
    static const char* names[] = {"undef", "disc", "line", "point", "circle", "rectangle", "sphere_marsaglia", "sphere"};
    for (uint32_t k = 0; k < 8; k++)
        if (std::strcmp(name, names[k]) == 0) return k;
    return 0;
}

namespace detail {
// comma-separated values of an environment key into v[0..n) (missing values keep their defaults)
inline void env_floats(const char* key, float* v, int n)
{
    const char* s = std::getenv(key);
    if (!s) return;
    for (int k = 0; k < n && *s; k++) {
        char* end = nullptr;
        const float x = std::strtof(s, &end);
        if (end == s) break;
        v[k] = x;
        s = *end == ',' ? end + 1 : end;
    }
}
}  // namespace detail

// the parameters with the reference's storch_FillGenstep_* environment overrides applied; type 0 (undef) when
// storch_FillGenstep_type names no torch type (the reference asserts)
inline TorchParams TorchParamsFromEnv()
{
    TorchParams p;
    detail::env_floats("storch_FillGenstep_pos", p.pos, 3);
    detail::env_floats("storch_FillGenstep_time", &p.time, 1);
    detail::env_floats("storch_FillGenstep_mom", p.mom, 3);
    detail::env_floats("storch_FillGenstep_wavelength", &p.wavelength, 1);
    detail::env_floats("storch_FillGenstep_distance", &p.distance, 1);
    detail::env_floats("storch_FillGenstep_weight", &p.weight, 1);
    detail::env_floats("storch_FillGenstep_zenith", p.zenith, 2);
    detail::env_floats("storch_FillGenstep_azimuth", p.azimuth, 2);
    detail::env_floats("storch_FillGenstep_radius", &p.radius, 1);
    if (const char* t = std::getenv("storch_FillGenstep_type")) p.type = TorchType(t);
    return p;
}

inline gbo_quad6 MakeGenstep_Torch(const TorchParams& p, int32_t numphoton)
{
    gbo_quad6 g;
    std::memset(&g, 0, sizeof(g));
    detail::put_u(g, 0, 0, GBO_GS_TORCH);
    detail::put_i(g, 0, 3, numphoton);
    for (int k = 0; k < 3; k++) g.q[1].f[k] = p.pos[k];
    g.q[1].f[3] = p.time;
    // normalize(float3) of the reference's smath: binary32 components over the binary32 length
    const float len = std::sqrt(p.mom[0] * p.mom[0] + p.mom[1] * p.mom[1] + p.mom[2] * p.mom[2]);
    const float inv = 1.f / len;
    for (int k = 0; k < 3; k++) g.q[2].f[k] = p.mom[k] * inv;
    g.q[2].f[3] = p.weight;
    g.q[3].f[3] = p.wavelength;
    g.q[4].f[0] = p.zenith[0];
    g.q[4].f[1] = p.zenith[1];
    g.q[4].f[2] = p.azimuth[0];
    g.q[4].f[3] = p.azimuth[1];
    g.q[5].f[0] = p.radius;
    g.q[5].f[1] = p.distance;
    detail::put_u(g, 5, 2, 255u);
    detail::put_u(g, 5, 3, p.type);
    return g;
}

}  // namespace gbo
