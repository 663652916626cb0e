// Gensteps of include/gbo_gensteps.hh for seeded random step values, and for the values of the reference's demo
// gensteps (sscint::FillGenstep, scerenkov::FillGenstep), written to the directory given as argv[1]:
//   inputs.bin : per random step 24 doubles (pre x y z t v, post x y z t v, step_length, charge, weight,
//                ScintillationTime, betaInverse, pmin_eV, pmax_eV, maxCos, maxSin2, MeanNumberOfPhotons1,
//                MeanNumberOfPhotons2, then trackid, pdg_code, matline as doubles) and 2 ints (numPhotons, scnt)
//   gs.bin     : per random step its scintillation then its Cerenkov genstep; then the two demo gensteps
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "G4CXOpticks_gb.hh"

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    const int n = argc > 2 ? std::atoi(argv[2]) : 1000;
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    std::vector<double> in;
    std::vector<int32_t> ints;
    std::vector<gbo_quad6> gs;
    for (int i = 0; i < n; i++) {
        gbo::TrackInfo t;
        gbo::StepPoints s;
        for (int k = 0; k < 3; k++) s.pre.pos[k] = 5000.0 * u(rng);
        for (int k = 0; k < 3; k++) s.post.pos[k] = s.pre.pos[k] + 3.0 * u(rng);
        s.pre.time = 100.0 * (1.0 + u(rng));
        s.post.time = s.pre.time + 0.01 * (1.0 + u(rng));
        s.pre.velocity = 150.0 * (1.0 + u(rng));
        s.post.velocity = 150.0 * (1.0 + u(rng));
        s.step_length = i % 3 == 0 ? -1.0 : 4.0 * (1.0 + u(rng));        // every third step: the chord
        t.charge = i % 2 ? -1.0 : 1.0;
        t.weight = 1.0 + 0.5 * u(rng);
        t.trackid = 1 + i;
        t.pdg_code = i % 2 ? 11 : -13;
        const double tau = 50.0 * (1.0 + u(rng));
        const double bi = 1.0 + 0.4 * (1.0 + u(rng)), pmin = 1.5 + 0.2 * u(rng), pmax = 6.0 + 3.0 * u(rng);
        const double maxCos = bi / 1.5, maxSin2 = (1.0 - maxCos) * (1.0 + maxCos);
        const double m1 = 50.0 * (1.0 + u(rng)), m2 = 50.0 * (1.0 + u(rng));
        const uint32_t matline = (uint32_t)(4 * i + 3);
        const int32_t np = 1 + i * 7, scnt = i % 2;
        gs.push_back(gbo::MakeGenstep_DsG4Scintillation_r4695(t, s, matline, np, scnt, tau));
        gs.push_back(gbo::MakeGenstep_G4Cerenkov_modified(t, s, matline, np, bi, pmin, pmax, maxCos, maxSin2, m1, m2));
        const double v[24] = {s.pre.pos[0], s.pre.pos[1], s.pre.pos[2], s.pre.time, s.pre.velocity,
                              s.post.pos[0], s.post.pos[1], s.post.pos[2], s.post.time, s.post.velocity,
                              s.step_length, t.charge, t.weight, tau, bi, pmin, pmax, maxCos, maxSin2, m1, m2,
                              (double)t.trackid, (double)t.pdg_code, (double)matline};
        in.insert(in.end(), v, v + 24);
        ints.push_back(np);
        ints.push_back(scnt);
    }
    // the reference's demo values: pos 100, time 20, DeltaPosition 1000 each, step_length 1000, code 1, charge 1,
    // weight 1, velocity 10 (scintillation: mean velocity; Cerenkov: 10 before, 20 after), ScintillationTime 10;
    // Cerenkov BetaInverse 1.5, photon energies 1.55 .. 15.5 eV, maxCos = 1.5 / 1.793 in binary32
    gbo::TrackInfo t;
    t.trackid = 0; t.pdg_code = 1; t.charge = 1.0; t.weight = 1.0;
    gbo::StepPoints s;
    s.pre = {{100.0, 100.0, 100.0}, 20.0, 10.0};
    s.post = {{1100.0, 1100.0, 1100.0}, 20.0, 10.0};
    s.step_length = 1000.0;
    gs.push_back(gbo::MakeGenstep_DsG4Scintillation_r4695(t, s, 0, n, 0, 10.0));
    s.post.velocity = 20.0;
    const float maxCos = 1.5f / 1.793f, maxSin2 = (1.f - maxCos) * (1.f + maxCos);
    gs.push_back(gbo::MakeGenstep_G4Cerenkov_modified(t, s, 3, n, 1.5, 1.55, 15.5, maxCos, maxSin2, 100.0, 200.0));
    FILE* f = std::fopen((dir + "/inputs.bin").c_str(), "wb");
    std::fwrite(in.data(), sizeof(double), in.size(), f);
    std::fwrite(ints.data(), sizeof(int32_t), ints.size(), f);
    std::fclose(f);
    f = std::fopen((dir + "/gs.bin").c_str(), "wb");
    std::fwrite(gs.data(), sizeof(gbo_quad6), gs.size(), f);
    std::fclose(f);
    // U4::CollectGenstep_* with the reference's DISABLE / ZEROPHO switches (environment of this process)
    gbo::U4::CollectGenstep_DsG4Scintillation_r4695(t, s, 0, 77, 0, 10.0);
    gbo::U4::CollectGenstep_G4Cerenkov_modified(t, s, 3, 88, 1.5, 1.55, 15.5, maxCos, maxSin2, 100.0, 200.0);
    std::printf("%lld", (long long)gbo::SEvt::GetNumGenstepFromGenstep(0));
    for (const gbo_quad6& q : gbo::SEvt::GetGenstep(0)) std::printf(" %u:%u", q.q[0].u[0], q.q[0].u[3]);
    std::printf("\n");
    return 0;
}
