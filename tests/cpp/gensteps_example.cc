// Writes gensteps made by include/gbo_gensteps.hh for fixed step values (scintillation, Cerenkov, and a torch
// genstep from the storch_FillGenstep_* environment), and the Cerenkov yield on a table, to the directory given as
// argv[1] (gs.bin: quad6 records; yield.txt: photons per mm at several betas).
#include <cstdio>
#include <string>
#include <vector>

#include "gbo_gensteps.hh"

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    // water n(E): 36 points from 200 to 700 nm, 1.360 at 200 nm falling linearly to 1.330 at 700 nm
    std::vector<double> e, n;
    for (int i = 35; i >= 0; i--) {
        const double wl = 200.0 + 500.0 * i / 35.0;
        e.push_back(gbo::HC_EVNM / wl);
        n.push_back(1.330 + 0.030 * (700.0 - wl) / 500.0);
    }
    gbo::TrackInfo t;
    t.trackid = 7; t.pdg_code = 13; t.charge = -1.0; t.weight = 1.0;
    gbo::StepPoints s;
    s.pre = {{10.0, -20.0, 30.0}, 1.5, 0.95 * 299.792458};
    s.post = {{10.6, -19.2, 31.5}, 1.508, 0.93 * 299.792458};
    std::vector<gbo_quad6> gs;
    gs.push_back(gbo::MakeGenstep_DsG4Scintillation_r4695(t, s, 11, 4321, 1, 12.5));
    gs.push_back(gbo::MakeGenstep_Cerenkov_FromTable(t, s, 7, 55, e.data(), n.data(), (int)n.size()));
    gs.push_back(gbo::MakeGenstep_Torch(gbo::TorchParamsFromEnv(), 1000));      // storch_FillGenstep_* from the env
    FILE* f = std::fopen((dir + "/gs.bin").c_str(), "wb");
    std::fwrite(gs.data(), sizeof(gbo_quad6), gs.size(), f);
    std::fclose(f);
    f = std::fopen((dir + "/yield.txt").c_str(), "w");
    for (double beta : {0.70, 0.74, 0.75, 0.8, 0.9, 0.99, 1.0})
        std::fprintf(f, "%.17g %.17g\n", beta, gbo::CerenkovMeanPhotonsPerMM(1.0, beta, e.data(), n.data(), (int)n.size()));
    std::fclose(f);
    return 0;
}
