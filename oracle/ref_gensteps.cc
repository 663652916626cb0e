// ref_gensteps.cc : test infrastructure (never linked into the library).  Compiles the reference's genstep structs
// and demo producers from the reference tree (sysrap/sscint.h, sysrap/scerenkov.h, sysrap/OpticksGenstep.h) and
// prints, as one JSON object on stdout:
//   * "offsets": the byte offset of every named field of sscint and scerenkov, read off the reference's structs;
//   * "enums": the reference's OpticksGenstep_* codes of the genstep kinds the host producers write;
//   * "scint_demo", "cerenkov_demo": sscint::FillGenstep / scerenkov::FillGenstep (the reference's fabricated demo
//     gensteps) for the photon count given as argv[1], 24 words each.
// (sysrap/storch.h's host producer includes sphoton.h's host part, which needs glm, absent here: the torch genstep
// is checked against storch.h's field list instead.)
// tests/golden/make_gensteps_golden.py stores the output as tests/golden/gensteps_ref.json, against which
// tests/test_cpp_gensteps.py checks include/gbo_gensteps.hh.
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "scuda.h"
#include "squad.h"
#include "sscint.h"
#include "scerenkov.h"
#include "OpticksGenstep.h"

static void words(const void* p, const char* key, bool comma)
{
    uint32_t w[24];
    std::memcpy(w, p, sizeof(w));
    std::printf("\"%s\": [", key);
    for (int i = 0; i < 24; i++) std::printf("\"%08x\"%s", w[i], i < 23 ? ", " : "");
    std::printf("]%s\n", comma ? "," : "");
}

#define OFF(T, f) std::printf("\"%s.%s\": %zu, ", #T, #f, offsetof(T, f))

int main(int argc, char** argv)
{
    const int n = argc > 1 ? std::atoi(argv[1]) : 1000;
    static_assert(sizeof(sscint) == 96 && sizeof(scerenkov) == 96, "quad6 layouts");
    std::printf("{\n\"offsets\": {");
    OFF(sscint, gentype); OFF(sscint, trackid); OFF(sscint, matline); OFF(sscint, numphoton);
    OFF(sscint, pos); OFF(sscint, time); OFF(sscint, DeltaPosition); OFF(sscint, step_length);
    OFF(sscint, code); OFF(sscint, charge); OFF(sscint, weight); OFF(sscint, meanVelocity);
    OFF(sscint, scnt); OFF(sscint, ScintillationTime);
    OFF(scerenkov, gentype); OFF(scerenkov, trackid); OFF(scerenkov, matline); OFF(scerenkov, numphoton);
    OFF(scerenkov, pos); OFF(scerenkov, time); OFF(scerenkov, DeltaPosition); OFF(scerenkov, step_length);
    OFF(scerenkov, code); OFF(scerenkov, charge); OFF(scerenkov, weight); OFF(scerenkov, preVelocity);
    OFF(scerenkov, BetaInverse); OFF(scerenkov, Wmin); OFF(scerenkov, Wmax); OFF(scerenkov, maxCos);
    OFF(scerenkov, maxSin2); OFF(scerenkov, MeanNumberOfPhotons1); OFF(scerenkov, MeanNumberOfPhotons2);
    std::printf("\"scerenkov.postVelocity\": %zu},\n", offsetof(scerenkov, postVelocity));
    std::printf("\"enums\": {\"DsG4Scintillation_r4695\": %d, \"G4Cerenkov_modified\": %d, \"TORCH\": %d, "
                "\"SCINTILLATION\": %d, \"CERENKOV\": %d},\n",
                (int)OpticksGenstep_DsG4Scintillation_r4695, (int)OpticksGenstep_G4Cerenkov_modified,
                (int)OpticksGenstep_TORCH, (int)OpticksGenstep_SCINTILLATION, (int)OpticksGenstep_CERENKOV);
    std::printf("\"numphoton\": %d,\n", n);
    quad6 q;
    q.zero();
    sscint::FillGenstep(*(sscint*)&q, 0, n, false);
    words(&q, "scint_demo", true);
    q.zero();
    scerenkov::FillGenstep(*(scerenkov*)&q, 3, n, false);
    words(&q, "cerenkov_demo", false);
    std::printf("}\n");
    return 0;
}
