// photon_file_example.cc : reads argv[1] with gbo::LoadPhotonsTxt, writes the photons' raw records to argv[2] and
// the same records in the hit text format to argv[3] (gbo::WriteHitsTxt).
#include <cstdio>

#include "gbo_photon_file.hh"

int main(int argc, char** argv)
{
    if (argc < 4) return 2;
    const std::vector<gbo_sphoton> p = gbo::LoadPhotonsTxt(argv[1]);
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 3;
    std::fwrite(p.data(), sizeof(gbo_sphoton), p.size(), f);
    std::fclose(f);
    return gbo::WriteHitsTxt(argv[3], p.data(), p.size()) ? 0 : 4;
}
