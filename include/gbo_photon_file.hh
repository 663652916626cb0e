// gbo_photon_file.hh : the text formats of the reference's photon-file application (src/GPUPhotonFileSource.h),
// header-only, for callers that feed input photons from a file and write hits as that application does.
//
//   LoadPhotonsTxt : one photon per line, 11 values "pos_x pos_y pos_z time mom_x mom_y mom_z pol_x pol_y pol_z
//                    wavelength"; blank lines and lines starting with '#' skipped, malformed lines skipped
//                    (load_photons_txt); the other sphoton fields are zero.
//   WriteHitsTxt   : "time wavelength  (x, y, z)  (mx, my, mz)  (px, py, pz)" per hit with the default stream
//                    formatting (EndOfEventAction).
#pragma once

#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "gbopticks.h"

namespace gbo {

inline std::vector<gbo_sphoton> LoadPhotonsTxt(const std::string& path)
{
    std::vector<gbo_sphoton> out;
    std::ifstream ifs(path);
    if (!ifs.is_open()) return out;
    std::string line;
    while (std::getline(ifs, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream ss(line);
        float v[11];
        bool ok = true;
        for (float& x : v) ok = ok && static_cast<bool>(ss >> x);
        if (!ok) continue;
        gbo_sphoton p{};
        p.pos[0] = v[0]; p.pos[1] = v[1]; p.pos[2] = v[2];
        p.time = v[3];
        p.mom[0] = v[4]; p.mom[1] = v[5]; p.mom[2] = v[6];
        p.pol[0] = v[7]; p.pol[1] = v[8]; p.pol[2] = v[9];
        p.wavelength = v[10];
        out.push_back(p);
    }
    return out;
}

inline bool WriteHitsTxt(const std::string& path, const gbo_sphoton* hits, size_t n)
{
    std::ofstream f(path);
    if (!f.is_open()) return false;
    for (size_t i = 0; i < n; i++) {
        const gbo_sphoton& h = hits[i];
        // the reference prints floats and doubles (G4ThreeVector components) with the default 6 significant digits
        f << (double)h.time << " " << (double)h.wavelength << "  (" << (double)h.pos[0] << ", " << (double)h.pos[1]
          << ", " << (double)h.pos[2] << ")  (" << (double)h.mom[0] << ", " << (double)h.mom[1] << ", "
          << (double)h.mom[2] << ")  (" << (double)h.pol[0] << ", " << (double)h.pol[1] << ", " << (double)h.pol[2]
          << ")" << std::endl;
    }
    return true;
}

}  // namespace gbo
