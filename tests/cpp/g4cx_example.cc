// Drives the engine through the G4CXOpticks-shaped C++ interface, the way a Geant4 application drives the
// reference (src/GPUPhotonSourceMinimal.h:87-146): SetGeometry, AddGenstep per genstep, simulate, GetNumHit,
// getHit, reset.  Inputs are raw little-endian arrays written by tests/test_cpp_interface.py into <dir>:
//   node.bin prim.bin solid.bin inst.bin itra.bin bnd.bin optical.bin icdf.bin gs.bin meta.txt
// Prints "hits <n> first_index <i> last_index <j>" and exits 0.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "G4CXOpticks_gb.hh"

template <typename T>
static std::vector<T> slurp(const std::string& path)
{
    std::ifstream f(path, std::ios::binary);
    std::vector<char> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<T> v(bytes.size() / sizeof(T));
    if (!v.empty()) std::memcpy(v.data(), bytes.data(), v.size() * sizeof(T));
    return v;
}

int main(int argc, char** argv)
{
    if (argc < 2) { std::fprintf(stderr, "usage: %s <dir>\n", argv[0]); return 2; }
    const std::string d = argv[1];
    auto node = slurp<gbo_csgnode>(d + "/node.bin");
    auto prim = slurp<gbo_csgprim>(d + "/prim.bin");
    auto solid = slurp<gbo_csgsolid>(d + "/solid.bin");
    auto inst = slurp<gbo_qat4>(d + "/inst.bin");
    auto itra = slurp<gbo_qat4>(d + "/itra.bin");
    auto bnd = slurp<float>(d + "/bnd.bin");
    auto optical = slurp<uint32_t>(d + "/optical.bin");
    auto icdf = slurp<float>(d + "/icdf.bin");
    auto gs = slurp<gbo_quad6>(d + "/gs.bin");
    int num_bnd = 0, hd = 0, event_id = 0;
    float nm0 = 0.f, nms = 0.f;
    std::ifstream meta(d + "/meta.txt");
    meta >> num_bnd >> nm0 >> nms >> hd >> event_id;

    gbo_geometry_desc g = {};
    g.node = node.data(); g.num_node = (int32_t)node.size();
    g.prim = prim.data(); g.num_prim = (int32_t)prim.size();
    g.solid = solid.data(); g.num_solid = (int32_t)solid.size();
    g.inst = inst.data(); g.num_inst = (int32_t)inst.size();
    g.itra = itra.empty() ? nullptr : itra.data(); g.num_itra = (int32_t)itra.size();
    g.bnd = bnd.data(); g.num_bnd = num_bnd; g.bnd_nx = 761;
    g.bnd_domain_low = nm0; g.bnd_domain_step = nms;
    g.optical = optical.data();
    g.icdf = icdf.data(); g.icdf_ny = 3; g.icdf_nx = 4096; g.hd_factor = hd;

    try {
        gbo::G4CXOpticks* gx = gbo::G4CXOpticks::SetGeometry(g);
        for (const gbo_quad6& q : gs) gbo::SEvt::AddGenstep(q);
        gx->simulate(event_id, false);
        const int64_t n = gbo::SEvt::GetNumHit(0);
        gbo_sphoton first = {}, last = {};
        if (n > 0) {
            gbo::SEvt::getHit(first, 0);
            gbo::SEvt::getHit(last, (unsigned)(n - 1));
        }
        std::printf("hits %lld first_index %u last_index %u\n", (long long)n, first.index, last.index);
        gx->reset(event_id);
        gbo::G4CXOpticks::Finalize();
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 1;
    }
    return 0;
}
