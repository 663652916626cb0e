// np_foundry_writer.cc : writes a CSGFoundry folder with the reference's own header-only NP writer (sysrap/NP.hh),
// in the layout of CSGFoundry::save_ (CSG/CSGFoundry.cc:2769-2800) plus the SSim/stree/standard optical tables of
// sstandard::serialize (sysrap/sstandard.h:197-213) with the metadata the reference attaches: the boundary
// table's wavelength domain (sstandard.h:503-506) and the scintillation inverse CDF's hd_factor (u4/U4Scint.h:444).
// Test infrastructure: compiled against the reference tree (GBO_REFERENCE_DIR) by tests/golden/make_csgfoundry_golden.py.
//
// Usage: np_foundry_writer <raw dir> <out dir>
//   <raw dir> holds the engine's arrays as raw little-endian files with a dims.txt of
//   "num_solid num_prim num_node num_inst num_itra num_tran num_plan num_bnd bnd_nx icdf_ny icdf_nx hd_factor
//    domain_low domain_step"; bnd.bin is float64, optical.bin int32, icdf.bin float64, the rest float32 / int32.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "NP.hh"

template <typename T>
static std::vector<T> read_raw(const std::string& path, size_t n)
{
    std::vector<T> v(n);
    if (n == 0) return v;
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
    return v;
}

int main(int argc, char** argv)
{
    if (argc < 3) return 2;
    const std::string raw = argv[1];
    const std::string out = std::string(argv[2]) + "/CSGFoundry";
    std::ifstream dims(raw + "/dims.txt");
    long num_solid, num_prim, num_node, num_inst, num_itra, num_tran, num_plan, num_bnd, bnd_nx, icdf_ny, icdf_nx;
    int hd_factor;
    float domain_low, domain_step;
    dims >> num_solid >> num_prim >> num_node >> num_inst >> num_itra >> num_tran >> num_plan >> num_bnd >> bnd_nx >>
        icdf_ny >> icdf_nx >> hd_factor >> domain_low >> domain_step;
    if (!dims) return 3;

    // CSGFoundry::save_ : the geometry arrays, each written only when non-empty
    const auto solid = read_raw<int>(raw + "/solid.bin", (size_t)num_solid * 12);
    const auto prim = read_raw<float>(raw + "/prim.bin", (size_t)num_prim * 16);
    const auto node = read_raw<float>(raw + "/node.bin", (size_t)num_node * 16);
    const auto plan = read_raw<float>(raw + "/plan.bin", (size_t)num_plan * 4);
    const auto tran = read_raw<float>(raw + "/tran.bin", (size_t)num_tran * 16);
    const auto itra = read_raw<float>(raw + "/itra.bin", (size_t)num_itra * 16);
    const auto inst = read_raw<float>(raw + "/inst.bin", (size_t)num_inst * 16);
    if (num_solid > 0) NP::Write(out.c_str(), "solid.npy", solid.data(), num_solid, 3, 4);
    if (num_prim > 0) NP::Write(out.c_str(), "prim.npy", prim.data(), num_prim, 4, 4);
    if (num_node > 0) NP::Write(out.c_str(), "node.npy", node.data(), num_node, 4, 4);
    if (num_plan > 0) NP::Write(out.c_str(), "plan.npy", plan.data(), num_plan, 1, 4);
    if (num_tran > 0) NP::Write(out.c_str(), "tran.npy", tran.data(), num_tran, 4, 4);
    if (num_itra > 0) NP::Write(out.c_str(), "itra.npy", itra.data(), num_itra, 4, 4);
    if (num_inst > 0) NP::Write(out.c_str(), "inst.npy", inst.data(), num_inst, 4, 4);

    // SSim/stree/standard : bnd (num_bnd, 4, 2, nx, 4) float64 with its domain, optical (num_bnd, 4, 4) int32,
    // icdf (ny, nx) float64 with its hd_factor
    const std::string std_dir = out + "/SSim/stree/standard";
    NP* bnd = NP::Make<double>(num_bnd, 4, 2, bnd_nx, 4);
    const auto bnd_raw = read_raw<double>(raw + "/bnd.bin", (size_t)bnd->num_values());
    std::copy(bnd_raw.begin(), bnd_raw.end(), bnd->values<double>());
    bnd->set_meta<float>("domain_low", domain_low);
    bnd->set_meta<float>("domain_high", domain_low + domain_step * float(bnd_nx - 1));
    bnd->set_meta<float>("domain_step", domain_step);
    bnd->set_meta<float>("domain_range", domain_step * float(bnd_nx - 1));
    bnd->save((std_dir + "/bnd.npy").c_str());
    NP* optical = NP::Make<int>(num_bnd, 4, 4);
    const auto opt_raw = read_raw<int>(raw + "/optical.bin", (size_t)optical->num_values());
    std::copy(opt_raw.begin(), opt_raw.end(), optical->values<int>());
    optical->save((std_dir + "/optical.npy").c_str());
    NP* icdf = NP::Make<double>(icdf_ny, icdf_nx);
    const auto icdf_raw = read_raw<double>(raw + "/icdf.bin", (size_t)icdf->num_values());
    std::copy(icdf_raw.begin(), icdf_raw.end(), icdf->values<double>());
    icdf->set_meta<int>("hd_factor", hd_factor);
    icdf->set_meta<int>("num_bins", (int)icdf_nx);
    icdf->save((std_dir + "/icdf.npy").c_str());
    std::printf("%s\n", out.c_str());
    return 0;
}
