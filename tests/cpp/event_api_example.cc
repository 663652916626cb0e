// event_api_example.cc : the engine-handle event API as a C caller binds it (gbo_event_submit / _wait /
// _num_hits / _copy_hits / _release from two producer threads).
// Usage: event_api_example <folder with node.bin ... gs.bin, meta.txt as g4cx_example reads> ; prints the hit count
// of each of four events submitted from two threads.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <thread>
#include <vector>

#include "gbopticks.h"

template <class T>
static std::vector<T> read_all(const std::string& path)
{
    std::vector<T> v;
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return v;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    v.resize((size_t)n / sizeof(T));
    if (std::fread(v.data(), sizeof(T), v.size(), f) != v.size()) v.clear();
    std::fclose(f);
    return v;
}

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    const std::string d = argv[1];
    auto node = read_all<gbo_csgnode>(d + "/node.bin");
    auto prim = read_all<gbo_csgprim>(d + "/prim.bin");
    auto solid = read_all<gbo_csgsolid>(d + "/solid.bin");
    auto inst = read_all<gbo_qat4>(d + "/inst.bin");
    auto itra = read_all<gbo_qat4>(d + "/itra.bin");
    auto bnd = read_all<float>(d + "/bnd.bin");
    auto optical = read_all<uint32_t>(d + "/optical.bin");
    auto icdf = read_all<float>(d + "/icdf.bin");
    auto gs = read_all<gbo_quad6>(d + "/gs.bin");
    int num_bnd = 0, hd = 0, event_id = 0;
    float dom0 = 60.f, domstep = 1.f;
    if (FILE* m = std::fopen((d + "/meta.txt").c_str(), "r")) {
        if (std::fscanf(m, "%d %f %f %d %d", &num_bnd, &dom0, &domstep, &hd, &event_id) != 5) return 3;
        std::fclose(m);
    }
    gbo_geometry_desc g{};
    g.node = node.data(); g.num_node = (int32_t)node.size();
    g.prim = prim.data(); g.num_prim = (int32_t)prim.size();
    g.solid = solid.data(); g.num_solid = (int32_t)solid.size();
    g.inst = inst.data(); g.num_inst = (int32_t)inst.size();
    g.itra = itra.data(); g.num_itra = (int32_t)itra.size();
    g.bnd = bnd.data(); g.num_bnd = num_bnd; g.bnd_nx = 761;
    g.bnd_domain_low = dom0; g.bnd_domain_step = domstep;
    g.optical = optical.data();
    g.icdf = icdf.data(); g.icdf_nx = 4096; g.icdf_ny = 3; g.hd_factor = hd;
    gbo_geometry* geo = nullptr;
    if (gbo_geometry_create(&g, &geo) != GBO_OK) { std::printf("create: %s\n", gbo_last_error()); return 4; }
    gbo_ticket t[4] = {0, 0, 0, 0};
    int rc[4] = {0, 0, 0, 0};
    auto producer = [&](int k0) {
        for (int k = k0; k < 4; k += 2) rc[k] = gbo_event_submit(geo, gs.data(), gs.size(), (uint32_t)(event_id + k), &t[k]);
    };
    std::thread a(producer, 0), b(producer, 1);
    a.join();
    b.join();
    for (int k = 0; k < 4; k++) {
        if (rc[k] != GBO_OK || gbo_event_wait(geo, t[k], 60'000'000'000ll) != GBO_OK) { std::printf("event %d: %s\n", k, gbo_last_error()); return 5; }
        const int64_t n = gbo_event_num_hits(geo, t[k]);
        std::vector<gbo_sphoton> hits((size_t)(n > 0 ? n : 0));
        if (n < 0 || gbo_event_copy_hits(geo, t[k], hits.data(), hits.size()) != GBO_OK) return 6;
        std::printf("event %d hits %lld first index %u\n", event_id + k, (long long)n, n > 0 ? hits[0].index : 0u);
        gbo_event_release(geo, t[k]);
    }
    gbo_geometry_destroy(geo);
    return 0;
}
