// accel_check.cc : invariants of the host-built acceleration structure (eic-opticks_gb300/csrc/gbo_accel.cpp) for
// one geometry given as the CSGFoundry-layout arrays node.bin, prim.bin, solid.bin, inst.bin in a folder.
//
//   * the TLAS leaves hold every instance exactly once;
//   * every child box contains the boxes beneath it (inner children) or its instances' world boxes (leaves);
//   * instances whose box has at least a quarter of the scene's box area are exactly those under the root's first
//     child (when other instances exist);
//   * every overlap-list entry is another instance whose world box meets the listing instance's box;
//   * no other instance's world box enters a clear ball;
//   * the deepest leaf fits the traversal stack (one entry per inner node on a path);
//   * each inner box lies inside its instance's box by the inside test's largest margin (or is empty) and carries
//     the same overlap list;
//   * is_identity is 1 exactly for identity instances and 2 exactly for inverses whose rotation block is 1 on the
//     diagonal and +0 elsewhere, and for those the single-leaf traversal's shortcut (pos + translation, dir
//     unchanged, for rays with no zero coordinate) equals the general transform bit for bit on seeded rays.
// Prints one summary line; exits non-zero on the first violation.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "gbo_accel.h"

using namespace gbo;

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

static bool contains(const float* lo, const float* hi, const float* blo, const float* bhi)
{
    for (int k = 0; k < 3; k++)
        if (blo[k] < lo[k] || bhi[k] > hi[k]) return false;
    return true;
}

static double area(const float* lo, const float* hi)
{
    const double a = (double)hi[0] - lo[0], b = (double)hi[1] - lo[1], c = (double)hi[2] - lo[2];
    return 2.0 * (a * b + b * c + c * a);
}

#define CHECK(cond, ...)                          \
    do {                                          \
        if (!(cond)) {                            \
            std::printf("FAIL: " __VA_ARGS__);    \
            std::printf("\n");                    \
            return 1;                             \
        }                                         \
    } while (0)

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    const std::string d = argv[1];
    const auto node = read_all<gbo_csgnode>(d + "/node.bin");
    const auto prim = read_all<gbo_csgprim>(d + "/prim.bin");
    const auto solid = read_all<gbo_csgsolid>(d + "/solid.bin");
    const auto inst = read_all<gbo_qat4>(d + "/inst.bin");
    AccelHost A;
    char err[256] = {0};
    CHECK(build_accel(node.data(), (int)node.size(), prim.data(), (int)prim.size(), solid.data(), (int)solid.size(),
                      inst.data(), (int)inst.size(), A, err, sizeof(err)) == 0, "build_accel: %s", err);
    const int n = (int)inst.size();
    CHECK((int)A.tlas_index.size() == n && (int)A.inst_box.size() == n, "sizes");
    CHECK(A.max_depth <= TLAS_STACK_DEPTH, "depth %d above the traversal stack", A.max_depth);

    // walk the two-child-box nodes: containment and instance coverage
    std::vector<int> seen(n, 0);
    std::vector<int> stack = {0};
    int leaves_at_root = 0;
    while (!stack.empty()) {
        const int ni = stack.back();
        stack.pop_back();
        CHECK(ni >= 0 && ni < (int)A.tlas2.size(), "node index %d", ni);
        const BvhNode2& nd = A.tlas2[ni];
        const float* lo[2] = {nd.lo0, nd.lo1};
        const float* hi[2] = {nd.hi0, nd.hi1};
        const int first[2] = {nd.first0, nd.first1}, count[2] = {nd.count0, nd.count1};
        for (int c = 0; c < 2; c++) {
            if (count[c] < 0) continue;
            if (count[c] == 0) {
                const BvhNode2& ch = A.tlas2[first[c]];
                if (ch.count0 >= 0) CHECK(contains(lo[c], hi[c], ch.lo0, ch.hi0), "node %d child %d box", ni, c);
                if (ch.count1 >= 0) CHECK(contains(lo[c], hi[c], ch.lo1, ch.hi1), "node %d child %d box", ni, c);
                stack.push_back(first[c]);
                continue;
            }
            if (ni == 0) leaves_at_root++;
            for (int k = 0; k < count[c]; k++) {
                const int ii = A.tlas_index[first[c] + k];
                CHECK(ii >= 0 && ii < n, "leaf instance %d", ii);
                seen[ii]++;
                CHECK(contains(lo[c], hi[c], A.inst_box[ii].lo, A.inst_box[ii].hi), "instance %d outside its leaf", ii);
            }
        }
    }
    for (int i = 0; i < n; i++) CHECK(seen[i] == 1, "instance %d in %d leaves", i, seen[i]);

    // containers hang off the root: the root's first child holds exactly them (when some instances are not)
    float alo[3] = {1e30f, 1e30f, 1e30f}, ahi[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            alo[k] = std::fmin(alo[k], A.inst_box[i].lo[k]);
            ahi[k] = std::fmax(ahi[k], A.inst_box[i].hi[k]);
        }
    std::vector<char> is_container(n, 0);
    int containers = 0;
    for (int i = 0; i < n; i++)
        if (area(A.inst_box[i].lo, A.inst_box[i].hi) >= 0.25 * area(alo, ahi)) { is_container[i] = 1; containers++; }
    if (containers > 0 && containers < n && n > 2) {
        const BvhNode2& r = A.tlas2[0];
        std::vector<int> under;                     // instances beneath the root's first child
        if (r.count0 > 0) {
            for (int k = 0; k < r.count0; k++) under.push_back(A.tlas_index[r.first0 + k]);
        } else if (r.count0 == 0) {
            std::vector<int> st = {r.first0};
            while (!st.empty()) {
                const BvhNode2& nd = A.tlas2[st.back()];
                st.pop_back();
                const int first[2] = {nd.first0, nd.first1}, count[2] = {nd.count0, nd.count1};
                for (int c = 0; c < 2; c++) {
                    if (count[c] == 0) st.push_back(first[c]);
                    for (int k = 0; k < count[c]; k++) under.push_back(A.tlas_index[first[c] + k]);
                }
            }
        }
        CHECK((int)under.size() == containers, "%zu instances under the root's first child, %d containers",
              under.size(), containers);
        for (int ii : under) CHECK(is_container[ii], "instance %d under the containers' child is no container", ii);
    }

    // overlap lists and clear balls
    int listed = 0, full = 0, balls = 0;
    for (int i = 0; i < n; i++) {
        const InstBox& bi = A.inst_box[i];
        if (bi.overlap_count < 0) { full++; continue; }
        for (int k = 0; k < bi.overlap_count; k++) {
            const int j = A.overlap[bi.overlap_first + k];
            CHECK(j >= 0 && j < n && j != i, "overlap entry %d of %d", j, i);
            const InstBox& bj = A.inst_box[j];
            bool meet = true;
            for (int a = 0; a < 3; a++) meet &= bj.lo[a] <= bi.hi[a] && bi.lo[a] <= bj.hi[a];
            CHECK(meet, "instance %d lists %d whose box does not meet its own", i, j);
            listed++;
        }
    }
    for (int i = 0; i < n; i++) {
        const float* c = &A.clear[4 * (size_t)i];
        if (!(c[3] > 0.f)) continue;
        balls++;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            double d2 = 0.0;
            for (int a = 0; a < 3; a++) {
                const double lo = A.inst_box[j].lo[a], hi = A.inst_box[j].hi[a];
                const double dd = c[a] < lo ? lo - c[a] : (c[a] > hi ? c[a] - hi : 0.0);
                d2 += dd * dd;
            }
            CHECK(d2 >= (double)c[3], "instance %d's box enters the clear ball of %d", j, i);
        }
    }
    CHECK(A.inner_box.size() == A.inst_box.size(), "inner box count");
    for (int i = 0; i < n; i++) {
        const InstBox &b = A.inst_box[i], &in = A.inner_box[i];
        CHECK(in.overlap_first == b.overlap_first && in.overlap_count == b.overlap_count, "inner box %d list", i);
        const bool empty = in.lo[0] == INFINITY;
        for (int k = 0; k < 3; k++) {
            const double lo = b.lo[k], hi = b.hi[k];
            const double m = 2e-6 * (std::fmax(std::fabs(lo), std::fabs(hi)) + std::fabs(lo) + std::fabs(hi)) + 1e-5;
            CHECK(empty ? (in.lo[k] == INFINITY && in.hi[k] == -INFINITY) : ((double)in.lo[k] >= lo + m &&
                  (double)in.hi[k] <= hi - m && in.lo[k] < in.hi[k]), "inner box %d axis %d", i, k);
        }
    }

    // instance classes and the translated-instance shortcut (binary32, no contraction: the operation order of the
    // device's general transform, inst_point / inst_vector)
    int shifted = 0;
    std::mt19937 gen(7);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    for (int i = 0; i < n; i++) {
        const InstDev& q = A.inst[i];
        const gbo_qat4& f = inst[i];
        const bool ident = f.q0.f[0] == 1.f && f.q0.f[1] == 0.f && f.q0.f[2] == 0.f && f.q1.f[0] == 0.f &&
                           f.q1.f[1] == 1.f && f.q1.f[2] == 0.f && f.q2.f[0] == 0.f && f.q2.f[1] == 0.f &&
                           f.q2.f[2] == 1.f && f.q3.f[0] == 0.f && f.q3.f[1] == 0.f && f.q3.f[2] == 0.f;
        const float* col[3] = {q.c0, q.c1, q.c2};
        bool unit = true;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                uint32_t bits;
                std::memcpy(&bits, col[j] + k, 4);
                unit = unit && bits == (j == k ? 0x3f800000u : 0u);
            }
        CHECK(q.is_identity == (ident ? 1 : (unit ? 2 : 0)), "instance %d classed %d", i, q.is_identity);
        if (q.is_identity != 2) continue;
        shifted++;
        for (int r = 0; r < 64; r++) {
            float p[3], v[3];
            for (int k = 0; k < 3; k++) {
                p[k] = 1000.f * u(gen);
                v[k] = u(gen);
            }
            for (int j = 0; j < 3; j++) {
                const float* c = col[j];
                const volatile float pj = ((c[0] * p[0] + c[1] * p[1]) + c[2] * p[2]) + c[3] * 1.f;
                const volatile float vj = ((c[0] * v[0] + c[1] * v[1]) + c[2] * v[2]) + c[3] * 0.f;
                const float ps = p[j] + c[3];
                CHECK(std::memcmp((const void*)&pj, &ps, 4) == 0 && std::memcmp((const void*)&vj, &v[j], 4) == 0,
                      "instance %d: translated shortcut differs from the transform", i);
            }
        }
    }
    std::printf("instances %d nodes %zu depth %d root leaves %d containers %d listed %d full %d balls %d "
                "translated %d\n", n, A.tlas2.size(), A.max_depth, leaves_at_root, containers, listed, full, balls,
                shifted);
    return 0;
}
