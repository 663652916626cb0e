// gbo_accel.cpp : host builder of the two-level acceleration structure (see gbo_accel.h).
#include "gbo_accel.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

namespace gbo {

namespace {

struct Box {
    double lo[3] = {1e300, 1e300, 1e300};
    double hi[3] = {-1e300, -1e300, -1e300};
    void grow(const double* p) { for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); } }
    void grow(const Box& b) { grow(b.lo); grow(b.hi); }
    bool empty() const { return lo[0] > hi[0]; }
    double area() const
    {
        if (empty()) return 0.0;
        double d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
        return 2.0 * (d0 * d1 + d1 * d2 + d2 * d0);
    }
    double centroid(int k) const { return 0.5 * (lo[k] + hi[k]); }
};

// AABBs are padded so that float round-off in the slab test never culls a hit on the surface itself
void pad(Box& b)
{
    double ext = 0.0;
    for (int k = 0; k < 3; k++) ext = std::max(ext, std::max(std::fabs(b.lo[k]), std::fabs(b.hi[k])));
    const double e = 1e-5 * ext + 1e-3;
    for (int k = 0; k < 3; k++) { b.lo[k] -= e; b.hi[k] += e; }
}

void invert_affine(const double m[3][3], const double t[3], double r[3][3], double it[3])
{
    double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                 m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    r[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / det;
    r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
    r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
    r[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / det;
    r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
    r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
    r[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / det;
    r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
    r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
    for (int j = 0; j < 3; j++) it[j] = -(t[0] * r[0][j] + t[1] * r[1][j] + t[2] * r[2][j]);
}

struct Builder {
    std::vector<Box> boxes;
    std::vector<int32_t>& index;
    std::vector<BvhNode>& nodes;
    int max_depth = 0;

    Builder(std::vector<int32_t>& idx, std::vector<BvhNode>& n) : index(idx), nodes(n) {}

    // forced_mid (begin < forced_mid < end): split there instead of by SAH
    int build(int begin, int end, int depth, int forced_mid = -1)
    {
        max_depth = std::max(max_depth, depth);
        Box bb, cb;
        for (int i = begin; i < end; i++) {
            bb.grow(boxes[index[i]]);
            double c[3] = {boxes[index[i]].centroid(0), boxes[index[i]].centroid(1), boxes[index[i]].centroid(2)};
            cb.grow(c);
        }
        int self = (int)nodes.size();
        nodes.push_back(BvhNode{});
        for (int k = 0; k < 3; k++) { nodes[self].bmin[k] = (float)bb.lo[k]; nodes[self].bmax[k] = (float)bb.hi[k]; }
        const int n = end - begin;
        if (n <= 2 || (depth >= 48 && n <= 255)) {      // leaf counts fit the 8-bit field of the traversal items
            nodes[self].left_first = begin;
            nodes[self].count = n;
            return self;
        }
        // binned SAH, 32 bins on each axis with a centroid spread; the cheapest split over the three axes; deep in
        // the tree a median split on the widest centroid axis, which bounds the remaining depth by log2(n)
        int mid = begin + n / 2;
        int axis = 0;
        for (int k = 1; k < 3; k++) if (cb.hi[k] - cb.lo[k] > cb.hi[axis] - cb.lo[axis]) axis = k;
        if (forced_mid > begin && forced_mid < end) {
            mid = forced_mid;
        } else if (depth >= TLAS_MEDIAN_DEPTH) {
            std::nth_element(index.begin() + begin, index.begin() + mid, index.begin() + end,
                             [&](int32_t a, int32_t c) { return boxes[a].centroid(axis) < boxes[c].centroid(axis); });
        } else if (cb.hi[axis] - cb.lo[axis] > 0.0) {
            constexpr int NB = 32;
            double best = 1e300;
            int best_axis = -1, best_split = -1;
            for (int ax = 0; ax < 3; ax++) {
                const double span = cb.hi[ax] - cb.lo[ax];
                if (!(span > 0.0)) continue;
                Box bin[NB];
                int cnt[NB] = {0};
                for (int i = begin; i < end; i++) {
                    int bi = (int)((boxes[index[i]].centroid(ax) - cb.lo[ax]) / span * NB);
                    bi = std::min(NB - 1, std::max(0, bi));
                    cnt[bi]++;
                    bin[bi].grow(boxes[index[i]]);
                }
                // right-to-left sweep of the suffix areas, then left-to-right over the split planes
                double right_area[NB];
                int right_cnt[NB];
                Box acc;
                int nacc = 0;
                for (int bi = NB - 1; bi >= 1; bi--) {
                    if (cnt[bi]) { acc.grow(bin[bi]); nacc += cnt[bi]; }
                    right_area[bi] = acc.area();
                    right_cnt[bi] = nacc;
                }
                Box left;
                int nl = 0;
                for (int sp = 1; sp < NB; sp++) {
                    if (cnt[sp - 1]) { left.grow(bin[sp - 1]); nl += cnt[sp - 1]; }
                    if (nl == 0 || right_cnt[sp] == 0) continue;
                    const double cost = left.area() * nl + right_area[sp] * right_cnt[sp];
                    if (cost < best) { best = cost; best_axis = ax; best_split = sp; }
                }
            }
            if (best_axis >= 0) {
                const int ax = best_axis;
                const double span = cb.hi[ax] - cb.lo[ax];
                auto it = std::partition(index.begin() + begin, index.begin() + end, [&](int32_t id) {
                    int bi = (int)((boxes[id].centroid(ax) - cb.lo[ax]) / span * NB);
                    bi = std::min(NB - 1, std::max(0, bi));
                    return bi < best_split;
                });
                mid = (int)(it - index.begin());
                axis = ax;
            }
            if (mid == begin || mid == end) {
                std::nth_element(index.begin() + begin, index.begin() + begin + n / 2, index.begin() + end,
                                 [&](int32_t a, int32_t c) { return boxes[a].centroid(axis) < boxes[c].centroid(axis); });
                mid = begin + n / 2;
            }
        }
        const int l = build(begin, mid, depth + 1);
        const int r = build(mid, end, depth + 1);
        (void)l;
        nodes[self].left_first = r;     // left child is always self+1
        nodes[self].count = 0;
        return self;
    }
};

}  // namespace

int build_accel(const gbo_csgnode* node, int num_node, const gbo_csgprim* prim, int num_prim,
                const gbo_csgsolid* solid, int num_solid, const gbo_qat4* inst, int num_inst, AccelHost& out,
                char* err, int errlen)
{
    out = AccelHost{};
    if (num_inst <= 0 || num_solid <= 0 || num_prim <= 0 || num_node <= 0) {
        std::snprintf(err, errlen, "empty geometry (nodes %d prims %d solids %d instances %d)", num_node, num_prim,
                      num_solid, num_inst);
        return 1;
    }
    if (num_inst > 0x10000) {
        std::snprintf(err, errlen, "%d instances exceed the 16-bit instance index of the photon record", num_inst);
        return 1;
    }
    out.solid.resize(num_solid);
    std::vector<Box> solid_box(num_solid);
    // per solid: the object-space boxes of its prims when every prim is a single untransformed, uncomplemented
    // box3 (its surface is then exactly its box's boundary); empty otherwise
    std::vector<std::vector<Box>> exact(num_solid);
    std::vector<char> all_exact(num_solid, 1);
    out.prim.resize(num_prim);
    for (int s = 0; s < num_solid; s++) {
        const gbo_csgsolid& so = solid[s];
        if (so.primOffset < 0 || so.numPrim < 0 || so.primOffset + so.numPrim > num_prim) {
            std::snprintf(err, errlen, "solid %d prim range [%d,+%d) outside %d prims", s, so.primOffset, so.numPrim, num_prim);
            return 1;
        }
        out.solid[s] = SolidDev{so.primOffset, so.numPrim};
        for (int k = 0; k < so.numPrim; k++) {
            const int pi = so.primOffset + k;
            const gbo_csgprim& pr = prim[pi];
            const int noff = pr.q0.i[1];
            const int nn = pr.q0.i[0];
            if (noff < 0 || nn <= 0 || noff + nn > num_node) {
                std::snprintf(err, errlen, "prim %d node range [%d,+%d) outside %d nodes", pi, noff, nn, num_node);
                return 1;
            }
            Box b;
            double lo[3] = {pr.q2.f[0], pr.q2.f[1], pr.q2.f[2]};
            double hi[3] = {pr.q2.f[3], pr.q3.f[0], pr.q3.f[1]};
            b.grow(lo);
            b.grow(hi);
            pad(b);
            PrimDev& pd = out.prim[pi];
            for (int j = 0; j < 3; j++) { pd.bmin[j] = (float)b.lo[j]; pd.bmax[j] = (float)b.hi[j]; }
            if (noff >= (1 << 30)) {
                std::snprintf(err, errlen, "prim %d node offset %d above 2^30", pi, noff);
                return 1;
            }
            // pure union trees of plain leaves (no complement, no phicut / halfspace) take the union fast path
            bool pure_union = nn > 1;
            for (int k = 0; k < nn && pure_union; k++) {
                const gbo_csgnode& nk = node[noff + k];
                const unsigned tc = nk.q3.u[2];
                if (tc == GBO_CSG_ZERO || tc == GBO_CSG_UNION) continue;
                if (tc < GBO_CSG_LEAF || tc == GBO_CSG_PHICUT || tc == GBO_CSG_HALFSPACE || (nk.q3.u[3] & 0x80000000u))
                    pure_union = false;
            }
            pd.node_offset = noff | (pure_union ? (1 << 30) : 0);
            const unsigned boundary = node[noff].q1.u[2];
            const unsigned gpi = pr.q3.u[3];
            pd.prim_boundary = ((gpi & 0xffffu) << 16) | (boundary & 0xffffu);
            solid_box[s].grow(b);
            const gbo_csgnode& nd = node[noff];
            const bool box_leaf = nn == 1 && nd.q3.u[2] == GBO_CSG_BOX3 && nd.q3.u[3] == 0u;
            if (box_leaf) {
                Box e;
                double lo2[3] = {-0.5 * nd.q0.f[0], -0.5 * nd.q0.f[1], -0.5 * nd.q0.f[2]};
                double hi2[3] = {0.5 * nd.q0.f[0], 0.5 * nd.q0.f[1], 0.5 * nd.q0.f[2]};
                e.grow(lo2);
                e.grow(hi2);
                exact[s].push_back(e);
            } else {
                all_exact[s] = 0;
            }
        }
    }
    out.inst.resize(num_inst);
    out.inst64.assign(12 * (size_t)num_inst, 0.0);
    std::vector<Box> inst_box(num_inst);
    for (int i = 0; i < num_inst; i++) {
        const gbo_qat4& q = inst[i];
        const int s = q.q1.i[3];
        if (s < 0 || s >= num_solid) {
            std::snprintf(err, errlen, "instance %d refers to solid %d of %d", i, s, num_solid);
            return 1;
        }
        double m[3][3] = {{q.q0.f[0], q.q0.f[1], q.q0.f[2]}, {q.q1.f[0], q.q1.f[1], q.q1.f[2]}, {q.q2.f[0], q.q2.f[1], q.q2.f[2]}};
        double t[3] = {q.q3.f[0], q.q3.f[1], q.q3.f[2]};
        double r[3][3], it[3];
        invert_affine(m, t, r, it);
        InstDev& d = out.inst[i];
        const bool ident = q.q0.f[0] == 1.f && q.q0.f[1] == 0.f && q.q0.f[2] == 0.f && q.q1.f[0] == 0.f &&
                           q.q1.f[1] == 1.f && q.q1.f[2] == 0.f && q.q2.f[0] == 0.f && q.q2.f[1] == 0.f &&
                           q.q2.f[2] == 1.f && q.q3.f[0] == 0.f && q.q3.f[1] == 0.f && q.q3.f[2] == 0.f;
        // columns of the inverse in the row-vector convention of sqat4::right_multiply
        for (int j = 0; j < 3; j++) {
            float* c = j == 0 ? d.c0 : (j == 1 ? d.c1 : d.c2);
            c[0] = (float)r[0][j];
            c[1] = (float)r[1][j];
            c[2] = (float)r[2][j];
            c[3] = (float)it[j];
            double* c64 = out.inst64.data() + 12 * (size_t)i + 4 * j;
            c64[0] = r[0][j];
            c64[1] = r[1][j];
            c64[2] = r[2][j];
            c64[3] = it[j];
        }
        d.solid = s;
        d.identity = (uint32_t)q.q2.i[3];
        // 2: the inverse's rotation block is exactly 1 on the diagonal and +0 elsewhere (a pure translation)
        bool shift = true;
        for (int j = 0; j < 3; j++) {
            const float* c = j == 0 ? d.c0 : (j == 1 ? d.c1 : d.c2);
            for (int k = 0; k < 3; k++) {
                uint32_t bits;
                std::memcpy(&bits, c + k, 4);
                shift = shift && bits == (k == j ? 0x3f800000u : 0u);
            }
            shift = shift && std::isfinite(c[3]);
        }
        d.is_identity = ident ? 1 : (shift ? 2 : 0);
        d.iindex = (uint32_t)i;
        const Box& sb = solid_box[s];
        Box wb;
        for (int cx = 0; cx < 2; cx++)
            for (int cy = 0; cy < 2; cy++)
                for (int cz = 0; cz < 2; cz++) {
                    double p[3] = {cx ? sb.hi[0] : sb.lo[0], cy ? sb.hi[1] : sb.lo[1], cz ? sb.hi[2] : sb.lo[2]};
                    double w[3];
                    for (int k = 0; k < 3; k++) w[k] = p[0] * m[0][k] + p[1] * m[1][k] + p[2] * m[2][k] + t[k];
                    wb.grow(w);
                }
        pad(wb);
        inst_box[i] = wb;
    }
    // instances made only of exact boxes under a translation: their world boxes, for the containment rule below
    std::vector<std::vector<Box>> inst_exact(num_inst);
    for (int i = 0; i < num_inst; i++) {
        const gbo_qat4& q = inst[i];
        const int s = q.q1.i[3];
        const bool translation_only = q.q0.f[0] == 1.f && q.q0.f[1] == 0.f && q.q0.f[2] == 0.f && q.q1.f[0] == 0.f &&
                                      q.q1.f[1] == 1.f && q.q1.f[2] == 0.f && q.q2.f[0] == 0.f && q.q2.f[1] == 0.f &&
                                      q.q2.f[2] == 1.f;
        if (!translation_only || !all_exact[s]) continue;
        for (const Box& e : exact[s]) {
            Box w;
            double lo[3], hi[3];
            for (int k = 0; k < 3; k++) { lo[k] = e.lo[k] + q.q3.f[k]; hi[k] = e.hi[k] + q.q3.f[k]; }
            w.grow(lo);
            w.grow(hi);
            inst_exact[i].push_back(w);
        }
    }
    // j cannot hold a hit inside i's box when each of j's prims is an exact box that either misses i's box or
    // contains it strictly (its surface, the box boundary, then lies outside i's box)
    auto cannot_hit_inside = [&](int j, const Box& bi) {
        if (inst_exact[j].empty()) return false;
        for (const Box& e : inst_exact[j]) {
            const double m = 1e-6 * (std::fabs(e.lo[0]) + std::fabs(e.hi[0]) + std::fabs(e.lo[1]) + std::fabs(e.hi[1]) +
                                     std::fabs(e.lo[2]) + std::fabs(e.hi[2])) + 1e-4;
            bool misses = false, contains = true;
            for (int k = 0; k < 3; k++) {
                if (e.hi[k] < bi.lo[k] || e.lo[k] > bi.hi[k]) misses = true;
                if (!(e.lo[k] + m < bi.lo[k] && bi.hi[k] < e.hi[k] - m)) contains = false;
            }
            if (!misses && !contains) return false;
        }
        return true;
    };
    // overlap lists: sort and sweep along x over the padded world boxes (closed intervals)
    {
        std::vector<int> by_x(num_inst);
        for (int i = 0; i < num_inst; i++) by_x[i] = i;
        std::sort(by_x.begin(), by_x.end(), [&](int a, int c) { return inst_box[a].lo[0] < inst_box[c].lo[0]; });
        std::vector<std::vector<int>> ov(num_inst);
        std::vector<char> full(num_inst, 0);
        for (int a = 0; a < num_inst; a++) {
            const int i = by_x[a];
            const Box& bi = inst_box[i];
            for (int c = a + 1; c < num_inst && inst_box[by_x[c]].lo[0] <= bi.hi[0]; c++) {
                const int j = by_x[c];
                const Box& bj = inst_box[j];
                if (bj.lo[1] > bi.hi[1] || bi.lo[1] > bj.hi[1] || bj.lo[2] > bi.hi[2] || bi.lo[2] > bj.hi[2]) continue;
                for (int e : {i, j}) {
                    const int other = e == i ? j : i;
                    if (full[e] || cannot_hit_inside(other, inst_box[e])) continue;
                    if ((int)ov[e].size() >= MAX_OVERLAP) { full[e] = 1; ov[e].clear(); continue; }
                    ov[e].push_back(other);
                }
            }
        }
        out.inst_box.resize(num_inst);
        out.inner_box.resize(num_inst);
        for (int i = 0; i < num_inst; i++) {
            InstBox& ib = out.inst_box[i];
            for (int k = 0; k < 3; k++) {
                // binary32 box inside the binary64 one, so that a point found inside it is inside the box the
                // overlaps were computed with
                float lo = (float)inst_box[i].lo[k], hi = (float)inst_box[i].hi[k];
                if ((double)lo < inst_box[i].lo[k]) lo = std::nextafter(lo, INFINITY);
                if ((double)hi > inst_box[i].hi[k]) hi = std::nextafter(hi, -INFINITY);
                ib.lo[k] = lo;
                ib.hi[k] = hi;
            }
            std::sort(ov[i].begin(), ov[i].end());
            ib.overlap_first = (int32_t)out.overlap.size();
            ib.overlap_count = full[i] ? -1 : (int32_t)ov[i].size();
            InstBox& in = out.inner_box[i];
            bool empty = false;
            for (int k = 0; k < 3; k++) {
                const double lo = ib.lo[k], hi = ib.hi[k];
                const double m = 2e-6 * (std::max(std::fabs(lo), std::fabs(hi)) + std::fabs(lo) + std::fabs(hi)) + 1e-5;
                float ilo = (float)(lo + m), ihi = (float)(hi - m);
                if ((double)ilo < lo + m) ilo = std::nextafter(ilo, INFINITY);
                if ((double)ihi > hi - m) ihi = std::nextafter(ihi, -INFINITY);
                in.lo[k] = ilo;
                in.hi[k] = ihi;
                empty = empty || !(ilo < ihi);
            }
            if (empty)
                for (int k = 0; k < 3; k++) { in.lo[k] = INFINITY; in.hi[k] = -INFINITY; }
            in.overlap_first = ib.overlap_first;
            in.overlap_count = ib.overlap_count;
            if (!full[i]) out.overlap.insert(out.overlap.end(), ov[i].begin(), ov[i].end());
        }
        if (out.overlap.empty()) out.overlap.push_back(0);
        // clear balls for the instances whose overlap lists overflowed (containers such as a world volume):
        // centred on the box centre, radius the distance to the nearest other box, a little less for rounding
        out.clear.assign(4 * (size_t)num_inst, 0.f);
        int done = 0;
        for (int i = 0; i < num_inst && done < 64; i++) {
            if (!full[i]) continue;
            done++;
            double c[3];
            for (int k = 0; k < 3; k++) c[k] = 0.5 * (inst_box[i].lo[k] + inst_box[i].hi[k]);
            double r2 = 1e300;
            for (int j = 0; j < num_inst; j++) {
                if (j == i) continue;
                double d2 = 0.0;
                for (int k = 0; k < 3; k++) {
                    const double d = c[k] < inst_box[j].lo[k] ? inst_box[j].lo[k] - c[k]
                                   : (c[k] > inst_box[j].hi[k] ? c[k] - inst_box[j].hi[k] : 0.0);
                    d2 += d * d;
                }
                r2 = std::min(r2, d2);
            }
            if (r2 >= 1e300) continue;                          // a single instance: its overlap list is empty
            const double r = std::sqrt(r2) * (1.0 - 1e-6) - 1e-3;
            if (r <= 0.0) continue;
            for (int k = 0; k < 3; k++) out.clear[4 * (size_t)i + k] = (float)c[k];
            out.clear[4 * (size_t)i + 3] = (float)(r * r);
        }
    }
    // Containers (instances whose box has at least a quarter of the area of the box of everything, e.g. a world
    // volume) hang off the root in their own subtree: inside the SAH split they would stretch every node on the
    // way down to their leaf to their own size, and a TLAS walk would descend that whole chain for any ray.
    out.tlas_index.resize(num_inst);
    int num_big = 0;
    {
        Box all;
        for (int i = 0; i < num_inst; i++) all.grow(inst_box[i]);
        const double big_area = 0.25 * all.area();
        for (int i = 0; i < num_inst; i++)
            if (inst_box[i].area() >= big_area) out.tlas_index[num_big++] = i;
        int k = num_big;
        for (int i = 0; i < num_inst; i++)
            if (inst_box[i].area() < big_area) out.tlas_index[k++] = i;
    }
    Builder b(out.tlas_index, out.tlas);
    b.boxes = inst_box;
    out.tlas.reserve(2 * num_inst);
    b.build(0, num_inst, 0, num_big > 0 && num_big < num_inst ? num_big : -1);
    out.max_depth = b.max_depth;
    if (out.max_depth > TLAS_STACK_DEPTH) {
        std::snprintf(err, errlen, "instance tree depth %d exceeds the %d-entry traversal stack", out.max_depth,
                      TLAS_STACK_DEPTH);
        return 1;
    }

    // two-child-box form: node k of tlas2 corresponds to inner node map[k] of tlas
    const std::vector<BvhNode>& t = out.tlas;
    std::vector<int> inner_id(t.size(), -1);
    std::vector<int> order;
    for (size_t i = 0; i < t.size(); i++)
        if (t[i].count == 0) { inner_id[i] = (int)order.size(); order.push_back((int)i); }
    auto child = [&](int ci, float* lo, float* hi, int32_t& first, int32_t& count) {
        for (int k = 0; k < 3; k++) { lo[k] = t[ci].bmin[k]; hi[k] = t[ci].bmax[k]; }
        if (t[ci].count > 0) { first = t[ci].left_first; count = t[ci].count; }
        else { first = inner_id[ci]; count = 0; }
    };
    if (order.empty()) {            // root is a leaf: one node whose second child is empty
        BvhNode2 n{};
        child(0, n.lo0, n.hi0, n.first0, n.count0);
        for (int k = 0; k < 3; k++) { n.lo1[k] = 0.f; n.hi1[k] = 0.f; }
        n.first1 = 0;
        n.count1 = -1;              // no second child: never visited
        out.tlas2.push_back(n);
    } else {
        for (int id : order) {
            BvhNode2 n{};
            child(id + 1, n.lo0, n.hi0, n.first0, n.count0);
            child(t[id].left_first, n.lo1, n.hi1, n.first1, n.count1);
            out.tlas2.push_back(n);
        }
    }
    return 0;
}

}  // namespace gbo
