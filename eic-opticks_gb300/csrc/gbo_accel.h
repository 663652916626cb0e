// gbo_accel.h : two-level acceleration structure replacing the reference's OptiX IAS/GAS.
//
// The reference builds one GAS per CSGSolid from CSGPrim AABBs and one IAS over the instance transforms
// (CSGOptiX/SBT.cc:247-495, GAS_Builder.cc, IAS_Builder.cc), then lets OptiX traverse them.  Here:
//   * level 1 (TLAS): a binned-SAH BVH over the world-space AABBs of all instances, built on the host;
//   * level 2: the prims of the instance's solid, each with an object-space AABB test before intersect_prim
//     (solids in these geometries hold a handful of prims);
//   * per instance, the list of other instances whose padded world boxes meet its own (at most MAX_OVERLAP;
//     instances made only of axis-aligned boxes that strictly contain it are left out, as their surfaces lie
//     outside it), and for instances with longer lists a clear ball no other instance's box enters: the
//     traversal uses them to skip the TLAS for steps that stay inside the photon's previous instance.
// Device layouts (all 16-byte aligned, read as float4/int4):
//   BvhNode  32 B : bmin.xyz, left-child-or-first-index ; bmax.xyz, count (0 for inner nodes)
//   InstDev  64 B : inverse transform as three float4 columns + (solid, identity, is_identity, iindex)
//   PrimDev  32 B : object AABB min.xyz + node offset (bit 30: pure union tree) ; AABB max.xyz +
//                   (globalPrimIdx<<16 | boundary)
//   InstBox  32 B : world box min.xyz + overlap list start ; max.xyz + overlap count (-1: use the TLAS)
//   clear    16 B : ball centre.xyz + radius^2 (0: none)
#pragma once
#include <cstdint>
#include <vector>
#include "../../include/gbo_types.h"

namespace gbo {

// Entries of the per-ray traversal stack.  A walk pushes at most one entry per inner node on its path, so a TLAS
// whose deepest leaf sits at depth <= TLAS_STACK_DEPTH never overflows it; the builder switches to median splits
// below TLAS_MEDIAN_DEPTH (at most 16 further levels for the 65,536-instance limit) and refuses any tree deeper
// than the stack, so no subtree is ever dropped.
constexpr int TLAS_STACK_DEPTH = 64;
constexpr int TLAS_MEDIAN_DEPTH = 40;

struct BvhNode {
    float bmin[3];
    int32_t left_first;
    float bmax[3];
    int32_t count;
};
static_assert(sizeof(BvhNode) == 32, "BvhNode is 32 bytes");

// Traversal node: the boxes of both children, so one 64 B load decides which children to visit and in which
// order.  For child c, count_c > 0 marks a leaf holding tlas_index[first_c .. first_c+count_c) (at most 255),
// count_c == 0 an inner node first_c, count_c < 0 an absent child (only in a root whose single child is a leaf).
struct BvhNode2 {
    float lo0[3]; int32_t first0;
    float hi0[3]; int32_t count0;
    float lo1[3]; int32_t first1;
    float hi1[3]; int32_t count1;
};
static_assert(sizeof(BvhNode2) == 64, "BvhNode2 is 64 bytes");

struct InstDev {
    float c0[4], c1[4], c2[4];     // columns of the inverse (object <- world) 3x4 transform: xyz rows + translation
    int32_t solid;
    uint32_t identity;             // sensor_identifier + 1, 0 : not a sensor
    int32_t is_identity;           // 1: identity, 2: pure translation (rotation block exactly 1 and +0), 0: other
    uint32_t iindex;
};
static_assert(sizeof(InstDev) == 64, "InstDev is 64 bytes");

struct PrimDev {
    float bmin[3];
    int32_t node_offset;
    float bmax[3];
    uint32_t prim_boundary;
};
static_assert(sizeof(PrimDev) == 32, "PrimDev is 32 bytes");

// World box of an instance (padded, rounded inward to binary32) and its overlap list: the other instances whose
// boxes meet it, as a range of AccelHost::overlap (count -1: more than MAX_OVERLAP, use the TLAS).
struct InstBox {
    float lo[3];
    int32_t overlap_first;
    float hi[3];
    int32_t overlap_count;
};
static_assert(sizeof(InstBox) == 32, "InstBox is 32 bytes");
constexpr int MAX_OVERLAP = 8;

struct SolidDev {
    int32_t prim_offset;
    int32_t num_prim;
};

struct AccelHost {
    std::vector<BvhNode> tlas;
    std::vector<BvhNode2> tlas2;         // traversal form of tlas (root is node 0; a single-leaf tree has one node)
    std::vector<int32_t> tlas_index;     // leaf ranges index into this permutation of instances
    std::vector<InstDev> inst;
    std::vector<double> inst64;          // the same inverse columns in binary64, 12 per instance (precision mode)
    std::vector<PrimDev> prim;
    std::vector<SolidDev> solid;
    std::vector<InstBox> inst_box;
    // per instance: inst_box shrunk on each axis by 2e-6 (max(|lo|, |hi|) + |lo| + |hi|) + 1e-5, rounded inward, with
    // the same overlap list fields: a point strictly inside it lies inside inst_box by more than the rounding of a
    // photon's position and of its segment's end (an empty box where the shrink consumes it)
    std::vector<InstBox> inner_box;
    std::vector<int32_t> overlap;
    // per instance (cx, cy, cz, r^2): a ball no other instance's box enters, for instances whose overlap list is
    // too long (r^2 = 0: none)
    std::vector<float> clear;
    int max_depth = 0;
};

// Builds the host-side structure from CSGFoundry-layout arrays. Returns 0 on success.
int build_accel(const gbo_csgnode* node, int num_node, const gbo_csgprim* prim, int num_prim,
                const gbo_csgsolid* solid, int num_solid, const gbo_qat4* inst, int num_inst, AccelHost& out,
                char* err, int errlen);

}  // namespace gbo
