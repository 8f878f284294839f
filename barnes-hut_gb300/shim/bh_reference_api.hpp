// The reference's C++ call surface for the single-rank `--fc tree` path,
// implemented over the C ABI of libbh_gpu.so (bh_reference_api.cpp).
//
// Compiled with -DBH_SHIM_USE_REFERENCE_HEADERS and the reference's include/
// directory on the path, the shim takes the reference's own types and
// declarations (body.h, bounding_box.h, linear_octree.h with its robin_hood
// OctreeMap, morton_keys.h, traversal.h, utility.h), and its definitions of
// generateMortonCodes, buildOctreeBottomUp and computeAccelerations link in
// place of src/morton_keys.cpp:65-98, src/linear_octree.cpp:13-107 and
// src/traversal.cpp:13-103.  sortBodiesByMortonKey is an inline function of
// include/utility.h, so that build keeps the header's body (its one-line
// replacement over bh_sort_bodies_by_morton_key is shown beside the C ABI).
// Without the macro this header declares types with the same names, layouts
// and semantics (std::unordered_map stands in for the OctreeMap container)
// and the shim also provides compute_local_bbox and sortBodiesByMortonKey.
#pragma once

#include <cstdint>
#include <vector>

#ifdef BH_SHIM_USE_REFERENCE_HEADERS
#include "body.h"
#include "bounding_box.h"
#include "exchange.h"
#include "linear_octree.h"
#include "morton_keys.h"
#include "traversal.h"
#include "utility.h"
#else
#include <limits>
#include <unordered_map>

// Vec3 and its aliases: include/body.h:4-10 (AoS, 24 bytes).
struct Vec3 {
    double x, y, z;
};
using Position = Vec3;
using Velocity = Vec3;
using Acceleration = Vec3;

// include/bounding_box.h:11-22: empty box is +inf / -inf.
struct BoundingBox {
    Position min{std::numeric_limits<double>::infinity(), std::numeric_limits<double>::infinity(),
                 std::numeric_limits<double>::infinity()};
    Position max{-std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                 -std::numeric_limits<double>::infinity()};
};

// include/linear_octree.h:15-57: a cell is (prefix, depth); the map holds
// mass and centre of mass per cell.
struct OctreeKey {
    uint64_t prefix;
    uint8_t depth;
    bool operator==(const OctreeKey& o) const noexcept { return prefix == o.prefix && depth == o.depth; }
};
struct OctreeKeyHash {
    size_t operator()(const OctreeKey& k) const noexcept
    {
        uint64_t x = k.prefix ^ (uint64_t{k.depth} * 0x9e3779b97f4a7c15ULL);
        x ^= x >> 30;
        x *= 0xbf58476d1ce4e5b9ULL;
        x ^= x >> 27;
        x *= 0x94d049bb133111ebULL;
        x ^= x >> 31;
        return (size_t)x;
    }
};
struct OctreeNode {
    double mass{0.0};
    double comX{0.0};
    double comY{0.0};
    double comZ{0.0};
    bool is_pseudo{false};
};
using OctreeMap = std::unordered_map<OctreeKey, OctreeNode, OctreeKeyHash>;

// include/linear_octree.h:60-65: one cell as the exchange sends it.
struct NodeRecord {
    uint64_t prefix;
    uint8_t depth;
    double mass;
    double comX, comY, comZ;
};

BoundingBox compute_local_bbox(const std::vector<Position>& points);

// include/utility.h:23-52 (in place; equal keys keep their input order)
void sortBodiesByMortonKey(std::vector<uint64_t>& mortonCodes, std::vector<Position>& pos, std::vector<double>& mass,
                           std::vector<Velocity>& vel, std::vector<uint64_t>& ids);
#endif

// src/morton_keys.cpp:65-98
std::vector<uint64_t> generateMortonCodes(const std::vector<Position>& raw, const BoundingBox& bb);

// src/linear_octree.cpp:13-107 (before any exchange: com = sum / mass)
OctreeMap buildOctreeBottomUp(const std::vector<uint64_t>& mortonCodes, const std::vector<Position>& positions,
                              const std::vector<double>& masses);

// src/traversal.cpp:13-103, bit for bit.  The map must be a single-rank tree
// of these keys (what buildOctreeBottomUp and the single-rank exchange make):
// its cells along a single-child chain carry equal values.  Pseudo-leaves
// (LET trees) are not supported and throw std::runtime_error.
#ifndef BH_SHIM_USE_REFERENCE_HEADERS
void computeAccelerations(const OctreeMap& tree, const std::vector<uint64_t>& key, const std::vector<Position>& pos,
                          double theta, double G, double soft2, const BoundingBox& global_bb,
                          std::vector<Acceleration>& out, int rank = 0);
#endif

// The LET data path (`--fc let` / `--fc let_direct` beyond one rank).
#ifndef BH_SHIM_USE_REFERENCE_HEADERS
// src/exchange.cpp:117-179, bit for bit.  `tree` must be a local tree of
// buildOctreeBottomUp (its depth-21 cells name its bodies' keys).
std::vector<NodeRecord> createInteractionListForRank(const OctreeMap& tree, const std::vector<BoundingBox>& remote_boxes,
                                                     const BoundingBox& global_bb, double theta2,
                                                     int max_traversal_depth);

// src/linear_octree.cpp:242-322; the records' own cells are marked
// is_pseudo.  Children are summed in octant order (the reference: in its
// hash map's order), so sums over several children agree to rounding.
OctreeMap buildTreeFromPseudoLeaves(const std::vector<NodeRecord>& remote_nodes);

// src/traversal.cpp:107-127.  Like the reference, merges the records'
// pseudo-leaf map into local_tree (mergeRecordsIntoTree), then walks it.
void computeAccelerationsWithLET(OctreeMap& local_tree, const std::vector<NodeRecord>& remote_nodes,
                                 const std::vector<uint64_t>& bodyKey, const std::vector<Position>& pos, double theta,
                                 double G, double soft2, const BoundingBox& global_bb, std::vector<Acceleration>& out,
                                 int rank);

// src/traversal.cpp:149-221: the local walk (bit for bit) plus the records
// summed directly in record order.
void computeAccelerationsWithRemoteDirectSum(const OctreeMap& local_tree, const std::vector<NodeRecord>& remote_nodes,
                                             const std::vector<uint64_t>& key, const std::vector<Position>& pos,
                                             double theta, double G, double soft2, const BoundingBox& global_bb,
                                             std::vector<Acceleration>& out, int rank = 0);
#endif
