// The reference's call surface over libbh_gpu.so (see bh_reference_api.hpp).
// Every call copies its vectors to a per-thread device context, runs the
// GB300 kernels and copies the results back; errors of the C ABI become
// std::runtime_error, the reference's own error channel (src/traversal.cpp:94).
#include "bh_reference_api.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>
#include <string>

#include "bh_gpu.h"

namespace {

void check(int rc, const char* what)
{
    if (rc != BH_OK) throw std::runtime_error(std::string(what) + ": " + bh_last_error());
}

struct Ctx {
    bh_context* c = nullptr;
    int64_t cap = 0;
    ~Ctx()
    {
        if (c) bh_context_destroy(c);
    }
    bh_context* get(int64_t n)
    {
        if (!c || cap < n) {
            if (c) bh_context_destroy(c);
            c = nullptr;
            check(bh_context_create(n, 0, &c), "bh_context_create");
            cap = n;
        }
        return c;
    }
};
thread_local Ctx g_ctx;

// Loads bodies with the caller's keys and sorts them (stable), returning the
// previous position of every sorted slot.
std::vector<int64_t> load_sorted(bh_context* c, const std::vector<uint64_t>& keys, const std::vector<Position>& pos,
                                 const std::vector<double>& mass)
{
    const int64_t n = (int64_t)keys.size();
    std::vector<Velocity> vel(n, Velocity{0.0, 0.0, 0.0});
    std::vector<uint64_t> ids(n);
    std::iota(ids.begin(), ids.end(), uint64_t{0});
    check(bh_set_bodies(c, n, &pos[0].x, &vel[0].x, mass.data(), ids.data()), "bh_set_bodies");
    check(bh_set_keys(c, keys.data()), "bh_set_keys");
    std::vector<int64_t> perm(n);
    check(bh_sort_bodies(c, perm.data()), "bh_sort_bodies");
    return perm;
}

}  // namespace

#ifndef BH_SHIM_USE_REFERENCE_HEADERS
BoundingBox compute_local_bbox(const std::vector<Position>& points)
{
    BoundingBox bb;
    if (points.empty()) return bb;
    double b[6];
    check(bh_compute_local_bbox(&points[0].x, (int64_t)points.size(), b), "bh_compute_local_bbox");
    bb.min = {b[0], b[1], b[2]};
    bb.max = {b[3], b[4], b[5]};
    return bb;
}
#endif

#ifndef BH_SHIM_USE_REFERENCE_HEADERS
void sortBodiesByMortonKey(std::vector<uint64_t>& mortonCodes, std::vector<Position>& pos, std::vector<double>& mass,
                           std::vector<Velocity>& vel, std::vector<uint64_t>& ids)
{
    if (pos.empty()) return;
    check(bh_sort_bodies_by_morton_key((int64_t)pos.size(), mortonCodes.data(), &pos[0].x, mass.data(), &vel[0].x,
                                       ids.data()),
          "bh_sort_bodies_by_morton_key");
}
#endif

std::vector<uint64_t> generateMortonCodes(const std::vector<Position>& raw, const BoundingBox& bb)
{
    std::vector<uint64_t> keys(raw.size());
    if (raw.empty()) return keys;
    const double b[6] = {bb.min.x, bb.min.y, bb.min.z, bb.max.x, bb.max.y, bb.max.z};
    check(bh_generate_morton_codes(&raw[0].x, (int64_t)raw.size(), b, keys.data()), "bh_generate_morton_codes");
    return keys;
}

OctreeMap buildOctreeBottomUp(const std::vector<uint64_t>& mortonCodes, const std::vector<Position>& positions,
                              const std::vector<double>& masses)
{
    OctreeMap tree;
    const int64_t n = (int64_t)mortonCodes.size();
    if (n == 0) return tree;
    bh_context* c = g_ctx.get(n);
    load_sorted(c, mortonCodes, positions, masses);
    check(bh_build_tree_options(c, 0), "bh_build_tree_options");
    int64_t nrec = 0, nnodes = 0, nleaves = 0;
    check(bh_tree_info(c, &nrec, &nnodes, &nleaves), "bh_tree_info");
    std::vector<uint64_t> prefix(nrec);
    std::vector<uint8_t> depth(nrec);
    std::vector<double> mass(nrec), com(3 * nrec);
    check(bh_export_tree(c, prefix.data(), depth.data(), mass.data(), com.data()), "bh_export_tree");
    tree.reserve((size_t)nrec);
    for (int64_t k = 0; k < nrec; ++k) {
        OctreeNode& nd = tree[OctreeKey{prefix[k], depth[k]}];
        nd.mass = mass[k];
        nd.comX = com[3 * k];
        nd.comY = com[3 * k + 1];
        nd.comZ = com[3 * k + 2];
    }
    return tree;
}

namespace {

// The device tree of `key` with the values of `tree` (which must be the
// single-rank tree of these keys): each device node stands for the deepest
// cell of a single-child chain and takes that cell's values; a cell missing
// from the map is massless (the reference's find() fails and skips it with
// its subtree).  Returns the sort permutation of the bodies.
std::vector<int64_t> load_map_tree(bh_context* c, const OctreeMap& tree, const std::vector<uint64_t>& key,
                                   const std::vector<Position>& pos, const BoundingBox& global_bb, const char* fn)
{
    for (const auto& kv : tree)
        if (kv.second.is_pseudo) throw std::runtime_error(std::string(fn) + ": pseudo-leaves (LET) are not supported");
    const int64_t n = (int64_t)key.size();
    const std::vector<double> unit(n, 1.0);
    std::vector<int64_t> perm = load_sorted(c, key, pos, unit);
    check(bh_build_tree_options(c, 0), "bh_build_tree_options");
    int64_t nrec = 0, nnodes = 0, nleaves = 0;
    check(bh_tree_info(c, &nrec, &nnodes, &nleaves), "bh_tree_info");
    if ((int64_t)tree.size() != nrec)
        throw std::runtime_error(std::string(fn) + ": the map is not the single-rank tree of these keys");
    std::vector<uint64_t> sp(nnodes);
    std::vector<uint8_t> sd(nnodes);
    check(bh_tree_slots(c, sp.data(), sd.data()), "bh_tree_slots");
    std::vector<double> m(nnodes, 0.0), com(3 * nnodes, 0.0);
    for (int64_t s = 0; s < nnodes; ++s) {
        const auto it = tree.find(OctreeKey{sp[s], sd[s]});
        if (it == tree.end()) continue;
        m[s] = it->second.mass;
        com[3 * s] = it->second.comX;
        com[3 * s + 1] = it->second.comY;
        com[3 * s + 2] = it->second.comZ;
    }
    check(bh_tree_set_slot_values(c, m.data(), com.data()), "bh_tree_set_slot_values");
    const double b[6] = {global_bb.min.x, global_bb.min.y, global_bb.min.z,
                         global_bb.max.x, global_bb.max.y, global_bb.max.z};
    check(bh_set_bbox(c, b), "bh_set_bbox");
    return perm;
}

struct RecordArrays {
    std::vector<uint64_t> prefix;
    std::vector<uint8_t> depth;
    std::vector<double> mass, com;
    explicit RecordArrays(const std::vector<NodeRecord>& r)
        : prefix(r.size()), depth(r.size()), mass(r.size()), com(3 * r.size())
    {
        for (size_t k = 0; k < r.size(); ++k) {
            prefix[k] = r[k].prefix;
            depth[k] = r[k].depth;
            mass[k] = r[k].mass;
            com[3 * k] = r[k].comX;
            com[3 * k + 1] = r[k].comY;
            com[3 * k + 2] = r[k].comZ;
        }
    }
};

}  // namespace

void computeAccelerations(const OctreeMap& tree, const std::vector<uint64_t>& key, const std::vector<Position>& pos,
                          double theta, double G, double soft2, const BoundingBox& global_bb,
                          std::vector<Acceleration>& out, int /*rank*/)
{
    const int64_t n = (int64_t)pos.size();
    out.resize((size_t)n);
    if (n == 0) return;
    bh_context* c = g_ctx.get(n);
    const std::vector<int64_t> perm = load_map_tree(c, tree, key, pos, global_bb, "computeAccelerations");
    std::vector<Acceleration> sorted((size_t)n);
    check(bh_compute_accelerations(c, theta, G, soft2, BH_MODE_PLAIN_FP64, &sorted[0].x), "bh_compute_accelerations");
    for (int64_t i = 0; i < n; ++i) out[(size_t)perm[i]] = sorted[(size_t)i];
}

std::vector<NodeRecord> createInteractionListForRank(const OctreeMap& tree, const std::vector<BoundingBox>& remote_boxes,
                                                     const BoundingBox& global_bb, double theta2,
                                                     int max_traversal_depth)
{
    if (tree.empty() || remote_boxes.empty()) return {};
    // The map's leaves name its bodies' keys; positions play no part.
    std::vector<uint64_t> keys;
    for (const auto& kv : tree)
        if (kv.first.depth == 21) keys.push_back(kv.first.prefix);
    if (keys.empty()) throw std::runtime_error("createInteractionListForRank: the map has no leaves");
    const std::vector<Position> pos(keys.size(), Position{0.0, 0.0, 0.0});
    bh_context* c = g_ctx.get((int64_t)keys.size());
    load_map_tree(c, tree, keys, pos, global_bb, "createInteractionListForRank");
    std::vector<double> boxes(6 * remote_boxes.size());
    for (size_t k = 0; k < remote_boxes.size(); ++k) {
        const BoundingBox& b = remote_boxes[k];
        const double v[6] = {b.min.x, b.min.y, b.min.z, b.max.x, b.max.y, b.max.z};
        std::copy(v, v + 6, boxes.begin() + 6 * (ptrdiff_t)k);
    }
    const double gb[6] = {global_bb.min.x, global_bb.min.y, global_bb.min.z,
                          global_bb.max.x, global_bb.max.y, global_bb.max.z};
    int64_t nnodes = 0;
    check(bh_tree_info(c, nullptr, &nnodes, nullptr), "bh_tree_info");
    std::vector<uint64_t> prefix(nnodes);
    std::vector<uint8_t> depth(nnodes);
    std::vector<double> mass(nnodes), com(3 * nnodes);
    int64_t k = 0;
    check(bh_let_export(c, boxes.data(), (int64_t)remote_boxes.size(), gb, theta2, max_traversal_depth, nnodes,
                        prefix.data(), depth.data(), mass.data(), com.data(), &k),
          "bh_let_export");
    std::vector<NodeRecord> out((size_t)k);
    for (int64_t i = 0; i < k; ++i)
        out[(size_t)i] = {prefix[i], depth[i], mass[i], com[3 * i], com[3 * i + 1], com[3 * i + 2]};
    return out;
}

OctreeMap buildTreeFromPseudoLeaves(const std::vector<NodeRecord>& remote_nodes)
{
    OctreeMap tree;
    if (remote_nodes.empty()) return tree;
    RecordArrays r(remote_nodes);
    int64_t cap = 0;
    for (uint8_t d : r.depth) cap += (d > 21 ? 21 : d) + 1;
    std::vector<uint64_t> prefix(cap);
    std::vector<uint8_t> depth(cap);
    std::vector<double> mass(cap), com(3 * cap);
    int64_t k = 0;
    check(bh_pseudo_leaf_tree(g_ctx.get(1), r.prefix.data(), r.depth.data(), r.mass.data(), r.com.data(),
                              (int64_t)remote_nodes.size(), cap, prefix.data(), depth.data(), mass.data(), com.data(),
                              &k),
          "bh_pseudo_leaf_tree");
    tree.reserve((size_t)k);
    for (int64_t i = 0; i < k; ++i) {
        OctreeNode& nd = tree[OctreeKey{prefix[i], depth[i]}];
        nd.mass = mass[i];
        nd.comX = com[3 * i];
        nd.comY = com[3 * i + 1];
        nd.comZ = com[3 * i + 2];
    }
    for (const NodeRecord& rec : remote_nodes) {  // the records' own cells
        if (!(rec.mass > 0.0) || !std::isfinite(rec.mass)) continue;
        const uint8_t d = rec.depth > 21 ? 21 : rec.depth;
        const uint64_t p = d == 0 ? 0 : rec.prefix & (~0ULL << (63 - 3 * d));
        tree[OctreeKey{p, d}].is_pseudo = true;
    }
    return tree;
}

void computeAccelerationsWithLET(OctreeMap& local_tree, const std::vector<NodeRecord>& remote_nodes,
                                 const std::vector<uint64_t>& bodyKey, const std::vector<Position>& pos, double theta,
                                 double G, double soft2, const BoundingBox& global_bb, std::vector<Acceleration>& out,
                                 int /*rank*/)
{
    const int64_t n = (int64_t)pos.size();
    out.resize((size_t)n);
    if (n > 0) {
        bh_context* c = g_ctx.get(n);
        const std::vector<int64_t> perm =
            load_map_tree(c, local_tree, bodyKey, pos, global_bb, "computeAccelerationsWithLET");
        RecordArrays r(remote_nodes);
        std::vector<Acceleration> sorted((size_t)n);
        check(bh_let_accelerations(c, r.prefix.data(), r.depth.data(), r.mass.data(), r.com.data(),
                                   (int64_t)remote_nodes.size(), theta, G, soft2, &sorted[0].x),
              "bh_let_accelerations");
        for (int64_t i = 0; i < n; ++i) out[(size_t)perm[i]] = sorted[(size_t)i];
    }
    if (remote_nodes.empty()) return;
    // The reference leaves the merged map in local_tree (mergeRecordsIntoTree).
    for (const auto& kv : buildTreeFromPseudoLeaves(remote_nodes)) {
        OctreeNode& nd = local_tree[kv.first];
        const double m0 = nd.mass, m1 = kv.second.mass, tot = m0 + m1;
        if (tot == 0) continue;
        nd.comX = (m0 * nd.comX + m1 * kv.second.comX) / tot;
        nd.comY = (m0 * nd.comY + m1 * kv.second.comY) / tot;
        nd.comZ = (m0 * nd.comZ + m1 * kv.second.comZ) / tot;
        nd.mass = tot;
    }
}

void computeAccelerationsWithRemoteDirectSum(const OctreeMap& local_tree, const std::vector<NodeRecord>& remote_nodes,
                                             const std::vector<uint64_t>& key, const std::vector<Position>& pos,
                                             double theta, double G, double soft2, const BoundingBox& global_bb,
                                             std::vector<Acceleration>& out, int /*rank*/)
{
    const int64_t n = (int64_t)pos.size();
    out.resize((size_t)n);
    if (n == 0) return;
    bh_context* c = g_ctx.get(n);
    const std::vector<int64_t> perm =
        load_map_tree(c, local_tree, key, pos, global_bb, "computeAccelerationsWithRemoteDirectSum");
    RecordArrays r(remote_nodes);
    std::vector<Acceleration> sorted((size_t)n);
    check(bh_let_direct_accelerations(c, nullptr, nullptr, r.mass.data(), r.com.data(), (int64_t)remote_nodes.size(),
                                      theta, G, soft2, &sorted[0].x),
          "bh_let_direct_accelerations");
    for (int64_t i = 0; i < n; ++i) out[(size_t)perm[i]] = sorted[(size_t)i];
}

#ifdef BH_SHIM_USE_REFERENCE_HEADERS
// Each definition above must be the function the reference's headers declare:
// a definition whose signature differed would add an overload, and taking the
// address of an overloaded name without a target type does not compile.
[[maybe_unused]] static const void* const kSameSignatures[] = {
    reinterpret_cast<const void*>(&generateMortonCodes),
    reinterpret_cast<const void*>(&buildOctreeBottomUp),
    reinterpret_cast<const void*>(&computeAccelerations),
    reinterpret_cast<const void*>(&createInteractionListForRank),
    reinterpret_cast<const void*>(&buildTreeFromPseudoLeaves),
    reinterpret_cast<const void*>(&computeAccelerationsWithLET),
    reinterpret_cast<const void*>(&computeAccelerationsWithRemoteDirectSum),
};
#endif
