// Oracle harness over the reference's own hot-path sources.
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
// reference's unmodified src/morton_keys.cpp, src/linear_octree.cpp,
// src/traversal.cpp, src/bounding_box.cpp and src/kepler_to_cartesian.cpp
// (see oracle/Makefile, target `ref`) into oracle/_ref/libbhref.so.  It is
// used to pin the C restatement (oracle/bh_oracle.c) and to generate the
// golden fixtures under tests/golden/.  Nothing in the product links it.
//
// Every entry point is a plain C function over flat arrays so that Python
// (ctypes) can drive it.  Positions/velocities/accelerations are AoS
// (x,y,z per body), exactly the layout of the reference's Vec3 (body.h:4-6).
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <vector>

#include "body.h"
#include "bounding_box.h"
#include "exchange.h"
#include "kepler_to_cartesian.h"
#include "linear_octree.h"
#include "morton_keys.h"
#include "traversal.h"
#include "utility.h"

namespace {

std::vector<Position> to_vec3(const double* p, int64_t n)
{
    std::vector<Position> v((size_t)n);
    if (n) std::memcpy(v.data(), p, sizeof(double) * 3 * (size_t)n);
    return v;
}

BoundingBox to_bbox(const double b[6])
{
    BoundingBox bb;
    bb.min = {b[0], b[1], b[2]};
    bb.max = {b[3], b[4], b[5]};
    return bb;
}

struct TreeHandle {
    OctreeMap map;
};

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// The single-rank effect of exchangeFullTrees (src/exchange.cpp:9-29): the
// local tree is serialised (linear_octree.cpp:169-176), all-gathered to
// itself unchanged, and merged into an empty map (linear_octree.cpp:178-204).
OctreeMap single_rank_exchange(const OctreeMap& local)
{
    std::vector<NodeRecord> recs = serializeTreeToRecords(local);
    OctreeMap full;
    mergeRecordsIntoTree(full, recs);
    return full;
}

}  // namespace

extern "C" {

// compute_local_bbox, src/bounding_box.cpp:23-44.  out = {minx,miny,minz,maxx,maxy,maxz}
void ref_compute_local_bbox(const double* pos, int64_t n, double out[6])
{
    BoundingBox bb = compute_local_bbox(to_vec3(pos, n));
    out[0] = bb.min.x; out[1] = bb.min.y; out[2] = bb.min.z;
    out[3] = bb.max.x; out[4] = bb.max.y; out[5] = bb.max.z;
}

// generateMortonCodes, src/morton_keys.cpp:65-98.
void ref_generate_morton_codes(const double* pos, int64_t n, const double bbox[6], uint64_t* out)
{
    std::vector<uint64_t> k = generateMortonCodes(to_vec3(pos, n), to_bbox(bbox));
    if (n) std::memcpy(out, k.data(), sizeof(uint64_t) * (size_t)n);
}

// sortBodiesByMortonKey, include/utility.h:23-52 (in place).
void ref_sort_bodies(int64_t n, uint64_t* keys, double* pos, double* mass, double* vel, uint64_t* ids)
{
    std::vector<uint64_t> k(keys, keys + n);
    std::vector<Position> p = to_vec3(pos, n);
    std::vector<double> m(mass, mass + n);
    std::vector<Velocity> v = to_vec3(vel, n);
    std::vector<uint64_t> id(ids, ids + n);
    sortBodiesByMortonKey(k, p, m, v, id);
    if (!n) return;
    std::memcpy(keys, k.data(), 8 * (size_t)n);
    std::memcpy(pos, p.data(), 24 * (size_t)n);
    std::memcpy(mass, m.data(), 8 * (size_t)n);
    std::memcpy(vel, v.data(), 24 * (size_t)n);
    std::memcpy(ids, id.data(), 8 * (size_t)n);
}

// buildOctreeBottomUp (src/linear_octree.cpp:13-107), optionally followed by
// the single-rank full-tree exchange (merge != 0), as main.cpp:239,248 do.
void* ref_build_tree(int64_t n, const uint64_t* keys, const double* pos, const double* mass, int merge)
{
    std::vector<uint64_t> k(keys, keys + n);
    std::vector<double> m(mass, mass + n);
    auto* h = new TreeHandle;
    h->map = buildOctreeBottomUp(k, to_vec3(pos, n), m);
    if (merge) h->map = single_rank_exchange(h->map);
    return h;
}

int64_t ref_tree_size(void* handle)
{
    return (int64_t)static_cast<TreeHandle*>(handle)->map.size();
}

// All nodes as records sorted by (depth, prefix), the order printTree and
// compareFlattened use (src/linear_octree.cpp:116-122, 214-221).
void ref_tree_records(void* handle, uint64_t* prefix, uint8_t* depth, double* mass, double* com)
{
    const OctreeMap& t = static_cast<TreeHandle*>(handle)->map;
    std::vector<std::pair<OctreeKey, OctreeNode>> v;
    v.reserve(t.size());
    for (const auto& kv : t) v.emplace_back(kv.first, kv.second);
    std::sort(v.begin(), v.end(), [](const auto& a, const auto& b) {
        if (a.first.depth != b.first.depth) return a.first.depth < b.first.depth;
        return a.first.prefix < b.first.prefix;
    });
    for (size_t i = 0; i < v.size(); ++i) {
        prefix[i] = v[i].first.prefix;
        depth[i] = v[i].first.depth;
        mass[i] = v[i].second.mass;
        com[3 * i + 0] = v[i].second.comX;
        com[3 * i + 1] = v[i].second.comY;
        com[3 * i + 2] = v[i].second.comZ;
    }
}

void ref_tree_free(void* handle) { delete static_cast<TreeHandle*>(handle); }

// computeAccelerations, src/traversal.cpp:13-103.
void ref_compute_accelerations(void* handle, int64_t n, const uint64_t* keys, const double* pos,
                               double theta, double G, double soft2, const double bbox[6], double* acc)
{
    const OctreeMap& t = static_cast<TreeHandle*>(handle)->map;
    std::vector<uint64_t> k(keys, keys + n);
    std::vector<Acceleration> out;
    computeAccelerations(t, k, to_vec3(pos, n), theta, G, soft2, to_bbox(bbox), out);
    if (n) std::memcpy(acc, out.data(), 24 * (size_t)n);
}

// The single-rank `--fc tree` step loop of src/main.cpp:191-282, run for
// `nsteps` steps starting at time *t (in/out).  The state arrays are updated
// in place and end up in the order of the last Morton sort, as in the
// reference.  phase_s (7 doubles, accumulated): kdk, bbox, keys, sort, build,
// merge, traversal.
void ref_simulate(int64_t n, double* pos, double* vel, double* mass, uint64_t* ids, double* acc,
                  double dt, double theta, double G, int64_t nsteps, double* t_io, double* phase_s)
{
    std::vector<Position> p = to_vec3(pos, n);
    std::vector<Velocity> v = to_vec3(vel, n);
    std::vector<Acceleration> a = to_vec3(acc, n);
    std::vector<double> m(mass, mass + n);
    std::vector<uint64_t> id(ids, ids + n);
    double t = *t_io;
    using clk = std::chrono::steady_clock;
    for (int64_t s = 0; s < nsteps; ++s, t += dt) {
        auto t0 = clk::now();
        if (t > 0) {
            #pragma omp parallel for
            for (size_t i = 0; i < p.size(); ++i) {
                v[i].x += 0.5 * dt * a[i].x;
                v[i].y += 0.5 * dt * a[i].y;
                v[i].z += 0.5 * dt * a[i].z;
            }
        }
        #pragma omp parallel for
        for (size_t i = 0; i < p.size(); ++i) {
            p[i].x += dt * v[i].x;
            p[i].y += dt * v[i].y;
            p[i].z += dt * v[i].z;
        }
        phase_s[0] += seconds_since(t0);
        t0 = clk::now();
        BoundingBox bb = compute_global_bbox(compute_local_bbox(p));
        phase_s[1] += seconds_since(t0);
        t0 = clk::now();
        std::vector<uint64_t> codes = generateMortonCodes(p, bb);
        phase_s[2] += seconds_since(t0);
        t0 = clk::now();
        sortBodiesByMortonKey(codes, p, m, v, id);
        phase_s[3] += seconds_since(t0);
        t0 = clk::now();
        OctreeMap local = buildOctreeBottomUp(codes, p, m);
        phase_s[4] += seconds_since(t0);
        t0 = clk::now();
        OctreeMap full = single_rank_exchange(local);
        phase_s[5] += seconds_since(t0);
        t0 = clk::now();
        computeAccelerations(full, codes, p, theta, G, 0.0, bb, a);
        phase_s[6] += seconds_since(t0);
        t0 = clk::now();
        #pragma omp parallel for
        for (size_t i = 0; i < p.size(); ++i) {
            v[i].x += 0.5 * dt * a[i].x;
            v[i].y += 0.5 * dt * a[i].y;
            v[i].z += 0.5 * dt * a[i].z;
        }
        phase_s[0] += seconds_since(t0);
    }
    *t_io = t;
    if (!n) return;
    std::memcpy(pos, p.data(), 24 * (size_t)n);
    std::memcpy(vel, v.data(), 24 * (size_t)n);
    std::memcpy(acc, a.data(), 24 * (size_t)n);
    std::memcpy(mass, m.data(), 8 * (size_t)n);
    std::memcpy(ids, id.data(), 8 * (size_t)n);
}

// convertKeplerToCartesian, src/kepler_to_cartesian.cpp:13-107.
// el = {e, a, i, omega(arg of periapsis), Omega(long. of asc. node), M, epoch, mu}
// (angles in radians); out = {x,y,z,vx,vy,vz}.
void ref_kepler_to_cartesian(const double* el, int64_t n, double* out)
{
    for (int64_t k = 0; k < n; ++k) {
        const double* e = el + 8 * k;
        OrbitalElements oe;
        oe.eccentricity = e[0];
        oe.semiMajorAxis = e[1];
        oe.inclination = e[2];
        oe.argOfPeriapsis = e[3];
        oe.longOfAscNode = e[4];
        oe.meanAnomaly = e[5];
        oe.epoch = e[6];
        oe.mu = e[7];
        Body* b = convertKeplerToCartesian(oe);
        double* o = out + 6 * k;
        o[0] = b->x; o[1] = b->y; o[2] = b->z;
        o[3] = b->vx; o[4] = b->vy; o[5] = b->vz;
        delete b;
    }
}

// createInteractionListForRank (src/exchange.cpp:117-179): the cells of the
// tree a remote rank whose domain is covered by `boxes` (nb x {min, max})
// needs, as NodeRecords; up to `cap` are written, the count is returned.
int64_t ref_let_export(TreeHandle* t, const double* boxes, int64_t nb, const double bb[6], double theta2,
                       int max_depth, uint64_t* prefix, uint8_t* depth, double* mass, double* com, int64_t cap)
{
    std::vector<BoundingBox> rb((size_t)nb);
    for (int64_t k = 0; k < nb; ++k) rb[(size_t)k] = to_bbox(boxes + 6 * k);
    const std::vector<NodeRecord> recs = createInteractionListForRank(t->map, rb, to_bbox(bb), theta2, max_depth);
    for (size_t k = 0; k < recs.size() && (int64_t)k < cap; ++k) {
        prefix[k] = recs[k].prefix;
        depth[k] = recs[k].depth;
        mass[k] = recs[k].mass;
        com[3 * k] = recs[k].comX;
        com[3 * k + 1] = recs[k].comY;
        com[3 * k + 2] = recs[k].comZ;
    }
    return (int64_t)recs.size();
}

// buildTreeFromPseudoLeaves (src/linear_octree.cpp:242-322) over m
// NodeRecords; the map is read back with ref_tree_size / ref_tree_records.
void* ref_pseudo_tree(const uint64_t* prefix, const uint8_t* depth, const double* mass, const double* com, int64_t m)
{
    std::vector<NodeRecord> recs((size_t)m);
    for (int64_t k = 0; k < m; ++k)
        recs[(size_t)k] = {prefix[k], depth[k], mass[k], com[3 * k], com[3 * k + 1], com[3 * k + 2]};
    auto* h = new TreeHandle();
    h->map = buildTreeFromPseudoLeaves(recs);
    return h;
}

// computeAccelerationsWithLET (src/traversal.cpp:107-127) on a copy of the
// tree `t` (the function merges the records into the map it is given) and
// computeAccelerationsWithRemoteDirectSum (:149-221), for n bodies with
// keys and positions; `direct` picks the second.
void ref_let_accelerations(void* handle, const uint64_t* prefix, const uint8_t* depth, const double* mass,
                           const double* com, int64_t m, int64_t n, const uint64_t* keys, const double* pos,
                           double theta, double G, double soft2, const double bb[6], int direct, double* acc)
{
    std::vector<NodeRecord> recs((size_t)m);
    for (int64_t k = 0; k < m; ++k)
        recs[(size_t)k] = {prefix[k], depth[k], mass[k], com[3 * k], com[3 * k + 1], com[3 * k + 2]};
    OctreeMap map = static_cast<TreeHandle*>(handle)->map;
    std::vector<uint64_t> key(keys, keys + n);
    std::vector<Acceleration> out;
    if (direct)
        computeAccelerationsWithRemoteDirectSum(map, recs, key, to_vec3(pos, n), theta, G, soft2, to_bbox(bb), out, 0);
    else
        computeAccelerationsWithLET(map, recs, key, to_vec3(pos, n), theta, G, soft2, to_bbox(bb), out, 0);
    for (int64_t i = 0; i < n; ++i) {
        acc[3 * i] = out[(size_t)i].x;
        acc[3 * i + 1] = out[(size_t)i].y;
        acc[3 * i + 2] = out[(size_t)i].z;
    }
}

}  // extern "C"
