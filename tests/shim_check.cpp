// Test driver for the C++ reference-API shim (tests/test_gpu_shim.py builds
// and runs it).  Reads a body set from a raw file, calls the reference-shaped
// functions in the order of src/main.cpp:212-263 (bbox, keys, sort, build,
// single-rank exchange, forces) and writes every result to a raw file.
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <algorithm>
#include <vector>

#include "bh_reference_api.hpp"

template <class T>
static void rd(std::ifstream& f, std::vector<T>& v, size_t n)
{
    v.resize(n);
    f.read(reinterpret_cast<char*>(v.data()), sizeof(T) * n);
}
template <class T>
static void wr(std::ofstream& f, const std::vector<T>& v)
{
    f.write(reinterpret_cast<const char*>(v.data()), sizeof(T) * v.size());
}

int main(int argc, char** argv)
{
    if (argc != 3) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    int64_t n = 0;
    double theta = 0.0;
    in.read(reinterpret_cast<char*>(&n), 8);
    in.read(reinterpret_cast<char*>(&theta), 8);
    std::vector<Position> pos;
    std::vector<Velocity> vel;
    std::vector<double> mass;
    std::vector<uint64_t> ids;
    rd(in, pos, n); rd(in, vel, n); rd(in, mass, n); rd(in, ids, n);
    const double G = 1.48812e-34;

    BoundingBox bb = compute_local_bbox(pos);
    std::vector<uint64_t> keys = generateMortonCodes(pos, bb);
    std::vector<uint64_t> sk = keys;
    sortBodiesByMortonKey(sk, pos, mass, vel, ids);
    OctreeMap tree = buildOctreeBottomUp(sk, pos, mass);
    // The single-rank exchange (src/exchange.cpp:9-29): every record merged
    // into an empty map, mass' = 0 + m, com' = (0*0 + m*c) / mass'.
    OctreeMap full;
    for (const auto& kv : tree) {
        OctreeNode& nd = full[kv.first];
        const double m0 = 0.0, c0 = 0.0, m1 = kv.second.mass;
        const double tot = m0 + m1;
        if (tot == 0) continue;
        nd.comX = (m0 * c0 + m1 * kv.second.comX) / tot;
        nd.comY = (m0 * c0 + m1 * kv.second.comY) / tot;
        nd.comZ = (m0 * c0 + m1 * kv.second.comZ) / tot;
        nd.mass = tot;
    }
    std::vector<Acceleration> acc;
    computeAccelerations(full, sk, pos, theta, G, 0.0, bb, acc);

    std::vector<std::pair<OctreeKey, OctreeNode>> recs(tree.begin(), tree.end());
    std::sort(recs.begin(), recs.end(), [](const auto& a, const auto& b) {
        return a.first.depth != b.first.depth ? a.first.depth < b.first.depth : a.first.prefix < b.first.prefix;
    });
    std::ofstream out(argv[2], std::ios::binary);
    const double bbv[6] = {bb.min.x, bb.min.y, bb.min.z, bb.max.x, bb.max.y, bb.max.z};
    out.write(reinterpret_cast<const char*>(bbv), sizeof(bbv));
    wr(out, keys); wr(out, ids); wr(out, pos);
    const int64_t nr = (int64_t)recs.size();
    out.write(reinterpret_cast<const char*>(&nr), 8);
    for (const auto& r : recs) {
        const double v[4] = {r.second.mass, r.second.comX, r.second.comY, r.second.comZ};
        out.write(reinterpret_cast<const char*>(&r.first.prefix), 8);
        out.write(reinterpret_cast<const char*>(&r.first.depth), 1);
        out.write(reinterpret_cast<const char*>(v), sizeof(v));
    }
    wr(out, acc);
    std::cout << "shim ok " << n << " bodies, " << nr << " cells" << std::endl;
    return 0;
}
