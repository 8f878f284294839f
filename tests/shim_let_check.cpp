// Test driver for the LET functions of the C++ reference-API shim
// (tests/test_shim.py builds and runs it).  Reads a local body set (sorted
// keys, positions, masses), received records and a remote domain's boxes,
// calls buildOctreeBottomUp, createInteractionListForRank,
// buildTreeFromPseudoLeaves, computeAccelerationsWithLET and
// computeAccelerationsWithRemoteDirectSum as src/main.cpp and
// src/exchange.cpp call them, and writes every result to a raw file.
#include <algorithm>
#include <cstdint>
#include <fstream>
#include <vector>

#include "bh_reference_api.hpp"

template <class T>
static void rd(std::ifstream& f, std::vector<T>& v, size_t n)
{
    v.resize(n);
    f.read(reinterpret_cast<char*>(v.data()), sizeof(T) * n);
}
template <class T>
static T rd1(std::ifstream& f)
{
    T v{};
    f.read(reinterpret_cast<char*>(&v), sizeof(T));
    return v;
}
template <class T>
static void wr1(std::ofstream& f, T v)
{
    f.write(reinterpret_cast<const char*>(&v), sizeof(T));
}

static void write_records(std::ofstream& f, std::vector<NodeRecord> r)
{
    std::sort(r.begin(), r.end(), [](const NodeRecord& a, const NodeRecord& b) {
        return a.depth != b.depth ? a.depth < b.depth : a.prefix < b.prefix;
    });
    wr1<int64_t>(f, (int64_t)r.size());
    for (const auto& x : r) {
        wr1(f, x.prefix);
        wr1(f, x.depth);
        wr1(f, x.mass);
        wr1(f, x.comX);
        wr1(f, x.comY);
        wr1(f, x.comZ);
    }
}

int main(int argc, char** argv)
{
    if (argc != 3) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    const int64_t n = rd1<int64_t>(in);
    const double theta = rd1<double>(in);
    std::vector<double> b6;
    rd(in, b6, 6);
    BoundingBox bb;
    bb.min = {b6[0], b6[1], b6[2]};
    bb.max = {b6[3], b6[4], b6[5]};
    std::vector<uint64_t> keys;
    std::vector<Position> pos;
    std::vector<double> mass;
    rd(in, keys, n); rd(in, pos, n); rd(in, mass, n);
    const int64_t m = rd1<int64_t>(in);
    std::vector<NodeRecord> recs((size_t)m);
    for (auto& r : recs) {
        r.prefix = rd1<uint64_t>(in);
        r.depth = rd1<uint8_t>(in);
        r.mass = rd1<double>(in);
        r.comX = rd1<double>(in);
        r.comY = rd1<double>(in);
        r.comZ = rd1<double>(in);
    }
    const int64_t nb = rd1<int64_t>(in);
    std::vector<BoundingBox> boxes((size_t)nb);
    for (auto& b : boxes) {
        std::vector<double> v;
        rd(in, v, 6);
        b.min = {v[0], v[1], v[2]};
        b.max = {v[3], v[4], v[5]};
    }
    const double theta2 = rd1<double>(in);
    const int max_depth = (int)rd1<int64_t>(in);
    if (!in) return 3;

    const double G = 1.48812e-34;
    std::ofstream out(argv[2], std::ios::binary);
    OctreeMap tree = buildOctreeBottomUp(keys, pos, mass);
    write_records(out, createInteractionListForRank(tree, boxes, bb, theta2, max_depth));
    const OctreeMap pt = buildTreeFromPseudoLeaves(recs);
    std::vector<NodeRecord> pr;
    int64_t npseudo = 0;
    for (const auto& kv : pt) {
        pr.push_back({kv.first.prefix, kv.first.depth, kv.second.mass, kv.second.comX, kv.second.comY,
                      kv.second.comZ});
        npseudo += kv.second.is_pseudo ? 1 : 0;
    }
    write_records(out, pr);
    wr1(out, npseudo);
    std::vector<Acceleration> acc;
    computeAccelerationsWithRemoteDirectSum(tree, recs, keys, pos, theta, G, 0.0, bb, acc);
    out.write(reinterpret_cast<const char*>(acc.data()), sizeof(Acceleration) * acc.size());
    computeAccelerationsWithLET(tree, recs, keys, pos, theta, G, 0.0, bb, acc, 0);
    out.write(reinterpret_cast<const char*>(acc.data()), sizeof(Acceleration) * acc.size());
    wr1<int64_t>(out, (int64_t)tree.size());  // the local map after the merge
    return out ? 0 : 4;
}
