// Oracle harness over the reference's own I/O code.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile (target `ref`)
// together with the reference's unmodified src/io.cpp and its vendored
// src/tinyxml2.cpp (plus the hot-path sources ref_harness.cpp drives) into
// oracle/_ref/libbhref.so.  tests/golden/make_golden.py uses it to write the
// I/O fixtures: what readCSV parses, the bytes writeSnapshot / updatePVDFile
// write, and the final_ref.csv / SUMMED_DIST_ERROR of the `-r` workflow.
//
// Plain C entry points over flat arrays for ctypes.
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <string>
#include <vector>

#include "body.h"
#include "bounding_box.h"
#include "cxxopts.hpp"
#include "exchange.h"
#include "io.h"
#include "linear_octree.h"
#include "morton_keys.h"
#include "parse_time.h"
#include "traversal.h"
#include "utility.h"

namespace {

std::vector<Position> to_vec3(const double* p, int64_t n)
{
    std::vector<Position> v((size_t)n);
    if (n) std::memcpy(v.data(), p, sizeof(double) * 3 * (size_t)n);
    return v;
}

// The option set of src/main.cpp:51-65 (names, types and defaults), so a
// ParseResult built here answers updatePVDFile's lookups exactly as the
// reference's driver does.
cxxopts::Options cli_options()
{
    cxxopts::Options opt("simulate", "Barnes-Hut");
    opt.add_options()
        ("h,help", "Print usage")
        ("f,file", "CSV file", cxxopts::value<std::string>())
        ("dt", "Time step", cxxopts::value<std::string>()->default_value("1d"))
        ("tend", "End time", cxxopts::value<std::string>()->default_value("1y"))
        ("vs", "Visualization step interval", cxxopts::value<std::string>()->default_value("10d"))
        ("o,outdir", "Output directory", cxxopts::value<std::string>()->default_value("sim_out"))
        ("b,bodies", "number of bodies", cxxopts::value<int>()->default_value("-1"))
        ("fc", "Force calculation", cxxopts::value<std::string>()->default_value("let"))
        ("theta", "BH opening angle", cxxopts::value<double>()->default_value("1.05"))
        ("max-depth", "LET depth", cxxopts::value<int>()->default_value("21"))
        ("bucket-bits", "histogram bits", cxxopts::value<int>()->default_value("18"))
        ("rebalance-interval", "rebalance steps", cxxopts::value<int>()->default_value("24"))
        ("r,reference", "reference run", cxxopts::value<bool>()->default_value("false"));
    return opt;
}

OctreeMap single_rank_exchange(const OctreeMap& local)
{
    std::vector<NodeRecord> recs = serializeTreeToRecords(local);
    OctreeMap full;
    mergeRecordsIntoTree(full, recs);
    return full;
}

}  // namespace

extern "C" {

// readCSV (src/io.cpp:16-81).  Returns the number of bodies read (copies
// at most `cap` of them), or -1 when the file cannot be opened.
int64_t ref_read_csv(const char* path, int body_count, uint64_t* ids, double* mass, double* pos, double* vel,
                     int64_t cap)
{
    std::vector<uint64_t> i;
    std::vector<double> m;
    std::vector<Position> p;
    std::vector<Velocity> v;
    if (!readCSV(path, i, m, p, v, body_count)) return -1;
    const int64_t n = (int64_t)m.size();
    const int64_t k = n < cap ? n : cap;
    if (k > 0) {
        std::memcpy(ids, i.data(), 8 * (size_t)k);
        std::memcpy(mass, m.data(), 8 * (size_t)k);
        std::memcpy(pos, p.data(), 24 * (size_t)k);
        std::memcpy(vel, v.data(), 24 * (size_t)k);
    }
    return n;
}

// writeSnapshot (src/io.cpp:84-232): <vs_dir>/<rank>/sim.<vs_counter>.vtp.
void ref_write_snapshot(int rank, int vs_counter, int64_t n, const uint64_t* ids, const double* mass,
                        const double* pos, const double* vel, const double* acc, const char* vs_dir)
{
    std::vector<uint64_t> i(ids, ids + n);
    std::vector<double> m(mass, mass + n);
    writeSnapshot(rank, vs_counter, i, m, to_vec3(pos, n), to_vec3(vel, n), to_vec3(acc, n), vs_dir);
}

// updatePVDFile (src/io.cpp:234-298) with the ParseResult of `argv` (argc
// strings, argv[0] the program name) under main.cpp's option set.
void ref_update_pvd(int argc, const char** argv, int size, int vs_counter, double current_time, const char* vs_dir)
{
    cxxopts::Options opt = cli_options();
    const auto args = opt.parse(argc, argv);
    updatePVDFile(args, size, vs_counter, current_time, vs_dir);
}

// saveReferenceCSV (src/io.cpp:716-722): <dir>/final_ref.csv.
void ref_save_reference_csv(const char* dir, int64_t n, const double* pos, const uint64_t* ids)
{
    std::vector<uint64_t> i(ids, ids + n);
    saveReferenceCSV(dir, to_vec3(pos, n), i);
}

// loadReferenceCSV (src/io.cpp:725-756); 0, or -1 when the file is missing.
int ref_load_reference_csv(const char* dir, int num_bodies, double* pos_out)
{
    try {
        std::vector<Position> p = loadReferenceCSV(dir, num_bodies);
        if (num_bodies > 0) std::memcpy(pos_out, p.data(), 24 * (size_t)num_bodies);
        return 0;
    } catch (const std::runtime_error&) {
        return -1;
    }
}

// computeDistanceSum (src/io.cpp:759-779) on one rank.
double ref_compute_distance_sum(int64_t n, const double* pos, const uint64_t* ids, int64_t nref,
                                const double* ref_pos)
{
    std::vector<uint64_t> i(ids, ids + n);
    return computeDistanceSum(to_vec3(pos, n), i, to_vec3(ref_pos, nref));
}

// The reference driver (src/main.cpp:44-345) on one rank for the tree
// force path, on the given command line (main.cpp's options): readCSV, the
// t < tend step loop of :191-282 with the snapshot schedule of :283-320
// (writeSnapshot + updatePVDFile), then performReferenceAndErrorAnalysis
// (:353-417: -r saves reference/final_ref.csv, otherwise an existing one is
// compared).  On one rank the collectives, the domain update and the
// rebalancing leave the state unchanged and are not replayed; the LET
// branches are not taken.  Relative paths resolve against the current
// directory.  Returns 0, or -1 when the input file cannot be read; *summed
// is SUMMED_DIST_ERROR, *n_bodies the bodies loaded, *n_steps the steps run
// and *frames the snapshots written.
int ref_run_cli(int argc, const char** argv, double* summed, int64_t* n_bodies, int64_t* n_steps, int64_t* frames)
{
    cxxopts::Options opt = cli_options();
    const auto args = opt.parse(argc, argv);
    const double dt = parseTime(args["dt"].as<std::string>());
    const double t_end = parseTime(args["tend"].as<std::string>());
    const double vs_interval = parseTime(args["vs"].as<std::string>());
    const std::string out_dir = args["outdir"].as<std::string>();
    const double theta = args["theta"].as<double>();
    const int nbodies = args["bodies"].as<int>();
    const bool is_reference = args["reference"].as<bool>();
    const std::string ref_dir = "reference";

    std::vector<Position> pos;
    std::vector<Velocity> vel;
    std::vector<double> mass;
    std::vector<uint64_t> ids;
    if (!readCSV(args["file"].as<std::string>(), ids, mass, pos, vel, nbodies)) return -1;
    std::filesystem::create_directories(out_dir);
    if (is_reference) std::filesystem::create_directories(ref_dir);
    const int N_total = (int)mass.size();

    const double G = 1.48812e-34;
    std::vector<Acceleration> acc(pos.size());
    double next_vis_time = 0.0;
    int vis_step = 0;
    double t = 0.0;
    int64_t steps = 0;
    for (int step = 0; t < t_end; ++step, t += dt, ++steps) {
        if (t > 0) {
            for (size_t i = 0; i < pos.size(); ++i) {
                vel[i].x += 0.5 * dt * acc[i].x;
                vel[i].y += 0.5 * dt * acc[i].y;
                vel[i].z += 0.5 * dt * acc[i].z;
            }
        }
        for (size_t i = 0; i < pos.size(); ++i) {
            pos[i].x += dt * vel[i].x;
            pos[i].y += dt * vel[i].y;
            pos[i].z += dt * vel[i].z;
        }
        BoundingBox bb = compute_global_bbox(compute_local_bbox(pos));
        std::vector<uint64_t> codes = generateMortonCodes(pos, bb);
        sortBodiesByMortonKey(codes, pos, mass, vel, ids);
        OctreeMap full = single_rank_exchange(buildOctreeBottomUp(codes, pos, mass));
        computeAccelerations(full, codes, pos, theta, G, 0.0, bb, acc);
        for (size_t i = 0; i < pos.size(); ++i) {
            vel[i].x += 0.5 * dt * acc[i].x;
            vel[i].y += 0.5 * dt * acc[i].y;
            vel[i].z += 0.5 * dt * acc[i].z;
        }
        if (t >= next_vis_time || step == 0) {
            writeSnapshot(0, vis_step, ids, mass, pos, vel, acc, out_dir);
            updatePVDFile(args, 1, vis_step, t, out_dir);
            next_vis_time += vs_interval;
            vis_step++;
        }
    }
    double err = 0.0;
    if (is_reference) {
        saveReferenceCSV(ref_dir, pos, ids);
    } else if (std::filesystem::exists(std::filesystem::path(ref_dir) / "final_ref.csv")) {
        std::vector<Position> ref_positions = loadReferenceCSV(ref_dir, N_total);
        err = computeDistanceSum(pos, ids, ref_positions);
    }
    *summed = err;
    *n_bodies = N_total;
    *n_steps = steps;
    *frames = vis_step;
    return 0;
}

}  // extern "C"
