// simulate: the reference's single-rank driver (src/main.cpp)
// on libbh_gpu.so.  Same flags and printed lines, so the reference's
// benchmark scripts can drive it:
//
//   simulate -f bodies.csv --dt 1h --tend 10d --theta 1.05 [-b N] [-r]
//            [--fc let|tree|let_direct] [--steps K] [--vs 10d|none] [-o sim_out]
//            [--mode plain|fp64_list|fp32|fp32_group|learned] [--generate N --seed S] [--dump FILE]
//            [--model FILE --budget B --theta-max T --band D --frac F]
//
// --tend uses the reference's loop (`for (t = 0; t < t_end; t += dt)`, so
// 10d at 1h runs 241 steps); --steps overrides it.  -r writes the final
// positions to reference/final_ref.csv (io.cpp:716-722 layout); without -r
// an existing reference file is compared by body id and SUMMED_DIST_ERROR
// printed (io.cpp:759-780), with 4 decimals as main.cpp:333-334 prints it and
// again at full precision (SUMMED_DIST_ERROR_FULL, %.17g).  TOTAL_TIME covers
// the step loop (main.cpp:185,323).
// --dump writes the final state at full precision in the state-vector CSV
// layout (what -f reads), bodies in the engine's final (key-sorted) order.
//
// Snapshots follow main.cpp:176-177,283-320: after a step whose time t
// (before the step's t += dt) reaches the next visualisation time, and after
// the first step, the state goes to <outdir>/0/sim.<k>.vtp (writeSnapshot,
// io.cpp:84-232) and <outdir>/<stem>_dt.._tend.._theta.._bodies.._fc...pvd
// lists the frames (updatePVDFile, io.cpp:235-298); -o/--outdir defaults to
// sim_out and --vs to 10d, as in the reference.  --vs none turns them off.
// The download of a frame waits for the GPU; its file is written by a host
// thread while the next steps run.
//
// --mode selects the force form: plain (the reference's arithmetic, bit
// for bit), fp64_list (the reference's interaction set in FP64), fp32 (FP32
// far field, FP64 Sun and planet terms), fp32_group (fp32 with one
// acceptance test per warp group of 32 bodies) or learned (fp32 with the learned
// acceptance criterion: --model names a file written by bh_mlp_save, --budget
// is each body's relative error budget, default 1e-5; --theta-max bounds
// the candidates, default 3; --band and --frac tune the criterion, see
// bh_learned_set_criterion; --theta stays the fallback criterion).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <future>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "bh_gpu.h"

namespace {

// parseTime (include/parse_time.h:6-16): "1h", "2.5d", "1y" -> days.
double parse_time(const std::string& s)
{
    if (s.empty()) throw std::invalid_argument("empty time");
    const double v = std::stod(s.substr(0, s.size() - 1));
    switch (s.back()) {
    case 'h': return v / 24.0;
    case 'd': return v;
    case 'y': return v * 365.25;
    default: throw std::invalid_argument("unknown time unit: " + s);
    }
}

void die(const std::string& msg)
{
    std::cerr << "Error: " << msg << std::endl;
    std::exit(1);
}

void check(int rc, const char* what)
{
    if (rc != BH_OK) die(std::string(what) + ": " + bh_last_error());
}

}  // namespace

int main(int argc, char** argv)
{
    std::string file, fc = "let", mode_s = "plain", dt_s = "1d", tend_s = "1y", dump, vs_s = "10d",
                out_dir = "sim_out", model;
    double theta = 1.05, budget = 1e-5, theta_max = 3.0, band = 0.5, frac = 0.25;
    long long bodies = -1, steps = -1, generate = 0;
    unsigned long long seed = 1;
    bool reference = false;
    for (int a = 1; a < argc; ++a) {
        const std::string k = argv[a];
        auto val = [&]() -> std::string {
            if (a + 1 >= argc) die("missing value for " + k);
            return argv[++a];
        };
        if (k == "-f" || k == "--file") file = val();
        else if (k == "--dt") dt_s = val();
        else if (k == "--tend") tend_s = val();
        else if (k == "--vs") vs_s = val();
        else if (k == "-o" || k == "--outdir") out_dir = val();
        else if (k == "--max-depth" || k == "--bucket-bits" ||
                 k == "--rebalance-interval") val();  // visualisation / multi-rank options: accepted, unused
        else if (k == "-b" || k == "--bodies") bodies = std::stoll(val());
        else if (k == "--fc") fc = val();
        else if (k == "--theta") theta = std::stod(val());
        else if (k == "-r" || k == "--reference") reference = true;
        else if (k == "--steps") steps = std::stoll(val());
        else if (k == "--mode") mode_s = val();
        else if (k == "--generate") generate = std::stoll(val());
        else if (k == "--seed") seed = std::stoull(val());
        else if (k == "--dump") dump = val();
        else if (k == "--model") model = val();
        else if (k == "--budget") budget = std::stod(val());
        else if (k == "--theta-max") theta_max = std::stod(val());
        else if (k == "--band") band = std::stod(val());
        else if (k == "--frac") frac = std::stod(val());
        else if (k == "-h" || k == "--help") {
            std::cout << "simulate -f FILE [--dt 1h] [--tend 1y] [--theta 1.05] [-b N] [-r] [--steps K]\n"
                         "         [--fc let|tree|let_direct] (one rank: the same step)\n"
                         "         [--vs 10d|none] [-o sim_out] [--mode plain|fp64_list|fp32|fp32_group|learned]\n"
                         "         [--model FILE --budget 1e-5 --theta-max 3 --band 0.5 --frac 0.25]\n"
                         "         [--generate N --seed S] [--dump FILE]\n";
            return 0;
        } else die("unknown option " + k);
    }
    if (reference) std::cout << "Running in reference mode. Force calculation method will be 'tree'." << std::endl;
    // main.cpp:93-109: -r forces the "tree" policy; "tree" and "let_direct"
    // name their policies and any other value is "let" (the default).  On
    // one rank the exchange sends nothing, so all three compute
    // computeAccelerations over the local tree: the same step.  File names
    // carry the --fc string as given (io.cpp:247-254).
    int mode = BH_MODE_PLAIN_FP64;
    if (mode_s == "fp64_list") mode = BH_MODE_FP64_LIST;
    else if (mode_s == "fp32") mode = BH_MODE_FP32_FAR;
    else if (mode_s == "learned") mode = BH_MODE_LEARNED;
    else if (mode_s == "fp32_group") mode = BH_MODE_FP32_GROUP;
    else if (mode_s != "plain") die("unknown --mode " + mode_s);
    std::vector<float> params(BH_MLP_PARAMS), scale(BH_MLP_SCALE);
    if (mode == BH_MODE_LEARNED) {
        if (model.empty()) die("--mode learned needs --model FILE");
        check(bh_mlp_load(model.c_str(), params.data(), scale.data()), "bh_mlp_load");
    }
    const double dt = parse_time(dt_s), t_end = parse_time(tend_s);

    std::vector<uint64_t> ids;
    std::vector<double> mass, pos, vel;
    int64_t n = 0;
    bh_context* ctx = nullptr;
    if (generate > 0) {
        n = generate;
        ids.resize(n); mass.resize(n); pos.resize(3 * n); vel.resize(3 * n);
        check(bh_generate_system(seed, n, 0.10, 0.0, pos.data(), vel.data(), mass.data(), ids.data()),
              "bh_generate_system");
        check(bh_context_create(n > 0 ? n : 1, 0, &ctx), "bh_context_create");
        check(bh_set_bodies(ctx, n, pos.data(), vel.data(), mass.data(), ids.data()), "bh_set_bodies");
    } else {
        // readCSV on the GPU straight into the device state; the context is
        // sized by the file's line count (an upper bound on its rows).
        if (file.empty()) die("input file required (-f)");
        int64_t lines = 1;
        if (std::FILE* f = std::fopen(file.c_str(), "rb")) {
            std::vector<char> buf(1 << 20);
            size_t k;
            while ((k = std::fread(buf.data(), 1, buf.size(), f)) > 0) lines += std::count(buf.data(), buf.data() + k, '\n');
            std::fclose(f);
        }
        const int64_t cap = bodies > 0 ? std::min<int64_t>(lines, bodies) : lines;
        check(bh_context_create(cap > 0 ? cap : 1, 0, &ctx), "bh_context_create");
        check(bh_load_csv(ctx, file.c_str(), bodies, &n), "bh_load_csv");
        ids.resize(n); mass.resize(n); pos.resize(3 * n); vel.resize(3 * n);
    }
    if (mode == BH_MODE_LEARNED) {
        check(bh_learned_set_model(ctx, params.data(), scale.data(), budget, theta_max), "bh_learned_set_model");
        check(bh_learned_set_criterion(ctx, band, frac), "bh_learned_set_criterion");
    }
    std::cout << "Loaded " << n << " bodies\n";
    int64_t nsteps = steps;
    if (nsteps < 0) {
        nsteps = 0;
        for (double t = 0.0; t < t_end; t += dt) ++nsteps;
    }
    std::cout << "Starting simulation (dt=" << dt << ", tend=" << t_end << ")\n";

    const double G = 1.48812e-34;
    double t = 0.0;
    const bool frames = vs_s != "none";
    const double vs_interval = frames ? parse_time(vs_s) : 0.0;
    std::ostringstream pvd_name;  // updatePVDFile's file name (io.cpp:242-254)
    pvd_name << (file.empty() ? std::string("generated") : std::filesystem::path(file).stem().string()) << "_dt"
             << dt_s << "_tend" << tend_s << "_theta" << theta << "_bodies" << bodies << "_fc" << fc << ".pvd";
    const std::filesystem::path vs_dir(out_dir);
    if (frames) std::filesystem::create_directories(vs_dir / "0");
    std::vector<double> fpos, fvel, facc, fmass, frame_t;
    std::vector<uint64_t> fids;
    std::future<int> writer;
    double next_vis = 0.0;
    const auto t0 = std::chrono::high_resolution_clock::now();
    for (int64_t s = 0; s < nsteps;) {
        // Steps up to and including the next one that writes a frame.
        double tq = t;
        int64_t q = s;
        while (q < nsteps && !(frames && (tq >= next_vis || q == 0))) {
            tq += dt;
            ++q;
        }
        const int64_t run = q < nsteps ? q - s + 1 : nsteps - s;
        check(bh_step(ctx, dt, theta, G, run, mode, &t), "bh_step");
        s += run;
        if (q >= nsteps) break;
        if (writer.valid()) check(writer.get(), "bh_write_vtp");
        fpos.resize(3 * n); fvel.resize(3 * n); facc.resize(3 * n); fmass.resize(n); fids.resize(n);
        check(bh_get_bodies(ctx, fpos.data(), fvel.data(), fmass.data(), fids.data(), facc.data()), "bh_get_bodies");
        const int k = (int)frame_t.size();
        const std::string path = (vs_dir / "0" / ("sim." + std::to_string(k) + ".vtp")).string();
        writer = std::async(std::launch::async, [&, path]() {
            return bh_write_vtp(path.c_str(), 0, n, fids.data(), fmass.data(), fpos.data(), fvel.data(), facc.data());
        });
        frame_t.push_back(tq);
        std::ofstream pvd(vs_dir / pvd_name.str());
        pvd << "<VTKFile type=\"Collection\">\n    <Collection>\n";
        char ts[64];
        for (int f = 0; f < (int)frame_t.size(); ++f) {
            std::snprintf(ts, sizeof ts, "%.17g", frame_t[f]);
            pvd << "        <DataSet timestep=\"" << ts << "\" part=\"0\" file=\"0/sim." << f << ".vtp\"/>\n";
        }
        pvd << "    </Collection>\n</VTKFile>\n";
        std::cout << "Saved frame " << k << " at t=" << tq << std::endl;
        next_vis += vs_interval;
    }
    if (writer.valid()) check(writer.get(), "bh_write_vtp");
    const auto t1 = std::chrono::high_resolution_clock::now();
    check(bh_get_bodies(ctx, pos.data(), vel.data(), mass.data(), ids.data(), nullptr), "bh_get_bodies");
    bh_context_destroy(ctx);
    if (!dump.empty())
        check(bh_write_csv(dump.c_str(), n, ids.data(), mass.data(), pos.data(), vel.data()), "bh_write_csv");

    double summed = 0.0;
    const std::filesystem::path ref = std::filesystem::path("reference") / "final_ref.csv";
    if (reference) {
        std::filesystem::create_directories("reference");
        std::ofstream os(ref);
        os << "id,x,y,z\n";
        for (int64_t i = 0; i < n; ++i)
            os << ids[i] << "," << pos[3 * i] << "," << pos[3 * i + 1] << "," << pos[3 * i + 2] << "\n";
        std::cout << "Reference positions saved to reference/final_ref.csv" << std::endl;
    } else if (std::filesystem::exists(ref)) {
        std::vector<double> rp(3 * (size_t)n, 0.0);
        std::ifstream is(ref);
        std::string line;
        std::getline(is, line);
        while (std::getline(is, line)) {
            std::stringstream ss(line);
            std::string f;
            std::getline(ss, f, ',');
            const uint64_t id = std::stoull(f);
            double v[3];
            for (double& x : v) {
                std::getline(ss, f, ',');
                x = std::stod(f);
            }
            if (id < (uint64_t)n)
                for (int a = 0; a < 3; ++a) rp[3 * id + a] = v[a];
        }
        for (int64_t i = 0; i < n; ++i) {
            const uint64_t id = ids[i];
            if (id >= (uint64_t)n) continue;
            const double dx = pos[3 * i] - rp[3 * id], dy = pos[3 * i + 1] - rp[3 * id + 1],
                         dz = pos[3 * i + 2] - rp[3 * id + 2];
            summed += std::sqrt(dx * dx + dy * dy + dz * dz);
        }
    } else {
        std::cout << "Reference file not found at reference/final_ref.csv, skipping error analysis." << std::endl;
    }
    const double secs = std::chrono::duration<double>(t1 - t0).count();
    std::cout << std::fixed << std::setprecision(4);
    std::cout << "TOTAL_TIME          " << secs << std::endl;
    std::cout << "SUMMED_DIST_ERROR   " << summed << std::endl;
    char full[64];
    std::snprintf(full, sizeof full, "%.17g", summed);
    std::cout << "SUMMED_DIST_ERROR_FULL " << full << std::endl;
    std::cout << "BODY_STEPS_PER_S    " << std::setprecision(1) << (secs > 0 ? n * (double)nsteps / secs : 0.0)
              << std::endl;
    return 0;
}
