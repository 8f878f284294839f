// Host-side input: Kepler conversion, the seeded synthetic solar system and
// the reference's CSV format.  Plain C++; no GPU is touched here.
#include <cerrno>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <string>

#include "bh_common.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 2.0 * kPi;
constexpr double kG = 1.48812e-34;     // AU^3 kg^-1 day^-2 (src/main.cpp:174)
constexpr double kSunMass = 1.989e30;  // kg
constexpr double kJ2000 = 2451544.5;   // Julian date of the conversion epoch

// Masses (kg) and semi-major axes (AU) of the eight planets, the values of
// data/orbital_elements_raw_csvs/planets_and_moons.csv:2-9 of the reference.
struct Planet { double mass, a; };
constexpr Planet kPlanets[8] = {
    {3.301011e+23, 0.3870982252718477},  // Mercury
    {4.86732e+24, 0.723326849675607},    // Venus
    {5.972186e+24, 1.000371833994387},   // Earth
    {6.416928e+23, 1.52367818431121},    // Mars
    {1.89813e+27, 5.205108585205607},    // Jupiter
    {5.683191e+26, 9.581451990534042},   // Saturn
    {8.681013e+25, 19.22994588008584},   // Uranus
    {1.024096e+26, 30.10071183142183},   // Neptune
};

// One Kepler state conversion: mean anomaly propagated to J2000, Newton on
// E - e sin E = M (|dE| < 1e-8, at most 100 iterations), true anomaly,
// perifocal position/velocity, then the rotation by (Omega, i, omega).
// The sequence of operations is the one of convertKeplerToCartesian
// (src/kepler_to_cartesian.cpp:13-107) so that both give the same states.
void kepler_one(const double* q, double* o)
{
    const double e = q[0], a = q[1], inc = q[2], w = q[3], Om = q[4], epoch = q[6], mu = q[7];
    double M = q[5];
    const double nmot = std::sqrt(mu / std::pow(a, 3));
    M += nmot * (kJ2000 - epoch);
    M = std::fmod(M, 2 * M_PI);
    if (M < 0) M += 2 * M_PI;
    double E = M;
    for (int it = 0; it < 100; ++it) {
        const double f = E - e * std::sin(E) - M;
        const double fp = 1 - e * std::cos(E);
        const double d = -f / fp;
        E += d;
        if (std::fabs(d) < 1e-8) break;
    }
    const double nu = 2 * std::atan2(std::sqrt(1 + e) * std::sin(E / 2), std::sqrt(1 - e) * std::cos(E / 2));
    const double r = a * (1 - e * std::cos(E));
    const double xo = r * std::cos(nu), yo = r * std::sin(nu);
    const double h = std::sqrt(mu * a) / r;
    const double vxo = h * (-std::sin(E)), vyo = h * std::sqrt(1 - e * e) * std::cos(E);
    const double cO = std::cos(Om), sO = std::sin(Om), ci = std::cos(inc), si = std::sin(inc);
    const double cw = std::cos(w), sw = std::sin(w);
    const double R11 = cO * cw - sO * sw * ci, R12 = -cO * sw - sO * cw * ci;
    const double R21 = sO * cw + cO * sw * ci, R22 = -sO * sw + cO * cw * ci;
    const double R31 = sw * si, R32 = cw * si;
    o[0] = R11 * xo + R12 * yo;
    o[1] = R21 * xo + R22 * yo;
    o[2] = R31 * xo + R32 * yo;
    o[3] = R11 * vxo + R12 * vyo;
    o[4] = R21 * vxo + R22 * vyo;
    o[5] = R31 * vxo + R32 * vyo;
}

// Uniform double in [0,1) from the top 53 bits of one mt19937_64 draw
// (explicit, so the stream is the same with every C++ library).
struct Rng {
    std::mt19937_64 g;
    explicit Rng(uint64_t seed) : g(seed) {}
    double u() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
    double u(double lo, double hi) { return lo + (hi - lo) * u(); }
};

// strtod with std::stod's failure rules: no digits or out of range fails.
bool parse_double(const std::string& s, double* out)
{
    const char* p = s.c_str();
    char* end = nullptr;
    errno = 0;
    double v = std::strtod(p, &end);
    if (end == p || errno == ERANGE) return false;
    *out = v;
    return true;
}

}  // namespace

// One data row of readCSV (src/io.cpp:45-70): three skipped columns, then
// mass, position and velocity through std::stod.  As in the reference, a
// getline past the end of the row leaves `field` holding the previous
// column, which is then parsed again.
bool bh_parse_csv_row(const std::string& line, double v[7])
{
    std::stringstream ss(line);
    std::string field;
    for (int c = 0; c < 3; ++c) std::getline(ss, field, ',');
    for (int c = 0; c < 7; ++c) {
        std::getline(ss, field, ',');
        if (!parse_double(field, &v[c])) return false;
    }
    return true;
}

extern "C" int bh_kepler_to_cartesian(const double* el, int64_t n, double* out)
{
    if (n < 0 || (n > 0 && (!el || !out))) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_kepler_to_cartesian: bad arguments");
    for (int64_t k = 0; k < n; ++k) kepler_one(el + 8 * k, out + 6 * k);
    return BH_OK;
}

// Body layout in the generated arrays: 0 = Sun, 1..8 = planets, then the
// inner belt, the outer belt and the trojans, in that order.
//   inner belt : a U[2.1,3.3] AU, e U[0,0.3], i U[0,20] deg
//   outer belt : a U[30,50] AU,  e U[0,0.2], i U[0,30] deg
//   trojans    : a = 5.2 AU, e U[0,0.1], i U[0,20] deg, mean longitude
//                lambda_J +/- 60 deg + U[-30,30] deg (L4 or L5 alternately)
//   every asteroid: Omega, omega U[0,2pi); M U[0,2pi) (trojans: from lambda);
//   mass log-uniform on [1e12, 1e20] kg.
// Planets: e = i = Omega = omega = 0, M U[0,2pi).  mu = G * M_sun, epoch J2000.
extern "C" int bh_generate_system(uint64_t seed, int64_t n, double frac_outer, double frac_trojan, double* pos,
                                  double* vel, double* mass, uint64_t* ids)
{
    if (n < 9 || !pos || !vel || !mass || !ids || frac_outer < 0 || frac_trojan < 0 || frac_outer + frac_trojan > 1)
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_generate_system: need n >= 9 and fractions in [0,1]");
    Rng rng(seed);
    const double mu = kG * kSunMass;
    const double deg = kPi / 180.0;
    const int64_t nast = n - 9;
    const int64_t n_outer = (int64_t)std::llround(frac_outer * (double)nast);
    const int64_t n_troj = (int64_t)std::llround(frac_trojan * (double)nast);
    const int64_t n_inner = nast - n_outer - n_troj;
    double q[8], s[6];
    for (int a = 0; a < 3; ++a) pos[a] = vel[a] = 0.0;
    mass[0] = kSunMass;
    double lambda_j = 0.0;
    for (int p = 0; p < 8; ++p) {
        const double M = rng.u(0.0, kTwoPi);
        if (p == 4) lambda_j = M;
        q[0] = 0.0; q[1] = kPlanets[p].a; q[2] = 0.0; q[3] = 0.0; q[4] = 0.0; q[5] = M; q[6] = kJ2000; q[7] = mu;
        kepler_one(q, s);
        for (int a = 0; a < 3; ++a) { pos[3 * (1 + p) + a] = s[a]; vel[3 * (1 + p) + a] = s[3 + a]; }
        mass[1 + p] = kPlanets[p].mass;
    }
    const double lmin = std::log(1e12), lmax = std::log(1e20);
    for (int64_t k = 0; k < nast; ++k) {
        const int64_t b = 9 + k;
        double a, e, inc, Om, w, M;
        if (k < n_inner) {
            a = rng.u(2.1, 3.3); e = rng.u(0.0, 0.3); inc = rng.u(0.0, 20.0) * deg;
            Om = rng.u(0.0, kTwoPi); w = rng.u(0.0, kTwoPi); M = rng.u(0.0, kTwoPi);
        } else if (k < n_inner + n_outer) {
            a = rng.u(30.0, 50.0); e = rng.u(0.0, 0.2); inc = rng.u(0.0, 30.0) * deg;
            Om = rng.u(0.0, kTwoPi); w = rng.u(0.0, kTwoPi); M = rng.u(0.0, kTwoPi);
        } else {
            a = 5.2; e = rng.u(0.0, 0.1); inc = rng.u(0.0, 20.0) * deg;
            Om = rng.u(0.0, kTwoPi); w = rng.u(0.0, kTwoPi);
            const double side = ((k - n_inner - n_outer) & 1) ? -60.0 : 60.0;
            const double lam = lambda_j + (side + rng.u(-30.0, 30.0)) * deg;
            M = std::fmod(lam - Om - w, kTwoPi);
            if (M < 0) M += kTwoPi;
        }
        mass[b] = std::exp(rng.u(lmin, lmax));
        q[0] = e; q[1] = a; q[2] = inc; q[3] = w; q[4] = Om; q[5] = M; q[6] = kJ2000; q[7] = mu;
        kepler_one(q, s);
        for (int c = 0; c < 3; ++c) { pos[3 * b + c] = s[c]; vel[3 * b + c] = s[3 + c]; }
    }
    for (int64_t i = 0; i < n; ++i) ids[i] = (uint64_t)i;
    return BH_OK;
}

extern "C" int bh_read_csv(const char* path, int64_t body_count, int64_t* n_out, uint64_t* ids, double* mass,
                           double* pos, double* vel)
{
    if (!path || !n_out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_read_csv: null path or n_out");
    const bool fill = pos != nullptr;
    if (fill && (!ids || !mass || !vel)) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_read_csv: missing output arrays");
    std::ifstream f(path);
    if (!f.is_open()) return bh_fail(BH_ERR_IO, std::string("bh_read_csv: cannot open ") + path);
    std::string line;
    std::getline(f, line);  // header
    int64_t n = 0;
    while (std::getline(f, line)) {
        if (body_count > 0 && n >= body_count) break;
        double v[7];
        const bool ok = bh_parse_csv_row(line, v);
        if (!ok) {
            std::fprintf(stderr, "Warning: Could not parse line, skipping: \"%s\"\n", line.c_str());
            continue;
        }
        if (fill) {
            ids[n] = (uint64_t)n;
            mass[n] = v[0];
            for (int a = 0; a < 3; ++a) { pos[3 * n + a] = v[1 + a]; vel[3 * n + a] = v[4 + a]; }
        }
        ++n;
    }
    *n_out = n;
    return BH_OK;
}

extern "C" int bh_write_csv(const char* path, int64_t n, const uint64_t* ids, const double* mass, const double* pos,
                            const double* vel)
{
    if (!path || n < 0 || (n > 0 && (!ids || !mass || !pos || !vel)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_write_csv: bad arguments");
    FILE* f = std::fopen(path, "w");
    if (!f) return bh_fail(BH_ERR_IO, std::string("bh_write_csv: cannot open ") + path);
    std::fprintf(f, "id,name,class,mass,pos_x,pos_y,pos_z,vel_x,vel_y,vel_z\n");
    for (int64_t i = 0; i < n; ++i)
        std::fprintf(f, "%llu,b%llu,SYN,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g\n", (unsigned long long)ids[i],
                     (unsigned long long)ids[i], mass[i], pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], vel[3 * i],
                     vel[3 * i + 1], vel[3 * i + 2]);
    const bool bad = std::ferror(f) != 0;
    std::fclose(f);
    return bad ? bh_fail(BH_ERR_IO, "bh_write_csv: write failed") : BH_OK;
}

// writeSnapshot (src/io.cpp:84-232): one VTK XML PolyData file per snapshot
// with the same elements, array names, types and number formatting (the
// default stream formatting, 6 significant digits): Points "position";
// PointData "rank", "body_id", "velocity", "mass", "acceleration" (the
// magnitude); Verts "offsets" / "connectivity", one vertex per body.  An
// empty state writes no file (io.cpp:95).
extern "C" int bh_write_vtp(const char* path, int rank, int64_t n, const uint64_t* ids, const double* mass,
                            const double* pos, const double* vel, const double* acc)
{
    if (!path || n < 0 || n > INT32_MAX || (n > 0 && (!ids || !mass || !pos || !vel || !acc)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_write_vtp: bad arguments");
    if (n == 0) return BH_OK;
    std::ofstream os(path);
    if (!os) return bh_fail(BH_ERR_IO, std::string("bh_write_vtp: cannot open ") + path);
    const std::string I1 = "    ", I2 = I1 + I1, I3 = I2 + I1, I4 = I3 + I1;
    auto open_array = [&](const std::string& ind, const char* type, const char* name, int comps, bool tuples) {
        os << ind << "<DataArray type=\"" << type << "\" Name=\"" << name << "\"";
        if (comps > 0) os << " NumberOfComponents=\"" << comps << "\"";
        if (tuples) os << " NumberOfTuples=\"" << n << "\"";
        os << " format=\"ascii\">";
    };
    os << "<VTKFile type=\"PolyData\" version=\"0.1\">\n" << I1 << "<PolyData>\n";
    os << I2 << "<Piece NumberOfPoints=\"" << n << "\" NumberOfVerts=\"" << n << "\">\n";
    os << I3 << "<Points>\n";
    open_array(I4, "Float64", "position", 3, true);
    for (int64_t i = 0; i < n; ++i) os << pos[3 * i] << " " << pos[3 * i + 1] << " " << pos[3 * i + 2] << "\n";
    os << "</DataArray>\n" << I3 << "</Points>\n" << I3 << "<PointData>\n";
    open_array(I4, "Int32", "rank", 1, true);
    for (int64_t i = 0; i < n; ++i) os << rank << "\n";
    os << "</DataArray>\n";
    open_array(I4, "UInt64", "body_id", 1, true);
    for (int64_t i = 0; i < n; ++i) os << ids[i] << "\n";
    os << "</DataArray>\n";
    open_array(I4, "Float64", "velocity", 3, true);
    for (int64_t i = 0; i < n; ++i) os << vel[3 * i] << " " << vel[3 * i + 1] << " " << vel[3 * i + 2] << "\n";
    os << "</DataArray>\n";
    open_array(I4, "Float64", "mass", 1, true);
    for (int64_t i = 0; i < n; ++i) os << mass[i] << "\n";
    os << "</DataArray>\n";
    open_array(I4, "Float64", "acceleration", 1, true);
    for (int64_t i = 0; i < n; ++i) {
        const double ax = acc[3 * i], ay = acc[3 * i + 1], az = acc[3 * i + 2];
        os << std::sqrt(ax * ax + ay * ay + az * az) << "\n";
    }
    os << "</DataArray>\n" << I3 << "</PointData>\n" << I3 << "<Verts>\n";
    open_array(I4, "Int64", "offsets", 0, false);
    for (int64_t i = 1; i <= n; ++i) os << i << " ";
    os << "</DataArray>\n";
    open_array(I4, "Int64", "connectivity", 0, false);
    for (int64_t i = 0; i < n; ++i) os << i << " ";
    os << "</DataArray>\n" << I3 << "</Verts>\n" << I2 << "</Piece>\n" << I1 << "</PolyData>\n</VTKFile>\n";
    os.flush();
    return os ? BH_OK : bh_fail(BH_ERR_IO, "bh_write_vtp: write failed");
}

// Bucket boxes of a remote domain (src/exchange.cpp:45-71): the cell of
// depth bucket_bits / 3 that each bucket prefix names, in the reference's
// arithmetic (cell size span / 2^d; minimum corner bbox.min + (i 2^-d) span).
extern "C" int bh_let_bucket_boxes(const uint64_t* prefixes, int64_t n, int bucket_bits, const double bbox[6],
                                   double* boxes_out)
{
    if (n < 0 || !bbox || bucket_bits < 0 || bucket_bits > 63 || (n > 0 && (!prefixes || !boxes_out)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_let_bucket_boxes: bad arguments");
    const int d = bucket_bits / 3;
    const double span[3] = {bbox[3] - bbox[0], bbox[4] - bbox[1], bbox[5] - bbox[2]};
    const double scale = 1.0 / static_cast<double>(1ull << d);
    double cell[3];
    for (int a = 0; a < 3; ++a) cell[a] = span[a] / static_cast<double>(1 << d);
    for (int64_t k = 0; k < n; ++k) {
        const uint64_t bits = d == 0 ? 0 : prefixes[k] >> (63 - 3 * d);
        for (int a = 0; a < 3; ++a) {
            uint32_t v = 0;
            for (int b = 0; b < d; ++b) v |= static_cast<uint32_t>((bits >> (3 * b + a)) & 1u) << b;
            const double lo = bbox[a] + (static_cast<double>(v) * scale) * span[a];
            boxes_out[6 * k + a] = lo;
            boxes_out[6 * k + 3 + a] = lo + cell[a];
        }
    }
    return BH_OK;
}
