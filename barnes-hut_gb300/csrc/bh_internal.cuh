// Internal definitions shared by the CUDA translation units of libbh_gpu.so.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "bh_common.h"

#define BH_CUDA_TRY(expr)                                                               \
    do {                                                                                \
        cudaError_t bh_e_ = (expr);                                                     \
        if (bh_e_ != cudaSuccess)                                                       \
            return bh_fail(BH_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(bh_e_)); \
    } while (0)

// After a kernel launch: report a launch error, count the launch.
#define BH_LAUNCH_CHECK(ctx)        \
    do {                            \
        BH_CUDA_TRY(cudaGetLastError()); \
        ++(ctx)->launches;          \
    } while (0)

namespace bh {
struct MlpDev;

constexpr int kMaxDepth = 21;          // depth of a leaf (one body key)
constexpr int kSortPasses = 8;         // 8-bit digits over the 63-bit key
constexpr int kRadix = 256;
constexpr int kSortThreads = 512;      // onesweep tile: 512 threads x 8 keys
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

// SM count of the current device (cudaDevAttrMultiProcessorCount), read once
// per device and cached; grids are sized in multiples of it.  1 when the
// device cannot be queried (the launch that follows reports the error).
int num_sms();

// Device error word bits (OR-ed by kernels, read back by bh_context_sync).
enum : unsigned {
    kErrNonFinite = 1u << 0,
    kErrTimeout = 1u << 1,
    kErrOverflow = 1u << 2,
    kErrCapacity = 1u << 3,
};

// Bits of a key kept by mortonPrefix(key, d) (src/morton_keys.cpp:28-32).
__host__ __device__ inline uint64_t prefix_mask(int d)
{
    return d == 0 ? 0ull : (~0ull << (63 - 3 * d));
}

// Deepest depth at which two distinct keys share a cell: 0..20.
__device__ inline int common_depth(uint64_t a, uint64_t b)
{
    const int hb = 63 - __clzll((long long)(a ^ b));  // highest differing bit, 0..62
    return (62 - hb) / 3;
}

// 1/sqrt(x) in FP64 from the FP32 hardware estimate y0 (relative error below
// 2^-21 with the truncation below) and one third-order Householder step for
// f(y) = 1/y^2 - x:
//   e = 1 - x y0^2,   y1 = y0 (1 + e/2 + 3 e^2 / 8),
// whose truncation error is 5/16 e^3 (below 2^-61); with the roundings of
// the FP64 steps the result is within about one ulp.  Outside [2^-100, 2^100]
// (and for 0, inf, NaN), where the FP32 estimate cannot represent the value,
// the library's rsqrt.  The non-bit-exact FP64 walk and the direct terms use
// it: 5 FP64 operations instead of a full-precision square root sequence.
__device__ __forceinline__ double rsqrt_hh(double x)
{
    const long long xb = __double_as_longlong(x);
    const int xe = (int)(xb >> 52);             // biased exponent for x >= 0; < 0 for x < 0
    if (xe < 923 || xe > 1122) return rsqrt(x);  // outside [2^-100, 2^100): also 0, inf, NaN
    // x truncated to FP32 and the estimate widened back, on the bit patterns
    // (integer operations: the FP64 pipe, at 1/64 of the FP32 rate, is the
    // walk's bound).  Truncation adds at most 2^-23 to the estimate's error.
    const float xf = __int_as_float(((xe - 896) << 23) | (int)((xb >> 29) & 0x7FFFFF));
    const int yb = __float_as_int(rsqrtf(xf));
    const double y0 = __longlong_as_double(((long long)(((yb >> 23) & 0xFF) + 896) << 52) |
                                           ((long long)(yb & 0x7FFFFF) << 29));
    const double h = x * y0;
    const double e = fma(-h, y0, 1.0);
    const double t = e * fma(e, 0.375, 0.5);
    return fma(y0, t, y0);
}

__device__ __forceinline__ float narrow_trunc(double x);

// x^(-3/2), the r^-3 of a monopole term from r^2, for the non-bit-exact
// FP64 walk and the direct terms: the FP32 estimate y0 of x^-1/2 as in
// rsqrt_hh, e = 1 - x y0^2, and x^-3/2 = y0^3 (1 - e)^-3/2 =
// y0^3 (1 + 3/2 e + 15/8 e^2 + ...): with |e| < 2^-20 the next term is below
// 2^-58 relative.  Three FP64 operations:
//  * y0 has a 24-bit significand s, so y0^2 (s^2 < 2^48) is formed exactly
//    and y0^3 (s^3 < 2^72) rounded to nearest from integer products;
//  * the e^2 term is below 2^-39: FP32 gives it to 2^-61 and it is added to 1
//    exactly as a count of 2^-52 units (below 2^13);
//  * then e, f = 3/2 e + (1 + 15/8 e^2) and y0^3 f in FP64.
// Within 4 ulps of RN(1 / RN(x RN(sqrt(x)))) (checked by bh_selftest).
__device__ __forceinline__ double rcube_hh(double x)
{
    const long long xb = __double_as_longlong(x);
    const int xe = (int)(xb >> 52);
    if (xe < 923 || xe > 1122) {  // outside [2^-100, 2^100): also 0, inf, NaN
        const double r = rsqrt(x);
        return r * r * r;
    }
    const float xf = __int_as_float(((xe - 896) << 23) | (int)((xb >> 29) & 0x7FFFFF));
    const int yb = __float_as_int(rsqrtf(xf));
    const int ey = (yb >> 23) & 0xFF;  // y0 = s 2^(ey - 150), y0 in [2^-50, 2^50]
    const unsigned long long sy = (unsigned long long)((yb & 0x7FFFFF) | 0x800000);
    // y0^2 = s^2 2^(2 ey - 300) with s^2 in [2^46, 2^48): exact.
    const unsigned long long s2 = sy * sy;
    const int t2 = (int)(s2 >> 47);
    const double y2 = __longlong_as_double(((long long)(2 * ey - 300 + 46 + t2 + 1023) << 52) |
                                           (long long)((s2 << (6 - t2)) & 0xFFFFFFFFFFFFFull));
    // y0^3 = s^3 2^(3 ey - 450) with s^3 in [2^69, 2^72): the leading 53 bits,
    // rounded to nearest (half up).
    const unsigned long long plo = s2 * sy;
    const unsigned long long phi = __umul64hi(s2, sy);  // in [2^5, 2^8)
    const int lp = 31 - __clz((int)phi);                  // 5, 6 or 7
    const int sh = lp + 12;                               // bits below the leading 53
    const unsigned long long lo2 = plo + (1ull << (sh - 1));
    const unsigned long long hi2 = phi + (lo2 < plo ? 1ull : 0ull);
    unsigned long long top = (hi2 << (64 - sh)) | (lo2 >> sh);
    int p3 = 64 + lp;
    if (top >> 53) {  // the rounding carried into a new leading bit
        top >>= 1;
        ++p3;
    }
    const double y3 = __longlong_as_double(((long long)(p3 + 3 * ey - 450 + 1023) << 52) |
                                           (long long)(top & 0xFFFFFFFFFFFFFull));
    const double e = fma(-x, y2, 1.0);
    const float ef = narrow_trunc(e);
    // round(15/8 e^2 2^52), below 2^13, read from the significand of its sum
    // with 2^23 (an FP32 addition rounds it to an integer; no conversion
    // instruction, which would share the FP64 pipe)
    const int cu = __float_as_int(fmaf(1.875f * ef, ef * 0x1p52f, 0x1p23f)) - 0x4B000000;
    const double w = __longlong_as_double(0x3FF0000000000000ll + (long long)cu);  // 1 + 15/8 e^2
    return y3 * fma(e, 1.5, w);
}

// norm + quantise of generateMortonCodes (src/morton_keys.cpp:77-94):
// t = (v - lo)/span clamped to [0, 1 - 2^-53], then (uint32)(t * 2^21).
__device__ inline uint32_t quantise_exact(double v, double lo, double span)
{
    double t = __ddiv_rn(__dsub_rn(v, lo), span);
    if (t <= 0.0) t = 0.0;
    else if (t >= 1.0) t = __longlong_as_double(0x3FEFFFFFFFFFFFFFll);  // nextafter(1, 0)
    return __double2uint_rz(__dmul_rn(t, 2097152.0));
}

// The same integer with two FP64 operations in nearly every case (FP64 runs
// at 1/64 of the FP32 rate here, comparisons included).  inv21 is
// RN(1/span) 2^21, so u = RN(d inv21) = RN(d RN(1/span)) 2^21 exactly, within
// 3 ulps (relative 3 2^-53) of t 2^21 with t = RN(d/span): the two differ by
// less than 2^-30.  The integer and fractional parts of u come from its bits
// (integer operations); where u lies in [2, 2^21 - 2] (no clamp) and its
// fractional part is farther than 2^-24 from an integer, both truncate to the
// same integer.  Elsewhere the IEEE division decides.
__device__ inline uint32_t quantise(double v, double lo, double span, double inv21)
{
    const double u = __dmul_rn(__dsub_rn(v, lo), inv21);
    const long long ub = __double_as_longlong(u);
    const int ue = (int)(ub >> 52);  // the biased exponent for u > 0 (negative u: < 0)
    if (ue >= 1024 && ue <= 1043) {  // 2 <= u < 2^21
        const int sh = 1075 - ue;    // fraction bits of u: 32 .. 51
        const unsigned long long mant = ((unsigned long long)ub & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
        const unsigned long long ip = mant >> sh;
        const unsigned long long fr = mant & ((1ull << sh) - 1ull);
        const unsigned long long lim = 1ull << (sh - 24);
        if (ip <= (1ull << 21) - 3ull && fr > lim && fr < (1ull << sh) - lim) return (uint32_t)ip;
    }
    return quantise_exact(v, lo, span);
}

// RN((0 + RN(m c)) / m) for m > 0 with two FP64 operations in nearly every
// case: the centre of mass after the single-rank merge
// (linear_octree.cpp:194-202 with m0 = com0 = 0), and the centre of mass of a
// one-body leaf ((0 + x m) / m, linear_octree.cpp:28-38,95-104).
// p = RN(m c) and the product's rounding error e = p - m c are exact (the
// error of a floating-point product is a double, and one FMA computes it:
// the TwoProduct of Ogita, Rump and Oishi), so p / m = c + e / m with
// |e / m| <= ulp(c).  The correctly rounded quotient is therefore c, or the
// neighbour of c on the side of e, whichever is within ulp(c) / 2 of p / m:
// |e| against m ulp(c) / 2, compared exactly on the bit patterns after
// scaling |e| by a power of two (integer operations).  Powers of two
// (uneven spacing below), exact ties and exponents outside 2^+-200 take the
// IEEE division.
__device__ inline double merge_div(double m, double c)
{
    const double p = __dmul_rn(m, c);
    const long long cb = __double_as_longlong(c), mb = __double_as_longlong(m);
    const int ce = (int)((cb >> 52) & 0x7FF), me = (int)((mb >> 52) & 0x7FF);
    if (mb <= 0 || ce < 823 || ce > 1223 || me < 823 || me > 1223 || (cb & 0x000FFFFFFFFFFFFFll) == 0)
        return __ddiv_rn(__dadd_rn(0.0, p), m);
    const double e = fma(-c, m, p);
    const long long eb = __double_as_longlong(e);
    const long long ea = eb & 0x7FFFFFFFFFFFFFFFll;
    if (ea == 0) return c;
    // |e| 2^(1076 - ce) against m: |e| < m 2^(ce - 1076) = m ulp(c) / 2
    const long long es = ea + ((long long)(1076 - ce) << 52);
    if (es < mb) return c;
    if (es > mb) return __longlong_as_double(((eb ^ cb) >= 0) ? cb + 1 : cb - 1);
    return __ddiv_rn(__dadd_rn(0.0, p), m);
}

// 1/x to within about one ulp (not correctly rounded): the FP32 hardware
// estimate (x narrowed and the estimate widened on the bit patterns, integer
// operations) refined by one third-order Newton step, y1 = y0 (1 + e + e^2)
// with e = 1 - x y0, whose truncation error e^3 is below 2^-60.  Outside
// [2^-100, 2^100] (and for 0, negative, inf, NaN) the IEEE reciprocal.
__device__ __forceinline__ double rcp_nr(double x)
{
    const long long xb = __double_as_longlong(x);
    const int xe = (int)(xb >> 52);
    if (xe < 923 || xe > 1122) return __drcp_rn(x);
    const float xf = __int_as_float(((xe - 896) << 23) | (int)((xb >> 29) & 0x7FFFFF));
    const int yb = __float_as_int(__frcp_rn(xf));
    const double y0 = __longlong_as_double(((long long)(((yb >> 23) & 0xFF) + 896) << 52) |
                                           ((long long)(yb & 0x7FFFFF) << 29));
    const double e = fma(-x, y0, 1.0);
    return fma(y0, fma(e, e, e), y0);
}

// x truncated to FP32 on the bit patterns (integer operations; the FP64
// conversion instructions run on the slow FP64 pipe): relative error below
// 2^-23; magnitudes below 2^-126 give a signed zero, above 2^127 the
// converted value.  widen() is the exact inverse direction.
__device__ __forceinline__ float narrow_trunc(double x)
{
    const long long xb = __double_as_longlong(x);
    const int e = (int)((xb >> 52) & 0x7FF);
    const int sign = (int)((unsigned long long)xb >> 63) << 31;
    if (e <= 896) return __int_as_float(sign);
    if (e >= 1151) return __double2float_rn(x);
    return __int_as_float(sign | ((e - 896) << 23) | (int)((xb >> 29) & 0x7FFFFF));
}

// narrow_trunc(x - widen(narrow_trunc(x))): the part of x below its FP32
// truncation, itself truncated to FP32, from the bit patterns.  Where
// narrow_trunc keeps x's exponent, x - hi is x's low 29 significand bits
// times 2^(e - 1075), exactly; the FP64 subtraction is left for the other
// exponents.
__device__ __forceinline__ double widen(float f);
__device__ __forceinline__ float low_part(double x)
{
    const long long xb = __double_as_longlong(x);
    const int e = (int)((xb >> 52) & 0x7FF);
    if (e <= 896 || e >= 1151) return narrow_trunc(x - widen(narrow_trunc(x)));
    const unsigned low = (unsigned)(xb & 0x1FFFFFFFll);
    if (low == 0) return 0.0f;  // x - hi = +0.0
    const int p = 31 - __clz((int)low);  // leading bit of the remainder, 0..28
    const int ed = e - 52 + p;           // its FP64 exponent
    const unsigned sign = (unsigned)((unsigned long long)xb >> 63) << 31;
    if (ed <= 896) return __int_as_float((int)sign);
    const unsigned frac = low - (1u << p);
    const unsigned m23 = p <= 23 ? frac << (23 - p) : frac >> (p - 23);
    return __int_as_float((int)(sign | ((unsigned)(ed - 896) << 23) | m23));
}

__device__ __forceinline__ double widen(float f)
{
    const int b = __float_as_int(f);
    const int e = (b >> 23) & 0xFF;
    const long long sign = (long long)((unsigned)b >> 31) << 63;
    if (e == 0 || e == 0xFF) return (double)f;
    return __longlong_as_double(sign | ((long long)(e + 896) << 52) | ((long long)(b & 0x7FFFFF) << 29));
}

// RN(w / m) for m > 0 with four FP64 operations in nearly every case, given
// r = rcp_nr(m).  q0 = RN(w r) is within a few ulps of w/m; one correction
// q1 = q0 + (w - q0 m) r (Markstein's) brings it within one ulp, where the
// residual w - q1 m is exact (the remainder of a faithful quotient is a
// double).  RN(w/m) is then q1 or its neighbour on the residual's side,
// decided exactly on the bit patterns as in merge_div; a residual of an ulp
// times m or more (q1 not faithful), a power-of-two q1, a tie or exponents
// outside 2^+-200 take the IEEE division.
__device__ inline double div_exact(double w, double m, double r)
{
    const long long mb = __double_as_longlong(m);
    const int me = (int)((mb >> 52) & 0x7FF);
    const double q0 = w * r;
    const double rho = fma(-q0, m, w);
    const double q1 = fma(rho, r, q0);
    const double rho1 = fma(-q1, m, w);
    const long long qb = __double_as_longlong(q1);
    const int eq = (int)((qb >> 52) & 0x7FF);
    if (mb <= 0 || me < 823 || me > 1223 || eq < 823 || eq > 1223 || (qb & 0x000FFFFFFFFFFFFFll) == 0)
        return __ddiv_rn(w, m);
    const long long rb = __double_as_longlong(rho1);
    const long long ra = rb & 0x7FFFFFFFFFFFFFFFll;
    if (ra == 0) return q1;
    const long long es = ra + ((long long)(1076 - eq) << 52);  // |rho1| / (ulp(q1) / 2)
    if (es < mb) return q1;
    const long long es2 = ra + ((long long)(1075 - eq) << 52);  // |rho1| / ulp(q1)
    if (es2 >= mb) return __ddiv_rn(w, m);
    if (es > mb) return __longlong_as_double(((rb ^ qb) >= 0) ? qb + 1 : qb - 1);
    return __ddiv_rn(w, m);
}

// One node of the compressed octree as the traversal reads it (48 bytes).
// A node stands for the reference's chain of single-child nodes from depth
// `top` down to `depth` (all with identical mass and centre of mass), so it
// is accepted exactly when the reference would accept any node of the chain.
struct __align__(16) TreeRec {
    double cx, cy, cz;  // centre of mass after the single-rank merge
    double m;           // mass
    int32_t child;      // first child slot, or -1 for a leaf
    int32_t leaf;       // leaf id for a leaf, -1 otherwise
    uint8_t nchild;     // 0 for a leaf, 2..8 otherwise
    uint8_t depth;      // bottom depth of the chain (21 for a leaf)
    uint8_t top;        // top depth of the chain
    uint8_t pad0;
    int32_t pad1;
};
static_assert(sizeof(TreeRec) == 48, "TreeRec layout");

}  // namespace bh

// The context behind the opaque bh_context handle.
struct bh_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    int64_t cap = 0;  // bodies the buffers hold
    int64_t n = 0;    // bodies currently loaded
    double t = 0.0;   // simulation time (bh_step)
    void* alloc_base = nullptr;  // the single device allocation

    // Body state, structure of arrays, in the current (last sorted) order.
    double *px = nullptr, *py = nullptr, *pz = nullptr;
    double *vx = nullptr, *vy = nullptr, *vz = nullptr;
    double *ax = nullptr, *ay = nullptr, *az = nullptr;
    double* m = nullptr;
    uint64_t* id = nullptr;
    uint64_t* key = nullptr;
    // Second body set; the permutation gathers into it, then the sets swap.
    double *px2 = nullptr, *py2 = nullptr, *pz2 = nullptr;
    double *vx2 = nullptr, *vy2 = nullptr, *vz2 = nullptr;
    double* m2 = nullptr;
    uint64_t* id2 = nullptr;

    // Radix sort scratch.
    uint64_t* key_alt = nullptr;
    uint32_t* perm = nullptr;      // after the sort: previous position per slot
    uint32_t* perm_alt = nullptr;
    uint32_t* hist = nullptr;      // kSortPasses x 256 digit counts, then starts
    uint32_t* lookback = nullptr;  // kSortPasses x tiles x 256 status words
    uint32_t* tile_ctr = nullptr;  // kSortPasses tile counters
    int64_t max_tiles = 0;

    // Bounding box: 6 doubles, block partials and the last-block ticket.
    double* bbox = nullptr;
    double* bbox_part = nullptr;
    unsigned* bbox_ticket = nullptr;
    int bbox_blocks = 0;

    // Tree build (sizes in bodies; L <= n leaves, B <= n branching nodes).
    int32_t* head = nullptr;        // scan scratch, n + 1
    int32_t* leaf_first = nullptr;  // first body of each leaf, n + 1
    int32_t* body_leaf = nullptr;   // leaf id of each body
    uint64_t* leaf_key = nullptr;
    double4_32a* leaf_s = nullptr;  // leaf sums {m x, m y, m z, m}
    int8_t* cdep = nullptr;         // common depth of leaves j-1, j (boundary j), n + 1
    int32_t* bnd_pl = nullptr;      // boundary j: start leaf of the node it splits, n + 1
    int32_t* bnd_pr = nullptr;      // boundary j: end leaf (exclusive) of that node, n + 1
    int32_t* bnd_next = nullptr;    // boundary j: next boundary no deeper than j, n + 1
    int32_t* split_node = nullptr;  // boundary j: the branching node it splits, n + 1
    int8_t* split_rank = nullptr;   // boundary j: its rank among that node's splits, n + 1
    int32_t* ansv_blk = nullptr;    // per-block summaries of the boundary pass
    int32_t* rep_node = nullptr;    // branching-node id of a representative boundary
    int32_t* node_rep = nullptr;    // representative boundary of each node
    int32_t* node_a = nullptr;      // first leaf of each node
    int32_t* node_e = nullptr;      // end leaf (exclusive) of each node
    int32_t* node_nchild = nullptr;
    int32_t* node_cs = nullptr;     // first child slot
    uint8_t* node_depth = nullptr;
    double4_32a* node_s = nullptr;  // branching-node sums {m x, m y, m z, m}
    int32_t* slot_ref = nullptr;    // >= 0 leaf id, < 0 ~node id
    uint8_t* slot_top = nullptr;
    int32_t* depth_off = nullptr;   // 23 offsets into depth_nodes (by depth)
    int32_t* depth_nodes = nullptr; // node ids bucketed by depth
    bh::TreeRec* rec = nullptr;     // traversal records, slot 0 = root
    int32_t* counts = nullptr;      // device scalars: [0]=L, [1]=B, [2]=slots
    int32_t* scan_tmp = nullptr;    // block sums of the device scans
    bool tree_valid = false;
    bool keys_valid = false;   // keys and their digit histograms are current
    bool bbox_valid = false;
    bool sorted_valid = false; // bodies are in sorted-key order

    bool tree_far = false;      // the tree holds far-field masses (FP32 modes)
    bool tree_moments = false;  // the tree's second moments are current
    bool tree_rec = false;      // rec holds the tree's FP64 records (a fused far-field build leaves them out)
    bool build_merge = true;    // apply the single-rank exchange merge in builds
    int num_direct = BH_NUM_MASSIVE;  // bodies with id < num_direct: FP64 direct terms in FP32 modes

    // Traversal.
    unsigned long long* inter_count = nullptr;
    int32_t* body_count = nullptr;  // accepted interactions per body (last traversal)
    // FP32 node records (FP32 modes): centre of mass as hi + lo floats, G m,
    // and the topology word; 2n entries each.
    float4* fA = nullptr;   // {hi.x, hi.y, hi.z, G m}
    float4* fB = nullptr;   // {lo.x, lo.y, lo.z, bits of ref (child or leaf id)}
    uint32_t* fmeta = nullptr;  // nchild | depth << 8 | leaf << 16
    double4_32a* d4 = nullptr;  // FP64 walk: {cx, cy, cz, G m} per slot
    bool fnodes_fused = false;  // fA / fB / fmeta are current for rec and fnodes_G
    double fnodes_G = 0.0;
    float* fspread = nullptr;   // sqrt(Q / m) per slot (second moment about the centre of mass)
    double* leaf_q = nullptr;   // second moments of leaves and branching nodes
    double* node_q = nullptr;
    bh::MlpDev* mlp_dev = nullptr;      // learned model (bh_learned_set_model)
    double learn_theta_max = 0.0;
    double learn_budget = 0.0;   // per-body error budget of the learned criterion
    double learn_band = 0.5;     // decades around the allowance the network decides
    double learn_frac = 0.25;    // largest share of the remaining allowance one candidate takes
    unsigned long long* lstats = nullptr;  // candidates, network accepts, fallbacks, analytic accepts
    double* direct = nullptr;   // 4 doubles per direct body: x, y, z, G m (by id)
    int32_t* direct_present = nullptr;  // 1 when body id k was found

    // Phase timing (bh_set_profiling): CUDA events around each phase of a
    // step, read back at the next synchronisation.
    bool prof = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    struct Mark { int phase; cudaEvent_t a, b; };
    std::vector<Mark> marks;
    double phase_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int64_t launches = 0;  // kernels of this library enqueued so far
    // CUDA graphs of one kicked step, replayed while their configuration
    // holds; one per body set the step starts from (the sets alternate).
    bool graphs = true;
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        int64_t n = -1, launches = 0;
        int mode = -1, merge = -1, nd = -1;
        double dt = 0.0, theta = 0.0, G = 0.0;
        double learn[4] = {0.0, 0.0, 0.0, 0.0};  // learned walk: theta_max, budget, band, frac
    } sg[2];

    // Error word raised by kernels and a pinned mirror for readback.
    unsigned* err = nullptr;
    unsigned* h_err = nullptr;
    double* h_small = nullptr;  // pinned host scratch (64 doubles)
    void* let_buf = nullptr;    // locally essential tree export scratch (bh_let_export)
    size_t let_bytes = 0;
    void* imp_buf = nullptr;    // pseudo-leaf tree scratch (bh_pseudo_leaf_tree): records
    size_t imp_bytes = 0;
    void* imp_buf2 = nullptr;   // and entries / cells
    size_t imp_bytes2 = 0;
    void* letf_buf = nullptr;   // merged map of the LET force paths
    size_t letf_bytes = 0;
};

namespace bh {

// Kernel launch wrappers (defined in the .cu files).  Each enqueues on
// ctx->stream and returns BH_OK or a launch error.
int launch_drift_bbox(bh_context* ctx, double dt, bool kick, bool drift);
int launch_keys(bh_context* ctx, bool with_hist);
int launch_hist(bh_context* ctx);
int bbox_partial_bytes(int blocks);
size_t sort_smem_bytes();
int64_t scan_tmp_ints(int64_t n_max);
// Ints of the per-block summaries of the tree build's boundary pass for up
// to n bodies.
int64_t boundary_pass_ints(int64_t n);
int launch_sort(bh_context* ctx);
int launch_permute(bh_context* ctx);
// The permutation gathers into the second body set; the two sets then trade
// places (host pointers only).
void swap_body_sets(bh_context* ctx);
// Digit counts for sort_passes_raw (hist zeroed by the caller).
int launch_digit_hist(int64_t n, const uint64_t* keys, uint32_t* hist, cudaStream_t st);
// The onesweep passes over raw buffers (the allocation-free sort entry).
int sort_passes_raw(int64_t n, const uint64_t* keys_in, uint64_t* keys_out, uint32_t* vals_out, uint64_t* key_alt,
                    uint32_t* val_alt, uint32_t* hist, uint32_t* lookback, uint32_t* tile_ctr, unsigned* err,
                    cudaStream_t stream);
// Builds the octree over the sorted bodies with the given masses (ctx->m
// for the reference's tree; the far-field masses for the FP32 modes);
// `moments` also computes the second moments (spread per slot).
// far_fused: the far-field tree of an FP32 form, whose centres of mass need
// no bit-exact quotient; the FP32 node records for G are written too.
// far_masses: the bodies with id < num_direct count as massless (the FP32
// forms' far-field tree).
int launch_build(bh_context* ctx, const double* mass, bool moments = false, bool far_fused = false, double G = 0.0,
                 bool far_masses = false);
// The FP64 records of the current tree, written by a rebuild of its node
// values where the last build left them out (no-op otherwise).
int ensure_rec(bh_context* ctx);
// Waits for the context's stream and turns a raised device error word into
// a status (clearing the word).
int finish(bh_context* ctx, const char* fn);
// Positions and G m of the bodies with id < num_direct (ctx->direct, by id).
int launch_direct_extract(bh_context* ctx, double G);

int launch_traverse(bh_context* ctx, double theta, double G, double soft2, int mode, double kick_h);
int launch_traverse_masked(bh_context* ctx, double theta, double G, double soft2, double kick_h, bool fp64,
                           bool group = false);
int launch_traverse_learned(bh_context* ctx, double theta, double G, double soft2, double kick_h);
// FP32 node records (hi/lo centres, G m, topology) from the FP64 records.
int launch_fp32_nodes(bh_context* ctx, double G);

// Device-wide exclusive scan of n int32 values (in may equal out); the
// total is written to *total (device pointer).  n is read from n_dev when
// n_dev != nullptr (device-side count, at most n_max), else n_max is used.
int device_exclusive_scan(bh_context* ctx, const int32_t* in, int32_t* out, int64_t n_max,
                          const int32_t* n_dev, int32_t* total);
// The leaves of n sorted keys (runs of equal keys) from a scan of their head
// flags: body_leaf[i] (the leaf of body i), leaf_first[l] (its first body,
// with leaf_first[L] = n), leaf_key[l], and *total = L.
int device_number_leaves(bh_context* ctx, const uint64_t* key, int64_t n, int32_t* total, int32_t* body_leaf,
                         int32_t* leaf_first, uint64_t* leaf_key);
// The same over a caller's block-sum scratch of scan_tmp_ints(n_max) ints.
int device_exclusive_scan_tmp(bh_context* ctx, const int32_t* in, int32_t* out, int64_t n_max,
                              const int32_t* n_dev, int32_t* total, int32_t* tmp);

}  // namespace bh
