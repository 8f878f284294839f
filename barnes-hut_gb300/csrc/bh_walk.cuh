// Definitions shared by the masked warp walks: the FP64 list, FP32
// far-field and collection walks (bh_traverse_fp32.cu) and the learned walk
// (bh_traverse_learned.cu).
#pragma once

#include "bh_internal.cuh"
#include "bh_mlp.cuh"

namespace bh {
namespace {

constexpr int kWarps = 4;
constexpr int kThreads = 32 * kWarps;
constexpr int kStack = 512;   // sibling-range entries per warp
constexpr int kList = 96;     // staged interactions per warp
// The FP64 walk's: a longer list, so that each balanced evaluation spreads
// more pairs over the warp (fewer flushes), and a shorter stack, so that the
// block still fits 5 per SM.  The deepest stack measured is 202 entries
// (4M bodies, theta = 0.3); past the bound the walk reports an overflow.
constexpr int kStack64 = 352;
constexpr int kList64 = 128;
// The group form's list: longer, for fewer flushes (its entries carry no lane
// masks); 144 keeps 7 blocks per SM.  The per-body FP32 walk ran slower with
// it, the learned walk no faster.
constexpr int kListGroup = 144;
constexpr int kSegs = 63;     // FP64 list evaluation: run slots body + thread, 0..62
constexpr int kSlotBits = 28; // slot index bits of a stack entry (count - 1 in the top 3)
constexpr float kMargin = 1e-5f;  // relative margin of the FP32 group tests
constexpr float kAbsErr = 1e-6f;  // bound on FP32 coordinate error, relative to magnitudes

enum { kLearnNone = 0, kLearnInfer = 1, kLearnCollect = 2 };

// Per-block shared memory of the walk.  Tables a variant does not use shrink
// to one element, so that the FP32 walk fits 8 blocks (32 warps) per SM; the
// FP64 walk fits 5 (6 ran slower: the FP64 pipe is already 86 % busy).
template <bool kFP64, int kLearn, bool kGroup = false>
struct WalkSmem {
    static constexpr int kW64 = kFP64 ? kWarps : 1;      // FP64-only tables
    static constexpr bool kLL = kFP64;                    // leaf ids kept for the evaluation's own-leaf test
    static constexpr bool kF = kLearn == 1;              // network input rows
    static constexpr int kStk = kFP64 ? kStack64 : kStack;  // stack entries per warp
    static constexpr int kLst = kFP64 ? kList64 : kGroup ? kListGroup : kList;  // staged entries per warp
    int2 stack[kWarps][kStk];  // sibling ranges: {first | (count - 1) << 28, lane mask}
    // FP32 node data of the staged entries: {x, y, z, G m} per entry, or in
    // the plain FP32 walk entry pairs {x0, x1, y0, y1}, {z0, z1, w0, w1}
    float4 lst[kFP64 ? 1 : kWarps][kFP64 ? 1 : kLst];
    int lst_node[kWarps][kLst];
    int lst_leaf[kLL ? kWarps : 1][kLL ? kLst : 1];
    alignas(8) unsigned lst_mask[kWarps][kLst];
    float side2f[kMaxDepth + 1];
    double side2d[kMaxDepth + 1];
    float2 sthr[kMaxDepth + 1];  // group-test distances per depth: side sqrt(1 + margin) / theta, (1 - margin)
    float feat[kF ? kWarps : 1][kF ? 32 : 1][9];
    uint8_t plist[kW64][kFP64 ? kLst : 1][32];  // FP64: each lane's own entries, in order
    // FP64: the balanced evaluation's per-warp tables (see the flush).
    int poff[kW64][33];                     // first pair of each lane, then the total
    double bpos[kW64][3][kFP64 ? 32 : 1];   // the bodies' positions
    int bleaf[kW64][kFP64 ? 32 : 1];        // the bodies' leaf ids
    double seg[kW64][3][kFP64 ? kSegs : 1];  // each (thread, body) run's partial sums
    uint16_t segn[kW64][kFP64 ? kSegs : 1];  // and its interaction count
};

// The resident blocks per SM each layout is sized for, in the SM's 228 KB of
// shared memory (1 KB of it reserved per block); registers allow no more.
constexpr size_t kSmemPerSM = 228 * 1024, kSmemReserved = 1024;
static_assert(5 * (sizeof(WalkSmem<true, kLearnNone>) + kSmemReserved) <= kSmemPerSM, "FP64 walk: 5 blocks per SM");
static_assert(8 * (sizeof(WalkSmem<false, kLearnNone>) + kSmemReserved) <= kSmemPerSM, "FP32 walk: 8 blocks per SM");
static_assert(7 * (sizeof(WalkSmem<false, kLearnNone, true>) + kSmemReserved) <= kSmemPerSM,
              "group walk: 7 blocks per SM");

// Packed FP32 pairs (two floats in one 64-bit register): one f32x2
// instruction does two FP32 operations, each rounded as the scalar one.
using f32x2 = unsigned long long;

__device__ __forceinline__ f32x2 pk(float lo, float hi)
{
    f32x2 d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}

__device__ __forceinline__ void upk(f32x2 v, float& lo, float& hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b)
{
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b)
{
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c)
{
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

}  // namespace

struct FParams {
    int64_t n;
    const double* px;
    const double* py;
    const double* pz;
    const uint64_t* id;
    const int32_t* body_leaf;
    const float4* A;
    const float4* B;
    const uint32_t* meta;
    const TreeRec* rec;
    const double4_32a* d4;
    const float* spread;
    const double* bbox;
    double theta2;
    double soft2;
    double G;
    const double* direct;
    const int32_t* present;
    int nd;
    double kick_h;
    double* ax;
    double* ay;
    double* az;
    double* vx;
    double* vy;
    double* vz;
    unsigned long long* inter_count;
    int32_t* body_count;
    unsigned* err;
    int64_t max_pops;
    // learned criterion
    const MlpDev* mlp;
    float theta_max2;
    float l_budget;  // per-body error budget (relative to the group's direct-term acceleration)
    float l_band;    // analytic estimate decides outside +-l_band decades of the allowance
    float l_frac;    // a candidate may take at most this fraction of the remaining allowance
    unsigned long long* lstats;  // candidates, network accepts, fallbacks, analytic accepts
    // collection
    int32_t* c_group;
    int32_t* c_slot;
    uint32_t* c_mask;
    float* c_feat;
    float* c_ascale;
    unsigned long long* c_count;
    int64_t c_cap;
};

// Prepares the FP32 node records and the direct bodies and fills the walk's
// parameters (kick_h and the learned/collection fields are the caller's).
int prepare_walk(bh_context* ctx, double theta, double G, double soft2, bool fp64, FParams& p);

}  // namespace bh
