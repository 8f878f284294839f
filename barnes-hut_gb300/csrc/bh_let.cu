// Locally essential tree export on the GPU: the cells of this rank's tree
// that a remote rank needs, selected as createInteractionListForRank
// (src/exchange.cpp:117-179) selects them, and the remote domain's bucket
// boxes of exchangeEssentialTrees (src/exchange.cpp:45-71).
//
// The reference walks its hash map depth first from the root.  A cell is
// opened when s^2 >= theta2 * d^2 for any remote box (s the largest side of
// the cell's box from getBoundingBoxForCell, src/bounding_box.cpp:55-75; d^2
// min_distance_sq, :10-18) and its depth is below max_depth; otherwise it is
// kept.  Which cells are kept does not depend on the visiting order (each
// cell is reached through its ancestors only), so the GPU walks the
// compressed tree breadth first instead: one warp per frontier node, lanes
// over the remote boxes, one launch per chain level (at most 22).  A node
// stands for the chain of single-child cells from `top` to `depth`; the warp
// tests the chain's cells from the top down and either keeps one of them,
// stops (a failing depth-21 leaf below max_depth has no children and is
// dropped, as in the reference), or appends the node's children to the next
// frontier.  Every cell box and distance is evaluated with the reference's
// operation order in round-to-nearest FP64 without contraction, so the kept
// set is the reference's bit for bit.  The kept cells are compacted in slot
// order with the device scan.
#include "bh_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace {

constexpr int kLetThreads = 256;
constexpr int kLetWarps = kLetThreads / 32;
constexpr int kLetLevels = bh::kMaxDepth + 1;  // chain tops 0..21

struct LetGeom {
    double lo[3];    // global box minimum corner
    double span[3];  // global box extent per axis (max - min)
};

// std::max(a, b) of the reference: (a < b) ? b : a.
__device__ __forceinline__ double ref_max(double a, double b) { return (a < b) ? b : a; }

// Integer cell coordinate on one axis from the top 3 d bits of a prefix.
__device__ __forceinline__ uint32_t cell_axis(uint64_t prefix, int d, int axis)
{
    if (d == 0) return 0;
    const uint64_t bits = prefix >> (63 - 3 * d);
    uint32_t v = 0;
    for (int b = 0; b < d; ++b) v |= (uint32_t)((bits >> (3 * b + axis)) & 1ull) << b;
    return v;
}

// FP32 prescreen of the box tests.  With every coordinate of the cell, the
// boxes and the global box at most M in magnitude (2^-20 < M < 2^40), each
// FP32 separation e_f lies within 2^-22 M of the exact one (the two operand
// roundings, 2^-24 M each, and the FP32 subtraction's, 2^-23 M) and the
// reference's FP64 separation within 2^-52 M of it, so within delta =
// 2^-21 M of each other; the FP32 squares, sums and products stay within
// 2^-20 relative.  A test is decided in FP32 when s^2 clears theta^2 d^2 by
// those margins either way, and in FP64 otherwise.
struct LetScreen {
    int on;         // 0: every test in FP64
    float delta;    // 2^-21 M
    float theta2f;  // (float) theta2
};

constexpr int kLetGroup = 32;  // boxes per group of the prefilter

// Whether the cell (prefix, d) fails the opening test against any of the nb
// remote boxes; warp-uniform result.  Cell box: size = span / 2^d,
// min = gmin + (ix * 2^-d) * span, max = min + size (all RN).
//
// With the prescreen on, the boxes are first taken in groups of kLetGroup
// consecutive boxes (bucket order, so spatially close), each with the FP32
// hull of its members' FP32 copies (grpf: min of the minima, max of the
// maxima).  Every step of the prescreen's lower bound dlo is monotone in the
// box corners (RN subtraction, fmaxf, the FMA of non-negative terms), so a
// hull's dlo is at most each member's; a group whose hull the prescreen
// decides "does not open" holds no member the prescreen would not also
// decide so, and is skipped.  Only the remaining groups are tested box by
// box, exactly as before.
__device__ bool cell_opens(uint64_t prefix, int d, const LetGeom& g, const double* __restrict__ boxes,
                           const float* __restrict__ boxf, const float* __restrict__ grpf, int nb, double theta2,
                           LetScreen sc, int lane)
{
    const double scale = 1.0 / (double)(1ull << d);  // exact
    double lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // span / 2^d: the quotient by a power of two equals the product by
        // its exact reciprocal (the same real number, rounded once).
        const double size = __dmul_rn(g.span[a], scale);
        lo[a] = __dadd_rn(g.lo[a], __dmul_rn(__dmul_rn((double)cell_axis(prefix, d, a), scale), g.span[a]));
        hi[a] = __dadd_rn(lo[a], size);
    }
    double s = __dsub_rn(hi[0], lo[0]);
    s = ref_max(s, __dsub_rn(hi[1], lo[1]));
    s = ref_max(s, __dsub_rn(hi[2], lo[2]));
    const double s2 = __dmul_rn(s, s);
    const float s2f = (float)s2;
    float lof[3], hif[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lof[a] = (float)lo[a];
        hif[a] = (float)hi[a];
    }
    constexpr float kUp = 1.0f + 0x1p-20f, kDn = 1.0f - 0x1p-20f;
    // The prescreen's lower bound on d^2 for an FP32 box r (min xyz, max xyz).
    auto dlo_of = [&](const float* __restrict__ rf) {
        float dlo = 0.0f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float ef = fmaxf(0.0f, fmaxf(lof[a] - __ldg(rf + 3 + a), __ldg(rf + a) - hif[a]));
            const float l = fmaxf(ef - sc.delta, 0.0f);
            dlo = fmaf(l, l, dlo);
        }
        return dlo;
    };
    auto box_opens = [&](int k) {
        if (sc.on) {
            const float* rf = boxf + 6 * (int64_t)k;
            float dlo = 0.0f, dhi = 0.0f;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float ef = fmaxf(0.0f, fmaxf(lof[a] - __ldg(rf + 3 + a), __ldg(rf + a) - hif[a]));
                const float l = fmaxf(ef - sc.delta, 0.0f), h = ef + sc.delta;
                dlo = fmaf(l, l, dlo);
                dhi = fmaf(h, h, dhi);
            }
            if (s2f * kDn >= sc.theta2f * dhi * kUp) return true;
            if (s2f * kUp < sc.theta2f * dlo * kDn) return false;
        }
        const double* r = boxes + 6 * (int64_t)k;
        double e[3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
            e[a] = ref_max(0.0, ref_max(__dsub_rn(lo[a], __ldg(r + 3 + a)), __dsub_rn(__ldg(r + a), hi[a])));
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(e[0], e[0]), __dmul_rn(e[1], e[1])), __dmul_rn(e[2], e[2]));
        return s2 >= __dmul_rn(theta2, d2);
    };
    if (sc.on) {
        const int ng = (nb + kLetGroup - 1) / kLetGroup;
        for (int g0 = 0; g0 < ng; g0 += 32) {
            const int gi = g0 + lane;
            const bool maybe = gi < ng && !(s2f * kUp < sc.theta2f * dlo_of(grpf + 6 * (int64_t)gi) * kDn);
            unsigned todo = __ballot_sync(0xffffffffu, maybe);
            while (todo) {
                const int j = g0 + __ffs(todo) - 1;
                todo &= todo - 1;
                const int k = j * kLetGroup + lane;  // kLetGroup == 32: one box per lane
                const bool f = k < nb && box_opens(k);
                if (__any_sync(0xffffffffu, f)) return true;
            }
        }
        return false;
    }
    for (int k0 = 0; k0 < nb; k0 += 32) {
        const int k = k0 + lane;
        const bool f = k < nb && box_opens(k);
        if (__any_sync(0xffffffffu, f)) return true;
    }
    return false;
}

__global__ void let_seed_kernel(int32_t* __restrict__ q0, int32_t* __restrict__ cnt)
{
    q0[0] = 0;  // the root slot
    cnt[0] = 1;
}

// One chain level of the frontier: q_in[0 .. cnt_in) -> kept depths and the
// next level's nodes.
__global__ void __launch_bounds__(kLetThreads) let_level_kernel(
    const bh::TreeRec* __restrict__ rec, const int32_t* __restrict__ slot_ref, const int32_t* __restrict__ node_a,
    const uint64_t* __restrict__ leaf_key, const double* __restrict__ boxes, const float* __restrict__ boxf,
    const float* __restrict__ grpf, int nb, LetGeom g, double theta2, LetScreen sc, int max_depth, const int32_t* __restrict__ q_in,
    const int32_t* __restrict__ cnt_in, int32_t* __restrict__ q_out, int32_t* __restrict__ cnt_out,
    int32_t* __restrict__ keep)
{
    const int lane = threadIdx.x & 31;
    const int count = *cnt_in;
    const int nwarps = gridDim.x * kLetWarps;
    for (int w = blockIdx.x * kLetWarps + (threadIdx.x >> 5); w < count; w += nwarps) {
        const int32_t s = q_in[w];
        const bh::TreeRec r = rec[s];
        const int32_t ref = slot_ref[s];
        const uint64_t key = leaf_key[ref >= 0 ? ref : node_a[~ref]];
        int kept = -1;
        bool descend = false;
        for (int d = r.top;; ++d) {
            const bool opens = cell_opens(key & bh::prefix_mask(d), d, g, boxes, boxf, grpf, nb, theta2, sc, lane);
            if (!opens || d >= max_depth) { kept = d; break; }
            if (d < r.depth) continue;
            descend = r.nchild > 0;
            break;
        }
        if (lane == 0) {
            keep[s] = kept;
            if (descend) {
                const int32_t base = atomicAdd(cnt_out, (int32_t)r.nchild);
                for (int c = 0; c < r.nchild; ++c) q_out[base + c] = r.child + c;
            }
        }
    }
}

__global__ void let_flag_kernel(const int32_t* __restrict__ counts, const int32_t* __restrict__ keep,
                                int32_t* __restrict__ flag)
{
    const int32_t S = counts[2];
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x)
        flag[s] = keep[s] >= 0 ? 1 : 0;
}

__global__ void let_write_kernel(const int32_t* __restrict__ counts, const int32_t* __restrict__ keep,
                                 const int32_t* __restrict__ pos, const bh::TreeRec* __restrict__ rec,
                                 const int32_t* __restrict__ slot_ref, const int32_t* __restrict__ node_a,
                                 const uint64_t* __restrict__ leaf_key, uint64_t* __restrict__ o_prefix,
                                 uint8_t* __restrict__ o_depth, double* __restrict__ o_mass, double* __restrict__ o_com)
{
    const int32_t S = counts[2];
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const int d = keep[s];
        if (d < 0) continue;
        const int32_t o = pos[s];
        const int32_t ref = slot_ref[s];
        const uint64_t key = leaf_key[ref >= 0 ? ref : node_a[~ref]];
        const bh::TreeRec r = rec[s];
        o_prefix[o] = key & bh::prefix_mask(d);
        o_depth[o] = (uint8_t)d;
        o_mass[o] = r.m;
        o_com[3 * (int64_t)o] = r.cx;
        o_com[3 * (int64_t)o + 1] = r.cy;
        o_com[3 * (int64_t)o + 2] = r.cz;
    }
}

// Scratch for one export: frontier queues, kept depths, scan, outputs,
// remote boxes and the per-level counts; grown on demand, kept with the
// context.
struct LetLayout {
    size_t q0, q1, keep, flag, prefix, depth, mass, com, boxes, boxf, grpf, cnt, total;
};

LetLayout let_layout(int64_t S, int64_t nb)
{
    auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
    LetLayout L{};
    size_t o = 0;
    L.q0 = o; o += up(sizeof(int32_t) * S);
    L.q1 = o; o += up(sizeof(int32_t) * S);
    L.keep = o; o += up(sizeof(int32_t) * S);
    L.flag = o; o += up(sizeof(int32_t) * S);
    L.prefix = o; o += up(sizeof(uint64_t) * S);
    L.depth = o; o += up(S);
    L.mass = o; o += up(sizeof(double) * S);
    L.com = o; o += up(3 * sizeof(double) * S);
    L.boxes = o; o += up(6 * sizeof(double) * nb);
    L.boxf = o; o += up(6 * sizeof(float) * nb);
    L.grpf = o; o += up(6 * sizeof(float) * ((nb + kLetGroup - 1) / kLetGroup));
    L.cnt = o; o += up(sizeof(int32_t) * (kLetLevels + 2));
    L.total = o;
    return L;
}

// ---- buildTreeFromPseudoLeaves (src/linear_octree.cpp:242-322) ------------
//
// Every valid record (mass > 0 and finite; depth clamped to 21; prefix masked
// to its depth) contributes its own cell and the cell's ancestors.  A cell is
// named by its locational code (1 << 3e) | (prefix >> (63 - 3e)); the sort
// key of an entry is that code shifted left by one with an "ancestor" bit
// below it (depth-21 entries, always a record's own cell, keep the bare
// code, which sorts above every shifted one).  One sort thus orders the
// cells by (depth, prefix), groups each cell's entries, and puts the
// records' own entries first in record order (the radix sort is stable), so
// duplicate records are summed in input order, as the reference's insertion
// loop sums them.  Levels are then aggregated bottom up: a cell's
// sums are its own records' (mass, mass x com), then its children's, in
// octant order.  The reference adds children in the iteration order of its
// hash map, which no other program reproduces; sums over several children
// can therefore differ from it in the last bits.

__device__ __forceinline__ uint64_t loc_code(uint64_t key, int e)
{
    return (1ull << (3 * e)) | (e ? key >> (63 - 3 * e) : 0ull);
}

__device__ __forceinline__ int code_depth(uint64_t code) { return (63 - __clzll((long long)code)) / 3; }

// Sort key of an entry (see above) and its inverse.
__device__ __forceinline__ uint64_t entry_key(uint64_t code, int e, bool own)
{
    return e == bh::kMaxDepth ? code : (code << 1) | (own ? 0ull : 1ull);
}
__device__ __forceinline__ uint64_t key_code(uint64_t k) { return (k >> 63) ? k : (k >> 1); }
__device__ __forceinline__ bool key_own(uint64_t k) { return (k >> 63) || !(k & 1ull); }

__device__ __forceinline__ int clamp_depth(uint8_t d) { return d > bh::kMaxDepth ? bh::kMaxDepth : (int)d; }

__global__ void imp_count_kernel(int64_t m, const uint8_t* __restrict__ depth, const double* __restrict__ mass,
                                 int32_t* __restrict__ cnt)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const double w = mass[i];
        const bool valid = (w > 0.0) && isfinite(w);
        cnt[i] = valid ? clamp_depth(depth[i]) + 1 : 0;
    }
}

__global__ void imp_expand_kernel(int64_t m, const uint64_t* __restrict__ prefix, const uint8_t* __restrict__ depth,
                                  const int32_t* __restrict__ cnt, const int32_t* __restrict__ off,
                                  uint64_t* __restrict__ code, int32_t* __restrict__ ent_rec)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        if (!cnt[i]) continue;
        const int d = clamp_depth(depth[i]);
        const uint64_t key = prefix[i] & bh::prefix_mask(d);
        const int32_t o = off[i];
        for (int e = 0; e <= d; ++e) {
            code[o + e] = entry_key(loc_code(key, e), e, e == d);
            ent_rec[o + e] = (int32_t)i;
        }
    }
}

__global__ void imp_head_kernel(int64_t t, const uint64_t* __restrict__ code, int32_t* __restrict__ head)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < t; j += (int64_t)gridDim.x * blockDim.x)
        head[j] = (j == 0 || key_code(code[j]) != key_code(code[j - 1])) ? 1 : 0;
}

__global__ void imp_cells_kernel(int64_t t, const uint64_t* __restrict__ code, const int32_t* __restrict__ cidx,
                                 uint64_t* __restrict__ cell_code, int32_t* __restrict__ cell_start)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < t; j += (int64_t)gridDim.x * blockDim.x) {
        if (j == 0 || key_code(code[j]) != key_code(code[j - 1])) {
            cell_code[cidx[j]] = key_code(code[j]);
            cell_start[cidx[j]] = (int32_t)j;
        }
    }
}

// level_start[e] = first cell of depth e (e = 0..22; level 22 = the end).
__global__ void imp_levels_kernel(const uint64_t* __restrict__ cell_code, const int32_t* __restrict__ ncell,
                                  int32_t* __restrict__ level_start)
{
    const int e = threadIdx.x;
    if (e > bh::kMaxDepth + 1) return;
    const int32_t c = *ncell;
    if (e == bh::kMaxDepth + 1) { level_start[e] = c; return; }
    const uint64_t lo = 1ull << (3 * e);
    int32_t a = 0, b = c;
    while (a < b) {
        const int32_t mid = a + (b - a) / 2;
        if (cell_code[mid] < lo) a = mid + 1; else b = mid;
    }
    level_start[e] = a;
}

// One level of the bottom-up aggregation: cells [c0, c1) of depth e; the
// children are the cells of depth e + 1 in [k0, k1).
__global__ void imp_level_kernel(int e, int32_t c0, int32_t c1, int32_t k0, int32_t k1, int32_t ncell, int64_t t,
                                 const uint64_t* __restrict__ cell_code, const int32_t* __restrict__ cell_start,
                                 const uint64_t* __restrict__ skey, const uint32_t* __restrict__ perm,
                                 const int32_t* __restrict__ ent_rec, const double* __restrict__ mass,
                                 const double* __restrict__ com, double4_32a* __restrict__ acc)
{
    for (int32_t c = c0 + blockIdx.x * blockDim.x + threadIdx.x; c < c1; c += gridDim.x * blockDim.x) {
        const uint64_t code = cell_code[c];
        double m = 0.0, wx = 0.0, wy = 0.0, wz = 0.0;
        const int32_t j1 = (c + 1 < ncell) ? cell_start[c + 1] : (int32_t)t;
        for (int32_t j = cell_start[c]; j < j1 && key_own(skey[j]); ++j) {  // own entries come first
            const int32_t r = ent_rec[perm[j]];
            const double w = mass[r];
            m = __dadd_rn(m, w);
            wx = __dadd_rn(wx, __dmul_rn(com[3 * (int64_t)r], w));
            wy = __dadd_rn(wy, __dmul_rn(com[3 * (int64_t)r + 1], w));
            wz = __dadd_rn(wz, __dmul_rn(com[3 * (int64_t)r + 2], w));
        }
        if (k0 < k1) {
            const uint64_t first = code << 3;
            int32_t a = k0, b = k1;
            while (a < b) {
                const int32_t mid = a + (b - a) / 2;
                if (cell_code[mid] < first) a = mid + 1; else b = mid;
            }
            for (int32_t k = a; k < k1 && (cell_code[k] >> 3) == code; ++k) {
                const double4_32a q = acc[k];
                m = __dadd_rn(m, q.w);
                wx = __dadd_rn(wx, q.x);
                wy = __dadd_rn(wy, q.y);
                wz = __dadd_rn(wz, q.z);
            }
        }
        acc[c] = double4_32a{wx, wy, wz, m};
    }
}

__global__ void imp_out_kernel(int32_t ncell, const uint64_t* __restrict__ cell_code, const double4_32a* __restrict__ acc,
                               uint64_t* __restrict__ o_prefix, uint8_t* __restrict__ o_depth,
                               double* __restrict__ o_mass, double* __restrict__ o_com)
{
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
        const uint64_t code = cell_code[c];
        const int e = code_depth(code);
        o_prefix[c] = e ? (code ^ (1ull << (3 * e))) << (63 - 3 * e) : 0ull;
        o_depth[c] = (uint8_t)e;
        const double4_32a q = acc[c];
        o_mass[c] = q.w;
        const bool div = q.w > 1e-12;
        o_com[3 * (int64_t)c] = div ? __ddiv_rn(q.x, q.w) : q.x;
        o_com[3 * (int64_t)c + 1] = div ? __ddiv_rn(q.y, q.w) : q.y;
        o_com[3 * (int64_t)c + 2] = div ? __ddiv_rn(q.z, q.w) : q.z;
    }
}

struct Arena {
    char* base;
    size_t off;
    template <class T>
    T* take(int64_t n)
    {
        T* p = reinterpret_cast<T*>(base + off);
        off += ((size_t)std::max<int64_t>(n, 1) * sizeof(T) + 255) & ~(size_t)255;
        return p;
    }
};

int grow(void** buf, size_t* bytes, size_t want)
{
    if (*bytes >= want) return BH_OK;
    if (*buf) BH_CUDA_TRY(cudaFree(*buf));
    *buf = nullptr;
    *bytes = 0;
    if (cudaMalloc(buf, want) != cudaSuccess) {
        cudaGetLastError();
        return bh_fail(BH_ERR_OUT_OF_MEMORY, "pseudo-leaf tree: scratch allocation failed");
    }
    *bytes = want;
    return BH_OK;
}

}  // namespace

extern "C" {

int bh_let_export(bh_context* ctx, const double* boxes, int64_t nboxes, const double bbox[6], double theta2,
                  int max_depth, int64_t capacity, uint64_t* prefix, uint8_t* depth, double* mass, double* com,
                  int64_t* count_out)
{
    if (!ctx || !bbox || !count_out || nboxes < 0 || capacity < 0 || (nboxes > 0 && !boxes) ||
        nboxes > (int64_t)INT32_MAX)
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_let_export: bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    *count_out = 0;
    if (ctx->n == 0 || nboxes == 0) return BH_OK;
    if (!ctx->tree_valid) return bh_fail(BH_ERR_STATE, "bh_let_export: no tree built");
    int rc;
    if (ctx->tree_far) {  // the export carries the reference's tree: real masses
        if ((rc = bh::launch_build(ctx, ctx->m))) return rc;
        ctx->tree_far = ctx->tree_moments = false;
    }
    cudaStream_t st = ctx->stream;
    int32_t S = 0;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, ctx->counts + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    std::memcpy(&S, ctx->h_small, sizeof(int32_t));
    if (S <= 0) return BH_OK;

    const LetLayout L = let_layout(S, nboxes);
    if (ctx->let_bytes < L.total) {
        if (ctx->let_buf) BH_CUDA_TRY(cudaFree(ctx->let_buf));
        ctx->let_buf = nullptr;
        ctx->let_bytes = 0;
        if (cudaMalloc(&ctx->let_buf, L.total) != cudaSuccess) {
            cudaGetLastError();
            return bh_fail(BH_ERR_OUT_OF_MEMORY, "bh_let_export: scratch allocation failed");
        }
        ctx->let_bytes = L.total;
    }
    char* base = static_cast<char*>(ctx->let_buf);
    int32_t* q[2] = {reinterpret_cast<int32_t*>(base + L.q0), reinterpret_cast<int32_t*>(base + L.q1)};
    int32_t* keep = reinterpret_cast<int32_t*>(base + L.keep);
    int32_t* flag = reinterpret_cast<int32_t*>(base + L.flag);
    uint64_t* o_prefix = reinterpret_cast<uint64_t*>(base + L.prefix);
    uint8_t* o_depth = reinterpret_cast<uint8_t*>(base + L.depth);
    double* o_mass = reinterpret_cast<double*>(base + L.mass);
    double* o_com = reinterpret_cast<double*>(base + L.com);
    double* d_boxes = reinterpret_cast<double*>(base + L.boxes);
    float* d_boxf = reinterpret_cast<float*>(base + L.boxf);
    float* d_grpf = reinterpret_cast<float*>(base + L.grpf);
    int32_t* cnt = reinterpret_cast<int32_t*>(base + L.cnt);

    LetGeom g;
    for (int a = 0; a < 3; ++a) {
        g.lo[a] = bbox[a];
        g.span[a] = bbox[3 + a] - bbox[a];
    }
    BH_CUDA_TRY(cudaMemcpyAsync(d_boxes, boxes, sizeof(double) * 6 * nboxes, cudaMemcpyHostToDevice, st));
    // The FP32 prescreen's copies and bound (see LetScreen).
    std::vector<float> hf((size_t)(6 * nboxes));
    double mag = 0.0;
    bool finite = true;
    for (int64_t k = 0; k < 6 * nboxes; ++k) {
        hf[(size_t)k] = (float)boxes[k];
        finite = finite && std::isfinite(boxes[k]);
        mag = std::max(mag, std::fabs(boxes[k]));
    }
    for (int a = 0; a < 6; ++a) {
        finite = finite && std::isfinite(bbox[a]);
        mag = std::max(mag, std::fabs(bbox[a]));
    }
    LetScreen sc{0, 0.0f, (float)theta2};
    if (finite && theta2 >= 0.0 && theta2 < 1e30 && mag > 0x1p-20 && mag < 0x1p40) {
        sc.on = 1;
        sc.delta = (float)(mag * 0x1p-21);
    }
    // The prefilter's group hulls of the FP32 copies.
    const int64_t ngroups = (nboxes + kLetGroup - 1) / kLetGroup;
    std::vector<float> hg((size_t)(6 * ngroups));
    for (int64_t j = 0; j < ngroups; ++j) {
        float* h = &hg[(size_t)(6 * j)];
        for (int a = 0; a < 3; ++a) {
            h[a] = std::numeric_limits<float>::infinity();
            h[3 + a] = -std::numeric_limits<float>::infinity();
        }
        for (int64_t k = j * kLetGroup; k < std::min<int64_t>(nboxes, (j + 1) * kLetGroup); ++k)
            for (int a = 0; a < 3; ++a) {
                h[a] = std::min(h[a], hf[(size_t)(6 * k + a)]);
                h[3 + a] = std::max(h[3 + a], hf[(size_t)(6 * k + 3 + a)]);
            }
    }
    BH_CUDA_TRY(cudaMemcpyAsync(d_boxf, hf.data(), sizeof(float) * 6 * nboxes, cudaMemcpyHostToDevice, st));
    BH_CUDA_TRY(cudaMemcpyAsync(d_grpf, hg.data(), sizeof(float) * 6 * ngroups, cudaMemcpyHostToDevice, st));
    BH_CUDA_TRY(cudaMemsetAsync(keep, 0xff, sizeof(int32_t) * S, st));
    BH_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (kLetLevels + 2), st));
    let_seed_kernel<<<1, 1, 0, st>>>(q[0], cnt);
    BH_LAUNCH_CHECK(ctx);
    int dev_sms = 0;
    BH_CUDA_TRY(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const int64_t want = (S + kLetWarps - 1) / kLetWarps;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)dev_sms * 8));
    // Chain tops grow by at least one per level, and no cell is deeper than
    // 21, so kLetLevels launches drain every frontier.
    for (int lv = 0; lv < kLetLevels; ++lv) {
        let_level_kernel<<<grid, kLetThreads, 0, st>>>(ctx->rec, ctx->slot_ref, ctx->node_a, ctx->leaf_key, d_boxes,
                                                       d_boxf, d_grpf, (int)nboxes, g, theta2, sc, max_depth, q[lv & 1],
                                                       cnt + lv, q[(lv + 1) & 1], cnt + lv + 1, keep);
        BH_LAUNCH_CHECK(ctx);
    }
    const int sgrid = (int)std::min<int64_t>((S + 255) / 256, (int64_t)dev_sms * 16);
    let_flag_kernel<<<sgrid, 256, 0, st>>>(ctx->counts, keep, flag);
    BH_LAUNCH_CHECK(ctx);
    int32_t* total = cnt + kLetLevels + 1;
    if ((rc = bh::device_exclusive_scan(ctx, flag, flag, S, ctx->counts + 2, total))) return rc;
    let_write_kernel<<<sgrid, 256, 0, st>>>(ctx->counts, keep, flag, ctx->rec, ctx->slot_ref, ctx->node_a,
                                            ctx->leaf_key, o_prefix, o_depth, o_mass, o_com);
    BH_LAUNCH_CHECK(ctx);
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, total, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(ctx->h_small) + 8, cnt + kLetLevels, sizeof(int32_t),
                                cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    int32_t k = 0, spill = 0;
    std::memcpy(&k, ctx->h_small, sizeof(int32_t));
    std::memcpy(&spill, reinterpret_cast<char*>(ctx->h_small) + 8, sizeof(int32_t));
    if (spill != 0) return bh_fail(BH_ERR_OVERFLOW, "bh_let_export: frontier deeper than the tree");
    *count_out = k;
    if (k > capacity) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_let_export: capacity below the exported count");
    if (k == 0) return BH_OK;
    if (!prefix || !depth || !mass || !com) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_let_export: null array");
    BH_CUDA_TRY(cudaMemcpyAsync(prefix, o_prefix, sizeof(uint64_t) * k, cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaMemcpyAsync(depth, o_depth, k, cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaMemcpyAsync(mass, o_mass, sizeof(double) * k, cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaMemcpyAsync(com, o_com, 3 * sizeof(double) * k, cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    return BH_OK;
}

}  // extern "C"

namespace {

// The device map of buildTreeFromPseudoLeaves: n cells sorted by
// locational code, in ctx->imp_buf2.
struct PseudoCells {
    int32_t n = 0;
    const uint64_t* code = nullptr;
    const uint64_t* prefix = nullptr;
    const uint8_t* depth = nullptr;
    const double* mass = nullptr;
    const double* com = nullptr;  // 3 per cell
};

int pseudo_tree_device(bh_context* ctx, const uint64_t* prefix, const uint8_t* depth, const double* mass,
                       const double* com, int64_t m, PseudoCells* out)
{
    *out = PseudoCells{};
    // entries (record cells and their ancestors) are numbered in int32
    if (m > (int64_t)(INT32_MAX / (bh::kMaxDepth + 1)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "pseudo-leaf tree: too many records");
    if (m == 0) return BH_OK;
    cudaStream_t st = ctx->stream;
    int dev_sms = 0;
    BH_CUDA_TRY(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
    auto grid_for = [&](int64_t n) {
        return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 16 * (int64_t)dev_sms));
    };
    int rc;

    // Phase 1: the records, their entry counts and offsets.
    auto layout_a = [&](Arena& a, uint64_t** rp, uint8_t** rd, double** rm, double** rc3, int32_t** cnt,
                        int32_t** off, int32_t** tmp, int32_t** small) {
        *rp = a.take<uint64_t>(m); *rd = a.take<uint8_t>(m); *rm = a.take<double>(m); *rc3 = a.take<double>(3 * m);
        *cnt = a.take<int32_t>(m); *off = a.take<int32_t>(m); *tmp = a.take<int32_t>(bh::scan_tmp_ints(m));
        *small = a.take<int32_t>(64);  // [0] entries, [1] cells, [8..30] level starts
    };
    uint64_t* r_prefix; uint8_t* r_depth; double* r_mass; double* r_com; int32_t *cnt, *off, *tmp_a, *small;
    {
        Arena probe{nullptr, 0};
        layout_a(probe, &r_prefix, &r_depth, &r_mass, &r_com, &cnt, &off, &tmp_a, &small);
        if ((rc = grow(&ctx->imp_buf, &ctx->imp_bytes, probe.off))) return rc;
    }
    Arena a{static_cast<char*>(ctx->imp_buf), 0};
    layout_a(a, &r_prefix, &r_depth, &r_mass, &r_com, &cnt, &off, &tmp_a, &small);
    BH_CUDA_TRY(cudaMemcpyAsync(r_prefix, prefix, sizeof(uint64_t) * m, cudaMemcpyHostToDevice, st));
    BH_CUDA_TRY(cudaMemcpyAsync(r_depth, depth, m, cudaMemcpyHostToDevice, st));
    BH_CUDA_TRY(cudaMemcpyAsync(r_mass, mass, sizeof(double) * m, cudaMemcpyHostToDevice, st));
    BH_CUDA_TRY(cudaMemcpyAsync(r_com, com, 3 * sizeof(double) * m, cudaMemcpyHostToDevice, st));
    imp_count_kernel<<<grid_for(m), 256, 0, st>>>(m, r_depth, r_mass, cnt);
    BH_LAUNCH_CHECK(ctx);
    if ((rc = bh::device_exclusive_scan_tmp(ctx, cnt, off, m, nullptr, small, tmp_a))) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, small, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    int32_t t = 0;
    std::memcpy(&t, ctx->h_small, sizeof(int32_t));
    if (t == 0) return BH_OK;

    // Phase 2: t entries -> sorted codes -> cells -> level sums.
    const int64_t tiles = (t + bh::kSortTile - 1) / bh::kSortTile;
    uint64_t *code, *code_s, *key_alt, *cell_code, *d_prefix;
    uint32_t *val_alt, *perm, *hist, *lookback, *tile_ctr;
    int32_t *ent_rec, *head, *cell_start, *tmp_b;
    unsigned* err;
    double4_32a* acc;
    uint8_t* d_depth;
    double *d_mass, *d_com;
    auto layout_b = [&](Arena& b) {
        code = b.take<uint64_t>(t); code_s = b.take<uint64_t>(t); key_alt = b.take<uint64_t>(t);
        val_alt = b.take<uint32_t>(t); perm = b.take<uint32_t>(t); ent_rec = b.take<int32_t>(t);
        head = b.take<int32_t>(t); tmp_b = b.take<int32_t>(bh::scan_tmp_ints(t));
        hist = b.take<uint32_t>(bh::kSortPasses * bh::kRadix);
        lookback = b.take<uint32_t>(bh::kSortPasses * tiles * bh::kRadix);
        tile_ctr = b.take<uint32_t>(bh::kSortPasses); err = b.take<unsigned>(1);
        cell_code = b.take<uint64_t>(t); cell_start = b.take<int32_t>(t); acc = b.take<double4_32a>(t);
        d_prefix = b.take<uint64_t>(t); d_depth = b.take<uint8_t>(t); d_mass = b.take<double>(t);
        d_com = b.take<double>(3 * (int64_t)t);
    };
    {
        Arena probe{nullptr, 0};
        layout_b(probe);
        if ((rc = grow(&ctx->imp_buf2, &ctx->imp_bytes2, probe.off))) return rc;
    }
    Arena b{static_cast<char*>(ctx->imp_buf2), 0};
    layout_b(b);
    imp_expand_kernel<<<grid_for(m), 256, 0, st>>>(m, r_prefix, r_depth, cnt, off, code, ent_rec);
    BH_LAUNCH_CHECK(ctx);
    if (t == 1) {
        BH_CUDA_TRY(cudaMemcpyAsync(code_s, code, sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
        BH_CUDA_TRY(cudaMemsetAsync(perm, 0, sizeof(uint32_t), st));
        BH_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
    } else {
        BH_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(uint32_t) * bh::kSortPasses * bh::kRadix, st));
        BH_CUDA_TRY(cudaMemsetAsync(lookback, 0, sizeof(uint32_t) * bh::kSortPasses * tiles * bh::kRadix, st));
        BH_CUDA_TRY(cudaMemsetAsync(tile_ctr, 0, sizeof(uint32_t) * bh::kSortPasses, st));
        BH_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
        if ((rc = bh::launch_digit_hist(t, code, hist, st))) return rc;
        if ((rc = bh::sort_passes_raw(t, code, code_s, perm, key_alt, val_alt, hist, lookback, tile_ctr, err, st)))
            return rc;
    }
    imp_head_kernel<<<grid_for(t), 256, 0, st>>>(t, code_s, head);
    BH_LAUNCH_CHECK(ctx);
    if ((rc = bh::device_exclusive_scan_tmp(ctx, head, head, t, nullptr, small + 1, tmp_b))) return rc;
    imp_cells_kernel<<<grid_for(t), 256, 0, st>>>(t, code_s, head, cell_code, cell_start);
    BH_LAUNCH_CHECK(ctx);
    imp_levels_kernel<<<1, 32, 0, st>>>(cell_code, small + 1, small + 8);
    BH_LAUNCH_CHECK(ctx);
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, small, 32 * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(ctx->h_small) + 256, err, sizeof(unsigned),
                                cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    int32_t hs[32];
    unsigned h_err = 0;
    std::memcpy(hs, ctx->h_small, sizeof(hs));
    std::memcpy(&h_err, reinterpret_cast<char*>(ctx->h_small) + 256, sizeof(unsigned));
    if (h_err & bh::kErrTimeout) return bh_fail(BH_ERR_TIMEOUT, "pseudo-leaf tree: a bounded device wait gave up");
    const int32_t ncell = hs[1];
    const int32_t* ls = hs + 8;  // ls[0..22]

    // Bottom-up sums, deepest level first.
    for (int e = bh::kMaxDepth; e >= 0; --e) {
        const int32_t c0 = ls[e], c1 = ls[e + 1];
        if (c0 == c1) continue;
        const int32_t k1 = e < bh::kMaxDepth ? ls[e + 2] : c1;
        imp_level_kernel<<<grid_for(c1 - c0), 256, 0, st>>>(e, c0, c1, c1, k1, ncell, t, cell_code, cell_start,
                                                            code_s, perm, ent_rec, r_mass, r_com, acc);
        BH_LAUNCH_CHECK(ctx);
    }
    imp_out_kernel<<<grid_for(ncell), 256, 0, st>>>(ncell, cell_code, acc, d_prefix, d_depth, d_mass, d_com);
    BH_LAUNCH_CHECK(ctx);
    out->n = ncell;
    out->code = cell_code;
    out->prefix = d_prefix;
    out->depth = d_depth;
    out->mass = d_mass;
    out->com = d_com;
    return BH_OK;
}

}  // namespace

extern "C" int bh_pseudo_leaf_tree(bh_context* ctx, const uint64_t* prefix, const uint8_t* depth, const double* mass,
                                   const double* com, int64_t m, int64_t capacity, uint64_t* o_prefix,
                                   uint8_t* o_depth, double* o_mass, double* o_com, int64_t* count_out)
{
    if (!ctx || !count_out || m < 0 || capacity < 0 || (m > 0 && (!prefix || !depth || !mass || !com)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_pseudo_leaf_tree: bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    *count_out = 0;
    PseudoCells pc;
    int rc = pseudo_tree_device(ctx, prefix, depth, mass, com, m, &pc);
    if (rc) return rc;
    *count_out = pc.n;
    if (pc.n == 0) return BH_OK;
    if (pc.n > capacity)
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_pseudo_leaf_tree: capacity below the cell count");
    if (!o_prefix || !o_depth || !o_mass || !o_com)
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_pseudo_leaf_tree: null output array");
    cudaStream_t st = ctx->stream;
    BH_CUDA_TRY(cudaMemcpyAsync(o_prefix, pc.prefix, sizeof(uint64_t) * pc.n, cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaMemcpyAsync(o_depth, pc.depth, pc.n, cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaMemcpyAsync(o_mass, pc.mass, sizeof(double) * pc.n, cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaMemcpyAsync(o_com, pc.com, 3 * sizeof(double) * pc.n, cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    return BH_OK;
}

// ---- Forces with imported LET records --------------------------------------
//
// computeAccelerationsWithLET (src/traversal.cpp:107-127): the received
// records become a pseudo-leaf map, which mergeRecordsIntoTree
// (src/linear_octree.cpp:178-204) folds into the local map (a cell in both:
// com = (m0 c0 + m1 c1) / (m0 + m1), skipped when that mass is 0; a cell
// only in the pseudo map enters with m0 = 0), and computeAccelerations
// (src/traversal.cpp:13-103) walks the merged map.  The merged map is not
// the compressed tree of any body set, so it is built here as an explicit
// cell array: the local chains expanded into their cells, the pseudo cells
// appended, one stable sort of the locational codes, and a merge of equal
// codes.  Each body then walks it depth first with the reference's visiting
// order (children pushed in octant order, popped last first) and its IEEE
// operation sequence, so the result is the reference's on the same merged
// map.  computeAccelerationsWithRemoteDirectSum (:149-221) is the exact
// traversal of the local tree plus a direct sum over the records, in record
// order.
namespace {

constexpr int kLetStack = 192;  // DFS depth <= 7 * 21 + 1 entries

struct Side2 {
    double v[bh::kMaxDepth + 1];
};

__global__ void chain_count_kernel(const int32_t* __restrict__ counts, const bh::TreeRec* __restrict__ rec,
                                   int32_t* __restrict__ cnt)
{
    const int32_t S = counts[2];
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x)
        cnt[s] = (int32_t)rec[s].depth - (int32_t)rec[s].top + 1;
}

// Local cells (codes at [0, L)) and the pseudo cells appended at [L, L + R).
__global__ void chain_cells_kernel(const int32_t* __restrict__ counts, const bh::TreeRec* __restrict__ rec,
                                   const int32_t* __restrict__ slot_ref, const int32_t* __restrict__ node_a,
                                   const uint64_t* __restrict__ leaf_key, const int32_t* __restrict__ off,
                                   uint64_t* __restrict__ code, int32_t* __restrict__ cell_slot)
{
    const int32_t S = counts[2];
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const bh::TreeRec r = rec[s];
        const int32_t ref = slot_ref[s];
        const uint64_t key = leaf_key[ref >= 0 ? ref : node_a[~ref]];
        const int32_t o = off[s];
        for (int d = r.top; d <= r.depth; ++d) {
            code[o + d - r.top] = loc_code(key & bh::prefix_mask(d), d);
            cell_slot[o + d - r.top] = s;
        }
    }
}

__global__ void merge_head_kernel(int64_t t, const uint64_t* __restrict__ code, int32_t* __restrict__ head)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < t; j += (int64_t)gridDim.x * blockDim.x)
        head[j] = (j == 0 || code[j] != code[j - 1]) ? 1 : 0;
}

// One merged cell per distinct code.  Sorted entries of one code: the local
// cell (entry index < L) first, then the pseudo cell.
__global__ void merge_cells_kernel(int64_t t, int32_t L, const uint64_t* __restrict__ code,
                                   const uint32_t* __restrict__ perm, const int32_t* __restrict__ midx,
                                   const int32_t* __restrict__ cell_slot, const bh::TreeRec* __restrict__ rec,
                                   const double* __restrict__ p_mass, const double* __restrict__ p_com,
                                   uint64_t* __restrict__ m_code, double4_32a* __restrict__ m_val)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < t; j += (int64_t)gridDim.x * blockDim.x) {
        if (j > 0 && code[j] == code[j - 1]) continue;
        const uint32_t e0 = perm[j];
        double m0 = 0.0, x0 = 0.0, y0 = 0.0, z0 = 0.0;
        int32_t remote = -1;
        if ((int32_t)e0 < L) {
            const bh::TreeRec r = rec[cell_slot[e0]];
            m0 = r.m; x0 = r.cx; y0 = r.cy; z0 = r.cz;
            if (j + 1 < t && code[j + 1] == code[j]) remote = (int32_t)perm[j + 1] - L;
        } else {
            remote = (int32_t)e0 - L;
        }
        if (remote >= 0) {
            const double m1 = p_mass[remote];
            const double tot = __dadd_rn(m0, m1);
            if (tot != 0.0) {
                x0 = __ddiv_rn(__dadd_rn(__dmul_rn(m0, x0), __dmul_rn(m1, p_com[3 * (int64_t)remote])), tot);
                y0 = __ddiv_rn(__dadd_rn(__dmul_rn(m0, y0), __dmul_rn(m1, p_com[3 * (int64_t)remote + 1])), tot);
                z0 = __ddiv_rn(__dadd_rn(__dmul_rn(m0, z0), __dmul_rn(m1, p_com[3 * (int64_t)remote + 2])), tot);
                m0 = tot;
            }
        }
        const int32_t k = midx[j];
        m_code[k] = code[j];
        m_val[k] = double4_32a{x0, y0, z0, m0};
    }
}

// First child (index into the merged cells) and the octants present.
__global__ void merge_children_kernel(int32_t M, const uint64_t* __restrict__ m_code, int32_t* __restrict__ first,
                                      uint8_t* __restrict__ mask)
{
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < M; c += gridDim.x * blockDim.x) {
        const uint64_t code = m_code[c];
        uint8_t bits = 0;
        int32_t a = M;
        if (!(code >> 63)) {  // depth < 21
            const uint64_t lo = code << 3;
            int32_t b = M;
            a = c + 1;
            while (a < b) {
                const int32_t mid = a + (b - a) / 2;
                if (m_code[mid] < lo) a = mid + 1; else b = mid;
            }
            for (int32_t k = a; k < M && (m_code[k] >> 3) == code; ++k) bits |= (uint8_t)(1u << (m_code[k] & 7u));
        }
        first[c] = a;
        mask[c] = bits;
    }
}

__global__ void __launch_bounds__(128) merged_walk_kernel(
    int64_t n, const double* __restrict__ px, const double* __restrict__ py, const double* __restrict__ pz,
    const uint64_t* __restrict__ key, int32_t M, const uint64_t* __restrict__ m_code,
    const double4_32a* __restrict__ m_val, const int32_t* __restrict__ first, const uint8_t* __restrict__ mask,
    Side2 side2, double theta2, double G, double soft2, double* __restrict__ ax, double* __restrict__ ay,
    double* __restrict__ az, unsigned* __restrict__ err)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = px[i], y = py[i], z = pz[i];
        const uint64_t ki = key[i];
        double sx = 0.0, sy = 0.0, sz = 0.0;
        int32_t stack[kLetStack];
        int top = 0;
        if (M > 0 && m_code[0] == 1ull) stack[top++] = 0;
        while (top) {
            const int32_t c = stack[--top];
            const double4_32a v = m_val[c];
            if (v.w == 0.0) continue;
            const uint64_t code = m_code[c];
            const int dep = code_depth(code);
            if (dep == bh::kMaxDepth && ((code ^ (1ull << 63)) == ki)) continue;  // the body's own leaf
            const double dx = __dsub_rn(v.x, x), dy = __dsub_rn(v.y, y), dz = __dsub_rn(v.z, z);
            const double r2 = __dadd_rn(
                __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), soft2);
            if (dep == bh::kMaxDepth || side2.v[dep] < __dmul_rn(theta2, r2)) {
                const double inv = __ddiv_rn(1.0, __dsqrt_rn(r2));
                const double inv3 = __dmul_rn(__dmul_rn(inv, inv), inv);
                const double s = __dmul_rn(__dmul_rn(G, v.w), inv3);
                sx = __dadd_rn(sx, __dmul_rn(s, dx));
                sy = __dadd_rn(sy, __dmul_rn(s, dy));
                sz = __dadd_rn(sz, __dmul_rn(s, dz));
            } else {
                const uint8_t bits = mask[c];
                int32_t k = first[c];
                for (int oc = 0; oc < 8; ++oc) {
                    if (!((bits >> oc) & 1u)) continue;
                    if (top == kLetStack) {  // cannot happen below depth 22; flagged, never written past
                        atomicOr(err, bh::kErrOverflow);
                        top = 0;
                        break;
                    }
                    stack[top++] = k++;
                }
            }
        }
        ax[i] = sx;
        ay[i] = sy;
        az[i] = sz;
    }
}

// out += sum over records in record order (rm = mass * G).
constexpr int kDirectTile = 128;

__global__ void __launch_bounds__(kDirectTile) remote_direct_kernel(
    int64_t n, const double* __restrict__ px, const double* __restrict__ py, const double* __restrict__ pz, int64_t M,
    const double* __restrict__ rcom, const double* __restrict__ rmass, double G, double soft2,
    double* __restrict__ ax, double* __restrict__ ay, double* __restrict__ az)
{
    __shared__ double4_32a tile[kDirectTile];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool live = i < n;
    const double x = live ? px[i] : 0.0, y = live ? py[i] : 0.0, z = live ? pz[i] : 0.0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int64_t j0 = 0; j0 < M; j0 += kDirectTile) {
        const int64_t j = j0 + threadIdx.x;
        if (j < M)
            tile[threadIdx.x] = double4_32a{rcom[3 * j], rcom[3 * j + 1], rcom[3 * j + 2], __dmul_rn(rmass[j], G)};
        __syncthreads();
        const int cnt = (int)(M - j0 < kDirectTile ? M - j0 : kDirectTile);
        for (int k = 0; k < cnt; ++k) {
            const double4_32a q = tile[k];
            const double dx = __dsub_rn(q.x, x), dy = __dsub_rn(q.y, y), dz = __dsub_rn(q.z, z);
            const double r2 = __dadd_rn(
                __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), soft2);
            if (r2 <= 1e-12) continue;
            const double inv = __ddiv_rn(1.0, __dsqrt_rn(r2));
            const double inv3 = __dmul_rn(__dmul_rn(inv, inv), inv);
            const double s = __dmul_rn(q.w, inv3);
            sx = __dadd_rn(sx, __dmul_rn(s, dx));
            sy = __dadd_rn(sy, __dmul_rn(s, dy));
            sz = __dadd_rn(sz, __dmul_rn(s, dz));
        }
        __syncthreads();
    }
    if (live) {
        ax[i] = __dadd_rn(ax[i], sx);
        ay[i] = __dadd_rn(ay[i], sy);
        az[i] = __dadd_rn(az[i], sz);
    }
}

int download_acc(bh_context* ctx, double* acc_out)
{
    const int64_t n = ctx->n;
    std::vector<double> h(3 * (size_t)n);
    BH_CUDA_TRY(cudaMemcpyAsync(h.data(), ctx->ax, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(h.data() + n, ctx->ay, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(h.data() + 2 * n, ctx->az, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    for (int64_t i = 0; i < n; ++i) {
        acc_out[3 * i] = h[(size_t)i];
        acc_out[3 * i + 1] = h[(size_t)(n + i)];
        acc_out[3 * i + 2] = h[(size_t)(2 * n + i)];
    }
    return BH_OK;
}

int let_check(bh_context* ctx, const uint64_t* prefix, const uint8_t* depth, const double* mass, const double* com,
              int64_t m, double theta, double soft2, bool need_keys, const char* fn)
{
    if (!ctx || m < 0 || (m > 0 && (!mass || !com || (need_keys && (!prefix || !depth)))) || !(theta >= 0.0) ||
        !(soft2 >= 0.0))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, std::string(fn) + ": bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    if (ctx->n > 0 && !ctx->tree_valid) return bh_fail(BH_ERR_STATE, std::string(fn) + ": no tree built");
    if (ctx->tree_far) {  // the reference's local tree: real masses
        int rc = bh::launch_build(ctx, ctx->m);
        if (rc) return rc;
        ctx->tree_far = ctx->tree_moments = false;
    }
    return BH_OK;
}

}  // namespace

extern "C" int bh_let_accelerations(bh_context* ctx, const uint64_t* prefix, const uint8_t* depth,
                                    const double* mass, const double* com, int64_t m, double theta, double G,
                                    double soft2, double* acc_out)
{
    int rc = let_check(ctx, prefix, depth, mass, com, m, theta, soft2, true, "bh_let_accelerations");
    if (rc) return rc;
    const int64_t n = ctx->n;
    if (n == 0) return BH_OK;
    cudaStream_t st = ctx->stream;
    int dev_sms = 0;
    BH_CUDA_TRY(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
    auto grid_for = [&](int64_t k) {
        return (int)std::max<int64_t>(1, std::min<int64_t>((k + 255) / 256, 16 * (int64_t)dev_sms));
    };

    // The pseudo-leaf map (in imp_buf2) and the local cell count.
    PseudoCells pc;
    if ((rc = pseudo_tree_device(ctx, prefix, depth, mass, com, m, &pc))) return rc;
    int32_t S = 0;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, ctx->counts + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    std::memcpy(&S, ctx->h_small, sizeof(int32_t));
    const int64_t lmax = (int64_t)S * (bh::kMaxDepth + 1);
    if (lmax + pc.n > (int64_t)INT32_MAX) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_let_accelerations: map too large");

    auto layout1 = [&](Arena& a, int32_t** cnt, int32_t** off, int32_t** tmp, int32_t** small) {
        *cnt = a.take<int32_t>(S); *off = a.take<int32_t>(S); *tmp = a.take<int32_t>(bh::scan_tmp_ints(S));
        *small = a.take<int32_t>(64);
    };
    int32_t *cnt, *off, *tmp1, *small;
    {
        Arena probe{nullptr, 0};
        layout1(probe, &cnt, &off, &tmp1, &small);
        if ((rc = grow(&ctx->letf_buf, &ctx->letf_bytes, probe.off))) return rc;
    }
    Arena a1{static_cast<char*>(ctx->letf_buf), 0};
    layout1(a1, &cnt, &off, &tmp1, &small);
    chain_count_kernel<<<grid_for(S), 256, 0, st>>>(ctx->counts, ctx->rec, cnt);
    BH_LAUNCH_CHECK(ctx);
    if ((rc = bh::device_exclusive_scan_tmp(ctx, cnt, off, S, nullptr, small, tmp1))) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, small, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    int32_t L = 0;
    std::memcpy(&L, ctx->h_small, sizeof(int32_t));
    const int64_t t = (int64_t)L + pc.n;

    // Local cells + pseudo cells -> one stable sort -> merged cells.
    const int64_t tiles = (t + bh::kSortTile - 1) / bh::kSortTile;
    uint64_t *code, *code_s, *key_alt, *m_code;
    uint32_t *val_alt, *perm, *hist, *lookback, *tile_ctr;
    int32_t *cell_slot, *head, *tmp2, *first;
    unsigned* err;
    double4_32a* m_val;
    uint8_t* mask;
    auto layout2 = [&](Arena& b) {
        code = b.take<uint64_t>(t); code_s = b.take<uint64_t>(t); key_alt = b.take<uint64_t>(t);
        val_alt = b.take<uint32_t>(t); perm = b.take<uint32_t>(t); cell_slot = b.take<int32_t>(L);
        head = b.take<int32_t>(t); tmp2 = b.take<int32_t>(bh::scan_tmp_ints(t));
        hist = b.take<uint32_t>(bh::kSortPasses * bh::kRadix);
        lookback = b.take<uint32_t>(bh::kSortPasses * tiles * bh::kRadix);
        tile_ctr = b.take<uint32_t>(bh::kSortPasses); err = b.take<unsigned>(1);
        m_code = b.take<uint64_t>(t); m_val = b.take<double4_32a>(t); first = b.take<int32_t>(t);
        mask = b.take<uint8_t>(t);
    };
    {
        Arena probe{nullptr, 0};
        layout2(probe);
        size_t need = a1.off + probe.off;
        if (ctx->letf_bytes < need) {
            // grow keeps nothing: redo the local cell count after growing
            if ((rc = grow(&ctx->letf_buf, &ctx->letf_bytes, need))) return rc;
            Arena again{static_cast<char*>(ctx->letf_buf), 0};
            layout1(again, &cnt, &off, &tmp1, &small);
            chain_count_kernel<<<grid_for(S), 256, 0, st>>>(ctx->counts, ctx->rec, cnt);
            BH_LAUNCH_CHECK(ctx);
            if ((rc = bh::device_exclusive_scan_tmp(ctx, cnt, off, S, nullptr, small, tmp1))) return rc;
        }
    }
    Arena a2{static_cast<char*>(ctx->letf_buf), a1.off};
    layout2(a2);
    chain_cells_kernel<<<grid_for(S), 256, 0, st>>>(ctx->counts, ctx->rec, ctx->slot_ref, ctx->node_a, ctx->leaf_key,
                                                    off, code, cell_slot);
    BH_LAUNCH_CHECK(ctx);
    if (pc.n)
        BH_CUDA_TRY(cudaMemcpyAsync(code + L, pc.code, sizeof(uint64_t) * pc.n, cudaMemcpyDeviceToDevice, st));
    BH_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
    if (t == 1) {
        BH_CUDA_TRY(cudaMemcpyAsync(code_s, code, sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
        BH_CUDA_TRY(cudaMemsetAsync(perm, 0, sizeof(uint32_t), st));
    } else {
        BH_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(uint32_t) * bh::kSortPasses * bh::kRadix, st));
        BH_CUDA_TRY(cudaMemsetAsync(lookback, 0, sizeof(uint32_t) * bh::kSortPasses * tiles * bh::kRadix, st));
        BH_CUDA_TRY(cudaMemsetAsync(tile_ctr, 0, sizeof(uint32_t) * bh::kSortPasses, st));
        if ((rc = bh::launch_digit_hist(t, code, hist, st))) return rc;
        if ((rc = bh::sort_passes_raw(t, code, code_s, perm, key_alt, val_alt, hist, lookback, tile_ctr, err, st)))
            return rc;
    }
    merge_head_kernel<<<grid_for(t), 256, 0, st>>>(t, code_s, head);
    BH_LAUNCH_CHECK(ctx);
    if ((rc = bh::device_exclusive_scan_tmp(ctx, head, head, t, nullptr, small + 1, tmp2))) return rc;
    merge_cells_kernel<<<grid_for(t), 256, 0, st>>>(t, L, code_s, perm, head, cell_slot, ctx->rec, pc.mass, pc.com,
                                                    m_code, m_val);
    BH_LAUNCH_CHECK(ctx);
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, small, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    int32_t hs[2];
    std::memcpy(hs, ctx->h_small, sizeof(hs));
    const int32_t M = hs[1];
    merge_children_kernel<<<grid_for(M), 256, 0, st>>>(M, m_code, first, mask);
    BH_LAUNCH_CHECK(ctx);

    // The walk: the reference's side^2 table over the global box.
    double bb[6];
    BH_CUDA_TRY(cudaMemcpyAsync(bb, ctx->bbox, sizeof(bb), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    double Lside = bb[3] - bb[0];
    if (Lside < bb[4] - bb[1]) Lside = bb[4] - bb[1];
    if (Lside < bb[5] - bb[2]) Lside = bb[5] - bb[2];
    Side2 side2;
    for (int d = 0; d <= bh::kMaxDepth; ++d) {
        const double side = Lside / (double)(1ull << d);
        side2.v[d] = side * side;
    }
    const int wgrid = (int)std::max<int64_t>(1, std::min<int64_t>((n + 127) / 128, 64 * (int64_t)dev_sms));
    merged_walk_kernel<<<wgrid, 128, 0, st>>>(n, ctx->px, ctx->py, ctx->pz, ctx->key, M, m_code, m_val, first, mask,
                                              side2, theta * theta, G, soft2, ctx->ax, ctx->ay, ctx->az, err);
    BH_LAUNCH_CHECK(ctx);
    unsigned h_err = 0;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    std::memcpy(&h_err, ctx->h_small, sizeof(unsigned));
    if (h_err & bh::kErrTimeout) return bh_fail(BH_ERR_TIMEOUT, "bh_let_accelerations: a bounded device wait gave up");
    if (h_err & bh::kErrOverflow) return bh_fail(BH_ERR_OVERFLOW, "bh_let_accelerations: walk stack overflow");
    return acc_out ? download_acc(ctx, acc_out) : BH_OK;
}

extern "C" int bh_let_direct_accelerations(bh_context* ctx, const uint64_t* prefix, const uint8_t* depth,
                                           const double* mass, const double* com, int64_t m, double theta, double G,
                                           double soft2, double* acc_out)
{
    int rc = let_check(ctx, prefix, depth, mass, com, m, theta, soft2, false, "bh_let_direct_accelerations");
    if (rc) return rc;
    const int64_t n = ctx->n;
    if (n == 0) return BH_OK;
    cudaStream_t st = ctx->stream;
    if ((rc = bh::launch_traverse(ctx, theta, G, soft2, BH_MODE_PLAIN_FP64, 0.0))) return rc;
    if (m > 0) {
        auto layout = [&](Arena& a, double** rc3, double** rm) {
            *rc3 = a.take<double>(3 * m);
            *rm = a.take<double>(m);
        };
        double *rcom, *rmass;
        {
            Arena probe{nullptr, 0};
            layout(probe, &rcom, &rmass);
            if ((rc = grow(&ctx->letf_buf, &ctx->letf_bytes, probe.off))) return rc;
        }
        Arena a{static_cast<char*>(ctx->letf_buf), 0};
        layout(a, &rcom, &rmass);
        BH_CUDA_TRY(cudaMemcpyAsync(rcom, com, 3 * sizeof(double) * m, cudaMemcpyHostToDevice, st));
        BH_CUDA_TRY(cudaMemcpyAsync(rmass, mass, sizeof(double) * m, cudaMemcpyHostToDevice, st));
        const int64_t blocks = (n + kDirectTile - 1) / kDirectTile;
        remote_direct_kernel<<<(unsigned)blocks, kDirectTile, 0, st>>>(n, ctx->px, ctx->py, ctx->pz, m, rcom, rmass, G,
                                                                      soft2, ctx->ax, ctx->ay, ctx->az);
        BH_LAUNCH_CHECK(ctx);
    }
    if (acc_out) return download_acc(ctx, acc_out);
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    return BH_OK;
}
