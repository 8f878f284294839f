// Parallel bottom-up octree construction from the sorted Morton keys, with
// a level-synchronous monopole pass (no global atomics).
//
// Replaces buildOctreeBottomUp (src/linear_octree.cpp:13-107) followed by the
// single-rank full-tree exchange (src/exchange.cpp:9-29, whose effect is
// mergeRecordsIntoTree into an empty map, src/linear_octree.cpp:178-204).
//
// The reference's tree is uncompressed: every (depth, prefix) cell that holds
// a body exists, so most bodies hang below a chain of single-child cells.
// A single-child cell has exactly its child's mass and weighted position
// sums (the reference starts every sum at +0.0, and 0.0 + c == c for every c
// such a sum can hold), hence the same centre of mass.  This build therefore
// materialises only the cells with two or more children ("branching nodes")
// and the leaves; each stored node stands for the chain above it (depth
// range [top, depth]).  bh_export_tree expands the chains back into the
// reference's node set for parity checks.
//
// Terminology: leaves are the distinct keys K[0..L).  Boundary j (1 <= j < L)
// sits between leaves j-1 and j; cdep[j] is the deepest depth at which the
// two keys share a cell.  A branching node at depth D spanning leaves [a, e)
// has all interior boundaries with cdep >= D and at least one with
// cdep == D; its children are the depth-(D+1) cells inside it.  The node is
// identified by its first child boundary ("representative").
//
// Sums follow the reference's order exactly: a leaf sums its bodies in
// sorted order, a parent sums its children in octant order (= key order),
// each starting from 0.0; then com = sum/mass when mass > 0, then the merge
// step mass' = 0 + mass, com' = (0*0 + mass*com) / mass'.  All with IEEE
// double intrinsics (no contraction), so masses and centres of mass are bit
// for bit the reference's.
#include <climits>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kThreads = 256;

// 0.0 + v in round-to-nearest: v itself, except -0.0 -> +0.0.
__device__ __forceinline__ double plus_zero(double v)
{
    const long long b = __double_as_longlong(v);
    return __longlong_as_double(b == (long long)0x8000000000000000ull ? 0ll : b);
}

inline int grid_for(int64_t n, int threads, int max_blocks)
{
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (int)(b > max_blocks ? max_blocks : b);
}

// Leaf sums in body order (linear_octree.cpp:28-38) and boundary depths.
// kMoments: also the leaf's second moment about its centre of mass (the
// learned criterion's spread feature), sum_b m_b |x_b - c|^2.
// nzero > 0: the bodies with id < nzero count as massless (the FP32 forms'
// far-field tree, which leaves the Sun and planets to the direct terms).
template <bool kMoments>
__global__ void leaf_sum_kernel(const int32_t* __restrict__ counts, const int32_t* __restrict__ leaf_first,
                                const uint64_t* __restrict__ leaf_key, const double* __restrict__ px,
                                const double* __restrict__ py, const double* __restrict__ pz,
                                const double* __restrict__ m, const uint64_t* __restrict__ id, int nzero,
                                double4_32a* __restrict__ ls, int8_t* __restrict__ cdep, double* __restrict__ lq)
{
    auto mass = [&](int b) { return nzero > 0 && id[b] < (uint64_t)nzero ? 0.0 : m[b]; };
    const int L = counts[0];
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < L; l += gridDim.x * blockDim.x) {
        double sm = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
        const int b0 = leaf_first[l], b1 = leaf_first[l + 1];
        if (b1 == b0 + 1) {
            // One body: each sum is 0.0 + v, which is v except that -0.0
            // becomes +0.0; decided on the bit patterns (no FP64 addition).
            const double mb = mass(b0);
            sm = plus_zero(mb);
            sx = plus_zero(__dmul_rn(px[b0], mb));
            sy = plus_zero(__dmul_rn(py[b0], mb));
            sz = plus_zero(__dmul_rn(pz[b0], mb));
        } else {
            for (int b = b0; b < b1; ++b) {
                const double mb = mass(b);
                sm = __dadd_rn(sm, mb);
                sx = __dadd_rn(sx, __dmul_rn(px[b], mb));
                sy = __dadd_rn(sy, __dmul_rn(py[b], mb));
                sz = __dadd_rn(sz, __dmul_rn(pz[b], mb));
            }
        }
        ls[l] = double4_32a{sx, sy, sz, sm};
        cdep[l] = l == 0 ? (int8_t)-1 : (int8_t)common_depth(leaf_key[l - 1], leaf_key[l]);
        if (l == L - 1) cdep[L] = -1;  // right sentinel of the boundary pass
        if (kMoments) {
            double q = 0.0;
            if (b1 - b0 > 1 && sm > 0) {
                const double is = rcp_nr(sm);
                const double cx = sx * is, cy = sy * is, cz = sz * is;
                for (int b = b0; b < b1; ++b) {
                    const double dx = px[b] - cx, dy = py[b] - cy, dz = pz[b] - cz;
                    q += mass(b) * (dx * dx + dy * dy + dz * dz);
                }
            }
            lq[l] = q;
        }
    }
}

// ---- Tree structure from the boundary depths ---------------------------
// With d(j) = cdep[j] for the boundaries 1 <= j < L and d(0) = d(L) = -1,
// the branching node that boundary j splits (the cell of depth d(j) holding
// leaves j-1 and j) spans the leaves [pl(j), pr(j)) between the nearest
// shallower boundaries
//   pl(j) = max{k < j : d(k) < d(j)},   pr(j) = min{k > j : d(k) < d(j)};
// its splits are the boundaries of depth d(j) in between (at most 7: eight
// octants), and the first of them represents it (j is first exactly when
// max{k < j : d(k) <= d(j)} is pl(j)).  next(j) = min{k > j : d(k) <= d(j)}
// is j's next split when d(next(j)) = d(j).  These nearest-value queries are
// answered per warp, block and grid: a query looks inside its own warp first
// (the lanes below its depth, from ballots on the depth's bits), then in the
// other warps of its block (prefix / suffix over the warps' last and first
// positions below each of the 22 thresholds t, d <= t - 1, t = 0..21), then
// in the other blocks (prefix / suffix over the blocks' extreme positions,
// from a pass over block summaries).  No searches and no atomics.
constexpr int kNT = kMaxDepth + 1;  // thresholds t: d <= t - 1
constexpr int kBT = 1024;           // boundary positions per block
constexpr int kBW = kBT / 32;

__device__ __forceinline__ int bnd_depth(const int8_t* __restrict__ cdep, int L, int64_t j)
{
    return j <= L ? (int)cdep[j] : 127;  // cdep[0] = cdep[L] = -1; past L: no threshold
}

// A warp's last and first position below each threshold t (v < t, i.e.
// d <= t - 1), into wl[t] and wf[t] (-1 / INT_MAX where none is): lane l is
// the last below t exactly for t in (v_l, min of the later lanes' v], and
// the first for t in (v_l, min of the earlier lanes' v]; thresholds up to
// the warp's minimum have neither.  Two min-scans and a short loop per lane
// instead of one ballot per threshold.
__device__ __forceinline__ void warp_threshold_ends(int v, int lane, int wbase, int* wl, int* wf)
{
    int suf = v, pre = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_down_sync(0xffffffffu, suf, off);
        if (lane + off < 32) suf = min(suf, y);
        const int z = __shfl_up_sync(0xffffffffu, pre, off);
        if (lane >= off) pre = min(pre, z);
    }
    int s_next = __shfl_down_sync(0xffffffffu, suf, 1);
    if (lane == 31) s_next = 127;
    int p_prev = __shfl_up_sync(0xffffffffu, pre, 1);
    if (lane == 0) p_prev = 127;
    const int wmin = __shfl_sync(0xffffffffu, pre, 31);
    if (lane < kNT && lane <= wmin) {
        wl[lane] = -1;
        wf[lane] = INT_MAX;
    }
    const int lo = v + 1;  // v >= -1
    for (int t = lo; t <= min(s_next, kNT - 1); ++t) wl[t] = wbase + lane;
    for (int t = lo; t <= min(p_prev, kNT - 1); ++t) wf[t] = wbase + lane;
}

// Per block: for every threshold the last and the first position at or below it.
__global__ void __launch_bounds__(kBT) bnd_summary_kernel(const int32_t* __restrict__ counts,
                                                          const int8_t* __restrict__ cdep,
                                                          int32_t* __restrict__ blast, int32_t* __restrict__ bfirst)
{
    static_assert(kNT <= 32, "one lane per threshold");
    __shared__ int wl[kBW][kNT], wf[kBW][kNT];
    const int L = counts[0];
    const int64_t j = (int64_t)blockIdx.x * kBT + threadIdx.x;
    const int v = bnd_depth(cdep, L, j);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int wbase = (int)(j - lane);
    warp_threshold_ends(v, lane, wbase, wl[w], wf[w]);
    __syncthreads();
    // Warp t reduces threshold t over the block's warps (lane = warp).
    static_assert(kBW == 32 && kNT <= kBW, "one lane per warp, one warp per threshold");
    if (w < kNT) {
        const int t = w;
        int l = wl[lane][t], f = wf[lane][t];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            l = max(l, __shfl_xor_sync(0xffffffffu, l, off));
            f = min(f, __shfl_xor_sync(0xffffffffu, f, off));
        }
        if (lane == 0) {
            blast[(int64_t)blockIdx.x * kNT + t] = l;
            bfirst[(int64_t)blockIdx.x * kNT + t] = f;
        }
    }
}

// Exclusive scan of one int per thread over the block (max, or min with
// kMin), continued from `carry`; returns the thread's exclusive value and
// advances `carry` past the whole block.
template <bool kMin>
__device__ int block_excl_extreme(int x, int& carry, int* wsum)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    auto op = [](int a, int b) { return kMin ? min(a, b) : max(a, b); };
    const int ident = kMin ? INT_MAX : -1;
    int inc = x;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc = op(inc, y);
    }
    int ex = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) ex = ident;
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        int sw = lane < (int)(blockDim.x >> 5) ? wsum[lane] : ident;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, sw, off);
            if (lane >= off) sw = op(sw, y);
        }
        wsum[lane] = sw;
    }
    __syncthreads();
    const int res = op(carry, op(w ? wsum[w - 1] : ident, ex));
    carry = op(carry, wsum[(blockDim.x >> 5) - 1]);
    __syncthreads();
    return res;
}

// Two blocks per threshold: the blocks' exclusive prefix of last positions
// (max; blocks 0..kNT-1) and exclusive suffix of first positions (min;
// blocks kNT..2 kNT-1).
__global__ void __launch_bounds__(1024) bnd_scan_kernel(int nblk, const int32_t* __restrict__ blast,
                                                        const int32_t* __restrict__ bfirst,
                                                        int32_t* __restrict__ bpre, int32_t* __restrict__ bsuf)
{
    __shared__ int wsum[32];
    const int t = blockIdx.x % kNT;
    if (blockIdx.x < kNT) {
        int carry = -1;
        for (int base = 0; base < nblk; base += blockDim.x) {
            const int b = base + threadIdx.x;
            const int x = b < nblk ? blast[(int64_t)b * kNT + t] : -1;
            const int ex = block_excl_extreme<false>(x, carry, wsum);
            if (b < nblk) bpre[(int64_t)b * kNT + t] = ex;
        }
    } else {
        int carry = INT_MAX;
        for (int base = 0; base < nblk; base += blockDim.x) {
            const int b = nblk - 1 - (base + (int)threadIdx.x);
            const int x = b >= 0 ? bfirst[(int64_t)b * kNT + t] : INT_MAX;
            const int ex = block_excl_extreme<true>(x, carry, wsum);
            if (b >= 0) bsuf[(int64_t)b * kNT + t] = ex;
        }
    }
}

// Per boundary: the representative flag (flag[j], 0 for j = 0 and j >= L up
// to cap), pl, pr and next.
__global__ void __launch_bounds__(kBT) bnd_resolve_kernel(const int32_t* __restrict__ counts,
                                                          const int8_t* __restrict__ cdep,
                                                          const int32_t* __restrict__ bpre,
                                                          const int32_t* __restrict__ bsuf, int32_t* __restrict__ flag,
                                                          int32_t* __restrict__ pl, int32_t* __restrict__ pr,
                                                          int32_t* __restrict__ nxt, int64_t cap)
{
    __shared__ int wl[kBW][kNT], wf[kBW][kNT];
    const int L = counts[0];
    const int64_t j = (int64_t)blockIdx.x * kBT + threadIdx.x;
    const int v = bnd_depth(cdep, L, j);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int wbase = (int)(j - lane);
    warp_threshold_ends(v, lane, wbase, wl[w], wf[w]);
    // Inside the warp: the lanes whose depth is below this lane's (LT) and
    // at or below it (LE), from five ballots on the bits of v + 1 (past the
    // end, v = 127, counts as 30: above every depth).
    const int vq = min(v, 30) + 1;
    unsigned lt_m = 0u, eq_m = 0xffffffffu;
#pragma unroll
    for (int k = 4; k >= 0; --k) {
        const bool bit = (vq >> k) & 1;
        const unsigned b = __ballot_sync(0xffffffffu, bit);
        if (bit) {
            lt_m |= eq_m & ~b;
            eq_m &= b;
        } else {
            eq_m &= ~b;
        }
    }
    const unsigned le_m = lt_m | eq_m;
    __syncthreads();
    // Each warp's answer from outside it: exclusive prefix (max) and suffix
    // (min) over the warps, started from the other blocks'.  Warp t scans
    // threshold t, one lane per warp of the block.
    if (w < kNT) {
        const int t = w;
        int inc = wl[lane][t];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc = max(inc, y);
        }
        int ex = __shfl_up_sync(0xffffffffu, inc, 1);
        if (lane == 0) ex = -1;
        wl[lane][t] = max(bpre[(int64_t)blockIdx.x * kNT + t], ex);
        int sinc = wf[lane][t];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_down_sync(0xffffffffu, sinc, off);
            if (lane + off < 32) sinc = min(sinc, y);
        }
        int sex = __shfl_down_sync(0xffffffffu, sinc, 1);
        if (lane == 31) sex = INT_MAX;
        wf[lane][t] = min(bsuf[(int64_t)blockIdx.x * kNT + t], sex);
    }
    __syncthreads();
    if (j >= cap) return;
    int f = 0;
    if (j >= 1 && j < L) {
        const unsigned below = (1u << lane) - 1u, above = ~below & ~(1u << lane);
        auto prev = [&](unsigned mask, int t) {
            const unsigned m = mask & below;
            return m ? wbase + 31 - __clz(m) : wl[w][t];
        };
        auto next = [&](unsigned mask, int t) {
            const unsigned m = mask & above;
            return m ? wbase + __ffs(m) - 1 : wf[w][t];
        };
        const int PL = prev(lt_m, v), PLE = prev(le_m, v + 1);
        f = PLE == PL ? 1 : 0;
        pl[j] = PL;
        pr[j] = next(lt_m, v);
        nxt[j] = next(le_m, v + 1);
    }
    flag[j] = f;
}

// Each branching node from its representative: depth, leaf range and its
// splits (at most 7) with their ranks; child count = splits + 1.
__global__ void node_split_kernel(const int32_t* __restrict__ counts, const int8_t* __restrict__ cdep,
                                  const int32_t* __restrict__ flag, const int32_t* __restrict__ excl,
                                  const int32_t* __restrict__ pl, const int32_t* __restrict__ pr,
                                  const int32_t* __restrict__ nxt, int32_t* __restrict__ node_rep,
                                  int32_t* __restrict__ node_a, int32_t* __restrict__ node_e,
                                  uint8_t* __restrict__ node_depth, int32_t* __restrict__ node_nchild,
                                  int32_t* __restrict__ split_node, int8_t* __restrict__ split_rank,
                                  unsigned* __restrict__ err)
{
    const int L = counts[0];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
        if (j == 0 || !flag[j]) continue;
        const int b = excl[j];
        const int c = cdep[j];
        node_rep[b] = j;
        node_a[b] = pl[j];
        node_e[b] = pr[j];
        node_depth[b] = (uint8_t)c;
        int k = j, r = 0;
        for (;;) {
            split_node[k] = b;
            split_rank[k] = (int8_t)r;
            ++r;
            k = nxt[k];
            if (k >= L || cdep[k] != c || r >= 7) break;
        }
        if (k < L && cdep[k] == c) atomicOr(err, kErrOverflow);  // an eighth split: impossible for an octree
        node_nchild[b] = r + 1;
    }
}

// Child slots: every leaf and branching node finds its parent from the
// boundaries at its two ends (the deeper one splits the parent; both
// sentinels: the root) and its place among the parent's children from that
// split's rank.  Slot 0 is the root.
__global__ void node_place_kernel(const int32_t* __restrict__ counts, const int8_t* __restrict__ cdep,
                                  const int32_t* __restrict__ node_a, const int32_t* __restrict__ node_e,
                                  const uint8_t* __restrict__ node_depth, const int32_t* __restrict__ node_cs,
                                  const int32_t* __restrict__ split_node, const int8_t* __restrict__ split_rank,
                                  int32_t* __restrict__ slot_ref, uint8_t* __restrict__ slot_top,
                                  unsigned* __restrict__ err)
{
    const int L = counts[0], B = counts[1], S = counts[2];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L + B; i += gridDim.x * blockDim.x) {
        int a, e, ref;
        if (i < L) {
            a = i; e = i + 1; ref = i;
        } else {
            const int b = i - L;
            a = node_a[b]; e = node_e[b]; ref = ~b;
        }
        const int ca = a == 0 ? -1 : cdep[a];
        const int ce = e >= L ? -1 : cdep[e];
        int P = -1, s = 0, top = 0;
        if (ca >= 0 || ce >= 0) {
            const bool left = ca >= ce;
            const int k = left ? a : e;
            P = split_node[k];
            if ((unsigned)P >= (unsigned)B) {  // every boundary splits a node: a broken invariant
                atomicOr(err, kErrOverflow);
                continue;
            }
            s = node_cs[P] + 1 + split_rank[k] + (left ? 1 : 0);
            top = node_depth[P] + 1;
            if (s < 1 || s >= S) {
                atomicOr(err, kErrOverflow);
                continue;
            }
        }
        slot_ref[s] = ref;
        slot_top[s] = (uint8_t)top;
    }
}

// One node's sums from its children, in slot (= octant) order from 0.0
// (linear_octree.cpp:69-87), and with kMoments the second moment by the
// parallel-axis rule (see below).  The children's sums were written by the
// previous level's launch; loads bypass L1.
__device__ __forceinline__ double4_32a load_sums(const double4_32a* p)
{
    const double2 a = __ldcg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2*>(p) + 1);
    return double4_32a{a.x, a.y, b.x, b.y};
}

// A node has at most 8 children: their slot entries are loaded together,
// then their sums four at a time, before the additions (independent loads
// in flight instead of a chain of dependent ones), which still run in slot
// order.
template <bool kMoments>
__device__ void node_sums(int b, const int32_t* __restrict__ node_cs, const int32_t* __restrict__ node_nchild,
                          const int32_t* __restrict__ slot_ref, const double4_32a* ls, double4_32a* ns,
                          const double* lq, double* nq)
{
    const int s0 = node_cs[b] + 1, nc = node_nchild[b];
    int rr[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) rr[c] = c < nc ? slot_ref[s0 + c] : 0;
    double sm = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
#pragma unroll
    for (int h = 0; h < 8; h += 4) {
        if (h >= nc) break;
        double4_32a vv[4];
#pragma unroll
        for (int c = 0; c < 4; ++c)
            if (h + c < nc) vv[c] = load_sums(rr[h + c] >= 0 ? ls + rr[h + c] : ns + ~rr[h + c]);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (h + c < nc) {
                sm = __dadd_rn(sm, vv[c].w);
                sx = __dadd_rn(sx, vv[c].x);
                sy = __dadd_rn(sy, vv[c].y);
                sz = __dadd_rn(sz, vv[c].z);
            }
        }
    }
    ns[b] = double4_32a{sx, sy, sz, sm};
    if (kMoments) {
        // m_c |c_c - c|^2 = |w_c - m_c c|^2 / m_c: u = w_c - m_c c by FMA
        // keeps the cancellation in FP64; the division by m_c needs only
        // the feature's precision (an FP32 reciprocal, 2^-22).  Masses are
        // >= 0, so "> 0" is a test on the bit pattern.
        double q = 0.0;
        if (__double_as_longlong(sm) > 0) {
            const double is = rcp_nr(sm);
            const double gx = sx * is, gy = sy * is, gz = sz * is;
            for (int c = 0; c < nc; ++c) {
                const int r = slot_ref[s0 + c];
                const double4_32a v = load_sums(r >= 0 ? ls + r : ns + ~r);
                const double cq = __ldcg(r >= 0 ? lq + r : nq + ~r);
                if (__double_as_longlong(v.w) > 0) {
                    const double ux = fma(-v.w, gx, v.x), uy = fma(-v.w, gy, v.y), uz = fma(-v.w, gz, v.z);
                    const double uu = fma(ux, ux, fma(uy, uy, uz * uz));
                    q += cq + uu * widen(__frcp_rn(narrow_trunc(v.w)));
                }
            }
        }
        nq[b] = q;
    }
}

// Depth buckets of the branching nodes (depths 0..20), three kernels:
// per-block counts, a scan of each depth's block counts, per-block placement.
constexpr int kBucketThreads = 1024;
constexpr int kDepths = kMaxDepth;  // branching depths 0..20

__global__ void bucket_count_kernel(const int32_t* __restrict__ counts, const uint8_t* __restrict__ node_depth,
                                    int32_t* __restrict__ blk_cnt, int nblk)
{
    __shared__ int32_t c[kDepths];
    if (threadIdx.x < kDepths) c[threadIdx.x] = 0;
    __syncthreads();
    const int B = counts[1];
    const int b = blockIdx.x * kBucketThreads + threadIdx.x;
    if (b < B) atomicAdd(&c[node_depth[b]], 1);
    __syncthreads();
    if (threadIdx.x < kDepths) blk_cnt[threadIdx.x * nblk + blockIdx.x] = c[threadIdx.x];
}

// One block per depth: the exclusive scan of that depth's per-block counts
// (offsets within the depth's bucket) and the depth's total.
__global__ void __launch_bounds__(kBucketThreads) bucket_scan_kernel(int32_t* __restrict__ blk_cnt, int nblk,
                                                                      int32_t* __restrict__ depth_tot)
{
    __shared__ int32_t warp_tot[32];
    const int d = blockIdx.x;
    int32_t* c = blk_cnt + (int64_t)d * nblk;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int carry = 0;
    for (int base = 0; base < nblk; base += kBucketThreads) {
        const int i = base + threadIdx.x;
        const int v = i < nblk ? c[i] : 0;
        int x = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            int t = warp_tot[lane];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, t, off);
                if (lane >= off) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        if (i < nblk) c[i] = carry + (w > 0 ? warp_tot[w - 1] : 0) + x - v;
        carry += warp_tot[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) depth_tot[d] = carry;
}

// Each block: the depth offsets from the totals (block 0 also stores them
// for the level launches), then its nodes into their depth buckets.
__global__ void bucket_place_kernel(const int32_t* __restrict__ counts, const uint8_t* __restrict__ node_depth,
                                    const int32_t* __restrict__ blk_off, int nblk,
                                    const int32_t* __restrict__ depth_tot, int32_t* __restrict__ depth_off,
                                    int32_t* __restrict__ depth_nodes)
{
    __shared__ int32_t c[kDepths];
    __shared__ int32_t off[kDepths + 1];
    if (threadIdx.x < kDepths) c[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        int run = 0;
        for (int d = 0; d < kDepths; ++d) {
            off[d] = run;
            run += depth_tot[d];
        }
        off[kDepths] = run;
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x <= kDepths) depth_off[threadIdx.x] = off[threadIdx.x];
    const int B = counts[1];
    const int b = blockIdx.x * kBucketThreads + threadIdx.x;
    if (b < B) {
        const int d = node_depth[b];
        const int r = atomicAdd(&c[d], 1);  // order inside a bucket is irrelevant
        depth_nodes[off[d] + blk_off[d * nblk + blockIdx.x] + r] = b;
    }
}

// Monopole (and second moment) of the branching nodes at one depth, from
// the sums of the level below (node_sums).
template <bool kMoments>
__global__ void monopole_level_kernel(int depth, const int32_t* __restrict__ depth_off,
                                      const int32_t* __restrict__ depth_nodes, const int32_t* __restrict__ node_cs,
                                      const int32_t* __restrict__ node_nchild, const int32_t* __restrict__ slot_ref,
                                      const double4_32a* ls, double4_32a* ns, const double* lq, double* nq)
{
    const int lo = depth_off[depth], hi = depth_off[depth + 1];
    for (int k = lo + blockIdx.x * blockDim.x + threadIdx.x; k < hi; k += gridDim.x * blockDim.x)
        node_sums<kMoments>(depth_nodes[k], node_cs, node_nchild, slot_ref, ls, ns, lq, nq);
}

// com = w/m when m > 0 (linear_octree.cpp:95-104), then the merge of
// linear_octree.cpp:194-202 with m0 = com0 = 0.  A one-body leaf passes its
// body's position (one = true): its w is 0 + x m, so w/m is merge_div(m, x).
__device__ inline void finish_com(double m, double wx, double wy, double wz, TreeRec& r, int merge, bool one,
                                  double x, double y, double z)
{
    double cx = wx, cy = wy, cz = wz;
    if (m > 0) {
        if (one) { cx = merge_div(m, x); cy = merge_div(m, y); cz = merge_div(m, z); }
        else {
            const double r = rcp_nr(m);
            cx = div_exact(wx, m, r); cy = div_exact(wy, m, r); cz = div_exact(wz, m, r);
        }
    }
    if (!merge) {  // buildOctreeBottomUp's own output, before any exchange
        r.cx = cx; r.cy = cy; r.cz = cz; r.m = m;
        return;
    }
    const double tot = __dadd_rn(0.0, m);
    if (tot == 0) {
        r.cx = r.cy = r.cz = r.m = 0.0;
        return;
    }
    r.cx = merge_div(tot, cx);
    r.cy = merge_div(tot, cy);
    r.cz = merge_div(tot, cz);
    r.m = tot;
}

// The far-field tree of the FP32 forms (direct bodies' masses zeroed) is not
// the reference's tree, so its centres of mass need no bit-exact quotient:
// w times the refined reciprocal of m (within 2 ulps), no merge step.  The
// kernel also writes the FP32 walk's node records (hi + lo split of the
// centre, G m and the topology word), which the walk would otherwise make in
// a pass of its own.
// Masses are >= 0, so "m > 0" is a test on the bit pattern.  A leaf of one
// body takes the body's position (the quotient w/m would round it).
__device__ inline void far_com(double m, double wx, double wy, double wz, TreeRec& r)
{
    if (__double_as_longlong(m) > 0) {
        const double q = rcp_nr(m);
        r.cx = wx * q; r.cy = wy * q; r.cz = wz * q;
    } else {
        r.cx = wx; r.cy = wy; r.cz = wz;
    }
    r.m = m;
}

struct FarOut {
    float4* A;       // {hi.x, hi.y, hi.z, G m}
    float4* B;       // {lo.x, lo.y, lo.z, bits of child or leaf id}
    uint32_t* meta;  // nchild | depth << 8 | leaf << 16 | massless << 17
    double G;
};

template <bool kMoments, bool kFar>
__global__ void finalize_kernel(const int32_t* __restrict__ counts, const int32_t* __restrict__ slot_ref,
                                const uint8_t* __restrict__ slot_top, const double4_32a* __restrict__ ls,
                                const double4_32a* __restrict__ ns, const int32_t* __restrict__ node_cs,
                                const int32_t* __restrict__ node_nchild, const uint8_t* __restrict__ node_depth,
                                TreeRec* __restrict__ rec, const double* __restrict__ lq,
                                const double* __restrict__ nq, float* __restrict__ spread, int merge,
                                const int32_t* __restrict__ leaf_first, const double* __restrict__ px,
                                const double* __restrict__ py, const double* __restrict__ pz, FarOut far)
{
    const int S = counts[2];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const int r = slot_ref[s];
        TreeRec o;
        o.top = slot_top[s];
        o.pad0 = 0;
        o.pad1 = 0;
        const double4_32a v = r >= 0 ? ls[r] : ns[~r];
        if (r >= 0) {
            if (kFar) {
                const int b = leaf_first[r];
                if (leaf_first[r + 1] == b + 1 && __double_as_longlong(v.w) > 0) {
                    o.cx = px[b]; o.cy = py[b]; o.cz = pz[b]; o.m = v.w;
                } else {
                    far_com(v.w, v.x, v.y, v.z, o);
                }
            } else {
                const int b = leaf_first[r];
                const bool one = leaf_first[r + 1] == b + 1;
                finish_com(v.w, v.x, v.y, v.z, o, merge, one, one ? px[b] : 0.0, one ? py[b] : 0.0,
                           one ? pz[b] : 0.0);
            }
            o.child = -1;
            o.leaf = r;
            o.nchild = 0;
            o.depth = (uint8_t)kMaxDepth;
        } else {
            const int b = ~r;
            if (kFar) far_com(v.w, v.x, v.y, v.z, o);
            else finish_com(v.w, v.x, v.y, v.z, o, merge, false, 0.0, 0.0, 0.0);
            o.child = node_cs[b] + 1;
            o.leaf = -1;
            o.nchild = (uint8_t)node_nchild[b];
            o.depth = node_depth[b];
        }
        // The fused far-field build feeds only the FP32 walks, which read
        // the FP32 records below: the FP64 record is left out (ensure_rec
        // writes it when a diagnostic or export asks for it).
        if (!kFar) rec[s] = o;
        if (kFar) {  // the FP32 walk's records, as fp32_nodes_kernel makes them
            const bool leaf = o.child < 0;
            far.A[s] = make_float4(narrow_trunc(o.cx), narrow_trunc(o.cy), narrow_trunc(o.cz),
                                   narrow_trunc(far.G * o.m));
            far.B[s] = make_float4(low_part(o.cx), low_part(o.cy), low_part(o.cz),
                                   __int_as_float(leaf ? o.leaf : o.child));
            far.meta[s] = (uint32_t)o.nchild | ((uint32_t)o.depth << 8) | ((leaf ? 1u : 0u) << 16) |
                          ((__double_as_longlong(o.m) << 1) == 0 ? 1u << 17 : 0u);
        }
        if (kMoments) {  // a feature: FP32 after narrowing on the bit patterns
            const double m = v.w;
            const double q = r >= 0 ? lq[r] : nq[~r];
            spread[s] = __double_as_longlong(m) > 0 ? sqrtf(narrow_trunc(q) * __frcp_rn(narrow_trunc(m))) : 0.0f;
        }
    }
}

__global__ void slot_count_kernel(int32_t* counts, const int32_t* __restrict__ child_total)
{
    // S = 1 (root) + every child slot.
    counts[2] = 1 + *child_total;
}

}  // namespace

int64_t boundary_pass_ints(int64_t n)
{
    const int64_t nb = (n + 1 + kBT - 1) / kBT;
    return 4 * kNT * nb;
}

int launch_build(bh_context* ctx, const double* mass, bool moments, bool far_fused, double G, bool far_masses)
{
    const int nzero = far_masses ? (ctx->num_direct < 64 ? ctx->num_direct : 64) : 0;
    ctx->fnodes_fused = false;
    const int64_t n = ctx->n;
    if (n == 0) return BH_OK;
    cudaStream_t st = ctx->stream;
    const int maxb = 8 * bh::num_sms();
    const int g = grid_for(n, kThreads, maxb);

    // 1. leaves: ids, first bodies and keys from a scan of the keys' head flags
    int rc = device_number_leaves(ctx, ctx->key, n, ctx->counts + 0, ctx->body_leaf, ctx->leaf_first, ctx->leaf_key);
    if (rc) return rc;
    if (moments)
        leaf_sum_kernel<true><<<g, kThreads, 0, st>>>(ctx->counts, ctx->leaf_first, ctx->leaf_key, ctx->px, ctx->py,
                                                      ctx->pz, mass, ctx->id, nzero, ctx->leaf_s, ctx->cdep,
                                                      ctx->leaf_q);
    else
        leaf_sum_kernel<false><<<g, kThreads, 0, st>>>(ctx->counts, ctx->leaf_first, ctx->leaf_key, ctx->px, ctx->py,
                                                       ctx->pz, mass, ctx->id, nzero, ctx->leaf_s, ctx->cdep,
                                                       ctx->leaf_q);
    BH_LAUNCH_CHECK(ctx);

    // 2. branching nodes: the boundary pass (representative flags, node
    // ranges, split chains) -> node ids -> child counts -> child slots
    {
        const int nb = (int)((n + 1 + kBT - 1) / kBT);
        int32_t* blast = ctx->ansv_blk;
        int32_t* bfirst = blast + (int64_t)nb * kNT;
        int32_t* bpre = bfirst + (int64_t)nb * kNT;
        int32_t* bsuf = bpre + (int64_t)nb * kNT;
        bnd_summary_kernel<<<nb, kBT, 0, st>>>(ctx->counts, ctx->cdep, blast, bfirst);
        BH_LAUNCH_CHECK(ctx);
        bnd_scan_kernel<<<2 * kNT, 1024, 0, st>>>(nb, blast, bfirst, bpre, bsuf);
        BH_LAUNCH_CHECK(ctx);
        bnd_resolve_kernel<<<nb, kBT, 0, st>>>(ctx->counts, ctx->cdep, bpre, bsuf, ctx->head, ctx->bnd_pl, ctx->bnd_pr,
                                                ctx->bnd_next, n);
        BH_LAUNCH_CHECK(ctx);
    }
    // rep_node[j] = exclusive count of representatives before j, i.e. the
    // node id of boundary j when it is a representative.
    rc = device_exclusive_scan(ctx, ctx->head, ctx->rep_node, n, nullptr, ctx->counts + 1);
    if (rc) return rc;
    node_split_kernel<<<g, kThreads, 0, st>>>(ctx->counts, ctx->cdep, ctx->head, ctx->rep_node, ctx->bnd_pl,
                                              ctx->bnd_pr, ctx->bnd_next, ctx->node_rep, ctx->node_a, ctx->node_e,
                                              ctx->node_depth, ctx->node_nchild, ctx->split_node, ctx->split_rank,
                                              ctx->err);
    BH_LAUNCH_CHECK(ctx);
    rc = device_exclusive_scan(ctx, ctx->node_nchild, ctx->node_cs, n, ctx->counts + 1, ctx->counts + 3);
    if (rc) return rc;
    slot_count_kernel<<<1, 1, 0, st>>>(ctx->counts, ctx->counts + 3);
    BH_LAUNCH_CHECK(ctx);
    node_place_kernel<<<grid_for(2 * n, kThreads, maxb), kThreads, 0, st>>>(
        ctx->counts, ctx->cdep, ctx->node_a, ctx->node_e, ctx->node_depth, ctx->node_cs, ctx->split_node,
        ctx->split_rank, ctx->slot_ref, ctx->slot_top, ctx->err);
    BH_LAUNCH_CHECK(ctx);

    // 3./4. monopoles (and second moments), level by level, deepest first:
    // depth buckets of the branching nodes, then one launch per depth; each
    // node sums its children in slot order from 0.0.  No atomics.
    {
        const int nblk = (int)((n + kBucketThreads - 1) / kBucketThreads);
        bucket_count_kernel<<<nblk, kBucketThreads, 0, st>>>(ctx->counts, ctx->node_depth, ctx->scan_tmp, nblk);
        BH_LAUNCH_CHECK(ctx);
        int32_t* depth_tot = ctx->scan_tmp + (int64_t)kDepths * nblk;
        bucket_scan_kernel<<<kDepths, kBucketThreads, 0, st>>>(ctx->scan_tmp, nblk, depth_tot);
        BH_LAUNCH_CHECK(ctx);
        bucket_place_kernel<<<nblk, kBucketThreads, 0, st>>>(ctx->counts, ctx->node_depth, ctx->scan_tmp, nblk,
                                                             depth_tot, ctx->depth_off, ctx->depth_nodes);
        BH_LAUNCH_CHECK(ctx);
        for (int d = kMaxDepth - 1; d >= 0; --d) {
            if (moments)
                monopole_level_kernel<true><<<g, kThreads, 0, st>>>(d, ctx->depth_off, ctx->depth_nodes,
                                                                    ctx->node_cs, ctx->node_nchild, ctx->slot_ref,
                                                                    ctx->leaf_s, ctx->node_s, ctx->leaf_q,
                                                                    ctx->node_q);
            else
                monopole_level_kernel<false><<<g, kThreads, 0, st>>>(d, ctx->depth_off, ctx->depth_nodes,
                                                                     ctx->node_cs, ctx->node_nchild, ctx->slot_ref,
                                                                     ctx->leaf_s, ctx->node_s, ctx->leaf_q,
                                                                     ctx->node_q);
            BH_LAUNCH_CHECK(ctx);
        }
    }

    // 5. traversal records
    const int gs = grid_for(2 * n, kThreads, maxb);
    const FarOut far{ctx->fA, ctx->fB, ctx->fmeta, G};
#define BH_FINALIZE(M, F)                                                                                      \
    finalize_kernel<M, F><<<gs, kThreads, 0, st>>>(                                                            \
        ctx->counts, ctx->slot_ref, ctx->slot_top, ctx->leaf_s, ctx->node_s, ctx->node_cs, ctx->node_nchild,     \
        ctx->node_depth,                                                                                       \
        ctx->rec, ctx->leaf_q, ctx->node_q, ctx->fspread, ctx->build_merge ? 1 : 0, ctx->leaf_first, ctx->px,  \
        ctx->py, ctx->pz, far)
    if (far_fused) {
        if (moments) BH_FINALIZE(true, true);
        else BH_FINALIZE(false, true);
    } else {
        if (moments) BH_FINALIZE(true, false);
        else BH_FINALIZE(false, false);
    }
#undef BH_FINALIZE
    BH_LAUNCH_CHECK(ctx);
    if (far_fused) {
        ctx->fnodes_fused = true;
        ctx->fnodes_G = G;
    }
    ctx->tree_rec = !far_fused;
    return BH_OK;
}

int ensure_rec(bh_context* ctx)
{
    if (ctx->tree_rec || ctx->n == 0) return BH_OK;
    return launch_build(ctx, ctx->m, ctx->tree_moments, false, 0.0, ctx->tree_far);
}

}  // namespace bh
