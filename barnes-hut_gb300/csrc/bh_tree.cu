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
#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kThreads = 256;

inline int grid_for(int64_t n, int threads, int max_blocks)
{
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (int)(b > max_blocks ? max_blocks : b);
}

// First index v in (u, L] whose key leaves u's cell under `mask`.
__device__ int cell_end(const uint64_t* __restrict__ K, int L, int u, uint64_t mask)
{
    const uint64_t p = K[u] & mask;
    int lo = u, hi = L, step = 1;
    for (;;) {
        const int64_t probe = (int64_t)u + step;
        if (probe >= L) break;
        if ((K[probe] & mask) != p) { hi = (int)probe; break; }
        lo = (int)probe;
        step <<= 1;
    }
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if ((K[mid] & mask) == p) lo = mid; else hi = mid;
    }
    return hi;
}

// First index t in [0, u] whose key is in u's cell under `mask`.
__device__ int cell_start(const uint64_t* __restrict__ K, int u, uint64_t mask)
{
    const uint64_t p = K[u] & mask;
    int hi = u, lo = -1, step = 1;
    for (;;) {
        const int probe = u - step;
        if (probe < 0) break;
        if ((K[probe] & mask) != p) { lo = probe; break; }
        hi = probe;
        step <<= 1;
    }
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if ((K[mid] & mask) == p) hi = mid; else lo = mid;
    }
    return hi;
}

__device__ inline bool is_head(const uint64_t* __restrict__ key, int64_t i)
{
    return i == 0 || key[i] != key[i - 1];
}

__global__ void leaf_head_kernel(int64_t n, const uint64_t* __restrict__ key, int32_t* __restrict__ head)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        head[i] = is_head(key, i) ? 1 : 0;
}

// Leaf ids of bodies, first body and key of each leaf.
__global__ void leaf_scatter_kernel(int64_t n, const uint64_t* __restrict__ key, const int32_t* __restrict__ excl,
                                    int32_t* __restrict__ body_leaf, int32_t* __restrict__ leaf_first,
                                    uint64_t* __restrict__ leaf_key)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const bool h = is_head(key, i);
        const int32_t lid = h ? excl[i] : excl[i] - 1;
        body_leaf[i] = lid;
        if (h) {
            leaf_first[lid] = (int32_t)i;
            leaf_key[lid] = key[i];
        }
        if (i == n - 1) leaf_first[lid + 1] = (int32_t)n;
    }
}

// Leaf sums in body order (linear_octree.cpp:28-38) and boundary depths.
// kMoments: also the leaf's second moment about its centre of mass (the
// learned criterion's spread feature), sum_b m_b |x_b - c|^2.
template <bool kMoments>
__global__ void leaf_sum_kernel(const int32_t* __restrict__ counts, const int32_t* __restrict__ leaf_first,
                                const uint64_t* __restrict__ leaf_key, const double* __restrict__ px,
                                const double* __restrict__ py, const double* __restrict__ pz,
                                const double* __restrict__ m, double4_32a* __restrict__ ls, int8_t* __restrict__ cdep,
                                double* __restrict__ lq)
{
    const int L = counts[0];
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < L; l += gridDim.x * blockDim.x) {
        double sm = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
        const int b0 = leaf_first[l], b1 = leaf_first[l + 1];
        for (int b = b0; b < b1; ++b) {
            const double mb = m[b];
            sm = __dadd_rn(sm, mb);
            sx = __dadd_rn(sx, __dmul_rn(px[b], mb));
            sy = __dadd_rn(sy, __dmul_rn(py[b], mb));
            sz = __dadd_rn(sz, __dmul_rn(pz[b], mb));
        }
        ls[l] = double4_32a{sx, sy, sz, sm};
        cdep[l] = l == 0 ? (int8_t)-1 : (int8_t)common_depth(leaf_key[l - 1], leaf_key[l]);
        if (kMoments) {
            double q = 0.0;
            if (b1 - b0 > 1 && sm > 0) {
                const double is = rcp_nr(sm);
                const double cx = sx * is, cy = sy * is, cz = sz * is;
                for (int b = b0; b < b1; ++b) {
                    const double dx = px[b] - cx, dy = py[b] - cy, dz = pz[b] - cz;
                    q += m[b] * (dx * dx + dy * dy + dz * dz);
                }
            }
            lq[l] = q;
        }
    }
}

// flag[j] = 1 when boundary j is the first child boundary of its node.
__global__ void rep_flag_kernel(const int32_t* __restrict__ counts, const uint64_t* __restrict__ K,
                                const int8_t* __restrict__ cdep, int32_t* __restrict__ flag, int64_t cap)
{
    const int L = counts[0];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < cap; j += gridDim.x * blockDim.x) {
        int f = 0;
        if (j >= 1 && j < L) {
            const int D = cdep[j];
            const int t = cell_start(K, j - 1, prefix_mask(D + 1));
            f = (t == 0 || cdep[t] < D) ? 1 : 0;
        }
        flag[j] = f;
    }
}

// Node ids, first leaf, depth and child count of each branching node.
// excl is the exclusive scan of the flags: the node id of a representative.
__global__ void node_init_kernel(const int32_t* __restrict__ counts, const uint64_t* __restrict__ K,
                                 const int8_t* __restrict__ cdep, const int32_t* __restrict__ flag,
                                 const int32_t* __restrict__ excl, int32_t* __restrict__ node_rep,
                                 int32_t* __restrict__ node_a, uint8_t* __restrict__ node_depth,
                                 int32_t* __restrict__ node_nchild)
{
    const int L = counts[0];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
        if (j == 0 || !flag[j]) continue;
        const int b = excl[j];
        const int D = cdep[j];
        const uint64_t mc = prefix_mask(D + 1);
        const int a = cell_start(K, j - 1, mc);
        const int e = cell_end(K, L, j, prefix_mask(D));
        int nc = 1;  // the child [a, j)
        for (int u = j; u < e; u = cell_end(K, L, u, mc)) ++nc;
        node_rep[b] = j;
        node_a[b] = a;
        node_depth[b] = (uint8_t)D;
        node_nchild[b] = nc;
    }
}

// Child slots of every branching node; slot 0 is the root.
__global__ void node_children_kernel(const int32_t* __restrict__ counts, const uint64_t* __restrict__ K,
                                     const int32_t* __restrict__ rep_node, const int32_t* __restrict__ node_rep,
                                     const int32_t* __restrict__ node_a, const uint8_t* __restrict__ node_depth,
                                     const int32_t* __restrict__ node_cs, int32_t* __restrict__ slot_ref,
                                     uint8_t* __restrict__ slot_top, int32_t* __restrict__ leaf_parent,
                                     int32_t* __restrict__ node_parent)
{
    const int L = counts[0], B = counts[1];
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid == 0) {
        if (L == 1) {
            slot_ref[0] = 0;
            leaf_parent[0] = -1;
        } else {
            const int Dr = common_depth(K[0], K[L - 1]);
            const int root = rep_node[cell_end(K, L, 0, prefix_mask(Dr + 1))];
            slot_ref[0] = ~root;
            node_parent[root] = -1;
        }
        slot_top[0] = 0;
    }
    for (int b = gid; b < B; b += gridDim.x * blockDim.x) {
        const int D = node_depth[b];
        const uint64_t mc = prefix_mask(D + 1);
        const int a = node_a[b];
        const int e = cell_end(K, L, node_rep[b], prefix_mask(D));
        int s = node_cs[b] + 1;
        for (int u = a; u < e; ++s) {
            const int v = cell_end(K, L, u, mc);
            int ref;
            if (v - u == 1) {
                ref = u;
            } else {
                const int cd = common_depth(K[u], K[v - 1]);
                ref = ~rep_node[cell_end(K, L, u, prefix_mask(cd + 1))];
            }
            slot_ref[s] = ref;
            slot_top[s] = (uint8_t)(D + 1);
            if (ref >= 0) leaf_parent[ref] = b;
            else node_parent[~ref] = b;
            u = v;
        }
    }
}

// One node's sums from its children, in slot (= octant) order from 0.0
// (linear_octree.cpp:69-87), and with kMoments the second moment by the
// parallel-axis rule (see below).  Children may have been written by other
// threads of this launch: loads bypass L1.
__device__ __forceinline__ double4_32a load_sums(const double4_32a* p)
{
    const double2 a = __ldcg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2*>(p) + 1);
    return double4_32a{a.x, a.y, b.x, b.y};
}

template <bool kMoments>
__device__ void node_sums(int b, const int32_t* __restrict__ node_cs, const int32_t* __restrict__ node_nchild,
                          const int32_t* __restrict__ slot_ref, const double4_32a* ls, double4_32a* ns,
                          const double* lq, double* nq)
{
    const int s0 = node_cs[b] + 1, s1 = s0 + node_nchild[b];
    double sm = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
    for (int s = s0; s < s1; ++s) {
        const int r = slot_ref[s];
        const double4_32a v = load_sums(r >= 0 ? ls + r : ns + ~r);
        sm = __dadd_rn(sm, v.w);
        sx = __dadd_rn(sx, v.x);
        sy = __dadd_rn(sy, v.y);
        sz = __dadd_rn(sz, v.z);
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
            for (int s = s0; s < s1; ++s) {
                const int r = slot_ref[s];
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

constexpr int64_t kUpsweepMaxBodies = 1000000;

// Bottom-up sums without levels: one thread per leaf climbs towards the
// root; at each node the thread whose arrival completes the node's children
// (an atomic count) computes the node, the others stop.  No thread waits:
// each node is computed exactly once, after all its children.  A thread's
// writes are fenced before its arrival is counted.
template <bool kMoments>
__global__ void upsweep_kernel(const int32_t* __restrict__ counts, const int32_t* __restrict__ leaf_parent,
                               const int32_t* __restrict__ node_parent, const int32_t* __restrict__ node_cs,
                               const int32_t* __restrict__ node_nchild, const int32_t* __restrict__ slot_ref,
                               const double4_32a* ls, double4_32a* ns, const double* lq, double* nq,
                               unsigned* __restrict__ ctr)
{
    const int L = counts[0];
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < L; l += gridDim.x * blockDim.x) {
        int b = leaf_parent[l];
        bool wrote = false;  // the leaf's sums come from an earlier launch
        while (b >= 0) {
            if (wrote) __threadfence();
            const unsigned arrived = atomicAdd(ctr + b, 1u);
            if (arrived + 1u != (unsigned)node_nchild[b]) break;
            __threadfence();
            node_sums<kMoments>(b, node_cs, node_nchild, slot_ref, ls, ns, lq, nq);
            wrote = true;
            b = node_parent[b];
        }
    }
}

// Depth buckets of the branching nodes (depths 0..20), three kernels:
// per-block counts, one scan over (depth, block), per-block placement.
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

__global__ void bucket_scan_kernel(int32_t* __restrict__ blk_cnt, int nblk, int32_t* __restrict__ depth_off)
{
    // Single block: exclusive scan of kDepths*nblk counts, depth-major.
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t carry;
    const int total = kDepths * nblk;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < total; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < total ? blk_cnt[i] : 0;
        int x = v;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            int t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, t, off);
                if (lane >= off) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const int before = (w > 0 ? warp_tot[w - 1] : 0) + carry;
        if (i < total) {
            blk_cnt[i] = before + x - v;
            if (i % nblk == 0) depth_off[i / nblk] = before + x - v;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) depth_off[kDepths] = carry;
}

__global__ void bucket_place_kernel(const int32_t* __restrict__ counts, const uint8_t* __restrict__ node_depth,
                                    const int32_t* __restrict__ blk_off, int nblk, int32_t* __restrict__ depth_nodes)
{
    __shared__ int32_t c[kDepths];
    if (threadIdx.x < kDepths) c[threadIdx.x] = 0;
    __syncthreads();
    const int B = counts[1];
    const int b = blockIdx.x * kBucketThreads + threadIdx.x;
    if (b < B) {
        const int d = node_depth[b];
        const int r = atomicAdd(&c[d], 1);  // order inside a bucket is irrelevant
        depth_nodes[blk_off[d * nblk + blockIdx.x] + r] = b;
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
__device__ inline void far_com(double m, double wx, double wy, double wz, TreeRec& r)
{
    if (m > 0) {
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
                far_com(v.w, v.x, v.y, v.z, o);
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
        rec[s] = o;
        if (kFar) {  // the FP32 walk's records, as fp32_nodes_kernel makes them
            const float hx = narrow_trunc(o.cx), hy = narrow_trunc(o.cy), hz = narrow_trunc(o.cz);
            const float lx = narrow_trunc(o.cx - widen(hx));
            const float ly = narrow_trunc(o.cy - widen(hy));
            const float lz = narrow_trunc(o.cz - widen(hz));
            const bool leaf = o.child < 0;
            far.A[s] = make_float4(hx, hy, hz, narrow_trunc(far.G * o.m));
            far.B[s] = make_float4(lx, ly, lz, __int_as_float(leaf ? o.leaf : o.child));
            far.meta[s] = (uint32_t)o.nchild | ((uint32_t)o.depth << 8) | ((leaf ? 1u : 0u) << 16) |
                          ((o.m == 0.0 ? 1u : 0u) << 17);
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

int launch_build(bh_context* ctx, const double* mass, bool moments, bool far_fused, double G)
{
    ctx->fnodes_fused = false;
    const int64_t n = ctx->n;
    if (n == 0) return BH_OK;
    cudaStream_t st = ctx->stream;
    const int maxb = 8 * bh::num_sms();
    const int g = grid_for(n, kThreads, maxb);

    // 1. leaves
    leaf_head_kernel<<<g, kThreads, 0, st>>>(n, ctx->key, ctx->head);
    BH_LAUNCH_CHECK(ctx);
    int rc = device_exclusive_scan(ctx, ctx->head, ctx->head, n, nullptr, ctx->counts + 0);
    if (rc) return rc;
    leaf_scatter_kernel<<<g, kThreads, 0, st>>>(n, ctx->key, ctx->head, ctx->body_leaf, ctx->leaf_first, ctx->leaf_key);
    BH_LAUNCH_CHECK(ctx);
    if (moments)
        leaf_sum_kernel<true><<<g, kThreads, 0, st>>>(ctx->counts, ctx->leaf_first, ctx->leaf_key, ctx->px, ctx->py,
                                                      ctx->pz, mass, ctx->leaf_s, ctx->cdep, ctx->leaf_q);
    else
        leaf_sum_kernel<false><<<g, kThreads, 0, st>>>(ctx->counts, ctx->leaf_first, ctx->leaf_key, ctx->px, ctx->py,
                                                       ctx->pz, mass, ctx->leaf_s, ctx->cdep, ctx->leaf_q);
    BH_LAUNCH_CHECK(ctx);

    // 2. branching nodes: representative flags -> ids -> ranges/child counts
    rep_flag_kernel<<<g, kThreads, 0, st>>>(ctx->counts, ctx->leaf_key, ctx->cdep, ctx->head, n);
    BH_LAUNCH_CHECK(ctx);
    // rep_node[j] = exclusive count of representatives before j, i.e. the
    // node id of boundary j when it is a representative.
    rc = device_exclusive_scan(ctx, ctx->head, ctx->rep_node, n, nullptr, ctx->counts + 1);
    if (rc) return rc;
    node_init_kernel<<<g, kThreads, 0, st>>>(ctx->counts, ctx->leaf_key, ctx->cdep, ctx->head, ctx->rep_node,
                                             ctx->node_rep, ctx->node_a, ctx->node_depth, ctx->node_nchild);
    BH_LAUNCH_CHECK(ctx);
    rc = device_exclusive_scan(ctx, ctx->node_nchild, ctx->node_cs, n, ctx->counts + 1, ctx->counts + 3);
    if (rc) return rc;
    slot_count_kernel<<<1, 1, 0, st>>>(ctx->counts, ctx->counts + 3);
    BH_LAUNCH_CHECK(ctx);
    node_children_kernel<<<g, kThreads, 0, st>>>(ctx->counts, ctx->leaf_key, ctx->rep_node, ctx->node_rep,
                                                 ctx->node_a, ctx->node_depth, ctx->node_cs, ctx->slot_ref,
                                                 ctx->slot_top, ctx->leaf_parent, ctx->node_parent);
    BH_LAUNCH_CHECK(ctx);

    // 3./4. monopoles (and second moments), deepest first.  Below a
    // million bodies one launch climbs from the leaves (launch overheads
    // dominate there); above, the level-synchronous pass keeps more loads in
    // flight.  Both sum each node's children in slot order from 0.0.
    if (n < kUpsweepMaxBodies) {
        BH_CUDA_TRY(cudaMemsetAsync(ctx->node_ctr, 0, sizeof(unsigned) * (size_t)n, st));
        if (moments)
            upsweep_kernel<true><<<g, kThreads, 0, st>>>(ctx->counts, ctx->leaf_parent, ctx->node_parent,
                                                         ctx->node_cs, ctx->node_nchild, ctx->slot_ref,
                                                         ctx->leaf_s, ctx->node_s, ctx->leaf_q, ctx->node_q,
                                                         ctx->node_ctr);
        else
            upsweep_kernel<false><<<g, kThreads, 0, st>>>(ctx->counts, ctx->leaf_parent, ctx->node_parent,
                                                          ctx->node_cs, ctx->node_nchild, ctx->slot_ref,
                                                          ctx->leaf_s, ctx->node_s, ctx->leaf_q, ctx->node_q,
                                                          ctx->node_ctr);
        BH_LAUNCH_CHECK(ctx);
    } else {
        const int nblk = (int)((n + kBucketThreads - 1) / kBucketThreads);
        bucket_count_kernel<<<nblk, kBucketThreads, 0, st>>>(ctx->counts, ctx->node_depth, ctx->scan_tmp, nblk);
        BH_LAUNCH_CHECK(ctx);
        bucket_scan_kernel<<<1, 1024, 0, st>>>(ctx->scan_tmp, nblk, ctx->depth_off);
        BH_LAUNCH_CHECK(ctx);
        bucket_place_kernel<<<nblk, kBucketThreads, 0, st>>>(ctx->counts, ctx->node_depth, ctx->scan_tmp, nblk,
                                                             ctx->depth_nodes);
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
    return BH_OK;
}

}  // namespace bh
