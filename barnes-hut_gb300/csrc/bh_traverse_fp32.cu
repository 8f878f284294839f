// The masked warp walk behind BH_MODE_FP64_LIST and BH_MODE_FP32_FAR, and
// the collection of training pairs for the learned criterion (the learned
// walk itself, BH_MODE_LEARNED, is bh_traverse_learned.cu).  No reference
// counterpart: the reference walks one body at a
// time (src/traversal.cpp:53-102).
//
// A warp owns 32 Morton-consecutive bodies.  Stack entries are sibling
// ranges (first child slot, number of children, mask of the lanes that still
// need them): an opened node pushes one entry.  Each iteration pops whole
// ranges from the top, up to 32 nodes, and classifies them one per lane
// against the group's bounding box (group-relative FP32 coordinates):
//   accept-all : side^2 < theta^2 dmin^2 (every body is at least dmin away),
//   open-all   : side^2 > theta^2 dmax^2 (no body is farther than dmax),
//   mixed      : each lane of the mask applies its own body's test.
// (both group tests allow for the FP32 rounding of the coordinates with an
// absolute bound and a relative margin, so every body's own FP64 test agrees
// with them).  Lanes that accept a node take it into a staged
// interaction list with their mask bit; the others carry it down to the
// children.  Each body therefore interacts with exactly the nodes its own
// walk at theta accepts.
//
// BH_MODE_FP64_LIST: per-lane tests in FP64 with the reference's rounding,
//   interactions in FP64 (rcube_hh + FMA) from the FP64 node records, on the
//   reference's tree.
// BH_MODE_FP32_FAR: precision form.  The bodies with id < num_direct (Sun and
//   planets) are taken out of the tree (masses zeroed before the build) and
//   summed directly in FP64.  Far-field interactions run in FP32 on
//   displacements relative to the warp's group centre g: node centres are
//   stored as float pairs hi + lo (formed in FP64 once per node), g is a
//   float, so (hi - g) + lo is the FP64 displacement rounded to FP32 without
//   one FP64 instruction per visit (the FP64 pipe is 1/60 of the FP32 one
//   here, and three FP64 subtractions per visit would cost more than the
//   interaction).  FP32 partials of each staged list are added into FP64
//   accumulators.
// Collection (bh_learned_collect): the FP32 walk with the theta test only,
//   recording every candidate's group, slot, lane mask and raw features.
#include <climits>

#include "bh_walk.cuh"

namespace bh {
namespace {

// FP32 node records from the FP64 ones.
// d4 (FP64 walk only): {cx, cy, cz, G m} per slot, the FP64 evaluation's
// 32-byte record.
__global__ void fp32_nodes_kernel(const int32_t* __restrict__ counts, const TreeRec* __restrict__ rec, double G,
                                  float4* __restrict__ A, float4* __restrict__ B, uint32_t* __restrict__ meta,
                                  double4_32a* __restrict__ d4)
{
    const int S = counts[2];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const TreeRec r = rec[s];
        if (d4) d4[s] = double4_32a{r.cx, r.cy, r.cz, G * r.m};
        // hi + lo splits by truncation on the bit patterns: c - hi is exact,
        // and hi + lo represents c to about 2^-46 relative.
        const bool leaf = r.child < 0;
        A[s] = make_float4(narrow_trunc(r.cx), narrow_trunc(r.cy), narrow_trunc(r.cz), narrow_trunc(G * r.m));
        B[s] = make_float4(low_part(r.cx), low_part(r.cy), low_part(r.cz), __int_as_float(leaf ? r.leaf : r.child));
        meta[s] = (uint32_t)r.nchild | ((uint32_t)r.depth << 8) | ((leaf ? 1u : 0u) << 16) |
                  ((__double_as_longlong(r.m) << 1) == 0 ? 1u << 17 : 0u);
    }
}

// Positions and G m of the direct bodies, indexed by id.
__global__ void direct_extract_kernel(int64_t n, const double* __restrict__ px, const double* __restrict__ py,
                                      const double* __restrict__ pz, const double* __restrict__ m,
                                      const uint64_t* __restrict__ id, int nd, double G, double* __restrict__ direct,
                                      int32_t* __restrict__ present)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = id[i];
        if (k < (uint64_t)nd) {
            direct[4 * k] = px[i];
            direct[4 * k + 1] = py[i];
            direct[4 * k + 2] = pz[i];
            direct[4 * k + 3] = G * m[i];
            present[k] = 1;
        }
    }
}

}  // namespace

namespace {

template <bool kFP64, int kLearn, bool kGroup = false>
__global__ void __launch_bounds__(kThreads) traverse_masked_kernel(FParams p)
{
    static_assert(kLearn != kLearnInfer, "the learned walk is traverse_learned_kernel");
    static_assert(!kGroup || (!kFP64 && kLearn == kLearnNone), "the group test is an FP32 far-field walk");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WalkSmem<kFP64, kLearn, kGroup>& sm = *reinterpret_cast<WalkSmem<kFP64, kLearn, kGroup>*>(smem_raw);
    if (threadIdx.x <= kMaxDepth) {
        const double dx = __dsub_rn(p.bbox[3], p.bbox[0]);
        const double dy = __dsub_rn(p.bbox[4], p.bbox[1]);
        const double dz = __dsub_rn(p.bbox[5], p.bbox[2]);
        double L = dx;
        if (L < dy) L = dy;
        if (L < dz) L = dz;
        const double side = __ddiv_rn(L, (double)(1ull << threadIdx.x));
        sm.side2d[threadIdx.x] = __dmul_rn(side, side);
        const float s2f = (float)sm.side2d[threadIdx.x];
        sm.side2f[threadIdx.x] = s2f;
        if (!kFP64) {
            // The FP32 walk's group-test distances: a node of this depth is
            // accepted by every body when dmin > S+ + err and opened by
            // every body when dmax < S- - err, S+- = side sqrt((1 +-
            // margin) / theta^2) (theta = 0: infinite, so that nothing is
            // accepted and all is opened).
            const float th2f = (float)p.theta2;
            sm.sthr[threadIdx.x] =
                make_float2(sqrtf(s2f * (1.0f + kMargin) / th2f), sqrtf(s2f * (1.0f - kMargin) / th2f));
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t group = (int64_t)blockIdx.x * kWarps + w;
    const int64_t base = group * 32;
    if (base >= p.n) return;
    const int64_t i = base + lane;
    const bool valid = i < p.n;
    const int64_t ii = valid ? i : base;  // idle lanes shadow the group's first body
    const double x = p.px[ii], y = p.py[ii], z = p.pz[ii];
    // The group centre g: the first body's position truncated to FP32 on the
    // bit patterns (any float near the group serves).
    const float gx = narrow_trunc(__shfl_sync(0xffffffffu, x, 0));
    const float gy = narrow_trunc(__shfl_sync(0xffffffffu, y, 0));
    const float gz = narrow_trunc(__shfl_sync(0xffffffffu, z, 0));
    const float rx = __double2float_rn(x - widen(gx));
    const float ry = __double2float_rn(y - widen(gy));
    const float rz = __double2float_rn(z - widen(gz));
    float bminx = rx, bminy = ry, bminz = rz, bmaxx = rx, bmaxy = ry, bmaxz = rz;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        bminx = fminf(bminx, __shfl_xor_sync(0xffffffffu, bminx, off));
        bminy = fminf(bminy, __shfl_xor_sync(0xffffffffu, bminy, off));
        bminz = fminf(bminz, __shfl_xor_sync(0xffffffffu, bminz, off));
        bmaxx = fmaxf(bmaxx, __shfl_xor_sync(0xffffffffu, bmaxx, off));
        bmaxy = fmaxf(bmaxy, __shfl_xor_sync(0xffffffffu, bmaxy, off));
        bmaxz = fmaxf(bmaxz, __shfl_xor_sync(0xffffffffu, bmaxz, off));
    }
    const unsigned full = __ballot_sync(0xffffffffu, valid);
    const int my_leaf = valid ? p.body_leaf[i] : -2;
    // The group's leaf ids span [leaf_lo, leaf_hi] (bodies in key order).
    int leaf_lo = valid ? my_leaf : INT_MAX, leaf_hi = valid ? my_leaf : INT_MIN;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        leaf_lo = min(leaf_lo, __shfl_xor_sync(0xffffffffu, leaf_lo, off));
        leaf_hi = max(leaf_hi, __shfl_xor_sync(0xffffffffu, leaf_hi, off));
    }
    const float theta2f = (float)p.theta2;
    const double theta2 = p.theta2, soft2 = p.soft2;
    const bool nosoft = (__double_as_longlong(soft2) << 1) == 0;  // soft2 is +-0
    if (kFP64) {
        sm.bpos[w][0][lane] = x;
        sm.bpos[w][1][lane] = y;
        sm.bpos[w][2][lane] = z;
        sm.bleaf[w][lane] = my_leaf;
        __syncwarp();
    }
    int2* stk = sm.stack[w];
    float4* L = kFP64 ? nullptr : sm.lst[w];
    int* LN = sm.lst_node[w];
    int* LL = WalkSmem<kFP64, kLearn, kGroup>::kLL ? sm.lst_leaf[w] : nullptr;
    unsigned* LM = sm.lst_mask[w];
    const unsigned me = 1u << lane;
    const unsigned lt = me - 1u;

    double adx = 0.0, ady = 0.0, adz = 0.0;
    unsigned cnt = 0;
    // The group form's own-leaf terms (evaluated where the leaf is met).
    float ox = 0.0f, oy = 0.0f, oz = 0.0f;

    // FP64 direct terms from the direct bodies first (FP32 modes): they set
    // the group's acceleration scale for the learned criterion.
    float ascale = 0.0f;
    if (!kFP64) {
        const uint64_t my_id = valid ? p.id[i] : ~0ull;
        for (int kk = 0; kk < p.nd; ++kk) {
            if (!p.present[kk] || my_id == (uint64_t)kk) continue;
            const double dx = p.direct[4 * kk] - x, dy = p.direct[4 * kk + 1] - y, dz = p.direct[4 * kk + 2] - z;
            const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, soft2)));
            // A body at the very position of a direct body shares its leaf,
            // which the reference skips (traversal.cpp:70): no term.
            if (__double_as_longlong(r2) == 0) continue;
            const double sc = p.direct[4 * kk + 3] * rcube_hh(r2);
            adx = fma(sc, dx, adx);
            ady = fma(sc, dy, ady);
            adz = fma(sc, dz, adz);
            ++cnt;
        }
        if (kLearn) {
            float a = valid ? (float)sqrt(adx * adx + ady * ady + adz * adz) : 3.0e38f;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) a = fminf(a, __shfl_xor_sync(0xffffffffu, a, off));
            ascale = a < 3.0e38f ? a : 0.0f;
        }
    }
    const float bmag = fmaxf(fmaxf(fmaxf(fabsf(bminx), fabsf(bmaxx)), fmaxf(fabsf(bminy), fabsf(bmaxy))),
                             fmaxf(fabsf(bminz), fabsf(bmaxz)));
    const float gextent = sqrtf((bmaxx - bminx) * (bmaxx - bminx) + (bmaxy - bminy) * (bmaxy - bminy) +
                                (bmaxz - bminz) * (bmaxz - bminz));
    const float bcx = 0.5f * (bminx + bmaxx), bcy = 0.5f * (bminy + bmaxy), bcz = 0.5f * (bminz + bmaxz);
    // Per-walk logarithms of the learned features (base 2).
    const float lext = kLearn ? __log2f(fmaxf(gextent, 1e-30f)) : 0.0f;
    const float lascale = kLearn ? __log2f(ascale) : 0.0f;

    int nlist = 0;
    int sp = 1;
    if (lane == 0) stk[0] = make_int2(0, (int)full);  // the root: a range of one slot
    __syncwarp();
    bool overflow = false;
    int64_t pops = 0;

    while (sp > 0 || nlist > 0) {
        if (sp > 0) {
            // Pop whole ranges from the top while they fit in 32 lanes.
            const int avail = sp < 32 ? sp : 32;
            int rfirst = 0, rcnt = 0;
            unsigned rmask = 0;
            if (lane < avail) {
                const int2 ent = stk[sp - 1 - lane];
                rfirst = ent.x & ((1 << kSlotBits) - 1);
                rcnt = (int)((unsigned)ent.x >> kSlotBits) + 1;
                rmask = (unsigned)ent.y;
            }
            int incl = rcnt;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += t;
            }
            const bool take = lane < avail && incl <= 32;
            const int R = __popc(__ballot_sync(0xffffffffu, take));
            const int T = __shfl_sync(0xffffffffu, incl, R - 1);
            const int rstart = incl - rcnt;
            const unsigned starts = __reduce_or_sync(0xffffffffu, take ? (1u << rstart) : 0u);
            const int rj = __popc(starts & ((2u << lane) - 1u)) - 1;
            const int f_r = __shfl_sync(0xffffffffu, rfirst, rj);
            const int s_r = __shfl_sync(0xffffffffu, rstart, rj);
            const unsigned m_r = __shfl_sync(0xffffffffu, rmask, rj);
            pops += T;
            if (sp - R + T > WalkSmem<kFP64, kLearn, kGroup>::kStk || pops > p.max_pops) {
                overflow = true;
                break;
            }
            const int k = T;
            int node = -1;
            unsigned M = 0, A = 0;
            int nc = 0, ref = 0, depth = 0;
            bool leaf = false, mixed = false, cand = false;
            float dmin2 = 0.f, dmax2 = 0.f, s2 = 0.f, nerr = 0.f;
            float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lane < k) {
                node = f_r + (lane - s_r);
                M = m_r;
                const float4 a = __ldg(p.A + node);
                const float4 b = __ldg(p.B + node);
                const uint32_t mt = __ldg(p.meta + node);
                const float cx = (a.x - gx) + b.x, cy = (a.y - gy) + b.y, cz = (a.z - gz) + b.z;
                e = make_float4(cx, cy, cz, a.w);
                ref = __float_as_int(b.w);
                leaf = (mt >> 16) & 1u;
                depth = (mt >> 8) & 0xFF;
                if ((mt >> 17) & 1u) {
                    M = 0;  // massless: skipped with its subtree (traversal.cpp:66)
                } else if (leaf) {
                    A = M;  // leaves are always accepted; the own leaf is handled at evaluation
                } else {
                    const float ex = fmaxf(0.0f, fmaxf(bminx - cx, cx - bmaxx));
                    const float ey = fmaxf(0.0f, fmaxf(bminy - cy, cy - bmaxy));
                    const float ez = fmaxf(0.0f, fmaxf(bminz - cz, cz - bmaxz));
                    const float fx = fmaxf(fabsf(cx - bminx), fabsf(cx - bmaxx));
                    const float fy = fmaxf(fabsf(cy - bminy), fabsf(cy - bmaxy));
                    const float fz = fmaxf(fabsf(cz - bminz), fabsf(cz - bmaxz));
                    dmin2 = ex * ex + ey * ey + ez * ez;
                    dmax2 = fx * fx + fy * fy + fz * fz;
                    nc = (int)(mt & 0xFF);
                    // Absolute error of the FP32 group-relative distances.
                    const float err = kAbsErr * (fmaxf(fabsf(cx), fmaxf(fabsf(cy), fabsf(cz))) + bmag);
                    nerr = err;
                    if (kFP64) {
                        s2 = sm.side2f[depth];
                        const float dlo = fmaxf(sqrtf(dmin2) - err, 0.0f), dhi = sqrtf(dmax2) + err;
                        if (s2 * (1.0f + kMargin) < theta2f * dlo * dlo) A = M;
                        else if (s2 * (1.0f - kMargin) > theta2f * dhi * dhi) A = 0;
                        else mixed = true;
                    } else {
                        // The same tests squared on the distance side:
                        // side^2 (1 + margin) < theta^2 (dmin - err)^2 and
                        // side^2 (1 - margin) > theta^2 (dmax + err)^2, with
                        // no square roots.
                        if (kLearn) s2 = sm.side2f[depth];
                        const float2 st = sm.sthr[depth];
                        const float ta = st.x + err, to = st.y - err;
                        if (ta * ta < dmin2) {
                            A = M;
                        } else {
                            if (kLearn) cand = M != 0 && dmin2 > 0.0f && s2 < p.theta_max2 * dmin2;
                            if (to > 0.0f && to * to > dmax2) A = 0;
                            else mixed = true;
                        }
                    }
                }
            }
            __syncwarp();
            sp -= R;
            if (kLearn && !kFP64) {
                const unsigned cb = __ballot_sync(0xffffffffu, cand);
                if (cb) {
                    float f[kFeat];
#pragma unroll
                    for (int q = 0; q < kFeat; ++q) f[q] = 0.0f;
                    if (cand) {
                        // log10 of ratios as differences of base-2 logarithms
                        // of the (squared) lengths: hardware log2 estimates,
                        // no divisions and no square roots.  Training pairs
                        // are collected by this same code, so the network
                        // sees the same feature arithmetic it was trained on.
                        constexpr float kL = 0.30102999566f;  // log10(2)
                        const float l2dmin = __log2f(dmin2), l2s = __log2f(s2);
                        const float lspr = __log2f(fmaxf(__ldg(p.spread + node), 1e-8f * sqrtf(s2)));
                        const float dcx = e.x - bcx, dcy = e.y - bcy, dcz = e.z - bcz;
                        const float ldmin = 0.5f * l2dmin;
                        f[0] = kL * (0.5f * l2s - ldmin);
                        f[1] = kL * (lspr - ldmin);
                        f[2] = kL * (lext - ldmin);
                        f[3] = kL * (__log2f(e.w) - l2dmin - lascale);
                        f[4] = kL * 0.5f * (__log2f(dmax2) - l2dmin);
                        f[5] = (float)depth * (1.0f / kMaxDepth);
                        f[6] = kL * (lspr - 0.5f * l2s);
                        f[7] = kL * (0.5f * __log2f(fmaxf(dcx * dcx + dcy * dcy + dcz * dcz, 1e-36f)) - ldmin);
                    }
                    if (kLearn == kLearnCollect) {
                        const int leader = __ffs(cb) - 1;
                        unsigned long long basec = 0;
                        if (lane == leader) basec = atomicAdd(p.c_count, (unsigned long long)__popc(cb));
                        basec = __shfl_sync(0xffffffffu, basec, leader);
                        const unsigned long long slot = basec + __popc(cb & lt);
                        if (cand && (int64_t)slot < p.c_cap) {
                            p.c_group[slot] = (int32_t)group;
                            p.c_slot[slot] = node;
                            p.c_mask[slot] = M;
                            p.c_ascale[slot] = ascale;
#pragma unroll
                            for (int q = 0; q < kFeat; ++q) p.c_feat[slot * kFeat + q] = f[q];
                        }
                    }
                }
            }
            // Mixed nodes: every lane of the mask applies its own test.
            unsigned mb = __ballot_sync(0xffffffffu, mixed);
            if (kFP64) {
                while (mb) {
                    const int j = __ffs(mb) - 1;
                    mb &= mb - 1;
                    const unsigned Mj = __shfl_sync(0xffffffffu, M, j);
                    const int dj = __shfl_sync(0xffffffffu, depth, j);
                    bool acc = false;
                    // Each lane's FP64 test (the reference's rounding) decides
                    // only where the FP32 distance, with the same error
                    // allowance as the group tests, cannot.
                    const int nj = __shfl_sync(0xffffffffu, node, j);
                    const float cx = __shfl_sync(0xffffffffu, e.x, j);
                    const float cy = __shfl_sync(0xffffffffu, e.y, j);
                    const float cz = __shfl_sync(0xffffffffu, e.z, j);
                    const float ej = 2.0f * __shfl_sync(0xffffffffu, nerr, j);
                    const float dxf = cx - rx, dyf = cy - ry, dzf = cz - rz;
                    const float df = sqrtf(dxf * dxf + dyf * dyf + dzf * dzf);
                    const float lo = fmaxf(df - ej, 0.0f), hi = df + ej;
                    const float s2j = sm.side2f[dj], sf = (float)soft2;
                    const bool sure_acc = s2j * (1.0f + kMargin) < theta2f * (lo * lo + sf);
                    const bool sure_rej = s2j * (1.0f - kMargin) > theta2f * (hi * hi + sf * (1.0f + kMargin));
                    acc = sure_acc;
                    if (((Mj >> lane) & 1u) && !sure_acc && !sure_rej) {
                        const TreeRec r = p.rec[nj];
                        const double dx = __dsub_rn(r.cx, x), dy = __dsub_rn(r.cy, y), dz = __dsub_rn(r.cz, z);
                        const double r2 = __dadd_rn(
                            __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), soft2);
                        acc = sm.side2d[dj] < __dmul_rn(theta2, r2);
                    }
                    const unsigned Aj = __ballot_sync(0xffffffffu, acc) & Mj;
                    if (lane == j) A = Aj;
                }
            } else if (mb) {
                // The mixed nodes {c, side^2} go to free entry slots past the
                // staged list (from the first even position, which leaves the
                // last entry pair whole; the list holds at most its capacity
                // less 32 entries here), and every lane tests its body
                // against each of them, read by broadcast.  Lane q keeps the
                // lanes that accept slot q.
                unsigned res = 0;
                float4* X = L + ((nlist + 1) & ~1);
                const int nm = __popc(mb);
                const int slot = __popc(mb & lt);
                if (kGroup) {
                    // Slots in the list's entry-pair layout, tested two at a
                    // time in packed FP32 pairs (an odd count leaves a stale
                    // second half, whose result no lane reads).  The per-body
                    // form keeps one slot at a time: the pairs' registers
                    // would cost it a resident block per SM.
                    if (mixed) {
                        float* P = reinterpret_cast<float*>(X + (slot & ~1)) + (slot & 1);
                        P[0] = e.x;
                        P[2] = e.y;
                        P[4] = e.z;
                        P[6] = sm.side2f[depth];
                    }
                    __syncwarp();
                    const f32x2 qx = pk(rx, rx), qy = pk(ry, ry), qz = pk(rz, rz), qt = pk(theta2f, theta2f);
                    for (int q = 0; q < nm; q += 2) {
                        const ulonglong2 xy = *reinterpret_cast<const ulonglong2*>(X + q);
                        const ulonglong2 zs = *reinterpret_cast<const ulonglong2*>(X + q + 1);
                        const f32x2 dx = sub2(xy.x, qx), dy = sub2(xy.y, qy), dz = sub2(zs.x, qz);
                        float t0, t1, s0, s1;
                        upk(mul2(qt, fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)))), t0, t1);
                        upk(zs.y, s0, s1);
                        const unsigned b0 = __ballot_sync(0xffffffffu, s0 < t0);
                        const unsigned b1 = __ballot_sync(0xffffffffu, s1 < t1);
                        if (lane == q) res = b0;
                        if (lane == q + 1) res = b1;
                    }
                } else {
                    if (mixed) X[slot] = make_float4(e.x, e.y, e.z, sm.side2f[depth]);
                    __syncwarp();
#pragma unroll 2
                    for (int q = 0; q < nm; ++q) {
                        const float4 v = X[q];
                        const float dx = v.x - rx, dy = v.y - ry, dz = v.z - rz;
                        const unsigned bq = __ballot_sync(0xffffffffu, v.w < theta2f * (dx * dx + dy * dy + dz * dz));
                        if (lane == q) res = bq;
                    }
                }
                const unsigned acc = __shfl_sync(0xffffffffu, res, slot & 31);
                // The group form accepts a mixed node only when every body
                // of the mask does, and otherwise opens it for all of them.
                if (mixed) A = kGroup ? ((acc & M) == M ? M : 0u) : acc & M;
                __syncwarp();
            }
            if (!kFP64 && kLearn == kLearnNone) {
                // A body never interacts with its own leaf (traversal.cpp:70,
                // the FP32 form has no chain rule for it): its lanes leave
                // the leaf's mask here, so the evaluation needs no leaf test.
                const bool own_cand = A != 0 && leaf && ref >= leaf_lo && ref <= leaf_hi;
                unsigned oc = __ballot_sync(0xffffffffu, own_cand);
                while (oc) {
                    const int j = __ffs(oc) - 1;
                    oc &= oc - 1u;
                    const int lj = __shfl_sync(0xffffffffu, ref, j);
                    const unsigned own = __ballot_sync(0xffffffffu, my_leaf == lj);
                    if (lane == j) A &= ~own;
                    if (kGroup) {
                        // The group form stages only entries that all its
                        // lanes take: an own leaf is evaluated here, for the
                        // lanes of its mask that do not belong to it.
                        const unsigned Aj = __shfl_sync(0xffffffffu, A, j);
                        const float cx = __shfl_sync(0xffffffffu, e.x, j);
                        const float cy = __shfl_sync(0xffffffffu, e.y, j);
                        const float cz = __shfl_sync(0xffffffffu, e.z, j);
                        const float gm = __shfl_sync(0xffffffffu, e.w, j);
                        if (Aj & me) {
                            const float dx = cx - rx, dy = cy - ry, dz = cz - rz;
                            const float inv = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, (float)soft2))));
                            const float sc = gm * (inv * inv * inv);
                            ox = fmaf(sc, dx, ox);
                            oy = fmaf(sc, dy, oy);
                            oz = fmaf(sc, dz, oz);
                            ++cnt;
                        }
                    }
                }
                if (kGroup && own_cand) A = 0;  // evaluated above, not staged
            }
            // Stage the accepted (node, lanes) entries.
            const bool stage = A != 0;
            const unsigned am = __ballot_sync(0xffffffffu, stage);
            if (stage) {
                const int pos = nlist + __popc(am & lt);
                if (!kFP64) {  // entry pairs {x0, x1, y0, y1}, {z0, z1, w0, w1}
                    float* P = reinterpret_cast<float*>(L + (pos & ~1)) + (pos & 1);
                    P[0] = e.x;
                    P[2] = e.y;
                    P[4] = e.z;
                    P[6] = e.w;
                }
                if (kFP64) LN[pos] = node;
                if (WalkSmem<kFP64, kLearn, kGroup>::kLL) LL[pos] = leaf ? ref : -1;  // for the own-leaf test
                LM[pos] = A;
            }
            nlist += __popc(am);
            // Push one sibling range per opened node, with the lanes that
            // still need it.
            const unsigned rest = M & ~A;
            const bool push = !leaf && nc > 0 && rest != 0;
            const unsigned pm = __ballot_sync(0xffffffffu, push);
            if (push) stk[sp + __popc(pm & lt)] = make_int2(ref | ((nc - 1) << kSlotBits), (int)rest);
            sp += __popc(pm);
            __syncwarp();
        }
        if (nlist > WalkSmem<kFP64, kLearn, kGroup>::kLst - 32 || (sp == 0 && nlist > 0)) {
            if (kLearn == kLearnCollect) {
                nlist = 0;  // collection evaluates nothing
                __syncwarp();
                continue;
            }
            if (kFP64) {
                // The (entry, body) pairs of the staged list, grouped by body,
                // are split evenly over the 32 threads: the FP64 pipe then
                // evaluates only pairs that count, however unevenly the
                // bodies' shares of the list are spread.  A thread sums its
                // consecutive pairs in registers while they belong to one
                // body, and stores each run's partial (a plain store: no
                // atomics and no FP64 work in divergent code) in slot
                // body + thread.  Along the pairs both indices only grow and
                // every new run increments at least one, so the slot of a run
                // is its own.  Each body's lane then adds the partials of its
                // runs, one per thread its pairs reach, in thread order.
                uint8_t (*PL)[32] = sm.plist[w];
                int* OFF = sm.poff[w];
                auto SG = sm.seg[w];  // [3][kSegs] in the FP64 walk
                uint16_t* SN = sm.segn[w];
                int mine = 0;
                for (int j = 0; j < nlist; ++j)
                    if (LM[j] & me) PL[mine++][lane] = (uint8_t)j;
                int incl = mine;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, off);
                    if (lane >= off) incl += t;
                }
                OFF[lane] = incl - mine;
                if (lane == 31) OFF[32] = incl;
                __syncwarp();
                const int P = OFF[32];
                const int per = (P + 31) >> 5;
                const int k0 = min(lane * per, P), k1 = min(k0 + per, P);
                int b = 0;  // the body of pair k0: the last lane whose first pair is <= k0
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (b + step < 32 && OFF[b + step] <= k0) b += step;
                double sx = 0.0, sy = 0.0, sz = 0.0;
                unsigned sn = 0;
                for (int t = 0; t < per; ++t) {
                    const int k = k0 + t;
                    const bool on = k < k1;
                    if (on) {
                        while (k >= OFF[b + 1]) {  // body b's run ends here
                            SG[0][b + lane] = sx;
                            SG[1][b + lane] = sy;
                            SG[2][b + lane] = sz;
                            SN[b + lane] = (uint16_t)sn;
                            sx = sy = sz = 0.0;
                            sn = 0;
                            ++b;
                        }
                    }
                    const int j = on ? PL[k - OFF[b]][b] : 0;
                    const double4_32a r = p.d4[LN[j]];
                    const double dx = r.x - sm.bpos[w][0][b], dy = r.y - sm.bpos[w][1][b],
                                 dz = r.z - sm.bpos[w][2][b];
                    bool take = on;
                    if (on && LL[j] == sm.bleaf[w][b]) {
                        // Own leaf: skipped at depth 21 unless a chain cell above
                        // it (depths top..20) accepts (traversal.cpp:70,78).  At
                        // zero displacement and no softening r^2 is 0 and no
                        // cell accepts (decided on the bit patterns).
                        if (nosoft && ((__double_as_longlong(dx) | __double_as_longlong(dy) |
                                        __double_as_longlong(dz)) << 1) == 0) {
                            take = false;
                        } else {
                            const double r2e = __dadd_rn(
                                __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), soft2);
                            take = p.rec[LN[j]].top <= kMaxDepth - 1 &&
                                   sm.side2d[kMaxDepth - 1] < __dmul_rn(theta2, r2e);
                        }
                    }
                    const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, soft2)));
                    // A pair not taken (an own leaf at r2 = 0, or a lane past
                    // its share) gets an argument on the fast path, so that no
                    // lane diverges into the out-of-range branch for it.
                    double sc = r.w * rcube_hh(take ? r2 : 1.0);
                    if (!take) sc = 0.0;
                    sx = fma(sc, dx, sx);
                    sy = fma(sc, dy, sy);
                    sz = fma(sc, dz, sz);
                    sn += take ? 1u : 0u;
                }
                if (k0 < k1) {
                    SG[0][b + lane] = sx;
                    SG[1][b + lane] = sy;
                    SG[2][b + lane] = sz;
                    SN[b + lane] = (uint16_t)sn;
                }
                __syncwarp();
                const int f0 = OFF[lane], f1 = OFF[lane + 1];  // this lane's body: its pairs
                if (f1 > f0) {
                    const int l1 = (f1 - 1) / per;
                    for (int l = f0 / per; l <= l1; ++l) {
                        adx += SG[0][lane + l];
                        ady += SG[1][lane + l];
                        adz += SG[2][lane + l];
                        cnt += SN[lane + l];
                    }
                }
                __syncwarp();
            } else {
                // Two entries per iteration in packed pairs (even, odd); an
                // odd count is padded with a zero entry taken by no lane.
                // Each half rounds as the scalar form; the two halves are
                // separate partial sums, added at the end.
                if (nlist & 1) {
                    if (lane == 0) {
                        // The pad entry: massless, and far enough away
                        // (r^2 = 3e36) that its r^-3 is 0 in FP32.
                        float* P = reinterpret_cast<float*>(L + (nlist - 1)) + 1;
                        P[0] = P[2] = P[4] = kGroup ? 1e18f : 0.0f;
                        P[6] = 0.0f;
                        LM[nlist] = 0u;
                    }
                    __syncwarp();
                }
                const f32x2 rx2 = pk(rx, rx), ry2 = pk(ry, ry), rz2 = pk(rz, rz);
                const f32x2 sf2 = pk((float)soft2, (float)soft2);
                f32x2 fx = 0ull, fy = 0ull, fz = 0ull;  // +0.0f pairs
                if (kGroup) {
                    // Every staged entry is taken by every lane: no masks.
                    for (int j = 0; j < nlist; j += 2) {
                        const ulonglong2 xy = *reinterpret_cast<const ulonglong2*>(L + j);
                        const ulonglong2 zw = *reinterpret_cast<const ulonglong2*>(L + j + 1);
                        const f32x2 dx = sub2(xy.x, rx2), dy = sub2(xy.y, ry2), dz = sub2(zw.x, rz2);
                        const f32x2 r2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, sf2)));
                        float r0, r1;
                        upk(r2, r0, r1);
                        const f32x2 inv = pk(rsqrtf(r0), rsqrtf(r1));
                        const f32x2 sc = mul2(zw.y, mul2(mul2(inv, inv), inv));
                        fx = fma2(sc, dx, fx);
                        fy = fma2(sc, dy, fy);
                        fz = fma2(sc, dz, fz);
                    }
                    cnt += (unsigned)nlist;
                } else
                for (int j = 0; j < nlist; j += 2) {
                    const ulonglong2 xy = *reinterpret_cast<const ulonglong2*>(L + j);
                    const ulonglong2 zw = *reinterpret_cast<const ulonglong2*>(L + j + 1);
                    const uint2 mj = *reinterpret_cast<const uint2*>(LM + j);
                    const f32x2 dx = sub2(xy.x, rx2), dy = sub2(xy.y, ry2), dz = sub2(zw.x, rz2);
                    const f32x2 r2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, sf2)));
                    float r0, r1;
                    upk(r2, r0, r1);
                    const f32x2 inv = pk(rsqrtf(r0), rsqrtf(r1));
                    float s0, s1;
                    upk(mul2(zw.y, mul2(mul2(inv, inv), inv)), s0, s1);
                    const bool t0 = (mj.x & me) != 0u, t1 = (mj.y & me) != 0u;
                    const f32x2 sc = pk(t0 ? s0 : 0.0f, t1 ? s1 : 0.0f);
                    fx = fma2(sc, dx, fx);
                    fy = fma2(sc, dy, fy);
                    fz = fma2(sc, dz, fz);
                    cnt += (t0 ? 1u : 0u) + (t1 ? 1u : 0u);
                }
                float fx0, fx1, fy0, fy1, fz0, fz1;
                upk(fx, fx0, fx1);
                upk(fy, fy0, fy1);
                upk(fz, fz0, fz1);
                // widen(): the exact conversion on the bit patterns (the
                // conversion instruction runs on the FP64 pipe, which the
                // direct terms already load)
                adx += widen(fx0 + fx1);
                ady += widen(fy0 + fy1);
                adz += widen(fz0 + fz1);
            }
            nlist = 0;
            __syncwarp();
        }
    }
    if (overflow && lane == 0) atomicOr(p.err, kErrOverflow);
    if (kLearn == kLearnCollect) return;
    if (kGroup) {
        adx += widen(ox);
        ady += widen(oy);
        adz += widen(oz);
    }

    if (valid) {
        p.ax[i] = adx;
        p.ay[i] = ady;
        p.az[i] = adz;
        if (p.body_count) p.body_count[i] = (int32_t)cnt;
        if (p.kick_h > 0.0) {
            p.vx[i] = p.vx[i] + p.kick_h * adx;
            p.vy[i] = p.vy[i] + p.kick_h * ady;
            p.vz[i] = p.vz[i] + p.kick_h * adz;
        }
    }
    if (p.inter_count) {
        unsigned long long c = valid ? cnt : 0ull;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
        if (lane == 0) atomicAdd(p.inter_count, c);
    }
}

int grid_n(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b < 1) b = 1;
    return (int)(b > 8 * bh::num_sms() ? 8 * bh::num_sms() : b);
}

template <bool kFP64, int kLearn, bool kGroup = false>
int launch_walk(bh_context* ctx, const FParams& p)
{
    const size_t smem = sizeof(WalkSmem<kFP64, kLearn, kGroup>);
    BH_CUDA_TRY(cudaFuncSetAttribute(traverse_masked_kernel<kFP64, kLearn, kGroup>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // The plain walks keep their working set in shared memory and L2 (L1
    // hit rates are low): shared memory takes the whole carveout, for more
    // resident blocks.  The learned walk reads the network's weights through
    // L1 and keeps the default split.
    if (kLearn == kLearnNone)
        BH_CUDA_TRY(cudaFuncSetAttribute(traverse_masked_kernel<kFP64, kLearn, kGroup>,
                                         cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared));
    const int64_t groups = (p.n + 31) / 32;
    const int64_t blocks = (groups + kWarps - 1) / kWarps;
    traverse_masked_kernel<kFP64, kLearn, kGroup><<<(unsigned)blocks, kThreads, smem, ctx->stream>>>(p);
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

}  // namespace

int launch_fp32_nodes(bh_context* ctx, double G)
{
    if (ctx->n == 0) return BH_OK;
    fp32_nodes_kernel<<<grid_n(2 * ctx->n), 256, 0, ctx->stream>>>(ctx->counts, ctx->rec, G, ctx->fA, ctx->fB,
                                                                    ctx->fmeta, nullptr);
    BH_LAUNCH_CHECK(ctx);
    ctx->fnodes_fused = true;
    ctx->fnodes_G = G;
    return BH_OK;
}

int launch_direct_extract(bh_context* ctx, double G)
{
    const int nd = ctx->num_direct < 64 ? ctx->num_direct : 64;
    if (ctx->n == 0 || nd <= 0) return BH_OK;
    BH_CUDA_TRY(cudaMemsetAsync(ctx->direct_present, 0, sizeof(int32_t) * 64, ctx->stream));
    direct_extract_kernel<<<grid_n(ctx->n), 256, 0, ctx->stream>>>(ctx->n, ctx->px, ctx->py, ctx->pz, ctx->m, ctx->id,
                                                                   nd, G, ctx->direct, ctx->direct_present);
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

int prepare_walk(bh_context* ctx, double theta, double G, double soft2, bool fp64, FParams& p)
{
    const int64_t n = ctx->n;
    const int nd = fp64 ? 0 : (ctx->num_direct < 64 ? ctx->num_direct : 64);
    if (fp64 || !ctx->fnodes_fused || ctx->fnodes_G != G) {  // else they are current (the build wrote them)
        if (int rc = ensure_rec(ctx)) return rc;
        fp32_nodes_kernel<<<grid_n(2 * n), 256, 0, ctx->stream>>>(ctx->counts, ctx->rec, G, ctx->fA, ctx->fB,
                                                                  ctx->fmeta, fp64 ? ctx->d4 : nullptr);
        BH_LAUNCH_CHECK(ctx);
        ctx->fnodes_fused = true;
        ctx->fnodes_G = G;
    }
    if (nd > 0) {
        int rc = launch_direct_extract(ctx, G);
        if (rc) return rc;
    }
    p = FParams{};
    p.n = n;
    p.px = ctx->px; p.py = ctx->py; p.pz = ctx->pz;
    p.id = ctx->id;
    p.body_leaf = ctx->body_leaf;
    p.A = ctx->fA; p.B = ctx->fB; p.meta = ctx->fmeta;
    p.rec = ctx->rec;
    p.d4 = ctx->d4;
    p.spread = ctx->fspread;
    p.bbox = ctx->bbox;
    p.theta2 = theta * theta;
    p.soft2 = soft2;
    p.G = G;
    p.direct = ctx->direct;
    p.present = ctx->direct_present;
    p.nd = nd;
    p.ax = ctx->ax; p.ay = ctx->ay; p.az = ctx->az;
    p.vx = ctx->vx; p.vy = ctx->vy; p.vz = ctx->vz;
    p.inter_count = ctx->inter_count;
    p.body_count = ctx->body_count;
    p.err = ctx->err;
    p.max_pops = 2 * n + 2;
    BH_CUDA_TRY(cudaMemsetAsync(ctx->inter_count, 0, sizeof(unsigned long long), ctx->stream));
    return BH_OK;
}

int launch_traverse_masked(bh_context* ctx, double theta, double G, double soft2, double kick_h, bool fp64,
                           bool group)
{
    if (ctx->n == 0) return BH_OK;
    if (2 * ctx->n >= (int64_t(1) << kSlotBits))
        return bh_fail(BH_ERR_CAPACITY, "masked walk: more than 2^27 bodies");
    FParams p;
    int rc = prepare_walk(ctx, theta, G, soft2, fp64, p);
    if (rc) return rc;
    p.kick_h = kick_h;
    if (fp64) return launch_walk<true, kLearnNone>(ctx, p);
    return group ? launch_walk<false, kLearnNone, true>(ctx, p) : launch_walk<false, kLearnNone>(ctx, p);
}

int launch_collect(bh_context* ctx, double theta, double G, double theta_max, int32_t* c_group, int32_t* c_slot,
                   uint32_t* c_mask, float* c_feat, float* c_ascale, unsigned long long* c_count, int64_t cap)
{
    if (ctx->n == 0) return BH_OK;
    if (2 * ctx->n >= (int64_t(1) << kSlotBits))
        return bh_fail(BH_ERR_CAPACITY, "masked walk: more than 2^27 bodies");
    if (!ctx->tree_moments) return bh_fail(BH_ERR_STATE, "collection: the tree was built without second moments");
    FParams p;
    int rc = prepare_walk(ctx, theta, G, 0.0, false, p);
    if (rc) return rc;
    p.kick_h = 0.0;
    p.theta_max2 = (float)(theta_max * theta_max);
    p.c_group = c_group; p.c_slot = c_slot; p.c_mask = c_mask; p.c_feat = c_feat; p.c_ascale = c_ascale;
    p.c_count = c_count;
    p.c_cap = cap;
    return launch_walk<false, kLearnCollect>(ctx, p);
}

}  // namespace bh
