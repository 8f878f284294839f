// The learned walk behind BH_MODE_LEARNED: the FP32 far-field walk of
// bh_traverse_fp32.cu (same groups, stack, staged list and FP64 direct
// terms) with a per-body error budget in place of the theta test for the
// candidates.  No reference counterpart: the reference accepts a node by
// theta alone (src/traversal.cpp:78).
//
// A candidate is a node the group test does not accept for the whole group
// but within theta_max of it (side < theta_max dmin).  Each group carries an
// allowance: budget x its smallest direct-term acceleration (the bodies'
// tightest budget), and every accepted candidate spends its estimated error
// from it.  The estimate is analytic, log10(G m s^2 / (dmin^4 a_scale)) with
// s the node's mass spread, unless it lies within l_band decades of the
// allowance; those candidates are deferred, and the network (8 -> 64 -> 64
// -> 1, BF16 mma.sync) predicts their log10 error in batches of up to 32.  A
// candidate may take at most l_frac of the remaining allowance, and the
// accepted errors of one iteration, in lane order, must fit in it (a prefix
// passes).  A candidate that is not accepted falls back to the theta test:
// each lane of its mask decides for itself, as in the plain walk.
// Candidates whose features fall outside the training range go the same way
// and are counted.
#include <climits>

#include "bh_walk.cuh"

namespace bh {
namespace {

constexpr int kPendFlush = 16;  // run the network once this many candidates wait
constexpr int kPendCap = 32;    // deferred candidates per warp

// The FP32 walk's shared memory (leaf ids and network rows included) and the
// deferred candidates.
struct LearnSmem : WalkSmem<false, kLearnInfer> {
    int pend_node[kWarps][kPendCap];
    unsigned pend_mask[kWarps][kPendCap];
};

// Five blocks per SM: the network's fragments and the deferral state take
// 96 registers.
__global__ void __launch_bounds__(kThreads, 5) traverse_learned_kernel(FParams p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LearnSmem& sm = *reinterpret_cast<LearnSmem*>(smem_raw);
    if (threadIdx.x <= kMaxDepth) {
        const double dx = __dsub_rn(p.bbox[3], p.bbox[0]);
        const double dy = __dsub_rn(p.bbox[4], p.bbox[1]);
        const double dz = __dsub_rn(p.bbox[5], p.bbox[2]);
        double L = dx;
        if (L < dy) L = dy;
        if (L < dz) L = dz;
        const double side = __ddiv_rn(L, (double)(1ull << threadIdx.x));
        sm.side2d[threadIdx.x] = __dmul_rn(side, side);
        sm.side2f[threadIdx.x] = (float)sm.side2d[threadIdx.x];
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
    // The group centre as the collection walk forms it (the features are
    // group-relative): the first body's position truncated to FP32.
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
    const float soft2f = (float)p.soft2;
    const double soft2 = p.soft2;
    int2* stk = sm.stack[w];
    float4* L = sm.lst[w];
    unsigned* LM = sm.lst_mask[w];
    const unsigned me = 1u << lane;
    const unsigned lt = me - 1u;

    double adx = 0.0, ady = 0.0, adz = 0.0;
    unsigned cnt = 0;

    // FP64 direct terms from the direct bodies first: they set the group's
    // acceleration scale, the unit of the error budget.
    {
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
    }
    float ascale = valid ? (float)sqrt(adx * adx + ady * ady + adz * adz) : 3.0e38f;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) ascale = fminf(ascale, __shfl_xor_sync(0xffffffffu, ascale, off));
    if (ascale >= 3.0e38f) ascale = 0.0f;
    const float bmag = fmaxf(fmaxf(fmaxf(fabsf(bminx), fabsf(bmaxx)), fmaxf(fabsf(bminy), fabsf(bmaxy))),
                             fmaxf(fabsf(bminz), fabsf(bmaxz)));
    const float gextent = sqrtf((bmaxx - bminx) * (bmaxx - bminx) + (bmaxy - bminy) * (bmaxy - bminy) +
                                (bmaxz - bminz) * (bmaxz - bminz));
    const float bcx = 0.5f * (bminx + bmaxx), bcy = 0.5f * (bminy + bmaxy), bcz = 0.5f * (bminz + bmaxz);
    // Per-walk logarithms of the learned features (base 2).
    const float lext = __log2f(fmaxf(gextent, 1e-30f));
    const float lascale = __log2f(ascale);
    unsigned long long ncand = 0, nacc = 0, nfall = 0, nana = 0;
    float grel = p.l_budget;  // remaining per-body allowance (units of a_scale)

    int nlist = 0;
    int sp = 1;
    if (lane == 0) stk[0] = make_int2(0, (int)full);  // the root: a range of one slot
    __syncwarp();
    bool overflow = false;
    int64_t pops = 0;

    int npend = 0;  // deferred candidates waiting for the network
    while (sp > 0 || nlist > 0 || npend > 0) {
        // The candidates the network must decide are deferred and evaluated
        // in batches: this iteration takes the deferred nodes instead of the
        // stack's when enough wait (or nothing else is left).
        const bool from_pend = npend > 0 && (npend >= kPendFlush || sp == 0);
        if (sp > 0 || from_pend) {
            int R = 0, T = 0, f_r = 0, s_r = 0;
            unsigned m_r = 0;
            float plerr = 0.0f;  // network's predicted log10 error of deferred row `lane`
            if (from_pend) {
                const float yrow = mlp_predict_warp(p.mlp, sm.feat[w], lane, npend);
                plerr = yrow * p.mlp->sc.lstd + p.mlp->sc.lmean;
                T = npend;
                if (sp + T > kStack) {
                    overflow = true;
                    break;
                }
            } else {
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
                R = __popc(__ballot_sync(0xffffffffu, take));
                T = __shfl_sync(0xffffffffu, incl, R - 1);
                const int rstart = incl - rcnt;
                const unsigned starts = __reduce_or_sync(0xffffffffu, take ? (1u << rstart) : 0u);
                const int rj = __popc(starts & ((2u << lane) - 1u)) - 1;
                f_r = __shfl_sync(0xffffffffu, rfirst, rj);
                s_r = __shfl_sync(0xffffffffu, rstart, rj);
                m_r = __shfl_sync(0xffffffffu, rmask, rj);
                pops += T;
                if (sp - R + T > kStack || pops > p.max_pops) {
                    overflow = true;
                    break;
                }
            }
            const int k = T;
            int node = -1;
            unsigned M = 0, A = 0;
            int nc = 0, ref = 0, depth = 0;
            bool leaf = false, mixed = false, cand = false;
            float dmin2 = 0.f, dmax2 = 0.f, s2 = 0.f;
            float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lane < k) {
                if (from_pend) {
                    node = sm.pend_node[w][lane];
                    M = sm.pend_mask[w][lane];
                } else {
                    node = f_r + (lane - s_r);
                    M = m_r;
                }
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
                    s2 = sm.side2f[depth];
                    nc = (int)(mt & 0xFF);
                    // Absolute error of the FP32 group-relative distances.
                    const float err = kAbsErr * (fmaxf(fabsf(cx), fmaxf(fabsf(cy), fabsf(cz))) + bmag);
                    const float dlo = fmaxf(sqrtf(dmin2) - err, 0.0f), dhi = sqrtf(dmax2) + err;
                    if (s2 * (1.0f + kMargin) < theta2f * dlo * dlo) {
                        A = M;
                    } else {
                        cand = !from_pend && M != 0 && dmin2 > 0.0f && s2 < p.theta_max2 * dmin2;
                        if (s2 * (1.0f - kMargin) > theta2f * dhi * dhi) A = 0;
                        else mixed = true;
                    }
                }
            }
            __syncwarp();
            sp -= R;
            if (from_pend) npend = 0;
            {
                // Per-body budget: the group's remaining allowance grel (the
                // smallest of its bodies' budgets, in units of a_scale) pays
                // for every accepted candidate's error.  The analytic
                // estimate log10(G m s^2 / (dmin^4 a_scale)) (s the spread)
                // accepts a candidate far below the allowance and leaves one
                // far above it to the theta test; the network predicts the
                // error of the others, deferred and evaluated in batches.
                // Out-of-range features: the theta test (the fallback).
                const MlpDev* md = p.mlp;
                const float lallow = grel > 0.0f ? __log10f(p.l_frac * grel) : -1e30f;
                bool take = false, defer = false;
                float lerr = 0.0f;
                if (from_pend) {
                    take = lane < k && M != 0 && plerr < lallow;
                    lerr = plerr;
                } else if (__ballot_sync(0xffffffffu, cand)) {
                    constexpr float kL = 0.30102999566f;  // log10(2)
                    float l2dmin = 0.0f, lspr = 0.0f, lest = 0.0f;
                    if (cand) {
                        l2dmin = __log2f(dmin2);
                        lspr = __log2f(fmaxf(__ldg(p.spread + node), 1e-8f * sqrtf(s2)));
                        lest = kL * (__log2f(e.w) - l2dmin - lascale) + 2.0f * kL * (lspr - 0.5f * l2dmin);
                    }
                    const bool sure = cand && lest + p.l_band < lallow;
                    const bool band = cand && !sure && lest - p.l_band <= lallow;
                    bool inr = false;
                    float zq[kFeat];
                    if (band) {
                        // the features, as the collection computes them
                        const float l2s = __log2f(s2);
                        const float dcx = e.x - bcx, dcy = e.y - bcy, dcz = e.z - bcz;
                        const float ldmin = 0.5f * l2dmin;
                        float f[kFeat];
                        f[0] = kL * (0.5f * l2s - ldmin);
                        f[1] = kL * (lspr - ldmin);
                        f[2] = kL * (lext - ldmin);
                        f[3] = kL * (__log2f(e.w) - l2dmin - lascale);
                        f[4] = kL * 0.5f * (__log2f(dmax2) - l2dmin);
                        f[5] = (float)depth * (1.0f / kMaxDepth);
                        f[6] = kL * (lspr - 0.5f * l2s);
                        f[7] = kL * (0.5f * __log2f(fmaxf(dcx * dcx + dcy * dcy + dcz * dcz, 1e-36f)) - ldmin);
                        inr = true;
#pragma unroll
                        for (int q = 0; q < kFeat; ++q) {
                            zq[q] = (f[q] - md->sc.mean[q]) * md->sc.inv_std[q];
                            inr = inr && zq[q] >= md->sc.lo[q] && zq[q] <= md->sc.hi[q];
                        }
                    }
                    const unsigned wb = __ballot_sync(0xffffffffu, band && inr);
                    const int slot = npend + __popc(wb & lt);
                    defer = band && inr && slot < kPendCap;
                    if (defer) {
                        float (*F)[9] = sm.feat[w];
#pragma unroll
                        for (int q = 0; q < kFeat; ++q) F[slot][q] = fminf(fmaxf(zq[q], -64.0f), 64.0f);
                        sm.pend_node[w][slot] = node;
                        sm.pend_mask[w][slot] = M;
                    }
                    npend = min(kPendCap, npend + __popc(wb));
                    take = sure;
                    lerr = lest;
                    if (cand) {
                        ++ncand;
                        if (band && !defer) ++nfall;  // outside the training range, or no room: theta
                    }
                }
                if (__any_sync(0xffffffffu, take)) {
                    // The accepted errors, in lane order, must fit in the
                    // allowance: a prefix of the candidates passes.
                    const float ec = take ? exp10f(lerr) : 0.0f;
                    float incl = ec;
#pragma unroll
                    for (int off = 1; off < 32; off <<= 1) {
                        const float t = __shfl_up_sync(0xffffffffu, incl, off);
                        if (lane >= off) incl += t;
                    }
                    take = take && incl <= grel;
                    float spent = take ? ec : 0.0f;
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) spent += __shfl_xor_sync(0xffffffffu, spent, off);
                    grel -= spent;
                }
                if (take) {
                    A = M;
                    mixed = false;
                    if (from_pend) ++nacc;
                    else ++nana;
                }
                if (defer) {  // decided later, when the network has run
                    A = 0;
                    M = 0;
                    mixed = false;
                }
                __syncwarp();
            }
            // Mixed nodes: every lane of the mask applies its own test.  The
            // nodes {c, side^2} go to free entry slots past the staged list
            // (from the first even position; the list holds at most
            // kList - 32 entries here), and every lane tests its body against
            // each of them, read by broadcast.  Lane q keeps the lanes that
            // accept slot q.
            const unsigned mb = __ballot_sync(0xffffffffu, mixed);
            if (mb) {
                float4* X = L + ((nlist + 1) & ~1);
                const int nm = __popc(mb);
                const int slot = __popc(mb & lt);
                if (mixed) X[slot] = make_float4(e.x, e.y, e.z, sm.side2f[depth]);
                __syncwarp();
                unsigned res = 0;
#pragma unroll 2
                for (int q = 0; q < nm; ++q) {
                    const float4 v = X[q];
                    const float dx = v.x - rx, dy = v.y - ry, dz = v.z - rz;
                    const unsigned bq = __ballot_sync(0xffffffffu, v.w < theta2f * (dx * dx + dy * dy + dz * dz));
                    if (lane == q) res = bq;
                }
                const unsigned accm = __shfl_sync(0xffffffffu, res, slot & 31);
                if (mixed) A = accm & M;
                __syncwarp();
            }
            // A body never interacts with its own leaf (traversal.cpp:70):
            // its lanes leave the leaf's mask here, so the evaluation needs
            // no leaf test.
            {
                const bool own_cand = A != 0 && leaf && ref >= leaf_lo && ref <= leaf_hi;
                unsigned oc = __ballot_sync(0xffffffffu, own_cand);
                while (oc) {
                    const int j = __ffs(oc) - 1;
                    oc &= oc - 1u;
                    const int lj = __shfl_sync(0xffffffffu, ref, j);
                    const unsigned own = __ballot_sync(0xffffffffu, my_leaf == lj);
                    if (lane == j) A &= ~own;
                }
            }
            // Stage the accepted (node, lanes) entries in pairs
            // {x0, x1, y0, y1}, {z0, z1, w0, w1}.
            const bool stage = A != 0;
            const unsigned am = __ballot_sync(0xffffffffu, stage);
            if (stage) {
                const int pos = nlist + __popc(am & lt);
                float* P = reinterpret_cast<float*>(L + (pos & ~1)) + (pos & 1);
                P[0] = e.x;
                P[2] = e.y;
                P[4] = e.z;
                P[6] = e.w;
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
        if (nlist > kList - 32 || (sp == 0 && nlist > 0)) {
            // Two entries per iteration in packed pairs (even, odd); an odd
            // count is padded with a zero entry taken by no lane.  Each half
            // rounds as the scalar form; the two halves are separate partial
            // sums, added at the end.
            if (nlist & 1) {
                if (lane == 0) {
                    float* P = reinterpret_cast<float*>(L + (nlist - 1)) + 1;
                    P[0] = P[2] = P[4] = P[6] = 0.0f;
                    LM[nlist] = 0u;
                }
                __syncwarp();
            }
            const f32x2 rx2 = pk(rx, rx), ry2 = pk(ry, ry), rz2 = pk(rz, rz);
            const f32x2 sf2 = pk(soft2f, soft2f);
            f32x2 fx = 0ull, fy = 0ull, fz = 0ull;  // +0.0f pairs
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
            adx += widen(fx0 + fx1);  // exact, on the bit patterns
            ady += widen(fy0 + fy1);
            adz += widen(fz0 + fz1);
            nlist = 0;
            __syncwarp();
        }
    }
    if (overflow && lane == 0) atomicOr(p.err, kErrOverflow);

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
    if (p.lstats) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            ncand += __shfl_down_sync(0xffffffffu, ncand, off);
            nacc += __shfl_down_sync(0xffffffffu, nacc, off);
            nfall += __shfl_down_sync(0xffffffffu, nfall, off);
            nana += __shfl_down_sync(0xffffffffu, nana, off);
        }
        if (lane == 0) {
            atomicAdd(p.lstats, ncand);
            atomicAdd(p.lstats + 1, nacc);
            atomicAdd(p.lstats + 2, nfall);
            atomicAdd(p.lstats + 3, nana);
        }
    }
}

}  // namespace

int launch_traverse_learned(bh_context* ctx, double theta, double G, double soft2, double kick_h)
{
    if (ctx->n == 0) return BH_OK;
    if (2 * ctx->n >= (int64_t(1) << kSlotBits))
        return bh_fail(BH_ERR_CAPACITY, "masked walk: more than 2^27 bodies");
    if (!ctx->mlp_dev) return bh_fail(BH_ERR_STATE, "learned mode: no model set (bh_learned_set_model)");
    if (!ctx->tree_moments) return bh_fail(BH_ERR_STATE, "learned mode: the tree was built without second moments");
    FParams p;
    int rc = prepare_walk(ctx, theta, G, soft2, false, p);
    if (rc) return rc;
    p.kick_h = kick_h;
    p.mlp = ctx->mlp_dev;
    p.theta_max2 = (float)(ctx->learn_theta_max * ctx->learn_theta_max);
    p.l_budget = (float)ctx->learn_budget;
    p.l_band = (float)ctx->learn_band;
    p.l_frac = (float)ctx->learn_frac;
    p.lstats = ctx->lstats;
    BH_CUDA_TRY(cudaMemsetAsync(ctx->lstats, 0, 4 * sizeof(unsigned long long), ctx->stream));
    const size_t smem = sizeof(LearnSmem);
    BH_CUDA_TRY(cudaFuncSetAttribute(traverse_learned_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t groups = (p.n + 31) / 32;
    const int64_t blocks = (groups + kWarps - 1) / kWarps;
    traverse_learned_kernel<<<(unsigned)blocks, kThreads, smem, ctx->stream>>>(p);
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

}  // namespace bh
