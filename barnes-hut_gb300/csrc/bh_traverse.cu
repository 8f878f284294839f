// Warp-cooperative Barnes-Hut traversal.
//
// Replaces computeAccelerations (src/traversal.cpp:13-103).  Each warp owns
// 32 Morton-consecutive bodies (one per lane) and walks the compressed
// octree once for all of them.
//
// BH_MODE_PLAIN_FP64 (exact): the warp runs the reference's depth-first walk
// over the union of the nodes its lanes need.  Children are pushed in octant
// order and popped last-in-first-out, exactly as the reference's per-body
// stack does, so every lane meets its own nodes in the reference's order.
// A lane that accepts a node the warp still opens marks the stack height;
// it sits out every node popped above that height (the node's subtree) and
// rejoins when the stack falls back below it.  Each lane applies the
// reference's test to its own body: leaf -> accept (own leaf -> skip),
// else side(depth)^2 < theta^2 r^2 with r the distance to the centre of
// mass.  Because every lane sees the same node, the node is first classified
// against the group's bounding box in FP32 (with allowances for rounding):
// accepted by all, opened by all, or undecided -- only then does each lane
// run the FP64 test.  Accepted nodes go to a per-lane list in walk order;
// the lists are evaluated in lockstep (each lane its own next node) with
// IEEE sqrt and division and no contraction, so every lane adds its terms in
// the reference's order and the result equals the reference bit for bit.
#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kTravWarps = 4;
constexpr int kTravThreads = 32 * kTravWarps;
// A root-to-leaf path has at most 22 nodes (depths strictly increase), each
// leaving at most 7 siblings behind, plus 8 children of the last node.
constexpr int kStackCap = 22 * 7 + 8 + 2;

struct TravParams {
    int64_t n;
    const double* px;
    const double* py;
    const double* pz;
    const int32_t* body_leaf;
    const TreeRec* rec;
    const float4* A;        // FP32 node records (group tests)
    const float4* B;
    const uint32_t* meta;
    const double* bbox;
    double theta2;
    double G;
    double soft2;
    double kick_h;  // > 0: also apply the second half kick v += kick_h * a
    int64_t max_pops;  // upper bound on tree slots (2n)
    double* ax;
    double* ay;
    double* az;
    double* vx;
    double* vy;
    double* vz;
    unsigned long long* inter_count;
    int32_t* body_count;
    unsigned* err;
};

// side(d)^2 = (L / 2^d)^2 with L the largest bbox span (traversal.cpp:31-43).
__device__ inline void fill_side2(const double* bbox, double* side2)
{
    if (threadIdx.x <= kMaxDepth) {
        const double dx = __dsub_rn(bbox[3], bbox[0]);
        const double dy = __dsub_rn(bbox[4], bbox[1]);
        const double dz = __dsub_rn(bbox[5], bbox[2]);
        double L = dx;
        if (L < dy) L = dy;
        if (L < dz) L = dz;
        const double side = __ddiv_rn(L, (double)(1ull << threadIdx.x));
        side2[threadIdx.x] = __dmul_rn(side, side);
    }
}

__device__ inline TreeRec load_rec(const TreeRec* __restrict__ rec, int s)
{
    const double2* p = reinterpret_cast<const double2*>(rec + s);
    const double2 a = __ldg(p);
    const double2 b = __ldg(p + 1);
    const int4 c = __ldg(reinterpret_cast<const int4*>(reinterpret_cast<const char*>(rec + s) + 32));
    TreeRec r;
    r.cx = a.x; r.cy = a.y; r.cz = b.x; r.m = b.y;
    r.child = c.x;
    r.leaf = c.y;
    r.nchild = (uint8_t)(c.z & 0xFF);
    r.depth = (uint8_t)((c.z >> 8) & 0xFF);
    r.top = (uint8_t)((c.z >> 16) & 0xFF);
    return r;
}

// Per-lane ordered interaction lists of the exact walk (slots).
constexpr int kPList = 48;
constexpr float kMargin = 1e-5f;
constexpr float kAbsErr = 1e-6f;

__global__ void __launch_bounds__(kTravThreads) traverse_exact_kernel(TravParams p)
{
    __shared__ int stack[kTravWarps][kStackCap];
    __shared__ int plist[kTravWarps][kPList][32];
    __shared__ double side2[kMaxDepth + 1];
    __shared__ float side2f[kMaxDepth + 1];
    fill_side2(p.bbox, side2);
    __syncthreads();
    if (threadIdx.x <= kMaxDepth) side2f[threadIdx.x] = (float)side2[threadIdx.x];
    __syncthreads();

    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t group = (int64_t)blockIdx.x * kTravWarps + w;
    const int64_t base = group * 32;
    if (base >= p.n) return;  // whole warp past the end
    const int64_t i = base + lane;
    const bool valid = i < p.n;
    const int64_t ii = valid ? i : base;
    const double px = p.px[ii], py = p.py[ii], pz = p.pz[ii];
    const int my_leaf = valid ? p.body_leaf[i] : -2;
    const double theta2 = p.theta2, G = p.G, soft2 = p.soft2;
    const float theta2f = (float)theta2;
    // Group box in group-relative FP32 coordinates (for the group tests).
    const float gx = __double2float_rn(__shfl_sync(0xffffffffu, px, 0));
    const float gy = __double2float_rn(__shfl_sync(0xffffffffu, py, 0));
    const float gz = __double2float_rn(__shfl_sync(0xffffffffu, pz, 0));
    const float rx = __double2float_rn(px - (double)gx);
    const float ry = __double2float_rn(py - (double)gy);
    const float rz = __double2float_rn(pz - (double)gz);
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
    const float bmag = fmaxf(fmaxf(fmaxf(fabsf(bminx), fabsf(bmaxx)), fmaxf(fabsf(bminy), fabsf(bmaxy))),
                             fmaxf(fabsf(bminz), fabsf(bmaxz)));
    int* stk = stack[w];
    int (*PL)[32] = plist[w];

    double ax = 0.0, ay = 0.0, az = 0.0;
    unsigned cnt = 0;
    int mine = 0;  // entries in this lane's list
    int sp = 1;
    int skip_sp = 0x7fffffff;
    if (lane == 0) stk[0] = 0;
    __syncwarp();
    bool overflow = false;
    int64_t pops = 0;

    // Evaluates every lane's list in order with the reference's arithmetic.
    auto flush = [&]() {
        int most = mine;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) most = max(most, __shfl_xor_sync(0xffffffffu, most, off));
        for (int q = 0; q < most; ++q) {
            const bool on = q < mine;
            const int s = on ? PL[q][lane] : 0;
            const TreeRec r = load_rec(p.rec, s);
            const double dx = __dsub_rn(r.cx, px), dy = __dsub_rn(r.cy, py), dz = __dsub_rn(r.cz, pz);
            const double r2 =
                __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), soft2);
            const double invR = __drcp_rn(__dsqrt_rn(r2));
            const double invR3 = __dmul_rn(__dmul_rn(invR, invR), invR);
            const double sc = __dmul_rn(__dmul_rn(G, r.m), invR3);
            if (on) {
                ax = __dadd_rn(ax, __dmul_rn(sc, dx));
                ay = __dadd_rn(ay, __dmul_rn(sc, dy));
                az = __dadd_rn(az, __dmul_rn(sc, dz));
            }
        }
        mine = 0;
        __syncwarp();
    };

    while (sp > 0) {
        if (++pops > p.max_pops) {
            overflow = true;
            break;
        }
        --sp;
        const int s = stk[sp];
        __syncwarp();
        const float4 a = __ldg(p.A + s);
        const float4 b = __ldg(p.B + s);
        const uint32_t mt = __ldg(p.meta + s);
        if (sp < skip_sp) skip_sp = 0x7fffffff;
        if ((mt >> 17) & 1u) continue;  // massless: skipped with its subtree (traversal.cpp:66)
        const bool active = valid && skip_sp == 0x7fffffff;
        const bool leaf = (mt >> 16) & 1u;
        const int depth = (mt >> 8) & 0xFF;
        bool accept = false, open = false;
        if (leaf) {
            if (active) {
                if (__float_as_int(b.w) != my_leaf) {
                    accept = true;
                } else {
                    // Own leaf: the reference skips it at depth 21, but a chain
                    // cell above it (depths top..20) may already accept.
                    const TreeRec r = load_rec(p.rec, s);
                    const double dx = __dsub_rn(r.cx, px), dy = __dsub_rn(r.cy, py), dz = __dsub_rn(r.cz, pz);
                    const double r2 = __dadd_rn(
                        __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), soft2);
                    accept = r.top <= kMaxDepth - 1 && side2[kMaxDepth - 1] < __dmul_rn(theta2, r2);
                }
            }
        } else {
            // The same node for every lane: classify it against the group box
            // (with allowances for FP32 rounding), test lane by lane in FP64
            // only when the box cannot decide.
            const float cx = (a.x - gx) + b.x, cy = (a.y - gy) + b.y, cz = (a.z - gz) + b.z;
            const float ex = fmaxf(0.0f, fmaxf(bminx - cx, cx - bmaxx));
            const float ey = fmaxf(0.0f, fmaxf(bminy - cy, cy - bmaxy));
            const float ez = fmaxf(0.0f, fmaxf(bminz - cz, cz - bmaxz));
            const float fx = fmaxf(fabsf(cx - bminx), fabsf(cx - bmaxx));
            const float fy = fmaxf(fabsf(cy - bminy), fabsf(cy - bmaxy));
            const float fz = fmaxf(fabsf(cz - bminz), fabsf(cz - bmaxz));
            const float err = kAbsErr * (fmaxf(fabsf(cx), fmaxf(fabsf(cy), fabsf(cz))) + bmag);
            const float dlo = fmaxf(sqrtf(ex * ex + ey * ey + ez * ez) - err, 0.0f);
            const float dhi = sqrtf(fx * fx + fy * fy + fz * fz) + err;
            const float s2 = side2f[depth];
            if (s2 * (1.0f + kMargin) < theta2f * dlo * dlo) {
                accept = active;
            } else if (s2 * (1.0f - kMargin) > theta2f * dhi * dhi) {
                open = active;
            } else if (__any_sync(0xffffffffu, active)) {
                const TreeRec r = load_rec(p.rec, s);
                if (active) {
                    const double dx = __dsub_rn(r.cx, px), dy = __dsub_rn(r.cy, py), dz = __dsub_rn(r.cz, pz);
                    const double r2 = __dadd_rn(
                        __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), soft2);
                    accept = side2[depth] < __dmul_rn(theta2, r2);
                    open = !accept;
                }
            }
        }
        if (accept) {
            PL[mine++][lane] = s;
            ++cnt;
        }
        const unsigned opened = __ballot_sync(0xffffffffu, open);
        if (opened) {
            if (accept) skip_sp = sp;  // sit out this node's subtree
            const int nc = (int)(mt & 0xFF);
            if (sp + nc > kStackCap) {
                overflow = true;
                break;
            }
            if (lane < nc) stk[sp + lane] = __float_as_int(b.w) + lane;
            __syncwarp();
            sp += nc;
        }
        if (__any_sync(0xffffffffu, mine == kPList)) flush();
    }
    flush();
    if (overflow && lane == 0) atomicOr(p.err, kErrOverflow);
    if (valid) {
        p.ax[i] = ax;
        p.ay[i] = ay;
        p.az[i] = az;
        if (p.body_count) p.body_count[i] = (int32_t)cnt;
        if (p.kick_h > 0.0) {
            p.vx[i] = __dadd_rn(p.vx[i], __dmul_rn(p.kick_h, ax));
            p.vy[i] = __dadd_rn(p.vy[i], __dmul_rn(p.kick_h, ay));
            p.vz[i] = __dadd_rn(p.vz[i], __dmul_rn(p.kick_h, az));
        }
    }
    if (p.inter_count) {
        unsigned long long c = valid ? cnt : 0ull;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
        if (lane == 0) atomicAdd(p.inter_count, c);
    }
}

}  // namespace

int launch_traverse(bh_context* ctx, double theta, double G, double soft2, int mode, double kick_h)
{
    const int64_t n = ctx->n;
    if (n == 0) return BH_OK;
    TravParams p;
    p.n = n;
    p.px = ctx->px; p.py = ctx->py; p.pz = ctx->pz;
    p.body_leaf = ctx->body_leaf;
    p.rec = ctx->rec;
    p.A = ctx->fA; p.B = ctx->fB; p.meta = ctx->fmeta;
    p.bbox = ctx->bbox;
    p.theta2 = theta * theta;
    p.G = G;
    p.soft2 = soft2;
    p.kick_h = kick_h;
    p.max_pops = 2 * n + 2;
    p.ax = ctx->ax; p.ay = ctx->ay; p.az = ctx->az;
    p.vx = ctx->vx; p.vy = ctx->vy; p.vz = ctx->vz;
    p.inter_count = ctx->inter_count;
    p.body_count = ctx->body_count;
    p.err = ctx->err;
    BH_CUDA_TRY(cudaMemsetAsync(ctx->inter_count, 0, sizeof(unsigned long long), ctx->stream));
    const int64_t groups = (n + 31) / 32;
    const int64_t blocks = (groups + kTravWarps - 1) / kTravWarps;
    switch (mode) {
    case BH_MODE_PLAIN_FP64: {
        const int rc = launch_fp32_nodes(ctx, G);
        if (rc) return rc;
        traverse_exact_kernel<<<(unsigned)blocks, kTravThreads, 0, ctx->stream>>>(p);
        break;
    }
    case BH_MODE_FP64_LIST:
        return launch_traverse_masked(ctx, theta, G, soft2, kick_h, true);
    case BH_MODE_FP32_FAR:
        return launch_traverse_masked(ctx, theta, G, soft2, kick_h, false);
    case BH_MODE_LEARNED:
        return launch_traverse_learned(ctx, theta, G, soft2, kick_h);
    case BH_MODE_FP32_GROUP:
        return launch_traverse_masked(ctx, theta, G, soft2, kick_h, false, true);
    default:
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_compute_accelerations: mode not available");
    }
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

}  // namespace bh
