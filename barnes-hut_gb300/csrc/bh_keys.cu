// Kick-drift with a fused bounding box, and the Morton-key kernel with the
// fused radix-sort digit histogram.
#include <cfloat>
#include <climits>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kBoxThreads = 256;

// Order-aware extremum: the reference keeps the FIRST body holding the
// extreme value (compute_local_bbox, src/bounding_box.cpp:33-41, replaces
// only on a strict comparison), so ties are broken towards the lower index.
// Values are compared as order-preserving integer images of their bit
// patterns (FP64 comparisons run on the slow FP64 pipe): for finite doubles
// ord(a) < ord(b) exactly when a < b, with -0 mapped to +0 so that the two
// zeros tie as they do in the reference's comparison.
struct Ext {
    long long k;  // ord(value)
    long long i;
};
__device__ inline long long ord(double v)
{
    long long b = __double_as_longlong(v);
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFll);
}
__device__ inline double unord(long long k) { return __longlong_as_double(k >= 0 ? k : (k ^ 0x7FFFFFFFFFFFFFFFll)); }
__device__ inline bool better_min(const Ext& a, const Ext& b) { return a.k < b.k || (a.k == b.k && a.i < b.i); }
__device__ inline bool better_max(const Ext& a, const Ext& b) { return b.k < a.k || (a.k == b.k && a.i < b.i); }

__device__ inline Ext shfl_ext(const Ext& e, int off)
{
    Ext r;
    r.k = __shfl_down_sync(0xffffffffu, e.k, off);
    r.i = __shfl_down_sync(0xffffffffu, e.i, off);
    return r;
}

// Finite: the exponent field is not all ones.
__device__ inline bool finite_bits(double v) { return ((__double_as_longlong(v) >> 52) & 0x7FF) != 0x7FF; }

// Block-wide reduction of the six extrema (min x,y,z then max x,y,z) into
// thread 0's `e`.
__device__ void block_reduce_box(Ext e[6])
{
    __shared__ Ext sh[kBoxThreads / 32][6];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            Ext o = shfl_ext(e[a], off);
            if (a < 3 ? better_min(o, e[a]) : better_max(o, e[a])) e[a] = o;
        }
    }
    if (lane == 0)
        for (int a = 0; a < 6; ++a) sh[w][a] = e[a];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kBoxThreads / 32; ++k)
            for (int a = 0; a < 6; ++a)
                if (a < 3 ? better_min(sh[k][a], e[a]) : better_max(sh[k][a], e[a])) e[a] = sh[k][a];
    }
}

// One launch: optional half kick v += (dt/2) a (src/main.cpp:193-200),
// optional drift x += dt v (:203-208), then the bounding box of the new
// positions (compute_local_bbox).  The last block to finish reduces the
// per-block partials (ticket pattern) and writes bbox[6].
__global__ void __launch_bounds__(kBoxThreads) drift_bbox_kernel(
    int64_t n, double* __restrict__ px, double* __restrict__ py, double* __restrict__ pz,
    double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz, const double* __restrict__ ax,
    const double* __restrict__ ay, const double* __restrict__ az, double dt, double h, int kick, int drift,
    Ext* __restrict__ part, double* __restrict__ bbox, unsigned* __restrict__ ticket, unsigned* __restrict__ err)
{
    Ext e[6];
    for (int a = 0; a < 3; ++a) { e[a] = {ord(DBL_MAX), LLONG_MAX}; e[3 + a] = {ord(-DBL_MAX), LLONG_MAX}; }
    // +-DBL_MAX with an index past every body loses every comparison with a
    // real (finite) coordinate; infinities and NaN are flagged below.
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x = px[i], y = py[i], z = pz[i];
        if (kick | drift) {
            double u = vx[i], v = vy[i], w = vz[i];
            if (kick) {
                u = __dadd_rn(u, __dmul_rn(h, ax[i]));
                v = __dadd_rn(v, __dmul_rn(h, ay[i]));
                w = __dadd_rn(w, __dmul_rn(h, az[i]));
                vx[i] = u; vy[i] = v; vz[i] = w;
            }
            if (drift) {
                x = __dadd_rn(x, __dmul_rn(dt, u));
                y = __dadd_rn(y, __dmul_rn(dt, v));
                z = __dadd_rn(z, __dmul_rn(dt, w));
                px[i] = x; py[i] = y; pz[i] = z;
            }
        }
        bad |= !(finite_bits(x) && finite_bits(y) && finite_bits(z));
        const double c[3] = {x, y, z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            Ext o{ord(c[a]), (long long)i};
            if (better_min(o, e[a])) e[a] = o;
            if (better_max(o, e[3 + a])) e[3 + a] = o;
        }
    }
    if (bad) atomicOr(err, kErrNonFinite);
    block_reduce_box(e);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        for (int a = 0; a < 6; ++a) part[blockIdx.x * 6 + a] = e[a];
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // Last block: reduce the partials (block count <= a few thousand).
    for (int a = 0; a < 3; ++a) { e[a] = {ord(DBL_MAX), LLONG_MAX}; e[3 + a] = {ord(-DBL_MAX), LLONG_MAX}; }
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        for (int a = 0; a < 6; ++a) {
            Ext o = part[b * 6 + a];
            if (a < 3 ? better_min(o, e[a]) : better_max(o, e[a])) e[a] = o;
        }
    }
    __syncthreads();
    block_reduce_box(e);
    if (threadIdx.x == 0) {
        // The extreme body's own value (keeps the sign of a zero, which the
        // integer image folds).
        for (int a = 0; a < 6; ++a) {
            const long long bi = e[a].i;
            const double* src = (a % 3 == 0) ? px : (a % 3 == 1) ? py : pz;
            bbox[a] = (bi >= 0 && bi < n) ? src[bi] : unord(e[a].k);
        }
        *ticket = 0u;
    }
}

// spread21 (src/morton_keys.cpp:11-19): bit k of v moves to bit 3k.
__device__ inline uint64_t spread21(uint32_t v)
{
    uint64_t x = v & 0x1FFFFFu;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}


constexpr int kKeyThreads = 512;

__global__ void __launch_bounds__(kKeyThreads) keys_kernel(int64_t n, const double* __restrict__ px,
                                                          const double* __restrict__ py,
                                                          const double* __restrict__ pz,
                                                          const double* __restrict__ bbox,
                                                          uint64_t* __restrict__ key, uint32_t* __restrict__ hist,
                                                          int with_hist)
{
    __shared__ uint32_t sh[kSortPasses * kRadix];
    if (with_hist)
        for (int k = threadIdx.x; k < kSortPasses * kRadix; k += blockDim.x) sh[k] = 0;
    const double lo0 = bbox[0], lo1 = bbox[1], lo2 = bbox[2];
    const double s0 = (bbox[3] == lo0) ? 1.0 : __dsub_rn(bbox[3], lo0);
    const double s1 = (bbox[4] == lo1) ? 1.0 : __dsub_rn(bbox[4], lo1);
    const double s2 = (bbox[5] == lo2) ? 1.0 : __dsub_rn(bbox[5], lo2);
    const double i0 = __drcp_rn(s0) * 2097152.0, i1 = __drcp_rn(s1) * 2097152.0, i2 = __drcp_rn(s2) * 2097152.0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t xi = quantise(px[i], lo0, s0, i0);
        const uint32_t yi = quantise(py[i], lo1, s1, i1);
        const uint32_t zi = quantise(pz[i], lo2, s2, i2);
        const uint64_t k = spread21(xi) | (spread21(yi) << 1) | (spread21(zi) << 2);
        key[i] = k;
        if (with_hist) {
#pragma unroll
            for (int p = 0; p < kSortPasses; ++p) atomicAdd(&sh[p * kRadix + ((k >> (8 * p)) & 0xFF)], 1u);
        }
    }
    if (!with_hist) return;
    __syncthreads();
    for (int k = threadIdx.x; k < kSortPasses * kRadix; k += blockDim.x)
        if (sh[k]) atomicAdd(&hist[k], sh[k]);
}

// Digit histograms of keys already in place (the stateless sort entry).
__global__ void __launch_bounds__(kKeyThreads) hist_kernel(int64_t n, const uint64_t* __restrict__ key,
                                                          uint32_t* __restrict__ hist)
{
    __shared__ uint32_t sh[kSortPasses * kRadix];
    for (int k = threadIdx.x; k < kSortPasses * kRadix; k += blockDim.x) sh[k] = 0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = key[i];
#pragma unroll
        for (int p = 0; p < kSortPasses; ++p) atomicAdd(&sh[p * kRadix + ((k >> (8 * p)) & 0xFF)], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kSortPasses * kRadix; k += blockDim.x)
        if (sh[k]) atomicAdd(&hist[k], sh[k]);
}

}  // namespace

int launch_hist(bh_context* ctx)
{
    if (ctx->n == 0) return BH_OK;
    BH_CUDA_TRY(cudaMemsetAsync(ctx->hist, 0, sizeof(uint32_t) * kSortPasses * kRadix, ctx->stream));
    int64_t want = (ctx->n + kKeyThreads * 4 - 1) / (kKeyThreads * 4);
    const int blocks = (int)(want < 1 ? 1 : (want > 4 * bh::num_sms() ? 4 * bh::num_sms() : want));
    hist_kernel<<<blocks, kKeyThreads, 0, ctx->stream>>>(ctx->n, ctx->key, ctx->hist);
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

int launch_drift_bbox(bh_context* ctx, double dt, bool kick, bool drift)
{
    if (ctx->n == 0) return BH_OK;
    const int blocks = ctx->bbox_blocks;
    drift_bbox_kernel<<<blocks, kBoxThreads, 0, ctx->stream>>>(
        ctx->n, ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy, ctx->vz, ctx->ax, ctx->ay, ctx->az, dt, 0.5 * dt,
        kick ? 1 : 0, drift ? 1 : 0, reinterpret_cast<Ext*>(ctx->bbox_part), ctx->bbox, ctx->bbox_ticket, ctx->err);
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

int bbox_partial_bytes(int blocks) { return blocks * 6 * (int)sizeof(Ext); }

int launch_keys(bh_context* ctx, bool with_hist)
{
    if (ctx->n == 0) return BH_OK;
    if (with_hist) BH_CUDA_TRY(cudaMemsetAsync(ctx->hist, 0, sizeof(uint32_t) * kSortPasses * kRadix, ctx->stream));
    int64_t want = (ctx->n + kKeyThreads * 4 - 1) / (kKeyThreads * 4);
    const int blocks = (int)(want < 1 ? 1 : (want > 4 * bh::num_sms() ? 4 * bh::num_sms() : want));
    keys_kernel<<<blocks, kKeyThreads, 0, ctx->stream>>>(ctx->n, ctx->px, ctx->py, ctx->pz, ctx->bbox, ctx->key,
                                                         ctx->hist, with_hist ? 1 : 0);
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

}  // namespace bh
