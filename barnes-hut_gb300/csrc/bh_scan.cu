// Device-wide exclusive scan of int32 values: per-block sums, then a
// down-sweep in which each block adds the sums before its own.  Used by the
// tree build to number leaves, branching nodes and child slots.  No block
// waits on another block.
#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;

__device__ inline int64_t scan_n(int64_t n_max, const int32_t* n_dev)
{
    if (!n_dev) return n_max;
    const int64_t v = *n_dev;
    return v < n_max ? v : n_max;
}

// Block-wide inclusive scan of one value per thread; returns the inclusive
// value and writes the block total to *total.
__device__ int32_t block_inclusive(int32_t x, int32_t* warp_tot, int32_t* total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int32_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, t, off);
            if (lane >= off) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const int32_t r = x + (w > 0 ? warp_tot[w - 1] : 0);
    if (threadIdx.x == blockDim.x - 1) *total = r;
    __syncthreads();
    return r;
}

// The scanned values: in[i], or with `key` the head flags of sorted keys
// (1 where key[i] starts a new run: the leaf numbering, with no pass to
// write the flags first).
__device__ __forceinline__ int32_t scan_value(const int32_t* in, const uint64_t* key, int64_t i)
{
    if (key) return (i == 0 || key[i] != key[i - 1]) ? 1 : 0;
    return in[i];
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const int32_t* __restrict__ in,
                                                                  const uint64_t* __restrict__ key, int64_t n_max,
                                                                  const int32_t* __restrict__ n_dev,
                                                                  int32_t* __restrict__ bsum)
{
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t total;
    const int64_t n = scan_n(n_max, n_dev);
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) s += scan_value(in, key, base + k);
    block_inclusive(s, warp_tot, &total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// Each block's offset is the sum of the block sums before it, read by the
// block itself (a few thousand at most), so no launch scans them; the last
// block also writes the total.
// With `key` (the leaf numbering) the sweep writes, instead of the scan, each
// body's leaf id and each leaf's first body and key (`leaves`).
struct LeafOut {
    int32_t* body_leaf;
    int32_t* leaf_first;  // L + 1 entries: the last is n
    uint64_t* leaf_key;
};

__global__ void __launch_bounds__(kScanThreads) scan_down_kernel(const int32_t* in, const uint64_t* __restrict__ key,
                                                                int32_t* out, int64_t n_max,
                                                                const int32_t* __restrict__ n_dev,
                                                                const int32_t* __restrict__ bsum,
                                                                int32_t* __restrict__ total_out, LeafOut leaves)
{
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t total;
    __shared__ int32_t before_s;
    // sum of bsum[0 .. blockIdx.x)
    {
        int32_t acc = 0;
        for (int k = threadIdx.x; k < (int)blockIdx.x; k += kScanThreads) acc += bsum[k];
        block_inclusive(acc, warp_tot, &total);
        if (threadIdx.x == 0) before_s = total;
        __syncthreads();
    }
    const int32_t before = before_s;
    const int64_t n = scan_n(n_max, n_dev);
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? scan_value(in, key, base + k) : 0;
        s += v[k];
    }
    const int32_t inc = block_inclusive(s, warp_tot, &total);
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *total_out = before + total;
    int32_t run = before + inc - s;
    if (key) {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            const int64_t i = base + k;
            if (i < n) {
                const int32_t lid = v[k] ? run : run - 1;
                leaves.body_leaf[i] = lid;
                if (v[k]) {
                    leaves.leaf_first[lid] = (int32_t)i;
                    leaves.leaf_key[lid] = key[i];
                }
                if (i == n - 1) leaves.leaf_first[lid + 1] = (int32_t)n;
            }
            run += v[k];
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

}  // namespace

int64_t scan_tmp_ints(int64_t n_max) { return (n_max + kScanBlock - 1) / kScanBlock + 64; }

int device_exclusive_scan(bh_context* ctx, const int32_t* in, int32_t* out, int64_t n_max, const int32_t* n_dev,
                          int32_t* total)
{
    return device_exclusive_scan_tmp(ctx, in, out, n_max, n_dev, total, ctx->scan_tmp);
}

int device_exclusive_scan_tmp(bh_context* ctx, const int32_t* in, int32_t* out, int64_t n_max, const int32_t* n_dev,
                              int32_t* total, int32_t* tmp)
{
    if (n_max <= 0) {
        BH_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(int32_t), ctx->stream));
        return BH_OK;
    }
    const int nb = (int)((n_max + kScanBlock - 1) / kScanBlock);
    scan_reduce_kernel<<<nb, kScanThreads, 0, ctx->stream>>>(in, nullptr, n_max, n_dev, tmp);
    BH_LAUNCH_CHECK(ctx);
    scan_down_kernel<<<nb, kScanThreads, 0, ctx->stream>>>(in, nullptr, out, n_max, n_dev, tmp, total, LeafOut{});
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

int device_number_leaves(bh_context* ctx, const uint64_t* key, int64_t n, int32_t* total, int32_t* body_leaf,
                         int32_t* leaf_first, uint64_t* leaf_key)
{
    if (n <= 0) {
        BH_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(int32_t), ctx->stream));
        return BH_OK;
    }
    const int nb = (int)((n + kScanBlock - 1) / kScanBlock);
    scan_reduce_kernel<<<nb, kScanThreads, 0, ctx->stream>>>(nullptr, key, n, nullptr, ctx->scan_tmp);
    BH_LAUNCH_CHECK(ctx);
    scan_down_kernel<<<nb, kScanThreads, 0, ctx->stream>>>(nullptr, key, nullptr, n, nullptr, ctx->scan_tmp, total,
                                                           LeafOut{body_leaf, leaf_first, leaf_key});
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

}  // namespace bh
