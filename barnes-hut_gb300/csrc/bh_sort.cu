// Onesweep LSD radix sort of the 63-bit Morton keys with a 32-bit payload
// (the body's previous position), and the permutation of the body arrays.
//
// Replaces sortBodiesByMortonKey (include/utility.h:23-52).  The reference
// index-sorts with std::sort and gathers pos/mass/vel/ids/keys; here the
// sort is a stable 8-pass LSD radix sort (8-bit digits) whose digit
// histograms for all passes come from the key kernel, and each pass is one
// kernel: tiles claim an id in launch order, rank their keys with warp
// ballots (one per digit bit), publish per-digit tile counts, and obtain their
// global offsets by a decoupled look-back over earlier tiles.  Every wait
// in the look-back is bounded; on expiry the kernel raises kErrTimeout
// and still publishes, so no tile can wait forever.
#include <utility>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kWarps = kSortThreads / 32;  // 16
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagIncl = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1;
constexpr int kSpinLimit = 1 << 22;
constexpr int kBatch = 8;  // look-back: predecessors read per round

struct SortSmem {
    uint32_t warp_hist[kWarps][kRadix];  // per-warp digit counts, then warp prefixes
    uint32_t digit_excl[kRadix];         // tile-local start of each digit
    uint32_t global_base[kRadix];        // global start minus tile-local start
    uint32_t scan[kRadix / 32];
    uint32_t tile;
    uint64_t keys[kSortTile];
    uint32_t vals[kSortTile];
};

// Exclusive scan over 256 values held one per thread by threads 0..255.
__device__ uint32_t scan256(uint32_t v, uint32_t* tmp)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) tmp[w] = x;
    __syncwarp();
    // 8 warps: a tiny serial pass by each thread over the warp totals.
    asm volatile("bar.sync 1, 256;");
    uint32_t before = 0;
    for (int k = 0; k < w; ++k) before += tmp[k];
    return before + x - v;
}

__global__ void hist_scan_kernel(uint32_t* __restrict__ hist)
{
    __shared__ uint32_t tmp[kRadix / 32];
    uint32_t* h = hist + blockIdx.x * kRadix;
    const uint32_t v = h[threadIdx.x];
    const uint32_t e = scan256(v, tmp);
    h[threadIdx.x] = e;
}

template <bool kFirst>
__global__ void __launch_bounds__(kSortThreads) onesweep_kernel(
    int64_t n, int shift, const uint64_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint64_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, const uint32_t* __restrict__ bucket_start,
    uint32_t* lookback, uint32_t* tile_ctr, unsigned* err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem& s = *reinterpret_cast<SortSmem*>(smem_raw);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;

    if (threadIdx.x == 0) s.tile = atomicAdd(tile_ctr, 1u);
    for (int k = threadIdx.x; k < kWarps * kRadix; k += kSortThreads) (&s.warp_hist[0][0])[k] = 0;
    __syncthreads();
    const uint32_t tile = s.tile;
    const int64_t base = (int64_t)tile * kSortTile;

    // Load: warp w owns keys [w*256, w*256+256) of the tile, item k at lane l
    // is key w*256 + k*32 + l, so (w, k, l) is the input order.
    uint64_t key[kSortItems];
    uint32_t val[kSortItems];
    uint32_t rank[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int64_t i = base + w * (32 * kSortItems) + k * 32 + lane;
        if (i < n) {
            key[k] = keys_in[i];
            val[k] = kFirst ? (uint32_t)i : vals_in[i];
        } else {
            key[k] = ~0ull;
            val[k] = 0;
        }
    }

    // Rank within the warp: peers holding the same digit are found with one
    // ballot per digit bit (a fixed cost; match.any takes longer the more
    // distinct digits a warp holds, as in the low passes); the lowest peer
    // bumps the warp's digit counter once.
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int64_t i = base + w * (32 * kSortItems) + k * 32 + lane;
        const bool valid = i < n;
        const uint32_t d = valid ? (uint32_t)((key[k] >> shift) & 0xFF) : 0u;
        // lanes past the end form their own peer set, apart from every digit
        const unsigned vb = __ballot_sync(0xffffffffu, valid);
        unsigned peers = valid ? vb : ~vb;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const bool bit = (d >> b) & 1u;
            const unsigned v = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? v : ~v;
        }
        const int leader = __ffs(peers) - 1;
        uint32_t old = 0;
        if (valid && lane == leader) {
            old = s.warp_hist[w][d];
            s.warp_hist[w][d] = old + __popc(peers);
        }
        old = __shfl_sync(0xffffffffu, old, leader);
        rank[k] = old + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();

    // Per digit: exclusive prefix over warps and the tile's total count.
    uint32_t tile_count = 0;
    if (threadIdx.x < kRadix) {
        const int d = threadIdx.x;
        uint32_t run = 0;
        for (int ww = 0; ww < kWarps; ++ww) {
            const uint32_t c = s.warp_hist[ww][d];
            s.warp_hist[ww][d] = run;
            run += c;
        }
        tile_count = run;
        volatile uint32_t* lb = lookback + (size_t)tile * kRadix;
        lb[d] = (tile == 0 ? kFlagIncl : kFlagAgg) | tile_count;
        s.digit_excl[d] = scan256(tile_count, s.scan);
    }

    // Decoupled look-back: thread d sums earlier tiles' counts of digit d,
    // reading kBatch predecessors per round (independent loads in flight)
    // and stopping at the nearest inclusive prefix.  A predecessor that has
    // not published yet is read again (bounded).
    if (threadIdx.x < kRadix) {
        const int d = threadIdx.x;
        uint32_t excl = 0;
        if (tile > 0) {
            const volatile uint32_t* lbv = lookback;
            int64_t k = (int64_t)tile - 1;
            int spins = 0;
            while (k >= 0) {
                uint32_t v[kBatch];
#pragma unroll
                for (int q = 0; q < kBatch; ++q) v[q] = k - q >= 0 ? lbv[(size_t)(k - q) * kRadix + d] : kFlagIncl;
                int used = 0;
                bool found = false, stall = false;
#pragma unroll
                for (int q = 0; q < kBatch; ++q) {
                    if (!found && !stall && k - q >= 0) {
                        const uint32_t f = v[q] & ~kCountMask;
                        if (f == 0u) {
                            stall = true;  // not published yet: read again from here
                        } else {
                            excl += v[q] & kCountMask;
                            ++used;
                            found = f == kFlagIncl;
                        }
                    }
                }
                if (found) break;
                if (stall) {
                    if (++spins > kSpinLimit) {
                        atomicOr(err, kErrTimeout);
                        break;
                    }
                    __nanosleep(32);
                }
                k -= used;
            }
            __threadfence();
            ((volatile uint32_t*)lookback)[(size_t)tile * kRadix + d] = kFlagIncl | ((excl + tile_count) & kCountMask);
        }
        s.global_base[d] = bucket_start[d] + excl - s.digit_excl[d];
    }
    __syncthreads();

    // Scatter into shared memory in tile-sorted order, then write out.
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int64_t i = base + w * (32 * kSortItems) + k * 32 + lane;
        if (i < n) {
            const uint32_t d = (uint32_t)((key[k] >> shift) & 0xFF);
            const uint32_t p = s.digit_excl[d] + s.warp_hist[w][d] + rank[k];
            if (p < (uint32_t)kSortTile) {
                s.keys[p] = key[k];
                s.vals[p] = val[k];
            }
        }
    }
    __syncthreads();
    const int64_t rem = n - base;
    const int cnt = rem < kSortTile ? (int)rem : kSortTile;
    for (int j = threadIdx.x; j < cnt; j += kSortThreads) {
        const uint64_t kk = s.keys[j];
        const uint32_t d = (uint32_t)((kk >> shift) & 0xFF);
        const uint32_t g = s.global_base[d] + (uint32_t)j;
        if ((int64_t)g < n) {  // always true unless a look-back wait gave up
            keys_out[g] = kk;
            vals_out[g] = s.vals[j];
        }
    }
}

constexpr int kPermThreads = 256;

// out[i] = in[perm[i]] for positions, velocities, masses and ids.
__global__ void __launch_bounds__(kPermThreads) permute_kernel(
    int64_t n, const uint32_t* __restrict__ perm, const double* __restrict__ px, const double* __restrict__ py,
    const double* __restrict__ pz, const double* __restrict__ vx, const double* __restrict__ vy,
    const double* __restrict__ vz, const double* __restrict__ m, const uint64_t* __restrict__ id,
    double* __restrict__ px2, double* __restrict__ py2, double* __restrict__ pz2, double* __restrict__ vx2,
    double* __restrict__ vy2, double* __restrict__ vz2, double* __restrict__ m2, uint64_t* __restrict__ id2)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t j = perm[i];
        if ((int64_t)j >= n) j = (uint32_t)i;  // only after a failed sort (error word set)
        px2[i] = px[j];
        py2[i] = py[j];
        pz2[i] = pz[j];
        vx2[i] = vx[j];
        vy2[i] = vy[j];
        vz2[i] = vz[j];
        m2[i] = m[j];
        id2[i] = id[j];
    }
}

}  // namespace

size_t sort_smem_bytes() { return sizeof(SortSmem); }

int launch_sort(bh_context* ctx)
{
    const int64_t n = ctx->n;
    if (n <= 1) {
        if (n == 1) BH_CUDA_TRY(cudaMemsetAsync(ctx->perm, 0, sizeof(uint32_t), ctx->stream));
        return BH_OK;
    }
    const size_t smem = sizeof(SortSmem);
    BH_CUDA_TRY(cudaFuncSetAttribute(onesweep_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    BH_CUDA_TRY(cudaFuncSetAttribute(onesweep_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t tiles = (n + kSortTile - 1) / kSortTile;
    BH_CUDA_TRY(cudaMemsetAsync(ctx->lookback, 0, sizeof(uint32_t) * kSortPasses * tiles * kRadix, ctx->stream));
    BH_CUDA_TRY(cudaMemsetAsync(ctx->tile_ctr, 0, sizeof(uint32_t) * kSortPasses, ctx->stream));
    hist_scan_kernel<<<kSortPasses, kRadix, 0, ctx->stream>>>(ctx->hist);
    BH_LAUNCH_CHECK(ctx);
    uint64_t* kin = ctx->key;
    uint64_t* kout = ctx->key_alt;
    uint32_t* vin = ctx->perm;
    uint32_t* vout = ctx->perm_alt;
    for (int p = 0; p < kSortPasses; ++p) {
        uint32_t* lb = ctx->lookback + (size_t)p * tiles * kRadix;
        if (p == 0)
            onesweep_kernel<true><<<(unsigned)tiles, kSortThreads, smem, ctx->stream>>>(
                n, 8 * p, kin, vin, kout, vout, ctx->hist + p * kRadix, lb, ctx->tile_ctr + p, ctx->err);
        else
            onesweep_kernel<false><<<(unsigned)tiles, kSortThreads, smem, ctx->stream>>>(
                n, 8 * p, kin, vin, kout, vout, ctx->hist + p * kRadix, lb, ctx->tile_ctr + p, ctx->err);
        BH_LAUNCH_CHECK(ctx);
        uint64_t* tk = kin; kin = kout; kout = tk;
        uint32_t* tv = vin; vin = vout; vout = tv;
    }
    // After an even number of passes the result is back in key / perm.
    return BH_OK;
}

int sort_passes_raw(int64_t n, const uint64_t* keys_in, uint64_t* keys_out, uint32_t* vals_out, uint64_t* key_alt,
                    uint32_t* val_alt, uint32_t* hist, uint32_t* lookback, uint32_t* tile_ctr, unsigned* err,
                    cudaStream_t stream)
{
    // The eight onesweep passes over caller-provided buffers: digit starts
    // from `hist` (counts on entry), pass 0 reads keys_in and writes the
    // alternate buffers, the last pass writes keys_out / vals_out.
    const size_t smem = sizeof(SortSmem);
    BH_CUDA_TRY(cudaFuncSetAttribute(onesweep_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    BH_CUDA_TRY(cudaFuncSetAttribute(onesweep_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t tiles = (n + kSortTile - 1) / kSortTile;
    hist_scan_kernel<<<kSortPasses, kRadix, 0, stream>>>(hist);
    BH_CUDA_TRY(cudaGetLastError());
    const uint64_t* kin = keys_in;
    const uint32_t* vin = nullptr;
    for (int p = 0; p < kSortPasses; ++p) {
        const bool to_out = (p & 1) != 0;
        uint64_t* kout = to_out ? keys_out : key_alt;
        uint32_t* vout = to_out ? vals_out : val_alt;
        uint32_t* lb = lookback + (size_t)p * tiles * kRadix;
        if (p == 0)
            onesweep_kernel<true><<<(unsigned)tiles, kSortThreads, smem, stream>>>(
                n, 8 * p, kin, vin, kout, vout, hist + p * kRadix, lb, tile_ctr + p, err);
        else
            onesweep_kernel<false><<<(unsigned)tiles, kSortThreads, smem, stream>>>(
                n, 8 * p, kin, vin, kout, vout, hist + p * kRadix, lb, tile_ctr + p, err);
        BH_CUDA_TRY(cudaGetLastError());
        kin = kout;
        vin = vout;
    }
    return BH_OK;
}

int launch_permute(bh_context* ctx)
{
    const int64_t n = ctx->n;
    if (n == 0) return BH_OK;
    int64_t want = (n + kPermThreads - 1) / kPermThreads;
    const int blocks = (int)(want > 8 * bh::num_sms() ? 8 * bh::num_sms() : want);
    permute_kernel<<<blocks, kPermThreads, 0, ctx->stream>>>(n, ctx->perm, ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy,
                                                             ctx->vz, ctx->m, ctx->id, ctx->px2, ctx->py2, ctx->pz2,
                                                             ctx->vx2, ctx->vy2, ctx->vz2, ctx->m2, ctx->id2);
    BH_LAUNCH_CHECK(ctx);
    swap_body_sets(ctx);
    return BH_OK;
}

void swap_body_sets(bh_context* ctx)
{
    std::swap(ctx->px, ctx->px2);
    std::swap(ctx->py, ctx->py2);
    std::swap(ctx->pz, ctx->pz2);
    std::swap(ctx->vx, ctx->vx2);
    std::swap(ctx->vy, ctx->vy2);
    std::swap(ctx->vz, ctx->vz2);
    std::swap(ctx->m, ctx->m2);
    std::swap(ctx->id, ctx->id2);
}

}  // namespace bh
