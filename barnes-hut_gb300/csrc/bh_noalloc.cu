// Allocation-free variant of the Morton-key radix sort.
//
// Some callers cannot let this library call cudaMalloc: a host simulation
// whose device memory is owned by its own pool or budget hands the engine
// device buffers it already holds and may not have a second allocator carve
// memory behind its back, and a caller in a time-critical loop cannot afford
// cudaMalloc's implicit device synchronisation or its failure under memory
// pressure in the middle of a run.  bh_sort_keys_noalloc serves them: the
// caller passes the keys and the output buffers, and every piece of scratch
// the sort needs (alternate key/permutation buffers, digit histograms,
// look-back words, tile counters, error word) lives in one file-scope
// __device__ array of fixed size, which every GPU that loads the library
// holds until the process exits.
//
// Host code never uses the array's name as an address (on the host it is
// only a stand-in symbol); the device address is obtained once per device
// with cudaGetSymbolAddress, with that device current, on the first call made
// on that device.  That first call should therefore come before any stream
// capture.  All calls share the array: it keeps the last call's contents, the
// parts that must start at zero are cleared on every call, and calls that
// overlap on the GPU (different streams, or different host threads on the
// same device) race on it.
#include <mutex>
#include <string>

#include "bh_internal.cuh"

namespace {

constexpr int64_t kMaxKeys = BH_NOALLOC_MAX_KEYS;
constexpr int64_t kMaxTiles = (kMaxKeys + bh::kSortTile - 1) / bh::kSortTile;

// Byte offsets of the pieces inside the scratch array (256-byte aligned).
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffKeyAlt = 0;
constexpr size_t kOffValAlt = align256(kOffKeyAlt + sizeof(uint64_t) * kMaxKeys);
constexpr size_t kOffHist = align256(kOffValAlt + sizeof(uint32_t) * kMaxKeys);
constexpr size_t kOffLookback = align256(kOffHist + sizeof(uint32_t) * bh::kSortPasses * bh::kRadix);
constexpr size_t kOffTileCtr = align256(kOffLookback + sizeof(uint32_t) * bh::kSortPasses * kMaxTiles * bh::kRadix);
constexpr size_t kOffErr = align256(kOffTileCtr + sizeof(uint32_t) * bh::kSortPasses);
constexpr size_t kScratchBytes = align256(kOffErr + sizeof(unsigned));

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up on the
// first call per device).
int scratch_address(int dev, unsigned char** out)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return bh_fail(BH_ERR_CUDA, std::string("bh_sort_keys_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[dev];
    return BH_OK;
}

constexpr int kHistThreads = 512;

__global__ void __launch_bounds__(kHistThreads) noalloc_hist_kernel(int64_t n, const uint64_t* __restrict__ key,
                                                                   uint32_t* __restrict__ hist)
{
    __shared__ uint32_t sh[bh::kSortPasses * bh::kRadix];
    for (int k = threadIdx.x; k < bh::kSortPasses * bh::kRadix; k += blockDim.x) sh[k] = 0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = key[i];
#pragma unroll
        for (int p = 0; p < bh::kSortPasses; ++p) atomicAdd(&sh[p * bh::kRadix + ((k >> (8 * p)) & 0xFF)], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < bh::kSortPasses * bh::kRadix; k += blockDim.x)
        if (sh[k]) atomicAdd(&hist[k], sh[k]);
}

}  // namespace

namespace bh {

// Digit counts of the eight passes (hist: kSortPasses x kRadix, zeroed by
// the caller) for sort_passes_raw.
int launch_digit_hist(int64_t n, const uint64_t* keys, uint32_t* hist, cudaStream_t st)
{
    int64_t blocks = (n + kHistThreads * 4 - 1) / (kHistThreads * 4);
    if (blocks > 4 * bh::num_sms()) blocks = 4 * bh::num_sms();
    if (blocks < 1) blocks = 1;
    noalloc_hist_kernel<<<(unsigned)blocks, kHistThreads, 0, st>>>(n, keys, hist);
    BH_CUDA_TRY(cudaGetLastError());
    return BH_OK;
}

}  // namespace bh

extern "C" int bh_sort_keys_noalloc(const uint64_t* keys_in, uint64_t* keys_out, uint32_t* perm_out, int64_t n,
                                    void* stream)
{
    if (n < 0 || (n > 0 && (!keys_in || !keys_out || !perm_out)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_sort_keys_noalloc: null buffer or negative n");
    if (n > kMaxKeys)
        return bh_fail(BH_ERR_CAPACITY, "bh_sort_keys_noalloc: n = " + std::to_string(n) +
                                            " exceeds the fixed scratch of " + std::to_string(kMaxKeys) + " keys");
    if (n == 0) return BH_OK;
    int dev = 0;
    BH_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_sort_keys_noalloc: device id");
    unsigned char* base = nullptr;
    int rc = scratch_address(dev, &base);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint64_t* key_alt = reinterpret_cast<uint64_t*>(base + kOffKeyAlt);
    uint32_t* val_alt = reinterpret_cast<uint32_t*>(base + kOffValAlt);
    uint32_t* hist = reinterpret_cast<uint32_t*>(base + kOffHist);
    uint32_t* lookback = reinterpret_cast<uint32_t*>(base + kOffLookback);
    uint32_t* tile_ctr = reinterpret_cast<uint32_t*>(base + kOffTileCtr);
    unsigned* err = reinterpret_cast<unsigned*>(base + kOffErr);

    if (n == 1) {
        if (keys_out != keys_in)
            BH_CUDA_TRY(cudaMemcpyAsync(keys_out, keys_in, sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
        BH_CUDA_TRY(cudaMemsetAsync(perm_out, 0, sizeof(uint32_t), st));
        BH_CUDA_TRY(cudaStreamSynchronize(st));
        return BH_OK;
    }
    // Clear what must start at zero: histograms, the look-back words of the
    // tiles this call uses, tile counters, the error word.
    const int64_t tiles = (n + bh::kSortTile - 1) / bh::kSortTile;
    BH_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(uint32_t) * bh::kSortPasses * bh::kRadix, st));
    BH_CUDA_TRY(cudaMemsetAsync(lookback, 0, sizeof(uint32_t) * bh::kSortPasses * tiles * bh::kRadix, st));
    BH_CUDA_TRY(cudaMemsetAsync(tile_ctr, 0, sizeof(uint32_t) * bh::kSortPasses, st));
    BH_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
    if ((rc = bh::launch_digit_hist(n, keys_in, hist, st))) return rc;
    if ((rc = bh::sort_passes_raw(n, keys_in, keys_out, perm_out, key_alt, val_alt, hist, lookback, tile_ctr, err,
                                  st)))
        return rc;
    unsigned h_err = 0;
    BH_CUDA_TRY(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    BH_CUDA_TRY(cudaStreamSynchronize(st));
    if (h_err & bh::kErrTimeout) return bh_fail(BH_ERR_TIMEOUT, "bh_sort_keys_noalloc: a bounded device wait gave up");
    return BH_OK;
}
