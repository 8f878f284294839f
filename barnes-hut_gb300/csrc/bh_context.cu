// The C ABI of libbh_gpu.so: context lifetime, device memory, host <-> device
// transfers, the hot path stage by stage, the step loop and the stateless
// host-buffer entry points.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "bh_internal.cuh"

namespace {

thread_local std::string g_last_error;

constexpr int64_t kMaxBodies = (1ll << 30) - 1;  // sort counts are 30-bit

// AoS (x,y,z per body) <-> SoA conversion kernels for the transfers.
__global__ void deinterleave_kernel(int64_t n, const double* __restrict__ aos, double* __restrict__ x,
                                    double* __restrict__ y, double* __restrict__ z)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = aos[3 * i];
        y[i] = aos[3 * i + 1];
        z[i] = aos[3 * i + 2];
    }
}

__global__ void interleave_kernel(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                                  const double* __restrict__ z, double* __restrict__ aos)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        aos[3 * i] = x[i];
        aos[3 * i + 1] = y[i];
        aos[3 * i + 2] = z[i];
    }
}

int grid256(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b < 1) b = 1;
    return (int)std::min<int64_t>(b, 8 * bh::num_sms());
}

// Carves one device allocation into aligned sub-buffers.
struct Carver {
    char* base = nullptr;
    size_t off = 0;
    template <class T>
    T* take(int64_t count)
    {
        off = (off + 255) & ~size_t(255);
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += sizeof(T) * (size_t)std::max<int64_t>(count, 1);
        return p;
    }
};

// Lays out every buffer of a context of capacity `cap`; with c.base null it
// only measures.
void layout(bh_context* ctx, Carver& c)
{
    const int64_t n = ctx->cap;
    // Body set A and B: pos/vel blocks are contiguous (3n) so that each can
    // serve as an AoS staging buffer for transfers.
    double* posA = c.take<double>(3 * n);
    double* velA = c.take<double>(3 * n);
    double* accA = c.take<double>(3 * n);
    double* posB = c.take<double>(3 * n);
    double* velB = c.take<double>(3 * n);
    ctx->px = posA; ctx->py = posA ? posA + n : nullptr; ctx->pz = posA ? posA + 2 * n : nullptr;
    ctx->vx = velA; ctx->vy = velA ? velA + n : nullptr; ctx->vz = velA ? velA + 2 * n : nullptr;
    ctx->ax = accA; ctx->ay = accA ? accA + n : nullptr; ctx->az = accA ? accA + 2 * n : nullptr;
    ctx->px2 = posB; ctx->py2 = posB ? posB + n : nullptr; ctx->pz2 = posB ? posB + 2 * n : nullptr;
    ctx->vx2 = velB; ctx->vy2 = velB ? velB + n : nullptr; ctx->vz2 = velB ? velB + 2 * n : nullptr;
    ctx->m = c.take<double>(n);
    ctx->m2 = c.take<double>(n);
    ctx->id = c.take<uint64_t>(n);
    ctx->id2 = c.take<uint64_t>(n);
    ctx->key = c.take<uint64_t>(n);
    ctx->key_alt = c.take<uint64_t>(n);
    ctx->perm = c.take<uint32_t>(n);
    ctx->perm_alt = c.take<uint32_t>(n);
    ctx->hist = c.take<uint32_t>(bh::kSortPasses * bh::kRadix);
    ctx->max_tiles = (n + bh::kSortTile - 1) / bh::kSortTile;
    ctx->lookback = c.take<uint32_t>(bh::kSortPasses * ctx->max_tiles * bh::kRadix);
    ctx->tile_ctr = c.take<uint32_t>(bh::kSortPasses);
    ctx->bbox = c.take<double>(8);
    ctx->bbox_blocks = (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 4 * bh::num_sms());
    ctx->bbox_part = reinterpret_cast<double*>(c.take<char>(bh::bbox_partial_bytes(ctx->bbox_blocks)));
    ctx->bbox_ticket = c.take<unsigned>(1);
    ctx->head = c.take<int32_t>(n + 1);
    ctx->leaf_first = c.take<int32_t>(n + 1);
    ctx->body_leaf = c.take<int32_t>(n);
    ctx->leaf_key = c.take<uint64_t>(n);
    ctx->leaf_s = c.take<double4_32a>(n);
    ctx->cdep = c.take<int8_t>(n + 1);
    ctx->bnd_pl = c.take<int32_t>(n + 1);
    ctx->bnd_pr = c.take<int32_t>(n + 1);
    ctx->bnd_next = c.take<int32_t>(n + 1);
    ctx->split_node = c.take<int32_t>(n + 1);
    ctx->split_rank = c.take<int8_t>(n + 1);
    ctx->ansv_blk = c.take<int32_t>(bh::boundary_pass_ints(n));
    ctx->rep_node = c.take<int32_t>(n);
    ctx->node_rep = c.take<int32_t>(n);
    ctx->node_a = c.take<int32_t>(n);
    ctx->node_e = c.take<int32_t>(n);
    ctx->node_nchild = c.take<int32_t>(n);
    ctx->node_cs = c.take<int32_t>(n);
    ctx->node_depth = c.take<uint8_t>(n);
    ctx->node_s = c.take<double4_32a>(n);
    ctx->slot_ref = c.take<int32_t>(2 * n);
    ctx->slot_top = c.take<uint8_t>(2 * n);
    ctx->depth_off = c.take<int32_t>(32);
    ctx->depth_nodes = c.take<int32_t>(n);
    ctx->rec = c.take<bh::TreeRec>(2 * n);
    ctx->counts = c.take<int32_t>(16);
    const int64_t nblk = (n + 1023) / 1024;
    ctx->scan_tmp = c.take<int32_t>(std::max<int64_t>(bh::scan_tmp_ints(2 * n), 21 * nblk + 64));
    ctx->inter_count = c.take<unsigned long long>(1);
    ctx->body_count = c.take<int32_t>(n);
    ctx->fA = c.take<float4>(2 * n);
    ctx->fB = c.take<float4>(2 * n);
    ctx->fmeta = c.take<uint32_t>(2 * n);
    ctx->d4 = c.take<double4_32a>(2 * n);
    ctx->fspread = c.take<float>(2 * n);
    ctx->leaf_q = c.take<double>(n);
    ctx->node_q = c.take<double>(n);
    ctx->lstats = c.take<unsigned long long>(4);
    ctx->direct = c.take<double>(4 * 64);
    ctx->direct_present = c.take<int32_t>(64);
    ctx->err = c.take<unsigned>(1);
}

int check_ctx(bh_context* ctx, const char* fn)
{
    if (!ctx) return bh_fail(BH_ERR_INVALID_ARGUMENT, std::string(fn) + ": null context");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return bh_fail(BH_ERR_CUDA, std::string(fn) + ": cudaSetDevice: " + cudaGetErrorString(e));
    return BH_OK;
}

void collect_phases(bh_context* ctx);

}  // namespace

// Waits for the stream and turns a raised device error word into a status.
int bh::num_sms()
{
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cache[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) return 1;
    cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

int bh::finish(bh_context* ctx, const char* fn)
{
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_err, ctx->err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (ctx->prof) collect_phases(ctx);
    const unsigned e = *ctx->h_err;
    if (!e) return BH_OK;
    BH_CUDA_TRY(cudaMemsetAsync(ctx->err, 0, sizeof(unsigned), ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (e & bh::kErrNonFinite) return bh_fail(BH_ERR_NONFINITE, std::string(fn) + ": non-finite position");
    if (e & bh::kErrTimeout) return bh_fail(BH_ERR_TIMEOUT, std::string(fn) + ": a bounded device wait gave up");
    if (e & bh::kErrOverflow) return bh_fail(BH_ERR_OVERFLOW, std::string(fn) + ": traversal stack overflow");
    return bh_fail(BH_ERR_CUDA, std::string(fn) + ": device error word set");
}

namespace {
using bh::finish;

int upload_vec3(bh_context* ctx, const double* host_aos, double* stage, double* x, double* y, double* z, int64_t n)
{
    BH_CUDA_TRY(cudaMemcpyAsync(stage, host_aos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
    deinterleave_kernel<<<grid256(n), 256, 0, ctx->stream>>>(n, stage, x, y, z);
    BH_LAUNCH_CHECK(ctx);
    return BH_OK;
}

int download_vec3(bh_context* ctx, double* host_aos, double* stage, const double* x, const double* y,
                  const double* z, int64_t n)
{
    interleave_kernel<<<grid256(n), 256, 0, ctx->stream>>>(n, x, y, z, stage);
    BH_LAUNCH_CHECK(ctx);
    BH_CUDA_TRY(cudaMemcpyAsync(host_aos, stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    return BH_OK;
}

cudaEvent_t next_event(bh_context* ctx)
{
    if (ctx->ev_used == ctx->ev_pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ctx->ev_pool.push_back(e);
    }
    return ctx->ev_pool[ctx->ev_used++];
}

// Phase markers: begin() records an event and returns it; end() records the
// closing event and remembers the pair (no-ops unless profiling).
cudaEvent_t phase_begin(bh_context* ctx)
{
    if (!ctx->prof) return nullptr;
    cudaEvent_t a = next_event(ctx);
    if (a) cudaEventRecord(a, ctx->stream);
    return a;
}

void phase_end(bh_context* ctx, int phase, cudaEvent_t a)
{
    if (!ctx->prof || !a) return;
    cudaEvent_t b = next_event(ctx);
    if (!b) return;
    cudaEventRecord(b, ctx->stream);
    ctx->marks.push_back({phase, a, b});
}

// After a synchronisation: fold the recorded phase pairs into phase_ms.
void collect_phases(bh_context* ctx)
{
    for (const auto& mk : ctx->marks) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, mk.a, mk.b) == cudaSuccess) ctx->phase_ms[mk.phase] += ms;
    }
    ctx->marks.clear();
    ctx->ev_used = 0;
}

// The whole step of src/main.cpp:191-282 (`--fc tree`, one rank).
// Phases: 0 kick+drift+bbox, 1 keys, 2 sort, 3 permute, 4 build, 5 forces+kick.
int step_once(bh_context* ctx, double dt, double theta, double G, int mode)
{
    const bool kick = ctx->t > 0;
    const bool far = mode >= BH_MODE_FP32_FAR;
    cudaEvent_t e = phase_begin(ctx);
    int rc = bh::launch_drift_bbox(ctx, dt, kick, true);
    phase_end(ctx, 0, e);
    e = phase_begin(ctx);
    if (!rc) rc = bh::launch_keys(ctx, true);
    phase_end(ctx, 1, e);
    e = phase_begin(ctx);
    if (!rc) rc = bh::launch_sort(ctx);
    phase_end(ctx, 2, e);
    e = phase_begin(ctx);
    if (!rc) rc = bh::launch_permute(ctx);
    phase_end(ctx, 3, e);
    e = phase_begin(ctx);
    const bool moments = mode == BH_MODE_LEARNED;
    if (!rc) rc = bh::launch_build(ctx, ctx->m, moments, far, G, far);
    ctx->tree_far = far;
    ctx->tree_moments = moments;
    phase_end(ctx, 4, e);
    e = phase_begin(ctx);
    if (!rc) rc = bh::launch_traverse(ctx, theta, G, 0.0, mode, 0.5 * dt);
    phase_end(ctx, 5, e);
    return rc;
}

// A step with the kick (every step of a run after its first) through a CUDA
// graph: captured from step_once on first use for this (bodies, mode, dt,
// theta, G, merge, direct-body count) configuration, then replayed, which
// enqueues the step's ~50 kernels with one call.  The step reads one body set
// and leaves the state in the other, so there is one graph per starting set;
// after a replay the host pointers trade places as step_once's permutation
// would make them.  The kernels read no host state that the key leaves out:
// buffers live in the context's single allocation, the learned model in a
// fixed device block, and the learned walk's scalar parameters (baked into
// its launch) are part of the key.
int step_graph(bh_context* ctx, double dt, double theta, double G, int mode)
{
    const int merge = ctx->build_merge ? 1 : 0;
    const double learn[4] = {ctx->learn_theta_max, ctx->learn_budget, ctx->learn_band, ctx->learn_frac};
    bh_context::StepGraph& g = ctx->sg[ctx->px < ctx->px2 ? 0 : 1];
    const bool same_learn = mode != BH_MODE_LEARNED || std::equal(learn, learn + 4, g.learn);
    if (!(g.exec && g.n == ctx->n && g.mode == mode && g.dt == dt && g.theta == theta && g.G == G &&
          g.merge == merge && g.nd == ctx->num_direct && same_learn)) {
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        const int64_t l0 = ctx->launches;
        BH_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
        const int rc = step_once(ctx, dt, theta, G, mode);
        bh::swap_body_sets(ctx);  // capturing ran no kernel: back to the starting set
        const int64_t captured = ctx->launches - l0;
        ctx->launches = l0;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
        if (rc || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return rc ? rc : bh_fail(BH_ERR_CUDA, std::string("bh_step: graph capture: ") + cudaGetErrorString(e));
        }
        e = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            g.exec = nullptr;
            return bh_fail(BH_ERR_CUDA, std::string("bh_step: graph instantiation: ") + cudaGetErrorString(e));
        }
        g.launches = captured;
        g.n = ctx->n;
        g.mode = mode;
        g.dt = dt;
        g.theta = theta;
        g.G = G;
        g.merge = merge;
        g.nd = ctx->num_direct;
        std::copy(learn, learn + 4, g.learn);
    }
    BH_CUDA_TRY(cudaGraphLaunch(g.exec, ctx->stream));
    bh::swap_body_sets(ctx);
    ctx->launches += g.launches;
    ctx->tree_far = mode >= BH_MODE_FP32_FAR;
    ctx->tree_moments = mode == BH_MODE_LEARNED;
    return BH_OK;
}

}  // namespace

int bh_fail(int status, const std::string& msg)
{
    g_last_error = msg;
    return status;
}

void bh_clear_error() { g_last_error.clear(); }

extern "C" {

const char* bh_last_error(void) { return g_last_error.c_str(); }

const char* bh_status_string(int status)
{
    switch (status) {
    case BH_OK: return "ok";
    case BH_ERR_INVALID_ARGUMENT: return "invalid argument";
    case BH_ERR_CUDA: return "CUDA error";
    case BH_ERR_OUT_OF_MEMORY: return "out of memory";
    case BH_ERR_CAPACITY: return "capacity exceeded";
    case BH_ERR_OVERFLOW: return "traversal overflow";
    case BH_ERR_TIMEOUT: return "device wait timed out";
    case BH_ERR_NONFINITE: return "non-finite position";
    case BH_ERR_STATE: return "call out of order";
    case BH_ERR_IO: return "I/O error";
    case BH_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

int bh_api_version(void) { return BH_API_VERSION; }

int bh_context_create(int64_t capacity, int device, bh_context** out)
{
    if (!out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_context_create: null out");
    *out = nullptr;
    if (capacity < 1 || capacity > kMaxBodies)
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_context_create: capacity must be in [1, 2^30)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return bh_fail(BH_ERR_NO_DEVICE, "bh_context_create: no CUDA device");
    }
    if (device < 0 || device >= ndev) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_context_create: bad device");
    BH_CUDA_TRY(cudaSetDevice(device));
    std::unique_ptr<bh_context> ctx(new bh_context);
    ctx->device = device;
    ctx->cap = capacity;
    Carver measure;
    layout(ctx.get(), measure);
    char* base = nullptr;
    cudaError_t e = cudaMalloc(&base, measure.off);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bh_fail(BH_ERR_OUT_OF_MEMORY, "bh_context_create: cudaMalloc of " + std::to_string(measure.off) + " bytes failed");
    }
    Carver carve;
    carve.base = base;
    layout(ctx.get(), carve);
    ctx->alloc_base = base;
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_err, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_small, 64 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(base, 0, measure.off, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(base);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        if (ctx->h_err) cudaFreeHost(ctx->h_err);
        if (ctx->h_small) cudaFreeHost(ctx->h_small);
        return bh_fail(BH_ERR_CUDA, std::string("bh_context_create: ") + cudaGetErrorString(e));
    }
    *out = ctx.release();
    return BH_OK;
}

int bh_context_destroy(bh_context* ctx)
{
    if (!ctx) return BH_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->alloc_base);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->h_err) cudaFreeHost(ctx->h_err);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->mlp_dev) cudaFree(ctx->mlp_dev);
    if (ctx->let_buf) cudaFree(ctx->let_buf);
    if (ctx->imp_buf) cudaFree(ctx->imp_buf);
    if (ctx->imp_buf2) cudaFree(ctx->imp_buf2);
    if (ctx->letf_buf) cudaFree(ctx->letf_buf);
    for (auto& g : ctx->sg)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    delete ctx;
    return BH_OK;
}

int bh_set_step_graphs(bh_context* ctx, int on)
{
    if (!ctx) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_set_step_graphs: null context");
    ctx->graphs = on != 0;
    return BH_OK;
}

int bh_set_profiling(bh_context* ctx, int on)
{
    if (!ctx) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_set_profiling: null context");
    ctx->prof = on != 0;
    for (double& v : ctx->phase_ms) v = 0.0;
    ctx->marks.clear();
    ctx->ev_used = 0;
    return BH_OK;
}

int bh_phase_times(bh_context* ctx, double ms_out[8], int64_t* launches_out)
{
    if (!ctx) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_phase_times: null context");
    if (ms_out)
        for (int k = 0; k < 8; ++k) ms_out[k] = ctx->phase_ms[k];
    if (launches_out) *launches_out = ctx->launches;
    return BH_OK;
}

int bh_context_sync(bh_context* ctx)
{
    int rc = check_ctx(ctx, "bh_context_sync");
    if (rc) return rc;
    return finish(ctx, "bh_context_sync");
}

int bh_context_stream(bh_context* ctx, void** stream_out)
{
    if (!ctx || !stream_out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_context_stream: null argument");
    *stream_out = (void*)ctx->stream;
    return BH_OK;
}

int bh_set_bodies(bh_context* ctx, int64_t n, const double* pos, const double* vel, const double* mass,
                  const uint64_t* ids)
{
    int rc = check_ctx(ctx, "bh_set_bodies");
    if (rc) return rc;
    if (n < 0) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_set_bodies: negative n");
    if (n > ctx->cap) return bh_fail(BH_ERR_CAPACITY, "bh_set_bodies: more bodies than the context capacity");
    if (n > 0 && (!pos || !vel || !mass || !ids)) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_set_bodies: null array");
    ctx->n = n;
    ctx->t = 0.0;
    ctx->tree_valid = ctx->keys_valid = ctx->bbox_valid = ctx->sorted_valid = false;
    if (n == 0) return BH_OK;
    // Staging: the second body set's pos and vel blocks (3n doubles each).
    if ((rc = upload_vec3(ctx, pos, ctx->px2, ctx->px, ctx->py, ctx->pz, n))) return rc;
    if ((rc = upload_vec3(ctx, vel, ctx->vx2, ctx->vx, ctx->vy, ctx->vz, n))) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->m, mass, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->id, ids, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, ctx->stream));
    BH_CUDA_TRY(cudaMemsetAsync(ctx->ax, 0, sizeof(double) * n, ctx->stream));
    BH_CUDA_TRY(cudaMemsetAsync(ctx->ay, 0, sizeof(double) * n, ctx->stream));
    BH_CUDA_TRY(cudaMemsetAsync(ctx->az, 0, sizeof(double) * n, ctx->stream));
    return finish(ctx, "bh_set_bodies");
}

int bh_set_accelerations(bh_context* ctx, const double* acc)
{
    int rc = check_ctx(ctx, "bh_set_accelerations");
    if (rc) return rc;
    if (ctx->n == 0) return BH_OK;
    if (!acc) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_set_accelerations: null array");
    if ((rc = upload_vec3(ctx, acc, ctx->px2, ctx->ax, ctx->ay, ctx->az, ctx->n))) return rc;
    return finish(ctx, "bh_set_accelerations");
}

int bh_get_bodies(bh_context* ctx, double* pos, double* vel, double* mass, uint64_t* ids, double* acc)
{
    int rc = check_ctx(ctx, "bh_get_bodies");
    if (rc) return rc;
    const int64_t n = ctx->n;
    if (n == 0) return BH_OK;
    if (pos && (rc = download_vec3(ctx, pos, ctx->px2, ctx->px, ctx->py, ctx->pz, n))) return rc;
    if (vel && (rc = download_vec3(ctx, vel, ctx->vx2, ctx->vx, ctx->vy, ctx->vz, n))) return rc;
    // The acceleration download reuses the position staging block after the
    // position copy on the same stream: stream order keeps them apart.
    if (acc && (rc = download_vec3(ctx, acc, ctx->px2, ctx->ax, ctx->ay, ctx->az, n))) return rc;
    if (mass) BH_CUDA_TRY(cudaMemcpyAsync(mass, ctx->m, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (ids) BH_CUDA_TRY(cudaMemcpyAsync(ids, ctx->id, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    return finish(ctx, "bh_get_bodies");
}

int bh_num_bodies(bh_context* ctx, int64_t* n_out)
{
    if (!ctx || !n_out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_num_bodies: null argument");
    *n_out = ctx->n;
    return BH_OK;
}

int bh_compute_bbox(bh_context* ctx, double bbox_out[6])
{
    int rc = check_ctx(ctx, "bh_compute_bbox");
    if (rc) return rc;
    if (ctx->n == 0) {
        if (bbox_out) {
            for (int a = 0; a < 3; ++a) { bbox_out[a] = INFINITY; bbox_out[3 + a] = -INFINITY; }
        }
        return BH_OK;
    }
    if ((rc = bh::launch_drift_bbox(ctx, 0.0, false, false))) return rc;
    if (bbox_out)
        BH_CUDA_TRY(cudaMemcpyAsync(bbox_out, ctx->bbox, 6 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    rc = finish(ctx, "bh_compute_bbox");
    ctx->bbox_valid = rc == BH_OK;
    return rc;
}

int bh_compute_keys(bh_context* ctx, uint64_t* keys_out)
{
    int rc = check_ctx(ctx, "bh_compute_keys");
    if (rc) return rc;
    if (!ctx->bbox_valid && ctx->n > 0) return bh_fail(BH_ERR_STATE, "bh_compute_keys: call bh_compute_bbox first");
    if ((rc = bh::launch_keys(ctx, true))) return rc;
    if (keys_out && ctx->n)
        BH_CUDA_TRY(cudaMemcpyAsync(keys_out, ctx->key, sizeof(uint64_t) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
    rc = finish(ctx, "bh_compute_keys");
    ctx->keys_valid = rc == BH_OK;
    ctx->tree_valid = ctx->sorted_valid = false;
    return rc;
}

int bh_sort_bodies(bh_context* ctx, int64_t* perm_out)
{
    int rc = check_ctx(ctx, "bh_sort_bodies");
    if (rc) return rc;
    if (!ctx->keys_valid && ctx->n > 0) return bh_fail(BH_ERR_STATE, "bh_sort_bodies: call bh_compute_keys first");
    if ((rc = bh::launch_sort(ctx))) return rc;
    if ((rc = bh::launch_permute(ctx))) return rc;
    std::vector<uint32_t> p;
    if (perm_out && ctx->n) {
        p.resize(ctx->n);
        BH_CUDA_TRY(cudaMemcpyAsync(p.data(), ctx->perm, sizeof(uint32_t) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    rc = finish(ctx, "bh_sort_bodies");
    if (rc) return rc;
    for (size_t i = 0; i < p.size(); ++i) perm_out[i] = (int64_t)p[i];
    ctx->keys_valid = false;  // histograms consumed; keys stay sorted
    ctx->tree_valid = false;
    ctx->sorted_valid = true;
    return BH_OK;
}

int bh_set_keys(bh_context* ctx, const uint64_t* keys)
{
    int rc = check_ctx(ctx, "bh_set_keys");
    if (rc) return rc;
    if (ctx->n == 0) return BH_OK;
    if (!keys) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_set_keys: null keys");
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->key, keys, sizeof(uint64_t) * ctx->n, cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = bh::launch_hist(ctx))) return rc;
    rc = finish(ctx, "bh_set_keys");
    ctx->keys_valid = rc == BH_OK;
    ctx->tree_valid = ctx->sorted_valid = false;
    return rc;
}

int bh_set_bbox(bh_context* ctx, const double bbox[6])
{
    int rc = check_ctx(ctx, "bh_set_bbox");
    if (rc) return rc;
    if (!bbox) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_set_bbox: null bbox");
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->bbox, bbox, 6 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    rc = finish(ctx, "bh_set_bbox");
    ctx->bbox_valid = rc == BH_OK;
    return rc;
}

int bh_build_tree_options(bh_context* ctx, int merge)
{
    int rc = check_ctx(ctx, "bh_build_tree_options");
    if (rc) return rc;
    ctx->build_merge = merge != 0;
    rc = bh_build_tree(ctx);
    ctx->build_merge = true;
    return rc;
}

int bh_build_tree(bh_context* ctx)
{
    int rc = check_ctx(ctx, "bh_build_tree");
    if (rc) return rc;
    if (!ctx->sorted_valid && ctx->n > 0) return bh_fail(BH_ERR_STATE, "bh_build_tree: call bh_sort_bodies first");
    if ((rc = bh::launch_build(ctx, ctx->m))) return rc;
    ctx->tree_far = ctx->tree_moments = false;
    rc = finish(ctx, "bh_build_tree");
    ctx->tree_valid = rc == BH_OK;
    return rc;
}

}  // extern "C"

namespace {

struct HostTree {
    int32_t L = 0, B = 0, S = 0;
    std::vector<bh::TreeRec> rec;
    std::vector<int32_t> slot_ref, node_a;
    std::vector<uint64_t> leaf_key;
};

int fetch_tree(bh_context* ctx, HostTree& h)
{
    if (int rc = bh::ensure_rec(ctx)) return rc;
    int32_t c[4];
    BH_CUDA_TRY(cudaMemcpyAsync(c, ctx->counts, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    h.L = c[0]; h.B = c[1]; h.S = c[2];
    h.rec.resize(h.S);
    h.slot_ref.resize(h.S);
    h.node_a.resize(std::max(h.B, 1));
    h.leaf_key.resize(h.L);
    BH_CUDA_TRY(cudaMemcpyAsync(h.rec.data(), ctx->rec, sizeof(bh::TreeRec) * h.S, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(h.slot_ref.data(), ctx->slot_ref, sizeof(int32_t) * h.S, cudaMemcpyDeviceToHost, ctx->stream));
    if (h.B) BH_CUDA_TRY(cudaMemcpyAsync(h.node_a.data(), ctx->node_a, sizeof(int32_t) * h.B, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(h.leaf_key.data(), ctx->leaf_key, sizeof(uint64_t) * h.L, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return BH_OK;
}

}  // namespace

extern "C" {

int bh_tree_info(bh_context* ctx, int64_t* n_records, int64_t* n_nodes, int64_t* n_leaves)
{
    int rc = check_ctx(ctx, "bh_tree_info");
    if (rc) return rc;
    if (!ctx->tree_valid) {
        if (ctx->n == 0) {
            if (n_records) *n_records = 0;
            if (n_nodes) *n_nodes = 0;
            if (n_leaves) *n_leaves = 0;
            return BH_OK;
        }
        return bh_fail(BH_ERR_STATE, "bh_tree_info: no tree built");
    }
    if (!n_records) {  // the counts alone: no copy of the tree
        int32_t c[4];
        BH_CUDA_TRY(cudaMemcpyAsync(c, ctx->counts, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream));
        BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        if (n_nodes) *n_nodes = c[2];
        if (n_leaves) *n_leaves = c[0];
        return BH_OK;
    }
    HostTree h;
    if ((rc = fetch_tree(ctx, h))) return rc;
    int64_t recs = 0;
    for (const auto& r : h.rec) recs += (int64_t)r.depth - r.top + 1;
    *n_records = recs;
    if (n_nodes) *n_nodes = h.S;
    if (n_leaves) *n_leaves = h.L;
    return BH_OK;
}

int bh_export_tree(bh_context* ctx, uint64_t* prefix, uint8_t* depth, double* mass, double* com)
{
    int rc = check_ctx(ctx, "bh_export_tree");
    if (rc) return rc;
    if (!ctx->tree_valid) return ctx->n == 0 ? BH_OK : bh_fail(BH_ERR_STATE, "bh_export_tree: no tree built");
    if (!prefix || !depth || !mass || !com) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_export_tree: null array");
    if (ctx->tree_far) {  // the export is the reference's tree: real masses
        if ((rc = bh::launch_build(ctx, ctx->m))) return rc;
        ctx->tree_far = ctx->tree_moments = false;
    }
    HostTree h;
    if ((rc = fetch_tree(ctx, h))) return rc;
    struct Out { uint64_t p; uint8_t d; int32_t s; };
    std::vector<Out> v;
    for (int32_t s = 0; s < h.S; ++s) {
        const bh::TreeRec& r = h.rec[s];
        const int32_t ref = h.slot_ref[s];
        const int32_t first = ref >= 0 ? ref : h.node_a[~ref];
        const uint64_t k = h.leaf_key[first];
        for (int d = r.top; d <= r.depth; ++d) v.push_back({k & bh::prefix_mask(d), (uint8_t)d, s});
    }
    std::sort(v.begin(), v.end(), [](const Out& a, const Out& b) { return a.d != b.d ? a.d < b.d : a.p < b.p; });
    for (size_t i = 0; i < v.size(); ++i) {
        const bh::TreeRec& r = h.rec[v[i].s];
        prefix[i] = v[i].p;
        depth[i] = v[i].d;
        mass[i] = r.m;
        com[3 * i] = r.cx;
        com[3 * i + 1] = r.cy;
        com[3 * i + 2] = r.cz;
    }
    return BH_OK;
}

int bh_tree_slots(bh_context* ctx, uint64_t* prefix, uint8_t* depth)
{
    int rc = check_ctx(ctx, "bh_tree_slots");
    if (rc) return rc;
    if (!ctx->tree_valid) return ctx->n == 0 ? BH_OK : bh_fail(BH_ERR_STATE, "bh_tree_slots: no tree built");
    if (!prefix || !depth) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_tree_slots: null array");
    HostTree h;
    if ((rc = fetch_tree(ctx, h))) return rc;
    for (int32_t s = 0; s < h.S; ++s) {
        const int32_t ref = h.slot_ref[s];
        const int32_t first = ref >= 0 ? ref : h.node_a[~ref];
        depth[s] = h.rec[s].depth;
        prefix[s] = h.leaf_key[first] & bh::prefix_mask(h.rec[s].depth);
    }
    return BH_OK;
}

int bh_tree_spread(bh_context* ctx, float* spread)
{
    int rc = check_ctx(ctx, "bh_tree_spread");
    if (rc) return rc;
    if (!ctx->tree_valid) return ctx->n == 0 ? BH_OK : bh_fail(BH_ERR_STATE, "bh_tree_spread: no tree built");
    if (!spread) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_tree_spread: null array");
    if (!ctx->tree_far || !ctx->tree_moments) {
        if ((rc = bh::launch_build(ctx, ctx->m, true, false, 0.0, true))) return rc;
        ctx->tree_far = ctx->tree_moments = true;
    }
    int32_t S = 0;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, ctx->counts + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    std::memcpy(&S, ctx->h_small, sizeof(int32_t));
    if (S > 0)
        BH_CUDA_TRY(cudaMemcpyAsync(spread, ctx->fspread, sizeof(float) * S, cudaMemcpyDeviceToHost, ctx->stream));
    return finish(ctx, "bh_tree_spread");
}

int bh_tree_set_slot_values(bh_context* ctx, const double* mass, const double* com)
{
    int rc = check_ctx(ctx, "bh_tree_set_slot_values");
    if (rc) return rc;
    if (!ctx->tree_valid) return ctx->n == 0 ? BH_OK : bh_fail(BH_ERR_STATE, "bh_tree_set_slot_values: no tree");
    if (!mass || !com) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_tree_set_slot_values: null array");
    HostTree h;
    if ((rc = fetch_tree(ctx, h))) return rc;
    for (int32_t s = 0; s < h.S; ++s) {
        h.rec[s].m = mass[s];
        h.rec[s].cx = com[3 * s];
        h.rec[s].cy = com[3 * s + 1];
        h.rec[s].cz = com[3 * s + 2];
    }
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->rec, h.rec.data(), sizeof(bh::TreeRec) * h.S, cudaMemcpyHostToDevice, ctx->stream));
    ctx->tree_far = ctx->tree_moments = false;
    ctx->fnodes_fused = false;
    return finish(ctx, "bh_tree_set_slot_values");
}

int bh_compute_accelerations(bh_context* ctx, double theta, double G, double soft2, int mode, double* acc_out)
{
    int rc = check_ctx(ctx, "bh_compute_accelerations");
    if (rc) return rc;
    if (!(theta >= 0.0) || !(soft2 >= 0.0)) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_compute_accelerations: theta and soft2 must be >= 0");
    if (ctx->n == 0) return BH_OK;
    if (!ctx->tree_valid) return bh_fail(BH_ERR_STATE, "bh_compute_accelerations: call bh_build_tree first");
    // The FP32 modes read a tree built over the far-field masses (direct
    // bodies zeroed); the FP64 modes the reference's tree.  Rebuild the
    // node values when the tree in place is the other kind.
    const bool far = mode >= BH_MODE_FP32_FAR;
    const bool moments = mode == BH_MODE_LEARNED;
    if (far != ctx->tree_far || (moments && !ctx->tree_moments)) {
        if ((rc = bh::launch_build(ctx, ctx->m, moments, false, 0.0, far))) return rc;
        ctx->tree_far = far;
        ctx->tree_moments = moments;
    }
    if ((rc = bh::launch_traverse(ctx, theta, G, soft2, mode, 0.0))) return rc;
    if (acc_out && (rc = download_vec3(ctx, acc_out, ctx->px2, ctx->ax, ctx->ay, ctx->az, ctx->n))) return rc;
    return finish(ctx, "bh_compute_accelerations");
}

int bh_interaction_counts(bh_context* ctx, int32_t* per_body)
{
    int rc = check_ctx(ctx, "bh_interaction_counts");
    if (rc) return rc;
    if (!per_body) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_interaction_counts: null out");
    if (ctx->n == 0) return BH_OK;
    BH_CUDA_TRY(cudaMemcpyAsync(per_body, ctx->body_count, sizeof(int32_t) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
    return finish(ctx, "bh_interaction_counts");
}

int bh_interaction_count(bh_context* ctx, int64_t* total_out)
{
    int rc = check_ctx(ctx, "bh_interaction_count");
    if (rc) return rc;
    if (!total_out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_interaction_count: null out");
    unsigned long long v = 0;
    BH_CUDA_TRY(cudaMemcpyAsync(&v, ctx->inter_count, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *total_out = (int64_t)v;
    return BH_OK;
}

int bh_step(bh_context* ctx, double dt, double theta, double G, int64_t nsteps, int mode, double* t_io)
{
    int rc = check_ctx(ctx, "bh_step");
    if (rc) return rc;
    if (nsteps < 0 || !(theta >= 0.0)) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_step: bad nsteps or theta");
    if (t_io) ctx->t = *t_io;
    for (int64_t s = 0; s < nsteps; ++s) {
        if (ctx->n > 0) {
            const bool graph = ctx->graphs && !ctx->prof && ctx->t > 0;
            if ((rc = graph ? step_graph(ctx, dt, theta, G, mode) : step_once(ctx, dt, theta, G, mode))) return rc;
        }
        ctx->t += dt;
    }
    rc = finish(ctx, "bh_step");
    if (t_io) *t_io = ctx->t;
    if (nsteps > 0 && ctx->n > 0) {
        ctx->tree_valid = ctx->sorted_valid = ctx->bbox_valid = rc == BH_OK;
        ctx->keys_valid = false;
    }
    return rc;
}

int bh_step_host(bh_context* ctx, int64_t n, double* pos, double* vel, double* mass, uint64_t* ids, double* acc,
                 double dt, double theta, double G, int64_t nsteps, int mode, double* t_io)
{
    int rc = check_ctx(ctx, "bh_step_host");
    if (rc) return rc;
    if (n < 0 || nsteps < 0 || !(theta >= 0.0))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_step_host: bad n, nsteps or theta");
    if (n > ctx->cap) return bh_fail(BH_ERR_CAPACITY, "bh_step_host: more bodies than the context capacity");
    if (n > 0 && (!pos || !vel || !mass || !ids || !acc))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_step_host: null array");
    // bh_set_bodies and bh_set_accelerations, without their waits: every
    // copy and kernel below runs in the order of the context's stream.
    ctx->n = n;
    ctx->t = t_io ? *t_io : 0.0;
    ctx->tree_valid = ctx->keys_valid = ctx->bbox_valid = ctx->sorted_valid = false;
    if (n > 0) {
        if ((rc = upload_vec3(ctx, pos, ctx->px2, ctx->px, ctx->py, ctx->pz, n))) return rc;
        if ((rc = upload_vec3(ctx, vel, ctx->vx2, ctx->vx, ctx->vy, ctx->vz, n))) return rc;
        BH_CUDA_TRY(cudaMemcpyAsync(ctx->m, mass, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        BH_CUDA_TRY(cudaMemcpyAsync(ctx->id, ids, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, ctx->stream));
        if ((rc = upload_vec3(ctx, acc, ctx->px2, ctx->ax, ctx->ay, ctx->az, n))) return rc;
    }
    // bh_step's loop, without its wait.
    for (int64_t s = 0; s < nsteps; ++s) {
        if (ctx->n > 0) {
            const bool graph = ctx->graphs && !ctx->prof && ctx->t > 0;
            if ((rc = graph ? step_graph(ctx, dt, theta, G, mode) : step_once(ctx, dt, theta, G, mode))) return rc;
        }
        ctx->t += dt;
    }
    // bh_get_bodies.
    if (n > 0) {
        if ((rc = download_vec3(ctx, pos, ctx->px2, ctx->px, ctx->py, ctx->pz, n))) return rc;
        if ((rc = download_vec3(ctx, vel, ctx->vx2, ctx->vx, ctx->vy, ctx->vz, n))) return rc;
        if ((rc = download_vec3(ctx, acc, ctx->px2, ctx->ax, ctx->ay, ctx->az, n))) return rc;
        BH_CUDA_TRY(cudaMemcpyAsync(mass, ctx->m, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        BH_CUDA_TRY(cudaMemcpyAsync(ids, ctx->id, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    rc = finish(ctx, "bh_step_host");
    if (t_io) *t_io = ctx->t;
    if (nsteps > 0 && ctx->n > 0) {
        ctx->tree_valid = ctx->sorted_valid = ctx->bbox_valid = rc == BH_OK;
        ctx->keys_valid = false;
    }
    return rc;
}

}  // extern "C"

// ---- stateless entry points over a per-thread default context ----------
namespace {

struct DefaultCtx {
    bh_context* ctx = nullptr;
    ~DefaultCtx() { if (ctx) bh_context_destroy(ctx); }
};
thread_local DefaultCtx g_default;

int default_ctx(int64_t n, bh_context** out)
{
    const int64_t want = std::max<int64_t>(n, 1);
    if (g_default.ctx && g_default.ctx->cap >= want) {
        *out = g_default.ctx;
        return BH_OK;
    }
    if (g_default.ctx) {
        bh_context_destroy(g_default.ctx);
        g_default.ctx = nullptr;
    }
    int rc = bh_context_create(want, 0, &g_default.ctx);
    if (rc) return rc;
    *out = g_default.ctx;
    return BH_OK;
}

}  // namespace

extern "C" {

int bh_compute_local_bbox(const double* pos, int64_t n, double bbox_out[6])
{
    if (n < 0 || !bbox_out || (n > 0 && !pos)) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_compute_local_bbox: bad arguments");
    if (n == 0) {
        for (int a = 0; a < 3; ++a) { bbox_out[a] = INFINITY; bbox_out[3 + a] = -INFINITY; }
        return BH_OK;
    }
    bh_context* ctx;
    int rc = default_ctx(n, &ctx);
    if (rc) return rc;
    if ((rc = check_ctx(ctx, "bh_compute_local_bbox"))) return rc;
    ctx->n = n;
    ctx->tree_valid = ctx->keys_valid = ctx->sorted_valid = false;
    if ((rc = upload_vec3(ctx, pos, ctx->px2, ctx->px, ctx->py, ctx->pz, n))) return rc;
    if ((rc = bh::launch_drift_bbox(ctx, 0.0, false, false))) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(bbox_out, ctx->bbox, 6 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    return finish(ctx, "bh_compute_local_bbox");
}

int bh_generate_morton_codes(const double* pos, int64_t n, const double bbox[6], uint64_t* keys_out)
{
    if (n < 0 || !bbox || (n > 0 && (!pos || !keys_out)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_generate_morton_codes: bad arguments");
    if (n == 0) return BH_OK;
    bh_context* ctx;
    int rc = default_ctx(n, &ctx);
    if (rc) return rc;
    if ((rc = check_ctx(ctx, "bh_generate_morton_codes"))) return rc;
    ctx->n = n;
    ctx->tree_valid = ctx->keys_valid = ctx->sorted_valid = ctx->bbox_valid = false;
    if ((rc = upload_vec3(ctx, pos, ctx->px2, ctx->px, ctx->py, ctx->pz, n))) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->bbox, bbox, 6 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = bh::launch_keys(ctx, false))) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(keys_out, ctx->key, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    return finish(ctx, "bh_generate_morton_codes");
}

int bh_sort_bodies_by_morton_key(int64_t n, uint64_t* keys, double* pos, double* mass, double* vel, uint64_t* ids)
{
    if (n < 0 || (n > 0 && (!keys || !pos || !mass || !vel || !ids)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_sort_bodies_by_morton_key: bad arguments");
    if (n == 0) return BH_OK;
    bh_context* ctx;
    int rc = default_ctx(n, &ctx);
    if (rc) return rc;
    if ((rc = check_ctx(ctx, "bh_sort_bodies_by_morton_key"))) return rc;
    ctx->n = n;
    if ((rc = upload_vec3(ctx, pos, ctx->px2, ctx->px, ctx->py, ctx->pz, n))) return rc;
    if ((rc = upload_vec3(ctx, vel, ctx->vx2, ctx->vx, ctx->vy, ctx->vz, n))) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->m, mass, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->id, ids, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->key, keys, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = bh::launch_hist(ctx))) return rc;
    if ((rc = bh::launch_sort(ctx))) return rc;
    if ((rc = bh::launch_permute(ctx))) return rc;
    // Downloads: pos and vel through the (now free) second body set.
    if ((rc = download_vec3(ctx, pos, ctx->px2, ctx->px, ctx->py, ctx->pz, n))) return rc;
    if ((rc = download_vec3(ctx, vel, ctx->vx2, ctx->vx, ctx->vy, ctx->vz, n))) return rc;
    BH_CUDA_TRY(cudaMemcpyAsync(mass, ctx->m, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(ids, ctx->id, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(keys, ctx->key, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    rc = finish(ctx, "bh_sort_bodies_by_morton_key");
    ctx->tree_valid = ctx->keys_valid = ctx->bbox_valid = ctx->sorted_valid = false;
    return rc;
}

}  // extern "C"
