// Diagnostics with no reference counterpart: the FP64 direct-sum sampler
// that every force error is measured against, and the invariants (energy, linear and
// angular momentum) whose drift is reported over a run.
#include <vector>

#include "bh_internal.cuh"

namespace {

constexpr int kDirThreads = 256;

__device__ double block_sum(double v, double* sh)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    __syncthreads();
    return t;
}

// One block per target: a = sum_i G m_i (x_i - x_j) / |x_i - x_j|^3 over all
// sources i != j, IEEE sqrt and division (the formula of traversal.cpp:79-82).
__global__ void __launch_bounds__(kDirThreads) direct_sum_kernel(int64_t n, const double* __restrict__ px,
                                                                const double* __restrict__ py,
                                                                const double* __restrict__ pz,
                                                                const double* __restrict__ m,
                                                                const int64_t* __restrict__ targets, double G,
                                                                double* __restrict__ out)
{
    __shared__ double sh[kDirThreads / 32];
    const int64_t j = targets[blockIdx.x];
    const double xj = px[j], yj = py[j], zj = pz[j];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        if (i == j) continue;
        const double dx = __dsub_rn(px[i], xj), dy = __dsub_rn(py[i], yj), dz = __dsub_rn(pz[i], zj);
        const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        if (r2 == 0.0) continue;
        const double invR = __drcp_rn(__dsqrt_rn(r2));
        const double s = __dmul_rn(__dmul_rn(G, m[i]), __dmul_rn(__dmul_rn(invR, invR), invR));
        ax = __dadd_rn(ax, __dmul_rn(s, dx));
        ay = __dadd_rn(ay, __dmul_rn(s, dy));
        az = __dadd_rn(az, __dmul_rn(s, dz));
    }
    ax = block_sum(ax, sh);
    ay = block_sum(ay, sh);
    az = block_sum(az, sh);
    if (threadIdx.x == 0) {
        out[3 * blockIdx.x] = ax;
        out[3 * blockIdx.x + 1] = ay;
        out[3 * blockIdx.x + 2] = az;
    }
}

// Per-block partial sums of K, L (3) and P (3).
__global__ void __launch_bounds__(kDirThreads) moments_kernel(int64_t n, const double* __restrict__ px,
                                                             const double* __restrict__ py,
                                                             const double* __restrict__ pz,
                                                             const double* __restrict__ vx,
                                                             const double* __restrict__ vy,
                                                             const double* __restrict__ vz,
                                                             const double* __restrict__ m, double* __restrict__ part)
{
    __shared__ double sh[kDirThreads / 32];
    double q[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = px[i], y = py[i], z = pz[i], u = vx[i], v = vy[i], w = vz[i], mi = m[i];
        q[0] += 0.5 * mi * (u * u + v * v + w * w);
        q[1] += mi * (y * w - z * v);
        q[2] += mi * (z * u - x * w);
        q[3] += mi * (x * v - y * u);
        q[4] += mi * u;
        q[5] += mi * v;
        q[6] += mi * w;
    }
    for (int k = 0; k < 7; ++k) {
        const double t = block_sum(q[k], sh);
        if (threadIdx.x == 0) part[blockIdx.x * 7 + k] = t;
    }
}

// Pairwise potential, exact FP64: block b takes bodies i = b, b + grid, ...
// and sums over j > i.  Partial per block.
__global__ void __launch_bounds__(kDirThreads) potential_pairs_kernel(int64_t n, const double* __restrict__ px,
                                                                     const double* __restrict__ py,
                                                                     const double* __restrict__ pz,
                                                                     const double* __restrict__ m, double G,
                                                                     double* __restrict__ part)
{
    __shared__ double sh[kDirThreads / 32];
    double u = 0.0;
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const double xi = px[i], yi = py[i], zi = pz[i], mi = m[i];
        for (int64_t j = i + 1 + threadIdx.x; j < n; j += blockDim.x) {
            const double dx = px[j] - xi, dy = py[j] - yi, dz = pz[j] - zi;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            if (r > 0) u -= G * mi * m[j] / r;
        }
    }
    const double t = block_sum(u, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

constexpr int64_t kExactPotentialMax = 1 << 17;

// Potential of the pairs that involve a massive body (id < nd), exact FP64.
// Each such pair counts once: a pair of two massive bodies by its higher id.
__global__ void __launch_bounds__(kDirThreads) potential_massive_kernel(
    int64_t n, const double* __restrict__ px, const double* __restrict__ py, const double* __restrict__ pz,
    const double* __restrict__ m, const uint64_t* __restrict__ id, int nd, const double* __restrict__ direct,
    const int32_t* __restrict__ present, double* __restrict__ part)
{
    __shared__ double sh[kDirThreads / 32];
    double u = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t idi = id[i];
        const double xi = px[i], yi = py[i], zi = pz[i], mi = m[i];
        for (int k = 0; k < nd; ++k) {
            if (!present[k] || idi == (uint64_t)k || (idi < (uint64_t)nd && idi < (uint64_t)k)) continue;
            const double dx = direct[4 * k] - xi, dy = direct[4 * k + 1] - yi, dz = direct[4 * k + 2] - zi;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            if (r > 0) u -= direct[4 * k + 3] * mi / r;
        }
    }
    const double t = block_sum(u, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Potential of all other pairs through the tree of far-field masses (the
// massive bodies zeroed): U = 1/2 sum_i m_i phi_i over the non-massive
// bodies, phi_i from the monopoles the theta criterion of the force walk
// accepts (side(depth)^2 < theta^2 r^2; leaves always, the own leaf never).
// One thread per body, depth-first with a private stack; a stack that would
// overflow raises the overflow bit of the error word and drops that subtree.
constexpr int kPotStack = 8 * bh::kMaxDepth + 8;

__global__ void __launch_bounds__(kDirThreads) potential_tree_kernel(
    int64_t n, const double* __restrict__ px, const double* __restrict__ py, const double* __restrict__ pz,
    const double* __restrict__ m, const uint64_t* __restrict__ id, int nd, const int32_t* __restrict__ body_leaf,
    const bh::TreeRec* __restrict__ rec, const double* __restrict__ bbox, double theta, double G,
    unsigned* __restrict__ err, double* __restrict__ part)
{
    __shared__ double sh[kDirThreads / 32];
    __shared__ double side2[bh::kMaxDepth + 1];
    if (threadIdx.x <= bh::kMaxDepth) {
        double L = bbox[3] - bbox[0];
        L = fmax(L, bbox[4] - bbox[1]);
        L = fmax(L, bbox[5] - bbox[2]);
        const double side = L / (double)(1ull << threadIdx.x);
        side2[threadIdx.x] = side * side;
    }
    __syncthreads();
    const double t2 = theta * theta;
    double u = 0.0;
    int32_t stack[kPotStack];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (id[i] < (uint64_t)nd) continue;
        const double x = px[i], y = py[i], z = pz[i];
        const int32_t own = body_leaf[i];
        double phi = 0.0;
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const bh::TreeRec r = rec[stack[--sp]];
            if (!(r.m > 0.0)) continue;
            const double dx = r.cx - x, dy = r.cy - y, dz = r.cz - z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r.nchild == 0) {
                if (r.leaf != own && r2 > 0.0) phi -= r.m / sqrt(r2);
                continue;
            }
            if (side2[r.depth] < t2 * r2) {
                phi -= r.m / sqrt(r2);
                continue;
            }
            if (sp + r.nchild > kPotStack) {
                atomicOr(err, bh::kErrOverflow);
                continue;
            }
            for (int c = r.nchild - 1; c >= 0; --c) stack[sp++] = r.child + c;
        }
        u += 0.5 * G * m[i] * phi;
    }
    const double t = block_sum(u, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Eight independent FMA chains per thread; the result is stored so the
// chains are live.
template <class T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T* out, int iters, T a, T b)
{
    T x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = (T)(threadIdx.x * 1e-3 + c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" {

int bh_direct_sum(bh_context* ctx, int64_t ns, const int64_t* targets, double G, double* acc_out)
{
    if (!ctx || ns < 0 || (ns > 0 && (!targets || !acc_out)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_direct_sum: bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    if (ns == 0) return BH_OK;
    for (int64_t k = 0; k < ns; ++k)
        if (targets[k] < 0 || targets[k] >= ctx->n)
            return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_direct_sum: target index out of range");
    int64_t* dt = nullptr;
    double* dout = nullptr;
    BH_CUDA_TRY(cudaMallocAsync(&dt, sizeof(int64_t) * ns, ctx->stream));
    BH_CUDA_TRY(cudaMallocAsync(&dout, sizeof(double) * 3 * ns, ctx->stream));
    BH_CUDA_TRY(cudaMemcpyAsync(dt, targets, sizeof(int64_t) * ns, cudaMemcpyHostToDevice, ctx->stream));
    direct_sum_kernel<<<(unsigned)ns, kDirThreads, 0, ctx->stream>>>(ctx->n, ctx->px, ctx->py, ctx->pz, ctx->m, dt, G,
                                                                     dout);
    BH_LAUNCH_CHECK(ctx);
    BH_CUDA_TRY(cudaMemcpyAsync(acc_out, dout, sizeof(double) * 3 * ns, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaFreeAsync(dt, ctx->stream));
    BH_CUDA_TRY(cudaFreeAsync(dout, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return BH_OK;
}

int bh_measure_fma_peak(bh_context* ctx, int fp64, double* tflops_out)
{
    if (!ctx || !tflops_out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_measure_fma_peak: bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    const int blocks = 8 * bh::num_sms(), threads = 256;
    const int iters = fp64 ? 2048 : 32768;
    void* out = nullptr;
    BH_CUDA_TRY(cudaMallocAsync(&out, sizeof(double) * blocks * threads, ctx->stream));
    cudaEvent_t a, b;
    BH_CUDA_TRY(cudaEventCreate(&a));
    BH_CUDA_TRY(cudaEventCreate(&b));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        BH_CUDA_TRY(cudaEventRecord(a, ctx->stream));
        if (fp64)
            fma_chain_kernel<double><<<blocks, threads, 0, ctx->stream>>>((double*)out, iters, 1.0000001, 1e-9);
        else
            fma_chain_kernel<float><<<blocks, threads, 0, ctx->stream>>>((float*)out, iters, 1.0000001f, 1e-9f);
        BH_LAUNCH_CHECK(ctx);
        BH_CUDA_TRY(cudaEventRecord(b, ctx->stream));
        BH_CUDA_TRY(cudaEventSynchronize(b));
        float ms = 0.f;
        BH_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
        if (rep > 0 && ms < best) best = ms;  // first launch is a warm-up
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    BH_CUDA_TRY(cudaFreeAsync(out, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *tflops_out = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
    return BH_OK;
}

int bh_invariants(bh_context* ctx, double G, double theta, double out[9])
{
    if (!ctx || !out || !(theta >= 0.0)) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_invariants: bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    const int64_t n = ctx->n;
    for (int k = 0; k < 9; ++k) out[k] = 0.0;
    if (n == 0) return BH_OK;
    const bool exact = theta == 0.0;
    if (exact && n > kExactPotentialMax)
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_invariants: exact pair potential limited to 131072 bodies");
    int rc = BH_OK;
    if (!exact) {
        // The tree part needs the tree of the current positions with the
        // massive bodies' masses zeroed.
        if (!ctx->tree_valid) {
            if ((rc = bh_compute_bbox(ctx, nullptr)) || (rc = bh_compute_keys(ctx, nullptr)) ||
                (rc = bh_sort_bodies(ctx, nullptr)) || (rc = bh_build_tree(ctx)))
                return rc;
        }
        if (!ctx->tree_far) {
            if ((rc = bh::launch_build(ctx, ctx->m, ctx->tree_moments, false, 0.0, true))) return rc;
            ctx->tree_far = true;
        }
        if ((rc = bh::ensure_rec(ctx))) return rc;
        if ((rc = bh::launch_direct_extract(ctx, G))) return rc;
    }
    // Every kernel below writes one partial per block into its own column.
    const int blocks = 8 * bh::num_sms();
    double* part = nullptr;
    BH_CUDA_TRY(cudaMallocAsync(&part, sizeof(double) * blocks * 9, ctx->stream));
    BH_CUDA_TRY(cudaMemsetAsync(part, 0, sizeof(double) * blocks * 9, ctx->stream));
    moments_kernel<<<blocks, kDirThreads, 0, ctx->stream>>>(n, ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy, ctx->vz,
                                                            ctx->m, part);
    BH_LAUNCH_CHECK(ctx);
    if (exact) {
        potential_pairs_kernel<<<blocks, kDirThreads, 0, ctx->stream>>>(n, ctx->px, ctx->py, ctx->pz, ctx->m, G,
                                                                        part + blocks * 7);
        BH_LAUNCH_CHECK(ctx);
    } else {
        const int nd = ctx->num_direct < 64 ? (ctx->num_direct > 0 ? ctx->num_direct : 0) : 64;
        potential_massive_kernel<<<blocks, kDirThreads, 0, ctx->stream>>>(
            n, ctx->px, ctx->py, ctx->pz, ctx->m, ctx->id, nd, ctx->direct, ctx->direct_present, part + blocks * 7);
        BH_LAUNCH_CHECK(ctx);
        potential_tree_kernel<<<blocks, kDirThreads, 0, ctx->stream>>>(
            n, ctx->px, ctx->py, ctx->pz, ctx->m, ctx->id, nd, ctx->body_leaf, ctx->rec, ctx->bbox, theta, G, ctx->err,
            part + blocks * 8);
        BH_LAUNCH_CHECK(ctx);
    }
    std::vector<double> h((size_t)blocks * 9);
    BH_CUDA_TRY(cudaMemcpyAsync(h.data(), part, sizeof(double) * blocks * 9, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaFreeAsync(part, ctx->stream));
    if ((rc = bh::finish(ctx, "bh_invariants"))) return rc;
    double q[7] = {0, 0, 0, 0, 0, 0, 0}, U = 0.0;
    for (int b = 0; b < blocks; ++b) {
        for (int k = 0; k < 7; ++k) q[k] += h[(size_t)b * 7 + k];
        U += h[(size_t)blocks * 7 + b] + h[(size_t)blocks * 8 + b];
    }
    out[0] = q[0] + U;
    out[1] = q[0];
    out[2] = U;
    for (int k = 0; k < 3; ++k) { out[3 + k] = q[1 + k]; out[6 + k] = q[4 + k]; }
    return BH_OK;
}

}  // extern "C"
