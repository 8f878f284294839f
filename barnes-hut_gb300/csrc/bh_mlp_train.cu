// Training of the acceptance network on the GPU with hand-written forward,
// backward and Adam kernels.  No reference counterpart.
//
// Loss: mean squared error of the standardised log10 error label.  Forward
// numerics are those of the inference path fused into the traversal: BF16
// weights and BF16 layer inputs, FP32 accumulation, bias first.  Gradients
// are taken with respect to the FP32 master weights (the BF16 rounding is
// treated as the identity), reduced deterministically (no atomics).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "bh_internal.cuh"
#include "bh_mlp.cuh"

namespace bh {
namespace {

constexpr int kFbThreads = 128;

struct Scratch {
    float *xb, *h1b, *h2b, *dh1, *dh2, *dy, *loss_part;
};

// One thread per sample: forward, loss, backward to the layer deltas.
__global__ void __launch_bounds__(kFbThreads) mlp_fwd_bwd_kernel(const float* __restrict__ X,
                                                                const float* __restrict__ T,
                                                                const int32_t* __restrict__ idx, int64_t off,
                                                                int B, float inv_b, const float* __restrict__ P,
                                                                Scratch s)
{
    __shared__ float W1[kHid * kFeat], b1[kHid], W2[kHid * kHid], b2[kHid], W3[kHid];
    __shared__ float b3;
    __shared__ float red[kFbThreads / 32];
    for (int k = threadIdx.x; k < kHid * kHid; k += blockDim.x) W2[k] = bf16r(P[kOffW2 + k]);
    for (int k = threadIdx.x; k < kHid * kFeat; k += blockDim.x) W1[k] = bf16r(P[kOffW1 + k]);
    for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
        b1[k] = P[kOffB1 + k];
        b2[k] = P[kOffB2 + k];
        W3[k] = bf16r(P[kOffW3 + k]);
    }
    if (threadIdx.x == 0) b3 = P[kOffB3];
    __syncthreads();
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    float l2 = 0.0f;
    if (b < B) {
        const int64_t sidx = idx ? (int64_t)idx[off + b] : off + b;
        float xb[kFeat];
#pragma unroll
        for (int k = 0; k < kFeat; ++k) xb[k] = bf16r(X[sidx * kFeat + k]);
        float h1[kHid];
#pragma unroll
        for (int i = 0; i < kHid; ++i) {
            float a = b1[i];
#pragma unroll
            for (int k = 0; k < kFeat; ++k) a = fmaf(W1[i * kFeat + k], xb[k], a);
            h1[i] = bf16r(fmaxf(a, 0.0f));
        }
        float h2[kHid];
        float y = b3;
#pragma unroll 4
        for (int i = 0; i < kHid; ++i) {
            float a = b2[i];
#pragma unroll
            for (int j = 0; j < kHid; ++j) a = fmaf(W2[i * kHid + j], h1[j], a);
            h2[i] = bf16r(fmaxf(a, 0.0f));
        }
#pragma unroll
        for (int i = 0; i < kHid; ++i) y = fmaf(W3[i], h2[i], y);
        const float diff = y - T[sidx];
        l2 = diff * diff;
        const float dy = 2.0f * diff * inv_b;
        s.dy[b] = dy;
#pragma unroll
        for (int k = 0; k < kFeat; ++k) s.xb[(int64_t)b * kFeat + k] = xb[k];
#pragma unroll
        for (int i = 0; i < kHid; ++i) {
            s.h1b[(int64_t)b * kHid + i] = h1[i];
            s.h2b[(int64_t)b * kHid + i] = h2[i];
            h2[i] = h2[i] > 0.0f ? dy * W3[i] : 0.0f;  // now dh2
            s.dh2[(int64_t)b * kHid + i] = h2[i];
        }
#pragma unroll 4
        for (int j = 0; j < kHid; ++j) {
            float a = 0.0f;
#pragma unroll
            for (int i = 0; i < kHid; ++i) a = fmaf(h2[i], W2[i * kHid + j], a);
            s.dh1[(int64_t)b * kHid + j] = h1[j] > 0.0f ? a : 0.0f;
        }
    }
    // block partial of the squared error
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l2 += __shfl_down_sync(0xffffffffu, l2, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int k = 0; k < kFbThreads / 32; ++k) t += red[k];
        s.loss_part[blockIdx.x] = t;
    }
}

// Block i reduces every gradient entry of hidden unit i over the batch.
__global__ void __launch_bounds__(256) mlp_grad_reduce_kernel(int B, int nloss, Scratch s, float* __restrict__ g,
                                                             float* __restrict__ loss_out, float inv_b)
{
    __shared__ float part[256];
    const int i = blockIdx.x, t = threadIdx.x;
    // dW2[i][j] = sum_b dh2[b][i] h1b[b][j]: 64 columns x 4 partial sums
    {
        const int j = t & 63, q = t >> 6;
        float a = 0.0f;
        for (int b = q; b < B; b += 4) a = fmaf(s.dh2[(int64_t)b * kHid + i], s.h1b[(int64_t)b * kHid + j], a);
        part[t] = a;
        __syncthreads();
        if (t < 64) g[kOffW2 + i * kHid + t] = (part[t] + part[t + 64]) + (part[t + 128] + part[t + 192]);
        __syncthreads();
    }
    // dW1[i][k] = sum_b dh1[b][i] xb[b][k]: 8 columns x 32 partial sums
    {
        const int k = t & 7, q = t >> 3;
        float a = 0.0f;
        for (int b = q; b < B; b += 32) a = fmaf(s.dh1[(int64_t)b * kHid + i], s.xb[(int64_t)b * kFeat + k], a);
        part[t] = a;
        __syncthreads();
        if (t < 8) {
            float r = 0.0f;
            for (int u = 0; u < 32; ++u) r += part[u * 8 + t];
            g[kOffW1 + i * kFeat + t] = r;
        }
        __syncthreads();
    }
    // db1[i], db2[i], dW3[i]: 3 sums x 64 partials (+ db3 and the loss in block 0)
    {
        const int which = t >> 6, q = t & 63;
        float a = 0.0f;
        if (which == 0)
            for (int b = q; b < B; b += 64) a += s.dh1[(int64_t)b * kHid + i];
        else if (which == 1)
            for (int b = q; b < B; b += 64) a += s.dh2[(int64_t)b * kHid + i];
        else if (which == 2)
            for (int b = q; b < B; b += 64) a = fmaf(s.dy[b], s.h2b[(int64_t)b * kHid + i], a);
        else if (i == 0)
            for (int b = q; b < B; b += 64) a += s.dy[b];
        part[t] = a;
        __syncthreads();
        if (t < 4) {
            float r = 0.0f;
            for (int u = 0; u < 64; ++u) r += part[t * 64 + u];
            if (t == 0) g[kOffB1 + i] = r;
            if (t == 1) g[kOffB2 + i] = r;
            if (t == 2) g[kOffW3 + i] = r;
            if (t == 3 && i == 0) g[kOffB3] = r;
        }
        if (i == 0 && t == 0 && loss_out) {
            float l = 0.0f;
            for (int u = 0; u < nloss; ++u) l += s.loss_part[u];
            loss_out[0] = l * inv_b;
            loss_out[1] += l * inv_b;  // running sum over the epoch
        }
    }
}

__global__ void adam_kernel(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float c1, float c2, float eps)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kParams) return;
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.0f - b1) * gk;
    const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    P[k] -= lr * (mk * c1) / (sqrtf(vk * c2) + eps);
}

struct DevBuf {
    std::vector<void*> ptrs;
    ~DevBuf()
    {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    T* alloc(size_t count)
    {
        void* p = nullptr;
        if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(count, 1)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

bool alloc_scratch(DevBuf& d, int B, Scratch& s)
{
    s.xb = d.alloc<float>((size_t)B * kFeat);
    s.h1b = d.alloc<float>((size_t)B * kHid);
    s.h2b = d.alloc<float>((size_t)B * kHid);
    s.dh1 = d.alloc<float>((size_t)B * kHid);
    s.dh2 = d.alloc<float>((size_t)B * kHid);
    s.dy = d.alloc<float>(B);
    s.loss_part = d.alloc<float>((B + kFbThreads - 1) / kFbThreads);
    return s.xb && s.h1b && s.h2b && s.dh1 && s.dh2 && s.dy && s.loss_part;
}

int fwd_bwd(const float* X, const float* T, const int32_t* idx, int64_t off, int B, const float* P, Scratch& s,
            float* g, float* loss, cudaStream_t st)
{
    const int blocks = (B + kFbThreads - 1) / kFbThreads;
    mlp_fwd_bwd_kernel<<<blocks, kFbThreads, 0, st>>>(X, T, idx, off, B, 1.0f / (float)B, P, s);
    BH_CUDA_TRY(cudaGetLastError());
    mlp_grad_reduce_kernel<<<kHid, 256, 0, st>>>(B, blocks, s, g, loss, 1.0f / (float)B);
    BH_CUDA_TRY(cudaGetLastError());
    return BH_OK;
}

}  // namespace
}  // namespace bh

using namespace bh;

extern "C" int bh_mlp_gradient(const float* params, const float* X, const float* T, int64_t n, float* grad_out,
                               float* loss_out)
{
    if (!params || !X || !T || !grad_out || n <= 0 || n > (1 << 20))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_mlp_gradient: bad arguments (n in [1, 2^20])");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return bh_fail(BH_ERR_NO_DEVICE, "bh_mlp_gradient: no CUDA device");
    }
    DevBuf d;
    float* dP = d.alloc<float>(kParams);
    float* dX = d.alloc<float>((size_t)n * kFeat);
    float* dT = d.alloc<float>(n);
    float* dG = d.alloc<float>(kParams);
    float* dL = d.alloc<float>(2);
    Scratch s;
    if (!dP || !dX || !dT || !dG || !dL || !alloc_scratch(d, (int)n, s))
        return bh_fail(BH_ERR_OUT_OF_MEMORY, "bh_mlp_gradient: device allocation failed");
    BH_CUDA_TRY(cudaMemcpy(dP, params, sizeof(float) * kParams, cudaMemcpyHostToDevice));
    BH_CUDA_TRY(cudaMemcpy(dX, X, sizeof(float) * n * kFeat, cudaMemcpyHostToDevice));
    BH_CUDA_TRY(cudaMemcpy(dT, T, sizeof(float) * n, cudaMemcpyHostToDevice));
    int rc = fwd_bwd(dX, dT, nullptr, 0, (int)n, dP, s, dG, dL, 0);
    if (rc) return rc;
    BH_CUDA_TRY(cudaMemcpy(grad_out, dG, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    if (loss_out) BH_CUDA_TRY(cudaMemcpy(loss_out, dL, sizeof(float), cudaMemcpyDeviceToHost));
    return BH_OK;
}

extern "C" int bh_mlp_train(const float* features, const float* labels, int64_t n, int epochs, int batch, float lr,
                            uint64_t seed, float* params_out, float* scale_out, float* loss_out)
{
    if (!features || !labels || !params_out || !scale_out || n < 16 || epochs < 1 || batch < 16 || batch > (1 << 16) ||
        !(lr > 0))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_mlp_train: bad arguments");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return bh_fail(BH_ERR_NO_DEVICE, "bh_mlp_train: no CUDA device");
    }
    // Standardisation from the data (host, FP64 sums).
    MlpScale sc;
    double mean[kFeat] = {0}, sq[kFeat] = {0}, lm = 0, ls = 0;
    for (int64_t r = 0; r < n; ++r) {
        for (int k = 0; k < kFeat; ++k) {
            const double v = features[r * kFeat + k];
            mean[k] += v;
            sq[k] += v * v;
        }
        lm += labels[r];
        ls += (double)labels[r] * labels[r];
    }
    for (int k = 0; k < kFeat; ++k) {
        const double mu = mean[k] / n, var = std::max(sq[k] / n - mu * mu, 1e-12);
        sc.mean[k] = (float)mu;
        sc.inv_std[k] = (float)(1.0 / std::sqrt(var));
        sc.lo[k] = 1e30f;
        sc.hi[k] = -1e30f;
    }
    sc.lmean = (float)(lm / n);
    sc.lstd = (float)std::sqrt(std::max(ls / n - (lm / n) * (lm / n), 1e-12));
    std::vector<float> Z((size_t)n * kFeat), TL(n);
    for (int64_t r = 0; r < n; ++r) {
        for (int k = 0; k < kFeat; ++k) {
            const float z = (features[r * kFeat + k] - sc.mean[k]) * sc.inv_std[k];
            Z[r * kFeat + k] = z;
            sc.lo[k] = std::min(sc.lo[k], z);
            sc.hi[k] = std::max(sc.hi[k], z);
        }
        TL[r] = (labels[r] - sc.lmean) / sc.lstd;
    }
    // He-normal initialisation, zero biases.
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    std::vector<float> P(kParams, 0.0f);
    for (int k = 0; k < kHid * kFeat; ++k) P[kOffW1 + k] = (float)(nd(rng) * std::sqrt(2.0 / kFeat));
    for (int k = 0; k < kHid * kHid; ++k) P[kOffW2 + k] = (float)(nd(rng) * std::sqrt(2.0 / kHid));
    for (int k = 0; k < kHid; ++k) P[kOffW3 + k] = (float)(nd(rng) * std::sqrt(1.0 / kHid));

    DevBuf d;
    float* dP = d.alloc<float>(kParams);
    float* dG = d.alloc<float>(kParams);
    float* dM = d.alloc<float>(kParams);
    float* dV = d.alloc<float>(kParams);
    float* dX = d.alloc<float>((size_t)n * kFeat);
    float* dT = d.alloc<float>(n);
    int32_t* dI = d.alloc<int32_t>(n);
    float* dL = d.alloc<float>(2);
    Scratch s;
    const int B = (int)std::min<int64_t>(batch, n);
    if (!dP || !dG || !dM || !dV || !dX || !dT || !dI || !dL || !alloc_scratch(d, B, s))
        return bh_fail(BH_ERR_OUT_OF_MEMORY, "bh_mlp_train: device allocation failed");
    BH_CUDA_TRY(cudaMemcpy(dP, P.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice));
    BH_CUDA_TRY(cudaMemset(dM, 0, sizeof(float) * kParams));
    BH_CUDA_TRY(cudaMemset(dV, 0, sizeof(float) * kParams));
    BH_CUDA_TRY(cudaMemcpy(dX, Z.data(), sizeof(float) * n * kFeat, cudaMemcpyHostToDevice));
    BH_CUDA_TRY(cudaMemcpy(dT, TL.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    std::vector<int32_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    int64_t step = 0;
    const int64_t nb = n / B;  // full batches only
    for (int e = 0; e < epochs; ++e) {
        std::shuffle(order.begin(), order.end(), rng);
        BH_CUDA_TRY(cudaMemcpy(dI, order.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        BH_CUDA_TRY(cudaMemset(dL, 0, 2 * sizeof(float)));
        for (int64_t k = 0; k < nb; ++k) {
            int rc = fwd_bwd(dX, dT, dI, k * B, B, dP, s, dG, dL, 0);
            if (rc) return rc;
            ++step;
            const float c1 = 1.0f / (1.0f - std::pow(b1, (float)step));
            const float c2 = 1.0f / (1.0f - std::pow(b2, (float)step));
            adam_kernel<<<(kParams + 255) / 256, 256>>>(dP, dG, dM, dV, lr, b1, b2, c1, c2, eps);
            BH_CUDA_TRY(cudaGetLastError());
        }
        float l[2] = {0.f, 0.f};
        BH_CUDA_TRY(cudaMemcpy(l, dL, 2 * sizeof(float), cudaMemcpyDeviceToHost));
        if (loss_out) loss_out[e] = l[1] / (float)std::max<int64_t>(nb, 1);  // mean batch loss of the epoch
    }
    BH_CUDA_TRY(cudaMemcpy(params_out, dP, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    std::memcpy(scale_out, &sc, sizeof(MlpScale));
    return BH_OK;
}
