// Learned acceptance: training-pair collection and labelling, model upload
// for the traversal's fused inference, and a standalone inference entry for
// checks.  No reference counterpart.
//
// A training pair is (warp group of 32 bodies, tree node) met by the FP32
// walk with the plain theta test, where theta would not accept the node for
// the whole group but theta_max would (the nodes the network is asked
// about).  Its label is log10 of the largest relative force error, over the
// group's bodies that reach the node, of accepting the node as one monopole
// instead of opening it: |a_mono - a_open| / a_scale, where a_open is the
// node's subtree summed by the plain per-body walk at theta_label (0.5) in
// FP64, and a_scale is the group's smallest direct-term acceleration (the
// Sun's pull dominates every body's acceleration).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "bh_internal.cuh"
#include "bh_mlp.cuh"

namespace bh {

int launch_collect(bh_context* ctx, double theta, double G, double theta_max, int32_t* c_group, int32_t* c_slot,
                   uint32_t* c_mask, float* c_feat, float* c_ascale, unsigned long long* c_count, int64_t cap);

namespace {

constexpr int kLW = 4;  // warps per block in the label kernel
constexpr int kLStack = 22 * 7 + 8 + 2;

__global__ void __launch_bounds__(32 * kLW) label_kernel(int64_t npairs, const int32_t* __restrict__ c_group,
                                                        const int32_t* __restrict__ c_slot,
                                                        const uint32_t* __restrict__ c_mask,
                                                        const float* __restrict__ c_ascale, int64_t n,
                                                        const double* __restrict__ px, const double* __restrict__ py,
                                                        const double* __restrict__ pz,
                                                        const int32_t* __restrict__ body_leaf,
                                                        const TreeRec* __restrict__ rec,
                                                        const double* __restrict__ bbox, double theta2, double G,
                                                        float* __restrict__ labels, unsigned* err)
{
    __shared__ int stack[kLW][kLStack];
    __shared__ double side2[kMaxDepth + 1];
    if (threadIdx.x <= kMaxDepth) {
        const double dx = bbox[3] - bbox[0], dy = bbox[4] - bbox[1], dz = bbox[5] - bbox[2];
        const double L = fmax(dx, fmax(dy, dz));
        const double side = L / (double)(1ull << threadIdx.x);
        side2[threadIdx.x] = side * side;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int* stk = stack[w];
    for (int64_t pr = (int64_t)blockIdx.x * kLW + w; pr < npairs; pr += (int64_t)gridDim.x * kLW) {
        const int64_t i = (int64_t)c_group[pr] * 32 + lane;
        const int s0 = c_slot[pr];
        const bool active = ((c_mask[pr] >> lane) & 1u) && i < n;
        const double x = active ? px[i] : 0.0, y = active ? py[i] : 0.0, z = active ? pz[i] : 0.0;
        const int my_leaf = active ? body_leaf[i] : -2;
        // the node as one monopole
        const TreeRec r0 = rec[s0];
        double mx = 0.0, my = 0.0, mz = 0.0;
        {
            const double dx = r0.cx - x, dy = r0.cy - y, dz = r0.cz - z;
            const double inv = rsqrt(dx * dx + dy * dy + dz * dz);
            const double sc = G * r0.m * inv * inv * inv;
            mx = sc * dx; my = sc * dy; mz = sc * dz;
        }
        // the node opened: per-lane walk of its subtree at theta_label
        double ox = 0.0, oy = 0.0, oz = 0.0;
        int sp = 1, skip_sp = 0x7fffffff;
        if (lane == 0) stk[0] = s0;
        __syncwarp();
        int pops = 0;
        while (sp > 0) {
            if (++pops > 4 * (int)n + 4) {
                atomicOr(err, kErrOverflow);
                break;
            }
            --sp;
            const int s = stk[sp];
            __syncwarp();
            const TreeRec r = rec[s];
            if (sp < skip_sp) skip_sp = 0x7fffffff;
            if (r.m == 0.0) continue;
            const bool on = active && skip_sp == 0x7fffffff;
            const bool leaf = r.child < 0;
            bool acc = false, open = false;
            if (on) {
                const double dx = r.cx - x, dy = r.cy - y, dz = r.cz - z;
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (leaf) acc = r.leaf != my_leaf;
                else { acc = side2[r.depth] < theta2 * r2; open = !acc; }
                if (acc) {
                    const double inv = rsqrt(r2);
                    const double sc = G * r.m * inv * inv * inv;
                    ox += sc * dx; oy += sc * dy; oz += sc * dz;
                }
            }
            const unsigned opened = __ballot_sync(0xffffffffu, open);
            if (opened) {
                if (acc && !leaf) skip_sp = sp;
                const int nc = r.nchild;
                if (sp + nc > kLStack) {
                    atomicOr(err, kErrOverflow);
                    break;
                }
                if (lane < nc) stk[sp + lane] = r.child + lane;
                __syncwarp();
                sp += nc;
            }
        }
        double e = 0.0;
        if (active) {
            const double ex = mx - ox, ey = my - oy, ez = mz - oz;
            e = sqrt(ex * ex + ey * ey + ez * ez);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) e = fmax(e, __shfl_xor_sync(0xffffffffu, e, off));
        // Errors below 1e-16 of the acceleration are rounding: floor there.
        if (lane == 0) labels[pr] = (float)fmax(log10(fmax(e, 1e-300) / (double)c_ascale[pr]), -16.0);
        __syncwarp();
    }
}

// Standalone inference over rows of raw features (checks of the fused path).
__global__ void predict_kernel(const MlpDev* __restrict__ M, const float* __restrict__ feat, int64_t n,
                               float* __restrict__ out, int32_t* __restrict__ in_range)
{
    __shared__ float F[4][32][9];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t row0 = ((int64_t)blockIdx.x * 4 + w) * 32;
    if (row0 >= n) return;
    const int64_t r = row0 + lane;
    bool inr = r < n;
    for (int q = 0; q < kFeat; ++q) {
        const float f = r < n ? feat[r * kFeat + q] : 0.0f;
        const float z = (f - M->sc.mean[q]) * M->sc.inv_std[q];
        inr = inr && z >= M->sc.lo[q] && z <= M->sc.hi[q];
        F[w][lane][q] = r < n ? fminf(fmaxf(z, -64.0f), 64.0f) : 0.0f;
    }
    __syncwarp();
    const float y = mlp_predict_warp(M, F[w], lane);
    if (r < n) {
        out[r] = y * M->sc.lstd + M->sc.lmean;
        if (in_range) in_range[r] = inr ? 1 : 0;
    }
}

// Host: the fragment layout of a model (see MlpDev).
void pack_model(const float* P, const float* scale, double budget_log10, MlpDev& m)
{
    auto bits = [](float v) -> uint32_t {
        const float r = bf16r(v);
        uint32_t u;
        std::memcpy(&u, &r, 4);
        return u >> 16;
    };
    auto pair = [&](float lo, float hi) -> uint32_t { return bits(lo) | (bits(hi) << 16); };
    const float* W1 = P + kOffW1;
    const float* W2 = P + kOffW2;
    for (int j = 0; j < 8; ++j)
        for (int lane = 0; lane < 32; ++lane) {
            const int g = lane >> 2, t = lane & 3, nrow = 8 * j + g;
            m.w1f[j][lane] = pair(W1[nrow * kFeat + 2 * t], W1[nrow * kFeat + 2 * t + 1]);
            for (int kk = 0; kk < 4; ++kk) {
                const int k0 = 16 * kk + 2 * t;
                m.w2f[j][kk][lane].x = pair(W2[nrow * kHid + k0], W2[nrow * kHid + k0 + 1]);
                m.w2f[j][kk][lane].y = pair(W2[nrow * kHid + k0 + 8], W2[nrow * kHid + k0 + 9]);
            }
        }
    for (int k = 0; k < kHid; ++k) {
        m.b1[k] = P[kOffB1 + k];
        m.b2[k] = P[kOffB2 + k];
        m.w3[k] = bf16r(P[kOffW3 + k]);
    }
    m.b3 = P[kOffB3];
    std::memcpy(&m.sc, scale, sizeof(MlpScale));
    m.log_thresh = (float)budget_log10;
    m.theta_max2 = 0.0f;
}

}  // namespace
}  // namespace bh

using namespace bh;

extern "C" {

int bh_learned_collect(bh_context* ctx, double theta, double theta_label, double theta_max, double G,
                       int64_t max_pairs, float* features_out, float* labels_out, int64_t* n_out)
{
    if (!ctx || max_pairs < 1 || !features_out || !labels_out || !n_out || !(theta > 0) || !(theta_label > 0) ||
        !(theta_max > theta))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_learned_collect: bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    *n_out = 0;
    if (ctx->n == 0) return BH_OK;
    if (!ctx->tree_valid) return bh_fail(BH_ERR_STATE, "bh_learned_collect: build the tree first");
    int rc;
    if (!ctx->tree_far || !ctx->tree_moments) {
        if ((rc = launch_build(ctx, ctx->m, true, false, 0.0, true))) return rc;
        ctx->tree_far = ctx->tree_moments = true;
    }
    if ((rc = ensure_rec(ctx))) return rc;
    cudaStream_t st = ctx->stream;
    int32_t *grp = nullptr, *slot = nullptr;
    uint32_t* mask = nullptr;
    float *feat = nullptr, *asc = nullptr, *lab = nullptr;
    unsigned long long* count = nullptr;
    auto cleanup = [&]() {
        cudaFree(grp); cudaFree(slot); cudaFree(mask); cudaFree(feat); cudaFree(asc); cudaFree(lab); cudaFree(count);
    };
    if (cudaMalloc(&grp, 4 * max_pairs) != cudaSuccess || cudaMalloc(&slot, 4 * max_pairs) != cudaSuccess ||
        cudaMalloc(&mask, 4 * max_pairs) != cudaSuccess || cudaMalloc(&feat, 4 * kFeat * max_pairs) != cudaSuccess ||
        cudaMalloc(&asc, 4 * max_pairs) != cudaSuccess || cudaMalloc(&lab, 4 * max_pairs) != cudaSuccess ||
        cudaMalloc(&count, 8) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return bh_fail(BH_ERR_OUT_OF_MEMORY, "bh_learned_collect: device allocation failed");
    }
    cudaMemsetAsync(count, 0, 8, st);
    rc = launch_collect(ctx, theta, G, theta_max, grp, slot, mask, feat, asc, count, max_pairs);
    if (rc) { cleanup(); return rc; }
    unsigned long long total = 0;
    cudaMemcpyAsync(&total, count, 8, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) { cleanup(); return bh_fail(BH_ERR_CUDA, "bh_learned_collect: collection failed"); }
    const int64_t np = (int64_t)total < max_pairs ? (int64_t)total : max_pairs;
    if (np > 0) {
        const int64_t blocks = std::min<int64_t>((np + kLW - 1) / kLW, 16 * bh::num_sms());
        label_kernel<<<(unsigned)blocks, 32 * kLW, 0, st>>>(np, grp, slot, mask, asc, ctx->n, ctx->px, ctx->py, ctx->pz,
                                                            ctx->body_leaf, ctx->rec, ctx->bbox,
                                                            theta_label * theta_label, G, lab, ctx->err);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { cleanup(); return bh_fail(BH_ERR_CUDA, std::string("label kernel: ") + cudaGetErrorString(e)); }
        ++ctx->launches;
        cudaMemcpyAsync(features_out, feat, 4 * kFeat * np, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(labels_out, lab, 4 * np, cudaMemcpyDeviceToHost, st);
    }
    cudaError_t e = cudaStreamSynchronize(st);
    cleanup();
    if (e != cudaSuccess) return bh_fail(BH_ERR_CUDA, std::string("bh_learned_collect: ") + cudaGetErrorString(e));
    *n_out = np;
    return bh_context_sync(ctx);
}

int bh_learned_set_model(bh_context* ctx, const float* params, const float* scale, double budget, double theta_max)
{
    if (!ctx || !params || !scale || !(budget > 0) || !(theta_max > 0))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_learned_set_model: bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    MlpDev m;
    pack_model(params, scale, std::log10(budget), m);
    m.theta_max2 = (float)(theta_max * theta_max);
    if (!ctx->mlp_dev) {
        if (cudaMalloc(&ctx->mlp_dev, sizeof(MlpDev)) != cudaSuccess) {
            cudaGetLastError();
            ctx->mlp_dev = nullptr;
            return bh_fail(BH_ERR_OUT_OF_MEMORY, "bh_learned_set_model: device allocation failed");
        }
    }
    BH_CUDA_TRY(cudaMemcpyAsync(ctx->mlp_dev, &m, sizeof(MlpDev), cudaMemcpyHostToDevice, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->learn_theta_max = theta_max;
    ctx->learn_budget = budget;
    return BH_OK;
}

int bh_learned_set_criterion(bh_context* ctx, double band, double frac)
{
    if (!ctx || !(band >= 0.0) || !(frac > 0.0) || !(frac <= 1.0))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_learned_set_criterion: need band >= 0 and 0 < frac <= 1");
    ctx->learn_band = band;
    ctx->learn_frac = frac;
    return BH_OK;
}

int bh_learned_stats(bh_context* ctx, int64_t out[4])
{
    if (!ctx || !out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_learned_stats: bad arguments");
    BH_CUDA_TRY(cudaSetDevice(ctx->device));
    unsigned long long v[4];
    BH_CUDA_TRY(cudaMemcpyAsync(v, ctx->lstats, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < 4; ++k) out[k] = (int64_t)v[k];
    return BH_OK;
}

namespace {
constexpr char kModelTag[8] = {'B', 'H', 'M', 'L', 'P', '0', '0', '1'};

void put_u32(unsigned char* b, uint32_t v)
{
    for (int k = 0; k < 4; ++k) b[k] = (unsigned char)(v >> (8 * k));
}

uint32_t get_u32(const unsigned char* b)
{
    uint32_t v = 0;
    for (int k = 0; k < 4; ++k) v |= (uint32_t)b[k] << (8 * k);
    return v;
}
}  // namespace

int bh_mlp_save(const char* path, const float* params, const float* scale)
{
    if (!path || !params || !scale) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_mlp_save: bad arguments");
    std::vector<unsigned char> buf(16 + 4 * (size_t)(kParams + kScaleFloats));
    std::memcpy(buf.data(), kModelTag, 8);
    put_u32(buf.data() + 8, (uint32_t)kParams);
    put_u32(buf.data() + 12, (uint32_t)kScaleFloats);
    size_t o = 16;
    for (int k = 0; k < kParams + kScaleFloats; ++k, o += 4) {
        uint32_t u;
        std::memcpy(&u, k < kParams ? params + k : scale + (k - kParams), 4);
        put_u32(buf.data() + o, u);
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return bh_fail(BH_ERR_IO, std::string("bh_mlp_save: cannot open ") + path);
    const bool ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    const bool closed = std::fclose(f) == 0;
    return ok && closed ? BH_OK : bh_fail(BH_ERR_IO, std::string("bh_mlp_save: write failed: ") + path);
}

int bh_mlp_load(const char* path, float* params_out, float* scale_out)
{
    if (!path || !params_out || !scale_out) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_mlp_load: bad arguments");
    FILE* f = std::fopen(path, "rb");
    if (!f) return bh_fail(BH_ERR_IO, std::string("bh_mlp_load: cannot open ") + path);
    std::vector<unsigned char> buf(16 + 4 * (size_t)(kParams + kScaleFloats) + 1);
    const size_t got = std::fread(buf.data(), 1, buf.size(), f);
    std::fclose(f);
    if (got != buf.size() - 1 || std::memcmp(buf.data(), kModelTag, 8) != 0 ||
        get_u32(buf.data() + 8) != (uint32_t)kParams || get_u32(buf.data() + 12) != (uint32_t)kScaleFloats)
        return bh_fail(BH_ERR_INVALID_ARGUMENT, std::string("bh_mlp_load: not a model file: ") + path);
    size_t o = 16;
    for (int k = 0; k < kParams + kScaleFloats; ++k, o += 4) {
        const uint32_t u = get_u32(buf.data() + o);
        std::memcpy(k < kParams ? params_out + k : scale_out + (k - kParams), &u, 4);
    }
    return BH_OK;
}

int bh_mlp_predict(const float* params, const float* scale, const float* features, int64_t n, float* out,
                   int32_t* in_range)
{
    if (!params || !scale || !features || !out || n < 0)
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_mlp_predict: bad arguments");
    if (n == 0) return BH_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return bh_fail(BH_ERR_NO_DEVICE, "bh_mlp_predict: no CUDA device");
    }
    MlpDev m;
    pack_model(params, scale, 0.0, m);
    MlpDev* dm = nullptr;
    float *df = nullptr, *dout = nullptr;
    int32_t* dr = nullptr;
    auto cleanup = [&]() { cudaFree(dm); cudaFree(df); cudaFree(dout); cudaFree(dr); };
    if (cudaMalloc(&dm, sizeof(MlpDev)) != cudaSuccess || cudaMalloc(&df, 4 * kFeat * n) != cudaSuccess ||
        cudaMalloc(&dout, 4 * n) != cudaSuccess || cudaMalloc(&dr, 4 * n) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return bh_fail(BH_ERR_OUT_OF_MEMORY, "bh_mlp_predict: device allocation failed");
    }
    cudaMemcpy(dm, &m, sizeof(MlpDev), cudaMemcpyHostToDevice);
    cudaMemcpy(df, features, 4 * kFeat * n, cudaMemcpyHostToDevice);
    const int64_t blocks = (n + 127) / 128;
    predict_kernel<<<(unsigned)blocks, 128>>>(dm, df, n, dout, dr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, 4 * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && in_range) e = cudaMemcpy(in_range, dr, 4 * n, cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) return bh_fail(BH_ERR_CUDA, std::string("bh_mlp_predict: ") + cudaGetErrorString(e));
    return BH_OK;
}

}  // extern "C"
