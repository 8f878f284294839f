// Self-checks of the arithmetic helpers that replace IEEE divisions and
// square roots on the hot path, against the IEEE operations themselves on
// seeded random and adversarial inputs (bh_selftest).  No reference
// counterpart.
#include "bh_internal.cuh"

namespace {

__device__ inline uint64_t mix64(uint64_t x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Uniform in [0, 1) from 53 random bits.
__device__ inline double unit(uint64_t r) { return (double)(r >> 11) * 0x1p-53; }

// A double with a random 52-bit mantissa and exponent e.
__device__ inline double with_exp(uint64_t r, int e)
{
    return __longlong_as_double((long long)(((uint64_t)(e + 1023) << 52) | (r & 0x000FFFFFFFFFFFFFull)));
}

// which = 0: merge_div(m, c) == RN((0 + RN(m c)) / m)
// which = 1: quantise(...) == quantise_exact(...)
// which = 2: rsqrt_hh(x) within 2 ulps of RN(1 / RN(sqrt(x)))
// which = 3: div_exact(w, m, rcp_nr(m)) == RN(w / m)
// which = 4: rcube_hh(x) within 4 ulps of RN(1 / RN(x RN(sqrt(x))))
// which = 5: low_part(x) == narrow_trunc(x - widen(narrow_trunc(x)))
__global__ void selftest_kernel(int which, int64_t n, uint64_t seed, unsigned long long* fails)
{
    unsigned long long bad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t r0 = mix64(seed ^ (uint64_t)i * 0x2545F4914F6CDD1Dull), r1 = mix64(r0), r2 = mix64(r1),
                       r3 = mix64(r2);
        if (which == 0) {
            // masses 2^-10 .. 2^110, centres 2^-40 .. 2^12 of either sign;
            // one case in 8 a power of two, one in 8 the largest mantissa.
            const double m = with_exp(r0, -10 + (int)(r1 % 120));
            double c = with_exp(r2, -40 + (int)(r3 % 52));
            const int kind = (int)((r3 >> 20) & 7);
            if (kind == 0) c = with_exp(0, -40 + (int)(r3 % 52));
            if (kind == 1) c = with_exp(~0ull, -40 + (int)(r3 % 52));
            if ((r3 >> 24) & 1) c = -c;
            const double want = __ddiv_rn(__dadd_rn(0.0, __dmul_rn(m, c)), m);
            const double got = bh::merge_div(m, c);
            bad += __double_as_longlong(want) != __double_as_longlong(got);
        } else if (which == 1) {
            // boxes of span 2^-10 .. 2^10 around offsets up to 2^8; points
            // uniform over the box +-10 %, one in 4 within 2^-30 of a cell
            // boundary of the 2^21 grid.
            const double lo = (unit(r0) - 0.5) * 512.0;
            const double span = with_exp(r1, -10 + (int)(r1 % 20));
            double v = lo + (unit(r2) * 1.2 - 0.1) * span;
            if ((r3 & 3) == 0) {
                const double k = (double)(r3 >> 43);  // 0 .. 2^21 - 1
                v = lo + (k * 0x1p-21) * span + (unit(r2) - 0.5) * 0x1p-30 * span;
            }
            const double inv = __drcp_rn(span) * 2097152.0;
            bad += bh::quantise(v, lo, span, inv) != bh::quantise_exact(v, lo, span);
        } else if (which == 3) {
            // sums over 2^-50 .. 2^120 of either sign (one in 8 a rounded
            // product m c, as a one-body sum is) over masses 2^-10 .. 2^110
            const double m = with_exp(r0, -10 + (int)(r1 % 120));
            double w = with_exp(r2, -50 + (int)(r3 % 170));
            if ((r3 >> 30) & 1) w = -w;
            if (((r3 >> 31) & 7) == 0) w = __dmul_rn(m, with_exp(r2, -20 + (int)(r3 % 40)));
            const double want = __ddiv_rn(w, m);
            const double got = bh::div_exact(w, m, bh::rcp_nr(m));
            bad += __double_as_longlong(want) != __double_as_longlong(got);
        } else if (which == 4) {
            const double x = with_exp(r0, -90 + (int)(r1 % 180));
            const double want = __drcp_rn(__dmul_rn(x, __dsqrt_rn(x)));
            const double got = bh::rcube_hh(x);
            const long long d = __double_as_longlong(want) - __double_as_longlong(got);
            bad += (d > 4 || d < -4);
        } else if (which == 5) {
            // either sign, exponents 2^-300 .. 2^300 (both ends of the FP32
            // range and past them); one in 8 with the low 29 bits clear, one
            // in 8 with only a few low bits set
            uint64_t bits = ((uint64_t)(723 + (int)(r1 % 600)) << 52) | (r0 & 0x000FFFFFFFFFFFFFull);
            const int kind = (int)((r2 >> 7) & 7);
            if (kind == 0) bits &= ~0x1FFFFFFFull;
            if (kind == 1) bits = (bits & ~0x1FFFFFFFull) | (r3 & 0xFFull);
            if ((r2 >> 3) & 1) bits |= 1ull << 63;
            const double x = __longlong_as_double((long long)bits);
            const float want = bh::narrow_trunc(x - bh::widen(bh::narrow_trunc(x)));
            bad += __float_as_int(want) != __float_as_int(bh::low_part(x));
        } else {
            const double x = with_exp(r0, -90 + (int)(r1 % 180));
            const double want = __drcp_rn(__dsqrt_rn(x));
            const double got = bh::rsqrt_hh(x);
            const long long d = __double_as_longlong(want) - __double_as_longlong(got);
            bad += (d > 2 || d < -2);
        }
    }
    if (bad) atomicAdd(fails, bad);
}

}  // namespace

extern "C" int bh_selftest(int which, int64_t n, uint64_t seed, int64_t* failures)
{
    if (which < 0 || which > 5 || n < 0 || !failures) return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_selftest: bad arguments");
    int dev = 0;
    BH_CUDA_TRY(cudaGetDevice(&dev));
    unsigned long long* d = nullptr;
    BH_CUDA_TRY(cudaMalloc(&d, sizeof(unsigned long long)));
    BH_CUDA_TRY(cudaMemset(d, 0, sizeof(unsigned long long)));
    const int64_t blocks64 = (n + 255) / 256;
    const int blocks = (int)(blocks64 < 1 ? 1 : (blocks64 > 8 * bh::num_sms() ? 8 * bh::num_sms() : blocks64));
    selftest_kernel<<<blocks, 256>>>(which, n, seed, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return bh_fail(BH_ERR_CUDA, std::string("bh_selftest: ") + cudaGetErrorString(e));
    *failures = (int64_t)h;
    return BH_OK;
}
