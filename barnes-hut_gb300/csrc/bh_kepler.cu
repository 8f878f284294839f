// Batched Kepler-to-Cartesian conversion on the GPU: one thread per body,
// the operation sequence of convertKeplerToCartesian
// (src/kepler_to_cartesian.cpp:13-107) as bh_kepler_to_cartesian restates it
// on the host (mean anomaly to J2000, Newton on E - e sin E = M with
// |dE| < 1e-8 and at most 100 iterations, true anomaly, perifocal state,
// rotation by Omega, i, omega), with CUDA's FP64 math functions.  Results
// agree with the host conversion to rounding (the math libraries differ in
// their last bits).  It moves the setup of multi-million-body systems off the
// host's scalar libm.
#include "bh_internal.cuh"

namespace {

constexpr double kJ2000Dev = 2451544.5;  // the conversion epoch of the host restatement

__global__ void kepler_kernel(int64_t n, const double* __restrict__ el, double* __restrict__ out)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const double* q = el + 8 * k;
        const double e = q[0], a = q[1], inc = q[2], w = q[3], Om = q[4], epoch = q[6], mu = q[7];
        double M = q[5];
        const double nmot = sqrt(mu / pow(a, 3.0));
        M += nmot * (kJ2000Dev - epoch);
        M = fmod(M, 2 * M_PI);
        if (M < 0) M += 2 * M_PI;
        double E = M;
        for (int it = 0; it < 100; ++it) {
            const double f = E - e * sin(E) - M;
            const double fp = 1 - e * cos(E);
            const double d = -f / fp;
            E += d;
            if (fabs(d) < 1e-8) break;
        }
        const double nu = 2 * atan2(sqrt(1 + e) * sin(E / 2), sqrt(1 - e) * cos(E / 2));
        const double r = a * (1 - e * cos(E));
        const double xo = r * cos(nu), yo = r * sin(nu);
        const double h = sqrt(mu * a) / r;
        const double vxo = h * (-sin(E)), vyo = h * sqrt(1 - e * e) * cos(E);
        const double cO = cos(Om), sO = sin(Om), ci = cos(inc), si = sin(inc);
        const double cw = cos(w), sw = sin(w);
        const double R11 = cO * cw - sO * sw * ci, R12 = -cO * sw - sO * cw * ci;
        const double R21 = sO * cw + cO * sw * ci, R22 = -sO * sw + cO * cw * ci;
        const double R31 = sw * si, R32 = cw * si;
        double* o = out + 6 * k;
        o[0] = R11 * xo + R12 * yo;
        o[1] = R21 * xo + R22 * yo;
        o[2] = R31 * xo + R32 * yo;
        o[3] = R11 * vxo + R12 * vyo;
        o[4] = R21 * vxo + R22 * vyo;
        o[5] = R31 * vxo + R32 * vyo;
    }
}

}  // namespace

extern "C" int bh_kepler_to_cartesian_gpu(const double* el, int64_t n, double* out)
{
    if (n < 0 || (n > 0 && (!el || !out)))
        return bh_fail(BH_ERR_INVALID_ARGUMENT, "bh_kepler_to_cartesian_gpu: bad arguments");
    if (n == 0) return BH_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return bh_fail(BH_ERR_NO_DEVICE, "bh_kepler_to_cartesian_gpu: no CUDA device");
    double *del = nullptr, *dout = nullptr;
    cudaError_t e = cudaMalloc(&del, sizeof(double) * 8 * n);
    if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(double) * 6 * n);
    if (e == cudaSuccess) e = cudaMemcpy(del, el, sizeof(double) * 8 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int64_t want = (n + 255) / 256;
        const int blocks = (int)(want > 16 * bh::num_sms() ? 16 * bh::num_sms() : want);
        kepler_kernel<<<blocks, 256>>>(n, del, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost);
    cudaFree(del);
    cudaFree(dout);
    if (e != cudaSuccess) return bh_fail(BH_ERR_CUDA, std::string("bh_kepler_to_cartesian_gpu: ") + cudaGetErrorString(e));
    return BH_OK;
}
