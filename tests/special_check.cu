// Test kernels of the GPU tests (not part of the library): evaluate the FP64
// transport's table-driven logarithm, sin/cos(pi u) and cos/sin(2 pi u) of
// Philox words, as the transport calls them, for comparison with 40-digit
// values and the host's libm, and its Newton-Raphson reciprocal.
#include <cstdint>

#include "mcd_device.cuh"

namespace {
__global__ void k_special(const uint32_t* w, int64_t n, double* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s, c;
    mcd::sincospi_word(w[i], &s, &c);
    out[5 * i] = mcd::ln_word(w[i]);
    out[5 * i + 1] = s;
    out[5 * i + 2] = c;
    mcd::cossin2pi_word(w[i], &out[5 * i + 3], &out[5 * i + 4]);
    // the adjoint's form of the same sin/cos, from the uniform as a double
    double s2, c2;
    mcd::sincospi_uniform(mcd::Ops<double>::unit(w[i]), &s2, &c2);
    if (s2 != s || c2 != c) out[5 * i + 1] = __longlong_as_double(0x7ff8000000000000ll);
}

__global__ void k_rcp(const double* d, int64_t n, double* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = mcd::rcp_pos(d[i]);
}
}  // namespace

// d (host, n, positive normal) -> out (host, n): the FP64 transport's 1/d
extern "C" int rcp_eval(const double* d, int64_t n, double* out) {
    double *dd = nullptr, *dout = nullptr;
    if (cudaMalloc(&dd, n * sizeof(double)) != cudaSuccess) return 1;
    if (cudaMalloc(&dout, n * sizeof(double)) != cudaSuccess) {
        cudaFree(dd);
        return 1;
    }
    int rc = 0;
    if (cudaMemcpy(dd, d, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) rc = 2;
    if (!rc) {
        k_rcp<<<(unsigned)((n + 255) / 256), 256>>>(dd, n, dout);
        if (cudaGetLastError() != cudaSuccess) rc = 3;
    }
    if (!rc && cudaMemcpy(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) rc = 4;
    cudaFree(dd);
    cudaFree(dout);
    return rc;
}

// words (host, n) -> out (host, 5 n: ln U, sin pi U, cos pi U, cos 2 pi U,
// sin 2 pi U); 0 on success
extern "C" int special_eval(const uint32_t* words, int64_t n, double* out) {
    uint32_t* dw = nullptr;
    double* dout = nullptr;
    if (cudaMalloc(&dw, n * sizeof(uint32_t)) != cudaSuccess) return 1;
    if (cudaMalloc(&dout, 5 * n * sizeof(double)) != cudaSuccess) {
        cudaFree(dw);
        return 1;
    }
    int rc = 0;
    if (cudaMemcpy(dw, words, n * sizeof(uint32_t), cudaMemcpyHostToDevice) != cudaSuccess) rc = 2;
    if (!rc) {
        k_special<<<(unsigned)((n + 255) / 256), 256>>>(dw, n, dout);
        if (cudaGetLastError() != cudaSuccess) rc = 3;
    }
    if (!rc && cudaMemcpy(out, dout, 5 * n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) rc = 4;
    cudaFree(dw);
    cudaFree(dout);
    return rc;
}
