// mcd_detector.cu - exit directions to detector coordinates
// (MC/tools/rotation.py:78-102, projOnDetector).
//
// The reference rotates each escape direction v by the conjugate of
// q_SD = (cos(alpha/2), sin(alpha/2), 0, 0), i.e. by -alpha about x, through
// the quaternion's rotation matrix (entries divided by |q|^2), subtracts the
// translation t = (x_PC, y_PC, L) and keeps the x and y components:
//     x = v_x - x_PC
//     y = m11 v_y + m12 v_z - y_PC,   m11 = 1 - 2 s^2 / n,  m12 = 2 s c / n,
// with c = cos(alpha/2), s = sqrt(1 - c^2), n = c^2 + s^2 (host, FP64, in the
// reference's order of operations).  L only enters the dropped z component.
//
// The map is bound by HBM traffic: 3 input planes and 2 output planes in the
// structure-of-arrays layout the transport kernels write (mcd_electron_out.dir
// = dx[n], dy[n], dz[n]).  Each thread moves 16-byte vectors of every plane
// when all five planes are 16-byte aligned; a scalar loop covers the rest.
// FP32 directions are projected in FP32: FP64 arithmetic would cap the map
// below HBM speed on this part.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/mcd.h"

namespace {

struct DetMatrix {
    double m11, m12, x_pc, y_pc;
};

DetMatrix det_matrix(double alpha_deg, double x_pc, double y_pc) {
    const double c = cos(alpha_deg * 3.141592653589793 / 180.0 / 2.0);
    const double s = sqrt(1.0 - c * c);
    // conj(q) = (c, -s, 0, 0): n = c^2 + s^2, rows 1-2 of its rotation matrix
    const double w = c, x = -s;
    const double n = w * w + x * x;
    DetMatrix d;
    d.m11 = 1.0 - 2.0 * (x * x) / n;
    d.m12 = 2.0 * (0.0 - x * w) / n;
    d.x_pc = x_pc;
    d.y_pc = y_pc;
    return d;
}

template <class T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
    static constexpr int N = 4;
};
template <>
struct Vec16<double> {
    using type = double2;
    static constexpr int N = 2;
};

template <class T>
__device__ __forceinline__ T det_x(T vx, T xpc) {
    return vx - xpc;
}
template <class T>
__device__ __forceinline__ T det_y(T vy, T vz, T m11, T m12, T ypc) {
    return (m11 * vy + m12 * vz) - ypc;
}

template <class T>
__global__ void __launch_bounds__(256) k_project_vec(const T* __restrict__ dir, int64_t n, T m11, T m12, T xpc,
                                                     T ypc, T* __restrict__ xy, int64_t nvec) {
    using V = typename Vec16<T>::type;
    const V* dx = reinterpret_cast<const V*>(dir);
    const V* dy = reinterpret_cast<const V*>(dir + n);
    const V* dz = reinterpret_cast<const V*>(dir + 2 * n);
    V* ox = reinterpret_cast<V*>(xy);
    V* oy = reinterpret_cast<V*>(xy + n);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nvec; i += stride) {
        const V a = __ldcs(dx + i), b = __ldcs(dy + i), c = __ldcs(dz + i);
        V rx, ry;
        if constexpr (Vec16<T>::N == 4) {
            rx = make_float4(det_x(a.x, xpc), det_x(a.y, xpc), det_x(a.z, xpc), det_x(a.w, xpc));
            ry = make_float4(det_y(b.x, c.x, m11, m12, ypc), det_y(b.y, c.y, m11, m12, ypc),
                             det_y(b.z, c.z, m11, m12, ypc), det_y(b.w, c.w, m11, m12, ypc));
        } else {
            rx = make_double2(det_x(a.x, xpc), det_x(a.y, xpc));
            ry = make_double2(det_y(b.x, c.x, m11, m12, ypc), det_y(b.y, c.y, m11, m12, ypc));
        }
        __stcs(ox + i, rx);
        __stcs(oy + i, ry);
    }
}

template <class T>
__global__ void __launch_bounds__(256) k_project_scalar(const T* __restrict__ dir, int64_t n, T m11, T m12, T xpc,
                                                        T ypc, T* __restrict__ xy, int64_t begin) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = begin + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        xy[i] = det_x(dir[i], xpc);
        xy[n + i] = det_y(dir[n + i], dir[2 * n + i], m11, m12, ypc);
    }
}

template <class T>
int project(const T* dir, int64_t n, const DetMatrix& d, T* xy, cudaStream_t st) {
    constexpr int N = Vec16<T>::N;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCD_ECUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MCD_ECUDA;
    const int block = 256;
    const int64_t cap = (int64_t)sms * 16;   // resident blocks: 16 x 256 threads per SM
    const T m11 = (T)d.m11, m12 = (T)d.m12, xpc = (T)d.x_pc, ypc = (T)d.y_pc;
    // all five planes start at dir + k n and xy + k n: aligned iff the bases
    // are and n is a multiple of the vector width
    const bool aligned = (reinterpret_cast<uintptr_t>(dir) % 16 == 0) && (reinterpret_cast<uintptr_t>(xy) % 16 == 0) &&
                         (n % N == 0);
    int64_t done = 0;
    if (aligned) {
        const int64_t nvec = n / N;
        if (nvec > 0) {
            int64_t grid = (nvec + block - 1) / block;
            if (grid > cap) grid = cap;
            k_project_vec<T><<<(unsigned)grid, block, 0, st>>>(dir, n, m11, m12, xpc, ypc, xy, nvec);
        }
        done = nvec * N;
    }
    if (done < n) {
        int64_t grid = (n - done + block - 1) / block;
        if (grid > cap) grid = cap;
        k_project_scalar<T><<<(unsigned)grid, block, 0, st>>>(dir, n, m11, m12, xpc, ypc, xy, done);
    }
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}

}  // namespace

extern "C" int mcd_project_detector(const void* dir, int64_t n, int32_t precision, double alpha_deg, double x_pc,
                                    double y_pc, double L, void* xy, void* stream) {
    (void)L;  // enters only the z component, which the projection drops
    if (n < 0) return MCD_EINVAL;
    if (precision != MCD_FP32 && precision != MCD_FP64) return MCD_EINVAL;
    if (n == 0) return MCD_OK;
    if (!dir || !xy) return MCD_EINVAL;
    const DetMatrix d = det_matrix(alpha_deg, x_pc, y_pc);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (precision == MCD_FP32)
        return project<float>(static_cast<const float*>(dir), n, d, static_cast<float*>(xy), st);
    return project<double>(static_cast<const double*>(dir), n, d, static_cast<double*>(xy), st);
}
