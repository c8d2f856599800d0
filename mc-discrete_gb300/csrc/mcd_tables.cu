// mcd_tables.cu - FP64 fill of the sampled energy-loss CDF tables.
//
// Restates probTable.computeBlock (MC/tools/probTables.py:415-462): for each
// E row, the trapezoid of dsigma/dW between consecutive float32 grid points
// W_k, W_k+1 (their float32 difference times the mean of the two values),
// a cumulative sum along W and a division by the row total.  An interval
// whose upper edge exceeds Wmax(E) = (E - Ef)/2, evaluated in float32 as the
// reference's float32 meshes are, is masked and stored as 0
// (MC/tools/probTables.py:428-439, 507).
//
// One warp per E row: each lane owns a contiguous run of intervals, sums it,
// the warp scans the 32 partial sums, and a second pass writes the
// normalised running sums.  dsigma/dW (MC/tools/extFunctions.py:159-219) is
// evaluated in FP64.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mcd_consts.h"

namespace mcd {

struct FillParams {
    const float* Es;
    const float* Ws;
    float* cdf32;
    double* cdf64;
    int32_t* nvalid;
    uint16_t* guide;
    int32_t nE, nW;
    int32_t kind;
    double nfree;  // Moller: valence electrons; Gryzinski: shell occupancy
    double Eb;     // Gryzinski binding energy
    float Ef32;
};

__device__ __forceinline__ double dcs(const FillParams& p, double E, double W) {
    const double eps = W / E;
    if (p.kind == MCD_TABLE_MOLLER) {
        if (!(eps < 1.0)) return 0.0;
        return p.nfree * kPiEfour * (1.0 / (eps * eps) + 1.0 / ((1.0 - eps) * (1.0 - eps)) - 1.0 / (eps * (1.0 - eps))) /
               (E * E * E);
    }
    const double epsB = p.Eb / E;
    if (!(eps < 1.0) || !(epsB < 1.0)) return 0.0;
    return p.nfree * kPiEfour * eps * pow(1.0 + epsB, -1.5) * pow(1.0 - eps, epsB / (epsB + eps)) *
           ((1.0 - epsB) + 4.0 * epsB * log(2.7 + sqrt((1.0 - eps) / epsB)) / (3.0 * eps)) / (W * W * W);
}

__global__ void __launch_bounds__(256) k_fill(const FillParams p) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + warp;
    if (row >= p.nE) return;
    const float e32 = p.Es[row];
    const double E = (double)e32;
    const float wmax = __fmul_rn(__fsub_rn(e32, p.Ef32), 0.5f);
    const int nint = p.nW - 1;
    const int per = (nint + 31) / 32;
    const int k0 = lane * per;
    const int k1 = min(k0 + per, nint);
    // pass 1: partial sum over this lane's intervals
    double part = 0.0;
    int valid = 0;
    if (k0 < k1) {
        float wa = p.Ws[k0];
        double fa = dcs(p, E, (double)wa);
        for (int k = k0; k < k1; ++k) {
            const float wb = p.Ws[k + 1];
            const double fb = dcs(p, E, (double)wb);
            if (wb <= wmax) {
                part += (double)__fsub_rn(wb, wa) * (fa + fb) / 2.0;
                ++valid;
            }
            wa = wb;
            fa = fb;
        }
    }
    // warp scan of the partial sums (exclusive)
    double incl = part;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const double total = __shfl_sync(0xffffffffu, incl, 31);
    const int nval = __reduce_add_sync(0xffffffffu, valid);
    double run = incl - part;
    // pass 2: normalised running sums
    if (k0 < k1) {
        float wa = p.Ws[k0];
        double fa = dcs(p, E, (double)wa);
        const size_t base = (size_t)row * nint;
        for (int k = k0; k < k1; ++k) {
            const float wb = p.Ws[k + 1];
            const double fb = dcs(p, E, (double)wb);
            double v = 0.0;
            float v32 = 0.0f;
            if (wb <= wmax) {
                run += (double)__fsub_rn(wb, wa) * (fa + fb) / 2.0;
                // the valid intervals are a prefix (Ws ascends), and the
                // reference's last valid entry is cum/cum = 1 exactly
                v = (k == nval - 1) ? 1.0 : fmin(run / total, 1.0);
                v32 = __double2float_rn(v);
            }
            p.cdf32[base + k] = v32;
            if (p.cdf64) p.cdf64[base + k] = v;
            wa = wb;
            fa = fb;
        }
    }
    if (lane == 0 && p.nvalid) p.nvalid[row] = nval;
    if (p.guide) {
        // guide[k] = first entry >= k/G among the unmasked prefix (as the
        // sampler's bisection sees the row); the row was written by this warp
        __syncwarp();
        const float* r = p.cdf32 + (size_t)row * nint;
        for (int k = lane; k <= MCD_GUIDE; k += 32) {
            const float q = (float)k / (float)MCD_GUIDE;
            int lo = 0, hi = nval;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                const float v = r[mid];
                if (v != 0.0f && v < q) lo = mid + 1; else hi = mid;
            }
            p.guide[(size_t)row * (MCD_GUIDE + 1) + k] = (uint16_t)lo;
        }
    }
}

}  // namespace mcd

using namespace mcd;

extern "C" int mcd_build_table(int kind, const mcd_material* mat, int shell, int32_t nE, int32_t nW,
                               const float* Es, const float* Ws, float* cdf32, double* cdf64, int32_t* nvalid,
                               uint16_t* guide, void* stream) {
    if (!mat || !Es || !Ws || !cdf32) return MCD_EINVAL;
    if (nE < 1 || nW < 2) return MCD_EINVAL;
    if (guide && nW - 1 > 65535) return MCD_EINVAL;   // column indices must fit 16 bits
    if (kind != MCD_TABLE_MOLLER && kind != MCD_TABLE_GRYZ) return MCD_EINVAL;
    FillParams p;
    p.Es = Es;
    p.Ws = Ws;
    p.cdf32 = cdf32;
    p.cdf64 = cdf64;
    p.nvalid = nvalid;
    p.guide = guide;
    p.nE = nE;
    p.nW = nW;
    p.kind = kind;
    p.Ef32 = (float)mat->fermi_e;
    if (kind == MCD_TABLE_MOLLER) {
        p.nfree = mat->n_val;
        p.Eb = 0.0;
    } else {
        if (shell < 0 || shell >= mat->n_shells) return MCD_EINVAL;
        p.nfree = mat->shell_n[shell];
        p.Eb = mat->shell_E[shell];
    }
    const int rows_per_block = 8;
    const unsigned grid = (unsigned)((nE + rows_per_block - 1) / rows_per_block);
    k_fill<<<grid, 32 * rows_per_block, 0, static_cast<cudaStream_t>(stream)>>>(p);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}
