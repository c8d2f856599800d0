// mcd_adjoint.cu - pathwise gradients of continuous-mode exit-energy tallies.
//
// Continuous mode (MC/tools/singleScatter.py:205-239) changes the energy
// only through E_{k+1} = E_k - s_k S(E_k), with s_k = -ln(U_k) / sigma'(E_k)
// the Rutherford step (MC/tools/scattering.py:802-826) and S the Bethe law
// (MC/tools/stoppingPowers.py:112-215).  With the random numbers and the
// event sequence frozen (the event k* in which an electron leaves through
// the surface is fixed), the exit energy E_{k*} is a smooth function of the
// Bethe mean ionisation energy J and of the density n, and its gradient is a
// scalar reverse sweep along that recursion:
//
//   lambda_{k*} = dL/dE_exit
//   dL/dJ      += lambda_{k+1} * (-s_k dS/dJ(E_k))
//   dL/dn      += lambda_{k+1} * (-(ds_k/dn S + s_k dS/dn))     (= 0: s ~ 1/n, S ~ n)
//   lambda_k    = lambda_{k+1} * (1 - ds_k/dE S - s_k dS/dE)
//
// The forward kernel runs the full transport (positions and directions decide
// k*) and stores E every 64 events; the backward kernel recomputes each
// 64-event segment from its checkpoint and the Philox counters, then sweeps
// it in reverse.  Tallies are Gaussian-soft bins of the exit energy of
// backscattered electrons, h_b = (1/N) sum exp(-(E - c_b)^2 / (2 sigma^2)),
// and the sum of exit energies.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mcd_device.cuh"

namespace mcd {

constexpr int kSeg = 64;  // events per checkpoint segment

struct AdjBuf {
    void* ckpt;        // T, max_ckpt x num_el (checkpoint-major)
    int32_t* kstar;    // exit event of 'bks' electrons, -1 otherwise
    void* E_exit;      // T
    int32_t max_ckpt;
};

struct SoftHist {
    int32_t nbins;
    double lo, width, inv2s2, inv_s2;
};

// Gaussian soft bins within 8 sigma of E: calls f(bin, weight, d = E - c_b)
template <class F>
__device__ __forceinline__ void soft_bins(const SoftHist& sh, double E, F f) {
    const double reach = 8.0 * rsqrt(2.0 * sh.inv2s2);
    int b0 = (int)floor((E - reach - sh.lo) / sh.width - 0.5);
    int b1 = (int)ceil((E + reach - sh.lo) / sh.width - 0.5);
    b0 = b0 < 0 ? 0 : b0;
    b1 = b1 > sh.nbins - 1 ? sh.nbins - 1 : b1;
    for (int b = b0; b <= b1; ++b) {
        const double d = E - (sh.lo + (b + 0.5) * sh.width);
        f(b, exp(-d * d * sh.inv2s2), d);
    }
}

template <class T, class C>
__device__ __forceinline__ T step_len(const C& c, T E, uint64_t elec, int64_t k) {
    const uint4 r = philox(make_uint4((uint32_t)k, (uint32_t)elec, (uint32_t)(elec >> 32), c.sim_id), c.key0,
                           c.key1);
    return -Ops<T>::ln_step(Ops<T>::unit(r.y)) * Ops<T>::div((T)1, sig_ruth<T>(c, E));
}

// dS/dE and dS/dJ_scale of the Bethe law at E (S itself returned in *S)
template <class T, class C>
__device__ __forceinline__ void stopping_derivs(const C& c, T E, T* S, T* SE, T* Sj) {
    const T s = stopping<T>(c, E);
    *S = s;
    if (c.bethe == MCD_BETHE_CLASSICAL) {
        *SE = Ops<T>::div(c.bP, E * E) - Ops<T>::div(s, E);
        *Sj = -Ops<T>::div(c.bP, E);                       // J dS/dJ, J = J0 * J_scale
    } else if (c.bethe == MCD_BETHE_JL) {
        *SE = Ops<T>::div(c.bP, E * (E + c.bkJ)) - Ops<T>::div(s, E);
        *Sj = Ops<T>::div(c.bP, E) * (Ops<T>::div(c.bkJ, E + c.bkJ) - (T)1);
    } else {
        *SE = Ops<T>::div(c.bX * c.bW, E * E) - Ops<T>::div(s, E);
        *Sj = (T)0;
    }
}

// d ln(sigma'_R)/dE
template <class T, class C>
__device__ __forceinline__ T dlnsig(const C& c, T E) {
    const T rel = c.ruth_r2 ? (T)2 * (Ops<T>::div((T)1, E + (T)511000) - Ops<T>::div((T)1, E + (T)1024000))
                            : (T)0;
    return rel - Ops<T>::div((T)1, E + c.aS);
}

template <class T>
__global__ void __launch_bounds__(256) k_adj_fwd(const SimConst<T> cp, const SoftHist sh, const AdjBuf buf,
                                                 double* hout, mcd_tally* tally, uint32_t* status) {
    __shared__ SimConst<T> c;  // see k_plain: constants are read from shared memory
    __shared__ double sh_h[MCD_HIST_E_MAX + 2];
    __shared__ unsigned long long s_cnt[9];
    if (threadIdx.x == 0) c = cp;
    for (int b = threadIdx.x; b < sh.nbins + 2; b += blockDim.x) sh_h[b] = 0.0;
    if (threadIdx.x < 9) s_cnt[threadIdx.x] = 0ull;
    __syncthreads();
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t st = 0;
    if (i < (uint64_t)c.num_el) {
        Lane<T> L;
        lane_init(L, c);
        const uint64_t elec = c.first + i;
        T* ck = static_cast<T*>(buf.ckpt);
        const size_t n = (size_t)c.num_el;
        int kstar = -1;
        while (L.outcome == MCD_OUT_NONE) {
            if ((L.step % kSeg) == 0) {
                const int64_t m = L.step / kSeg;
                if (m < buf.max_ckpt) ck[(size_t)m * n + i] = L.E;
            }
            EventOut<T> ev;
            cont_event<T, false>(L, c, elec, &ev);
            if (L.outcome == MCD_OUT_BKS) kstar = (int)(L.step - 1);
        }
        const bool bks = L.outcome == MCD_OUT_BKS;
        if (bks && kstar > 0 && (kstar - 1) / kSeg >= buf.max_ckpt) st |= MCD_FLAG_CKPT;
        buf.kstar[i] = bks ? kstar : -1;
        static_cast<T*>(buf.E_exit)[i] = L.E_row;
        if (bks) {
            const double E = (double)L.E_row;
            soft_bins(sh, E, [&](int b, double w, double) { if (w > 0.0) atomicAdd(&sh_h[b], w); });
            atomicAdd(&sh_h[sh.nbins], E);
            atomicAdd(&sh_h[sh.nbins + 1], 1.0);
        }
        atomicAdd(&s_cnt[L.outcome & 7], 1ull);
        atomicAdd(&s_cnt[8], (unsigned long long)L.step);
        if (L.flags & F_CLAMPED) st |= MCD_FLAG_CLAMPED;
        if (L.flags & F_LONG_PATH) st |= MCD_FLAG_LONG_PATH;
        if (L.outcome == MCD_OUT_LONG) st |= MCD_FLAG_LONG;
    }
    const uint32_t w = __reduce_or_sync(0xffffffffu, st);
    if ((threadIdx.x & 31) == 0 && w) atomicOr(status, w);
    __syncthreads();
    for (int b = threadIdx.x; b < sh.nbins + 2; b += blockDim.x)
        if (sh_h[b] != 0.0) atomicAdd(&hout[b], sh_h[b]);
    if (tally && threadIdx.x < 9 && s_cnt[threadIdx.x]) {
        if (threadIdx.x < 8) atomicAdd(&tally->outcome[threadIdx.x], s_cnt[threadIdx.x]);
        else atomicAdd(&tally->events, s_cnt[8]);
    }
}

template <class T>
__global__ void __launch_bounds__(128) k_adj_bwd(const SimConst<T> cp, const SoftHist sh, const AdjBuf buf,
                                                 const double* grad_h, double inv_n, double inv_j,
                                                 double inv_ns, double* grad) {
    __shared__ SimConst<T> c;
    __shared__ double red[2];
    if (threadIdx.x == 0) {
        c = cp;
        red[0] = red[1] = 0.0;
    }
    __syncthreads();
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double gj = 0.0, gn = 0.0;
    if (i < (uint64_t)c.num_el) {
        const int kstar = buf.kstar[i];
        if (kstar > 0 && (kstar - 1) / kSeg < buf.max_ckpt) {
            const T* ck = static_cast<const T*>(buf.ckpt);
            const size_t n = (size_t)c.num_el;
            const uint64_t elec = c.first + i;
            // lambda at the exit energy: derivative of the soft-bin weights + the sum
            const double Ex = (double)static_cast<const T*>(buf.E_exit)[i];
            double lam0 = grad_h[sh.nbins];
            soft_bins(sh, Ex, [&](int b, double w, double d) { lam0 += grad_h[b] * inv_n * (-d * sh.inv_s2) * w; });
            // the sweep runs in the transport precision: lambda is a product of
            // factors 1 + O(1e-2) and each step adds one term to the sums
            T lam = (T)lam0, sj = (T)0, sn = (T)0;
            const T ij = (T)inv_j, ins = (T)inv_ns;
            T Eseg[kSeg], sseg[kSeg];
            for (int m = (kstar - 1) / kSeg; m >= 0; --m) {
                const int k0 = m * kSeg;
                const int len = min(kSeg, kstar - k0);
                T E = ck[(size_t)m * n + i];
                for (int j = 0; j < len; ++j) {   // recompute the segment exactly as the forward did
                    const T s = step_len<T>(c, E, elec, k0 + j);
                    Eseg[j] = E;
                    sseg[j] = s;
                    E = E - Ops<T>::mul_rn(s, stopping<T>(c, E));
                }
                for (int j = len - 1; j >= 0; --j) {   // reverse sweep
                    const T Ek = Eseg[j], s = sseg[j];
                    T S, SE, Sj;
                    stopping_derivs<T>(c, Ek, &S, &SE, &Sj);
                    sj += lam * (-s * Sj * ij);
                    // ds/dn = -s/n and dS/dn = S/n: the two terms cancel
                    sn += lam * (-((-s * ins) * S + s * (S * ins)));
                    lam *= (T)1 + s * (dlnsig<T>(c, Ek) * S - SE);
                }
            }
            gj = (double)sj;
            gn = (double)sn;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        gj += __shfl_down_sync(0xffffffffu, gj, o);
        gn += __shfl_down_sync(0xffffffffu, gn, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&red[0], gj);
        atomicAdd(&red[1], gn);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(&grad[0], red[0]);
        atomicAdd(&grad[1], red[1]);
    }
}

// E_{k*}(J, n) along the frozen event sequence only (no geometry): the
// function the adjoint differentiates, for finite-difference checks.
template <class T>
__global__ void __launch_bounds__(256) k_adj_chain(const SimConst<T> cp, const SoftHist sh, const AdjBuf buf,
                                                   double* hout) {
    __shared__ SimConst<T> c;
    __shared__ double sh_h[MCD_HIST_E_MAX + 2];
    if (threadIdx.x == 0) c = cp;
    for (int b = threadIdx.x; b < sh.nbins + 2; b += blockDim.x) sh_h[b] = 0.0;
    __syncthreads();
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (uint64_t)c.num_el) {
        const int kstar = buf.kstar[i];
        if (kstar >= 0) {
            const uint64_t elec = c.first + i;
            T E = c.E0;
            for (int k = 0; k < kstar; ++k) {
                const T s = step_len<T>(c, E, elec, k);
                E = E - Ops<T>::mul_rn(s, stopping<T>(c, E));
            }
            const double Ed = (double)E;
            soft_bins(sh, Ed, [&](int b, double w, double) { if (w > 0.0) atomicAdd(&sh_h[b], w); });
            atomicAdd(&sh_h[sh.nbins], Ed);
            atomicAdd(&sh_h[sh.nbins + 1], 1.0);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < sh.nbins + 2; b += blockDim.x)
        if (sh_h[b] != 0.0) atomicAdd(&hout[b], sh_h[b]);
}

static int adj_args(const mcd_sim* sim, const mcd_material* mat, const mcd_softhist* hist,
                    const mcd_adjoint_buf* buf, SoftHist* sh, AdjBuf* ab) {
    if (!sim || !mat || !hist || !buf) return MCD_EINVAL;
    const int rc = check_sim(*sim, *mat, nullptr, nullptr);
    if (rc != MCD_OK) return rc;
    if (sim->mode != MCD_MODE_CONT) return MCD_EINVAL;
    if (hist->nbins < 1 || hist->nbins > MCD_HIST_E_MAX) return MCD_ETOOBIG;
    if (!(hist->sigma > 0) || !(hist->hi > hist->lo)) return MCD_EINVAL;
    if (!buf->ckpt || !buf->kstar || !buf->E_exit || buf->max_ckpt < 1) return MCD_EINVAL;
    if (!(sim->J_scale >= 0) || !(sim->n_scale >= 0)) return MCD_EINVAL;
    sh->nbins = hist->nbins;
    sh->lo = hist->lo;
    sh->width = (hist->hi - hist->lo) / hist->nbins;
    sh->inv2s2 = 1.0 / (2.0 * hist->sigma * hist->sigma);
    sh->inv_s2 = 1.0 / (hist->sigma * hist->sigma);
    ab->ckpt = buf->ckpt;
    ab->kstar = buf->kstar;
    ab->E_exit = buf->E_exit;
    ab->max_ckpt = buf->max_ckpt;
    return MCD_OK;
}

}  // namespace mcd

using namespace mcd;

extern "C" int mcd_adjoint_forward(const mcd_sim* sim, const mcd_material* mat, const mcd_softhist* hist,
                                   const mcd_adjoint_buf* buf, double* hist_out, mcd_tally* tally,
                                   uint32_t* status, void* stream) {
    SoftHist sh;
    AdjBuf ab;
    int rc = adj_args(sim, mat, hist, buf, &sh, &ab);
    if (rc != MCD_OK) return rc;
    if (!hist_out || !status) return MCD_EINVAL;
    const unsigned long long grid = ((unsigned long long)sim->num_el + 255) / 256;
    if (grid == 0) return MCD_OK;
    if (grid > 0x7fffffffull) return MCD_ETOOBIG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (sim->precision == MCD_FP64)
        k_adj_fwd<double><<<(unsigned)grid, 256, 0, st>>>(make_consts<double>(*sim, *mat, nullptr, nullptr), sh, ab,
                                                           hist_out, tally, status);
    else
        k_adj_fwd<float><<<(unsigned)grid, 256, 0, st>>>(make_consts<float>(*sim, *mat, nullptr, nullptr), sh, ab,
                                                          hist_out, tally, status);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}

extern "C" int mcd_adjoint(const mcd_sim* sim, const mcd_material* mat, const mcd_softhist* hist,
                           const mcd_adjoint_buf* buf, const double* grad_hist, double* grad, void* stream) {
    SoftHist sh;
    AdjBuf ab;
    int rc = adj_args(sim, mat, hist, buf, &sh, &ab);
    if (rc != MCD_OK) return rc;
    if (!grad_hist || !grad) return MCD_EINVAL;
    const unsigned long long grid = ((unsigned long long)sim->num_el + 127) / 128;
    if (grid == 0) return MCD_OK;
    if (grid > 0x7fffffffull) return MCD_ETOOBIG;
    const double inv_n = 1.0 / (double)sim->num_el;
    const double js = 1.0 / (sim->J_scale > 0 ? sim->J_scale : 1.0);
    const double ns = 1.0 / (sim->n_scale > 0 ? sim->n_scale : 1.0);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (sim->precision == MCD_FP64)
        k_adj_bwd<double><<<(unsigned)grid, 128, 0, st>>>(make_consts<double>(*sim, *mat, nullptr, nullptr), sh, ab,
                                                           grad_hist, inv_n, js, ns, grad);
    else
        k_adj_bwd<float><<<(unsigned)grid, 128, 0, st>>>(make_consts<float>(*sim, *mat, nullptr, nullptr), sh, ab,
                                                          grad_hist, inv_n, js, ns, grad);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}

extern "C" int mcd_adjoint_chain(const mcd_sim* sim, const mcd_material* mat, const mcd_softhist* hist,
                                 const mcd_adjoint_buf* buf, double* hist_out, void* stream) {
    SoftHist sh;
    AdjBuf ab;
    int rc = adj_args(sim, mat, hist, buf, &sh, &ab);
    if (rc != MCD_OK) return rc;
    if (!hist_out) return MCD_EINVAL;
    const unsigned long long grid = ((unsigned long long)sim->num_el + 255) / 256;
    if (grid == 0) return MCD_OK;
    if (grid > 0x7fffffffull) return MCD_ETOOBIG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (sim->precision == MCD_FP64)
        k_adj_chain<double><<<(unsigned)grid, 256, 0, st>>>(make_consts<double>(*sim, *mat, nullptr, nullptr), sh, ab,
                                                             hist_out);
    else
        k_adj_chain<float><<<(unsigned)grid, 256, 0, st>>>(make_consts<float>(*sim, *mat, nullptr, nullptr), sh, ab,
                                                            hist_out);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}
