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
    unsigned long long* queue;   // the forward pass's work queue, or nullptr
};

struct SoftHist {
    int32_t nbins;
    int32_t quantity;   // MCD_ADJ_EXIT_E or MCD_ADJ_MAX_DEPTH
    double lo, width, inv2s2, inv_s2;
    double inv_width, reach;   // 1 / width; 8 sigma
    // the same in FP32, for FP32 runs: their soft bins are evaluated in FP32
    // (and summed in FP64), so that an FP32 run issues no FP64 arithmetic
    // per electron -- the backward takes its electrons a few lanes at a time,
    // and the FP64 unit charges each of those instructions in full
    float f_lo, f_inv_width, f_width, f_inv2s2, f_inv_s2, f_reach;
};

constexpr int kDepthState = 8;   // E, z, d (3), y (3) per depth checkpoint

// Gaussian soft bins within 8 sigma of the quantity q, in the transport
// precision T: calls f(bin, weight, d = q - c_b)
template <class T, class F>
__device__ __forceinline__ void soft_bins(const SoftHist& sh, T q, F f) {
    T lo, w, iw, i2, reach;
    if constexpr (sizeof(T) == 8) {
        lo = sh.lo, w = sh.width, iw = sh.inv_width, i2 = sh.inv2s2, reach = sh.reach;
    } else {
        lo = sh.f_lo, w = sh.f_width, iw = sh.f_inv_width, i2 = sh.f_inv2s2, reach = sh.f_reach;
    }
    int b0 = (int)floor((q - reach - lo) * iw - (T)0.5);
    int b1 = (int)ceil((q + reach - lo) * iw - (T)0.5);
    b0 = b0 < 0 ? 0 : b0;
    b1 = b1 > sh.nbins - 1 ? sh.nbins - 1 : b1;
    for (int b = b0; b <= b1; ++b) {
        const T d = q - (lo + ((T)b + (T)0.5) * w);
        f(b, exp(-d * d * i2), d);
    }
}

template <class T, class C>
__device__ __forceinline__ T step_len(const C& c, T E, uint64_t elec, int64_t k) {
    const uint4 r = philox(make_uint4((uint32_t)k, (uint32_t)elec, (uint32_t)(elec >> 32), c.sim_id), c.key0,
                           c.key1);
    return -Ops<T>::ln_step_word(r.y) * Ops<T>::div((T)1, sig_ruth<T>(c, E));
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

// The forward pass: every electron's full transport, with its checkpoints
// every kSeg events.  With a queue word (buf.queue) the grid is resident and
// a lane that finishes its electron takes the next from the queue, so that
// lanes do not idle while the longest trajectory of their warp runs (one
// thread per electron kept about 18 of 32 lanes busy); without one, each
// warp takes `range` = 32 consecutive electrons, one per lane.
template <class T>
__global__ void __launch_bounds__(256) k_adj_fwd(const SimConst<T> cp, const SoftHist sh, const AdjBuf buf,
                                                 uint32_t range, double* hout, mcd_tally* tally,
                                                 uint32_t* status) {
    __shared__ SimConst<T> c;  // see k_plain: constants are read from shared memory
    __shared__ double sh_h[MCD_HIST_E_MAX + 2];
    __shared__ unsigned long long s_cnt[9];
    if (threadIdx.x == 0) c = cp;
    for (int b = threadIdx.x; b < sh.nbins + 2; b += blockDim.x) sh_h[b] = 0.0;
    if (threadIdx.x < 9) s_cnt[threadIdx.x] = 0ull;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const uint64_t n = (uint64_t)c.num_el;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint64_t pos = warp * range;
    const uint64_t end = buf.queue ? n : (pos + range < n ? pos + range : n);
    bool exhausted = false;
    const bool depth = sh.quantity == MCD_ADJ_MAX_DEPTH;
    T* ck = static_cast<T*>(buf.ckpt);
    uint32_t st = 0;
    Lane<T> L;
    uint64_t i = 0;
    bool have = false;
    int kstar = -1, mstar = 0;   // exit event; events up to the deepest point
    T zbest = (T)0;
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, !have);
        if (idle && !exhausted) {   // the idle lanes take the next electrons
            const unsigned cnt = (unsigned)__popc(idle);
            unsigned long long base = pos;
            if (buf.queue) {
                if (lane == 0) base = atomicAdd(buf.queue, (unsigned long long)cnt);
                base = __shfl_sync(0xffffffffu, base, 0);
            } else {
                pos += cnt;
            }
            const uint64_t j = base + (uint64_t)__popc(idle & lt);
            if (!have && j < end) {
                i = j;
                lane_init(L, c);
                kstar = -1;
                mstar = 0;
                zbest = (T)0;
                have = true;
            }
            if (base + cnt >= end) exhausted = true;
        }
        if (__ballot_sync(0xffffffffu, have) == 0u) {
            if (exhausted) break;
            continue;
        }
        if (!have) continue;
        if ((L.step % kSeg) == 0) {
            const int64_t m = L.step / kSeg;
            if (m < buf.max_ckpt) {
                if (!depth) {
                    ck[(size_t)m * n + i] = L.E;
                } else {
                    T* q = ck + (size_t)m * kDepthState * n + i;
                    q[0] = L.E;
                    q[n] = L.z;
                    q[2 * n] = L.dx;
                    q[3 * n] = L.dy;
                    q[4 * n] = L.dz;
                    q[5 * n] = L.yx;
                    q[6 * n] = L.yy;
                    q[7 * n] = L.yz;
                }
            }
        }
        EventOut<T> ev;
        cont_event<T, false>(L, c, c.first + i, &ev);
        if (L.outcome == MCD_OUT_BKS) kstar = (int)(L.step - 1);
        if (L.max_z > zbest) {
            zbest = L.max_z;
            mstar = (int)L.step;
        }
        if (L.outcome == MCD_OUT_NONE) continue;
        // the electron is done
        const bool bks = L.outcome == MCD_OUT_BKS;
        const int key = depth ? mstar : kstar;
        if (bks && key > 0 && (key - 1) / kSeg >= buf.max_ckpt) st |= MCD_FLAG_CKPT;
        buf.kstar[i] = bks ? key : -1;
        const T q = depth ? L.max_z : L.E_row;
        static_cast<T*>(buf.E_exit)[i] = q;
        if (bks) {
            // summed per block in FP64 (straight to the output the clustered
            // depths contend for a few addresses: 2.3 times slower)
            soft_bins<T>(sh, q, [&](int b, T w, T) { if (w > (T)0) atomicAdd(&sh_h[b], (double)w); });
            atomicAdd(&sh_h[sh.nbins], (double)q);
            atomicAdd(&sh_h[sh.nbins + 1], 1.0);
        }
        atomicAdd(&s_cnt[L.outcome & 7], 1ull);
        atomicAdd(&s_cnt[8], (unsigned long long)L.step);
        if (L.flags & F_CLAMPED) st |= MCD_FLAG_CLAMPED;
        if (L.flags & F_LONG_PATH) st |= MCD_FLAG_LONG_PATH;
        if (L.outcome == MCD_OUT_LONG) st |= MCD_FLAG_LONG;
        have = false;
    }
    const uint32_t w = __reduce_or_sync(0xffffffffu, st);
    if (lane == 0 && w) atomicOr(status, w);
    __syncthreads();
    for (int b = threadIdx.x; b < sh.nbins + 2; b += blockDim.x)
        if (sh_h[b] != 0.0) atomicAdd(&hout[b], sh_h[b]);
    if (tally && threadIdx.x < 9 && s_cnt[threadIdx.x]) {
        if (threadIdx.x < 8) atomicAdd(&tally->outcome[threadIdx.x], s_cnt[threadIdx.x]);
        else atomicAdd(&tally->events, s_cnt[8]);
    }
}

// Reverse sweep of the deepest depth Z = z_{m*} = sum_{k < m*} s_k d_z,k
// along the frozen sequence.  Per event k, with the step s(E), the energy
// update E' = E - s S(E), the Rutherford sin^2(theta/2) = s2(E) and the
// rotation of the frame (d, y, x = y cross d)
//     d' = d cos(theta) + x sin(theta) cos(phi) + y sin(theta) sin(phi)
//     y' = y cos(phi) - x sin(phi)
// the adjoints of (E, d, y) run backwards from zero at m* (Z does not
// depend on the state after m*), g = dL/dZ feeds the z term of every event:
//     lE  = lE' (1 + s dlnsig S - s dS/dE) - g d_z s dlnsig
//           + lD' . (-2 ds2/dE d + dsin(theta)/dE (x cos(phi) + y sin(phi)))
//     lD  = cos(theta) lD' + w cross y + g s e_z
//     lY  = sin(theta) sin(phi) lD' + cos(phi) lY' + d cross w,
//           w = sin(theta) cos(phi) lD' - sin(phi) lY'
//     dL/dJ += lE' (-s dS/dJ);  dL/dn += g d_z (-s / n)  (E' does not depend on n)
// (the renormalisation of d and y after each rotation is left out: it moves
// a unit vector by rounding only).  Each segment is recomputed from its
// checkpoint with the forward's own event code.
// The adjoints a depth sweep carries from one segment to the one before it,
// and the electron's parameter sums.
template <class T>
struct DepthAdj {
    T lE, ldx, ldy, ldz, lyx, lyy, lyz, sj, sn;
};

// Segment m of electron i's depth sweep (the segments run last to first).
template <class T, class C>
__device__ __forceinline__ void depth_segment(const C& c, const AdjBuf& buf, uint64_t i, uint64_t elec, int mstar,
                                              int m, T g, T ij, T ins, DepthAdj<T>& A) {
    const T* ck = static_cast<const T*>(buf.ckpt);
    const size_t n = (size_t)c.num_el;
    T lE = A.lE, ldx = A.ldx, ldy = A.ldy, ldz = A.ldz, lyx = A.lyx, lyy = A.lyy, lyz = A.lyz;
    T sj = A.sj, sn = A.sn;
    // the segment's recorded states (E, d and y before each event); the
    // event's step, polar angle and uniforms are recomputed from its Philox
    // block in the sweep (the recorded arrays pass through local memory,
    // and four more of them cost more traffic than the recomputation)
    T aE[kSeg], aD[3][kSeg], aY[3][kSeg];
    {
        const int k0 = m * kSeg;
        const int len = min(kSeg, mstar - k0);
        const T* q = ck + (size_t)m * kDepthState * n + i;
        Lane<T> L;
        lane_init(L, c);
        L.E = q[0];
        L.z = q[n];
        L.dx = q[2 * n];
        L.dy = q[3 * n];
        L.dz = q[4 * n];
        L.yx = q[5 * n];
        L.yy = q[6 * n];
        L.yz = q[7 * n];
        L.step = k0;
        for (int j = 0; j < len; ++j) {   // the forward's events, recorded
            aE[j] = L.E;
            aD[0][j] = L.dx;
            aD[1][j] = L.dy;
            aD[2][j] = L.dz;
            aY[0][j] = L.yx;
            aY[1][j] = L.yy;
            aY[2][j] = L.yz;
            EventOut<T> ev;
            cont_event<T, false>(L, c, elec, &ev);
        }
        for (int j = len - 1; j >= 0; --j) {   // reverse sweep
            const T E = aE[j];
            // the event's step and angles as cont_event_r computed them
            const uint4 r = philox(event_counter((uint32_t)(k0 + j), elec, c.sim_id), c.key0, c.key1);
            const T s = -Ops<T>::ln_step_word(r.y) * Ops<T>::div((T)1, sig_ruth<T>(c, E));
            const T a_r = Ops<T>::div(c.a0, E);
            const T s2 = Ops<T>::div(a_r * Ops<T>::unit(r.z), a_r + Ops<T>::unit_c(r.z));
            const T dx = aD[0][j], dy = aD[1][j], dz = aD[2][j];
            const T yx = aY[0][j], yy = aY[1][j], yz = aY[2][j];
            T S, SE, Sj;
            stopping_derivs<T>(c, E, &S, &SE, &Sj);
            const T dl = dlnsig<T>(c, E);
            // angles of the event
            T sp, cp;
            Ops<T>::sincos_pi(Ops<T>::unit(r.w), &sp, &cp);
            if (c.quirks & MCD_Q_HALF_PHI_FOLD) cp = fabs(cp);
            const T cph = (T)1 - (T)2 * sp * sp, sph = (T)2 * sp * cp;
            const T cth = (T)1 - (T)2 * s2;
            const T sth = (T)2 * Ops<T>::sqrt_(s2) * Ops<T>::sqrt_((T)1 - s2);
            // d s2 / dE with s2 = a U / (a + 1 - U), a = a0 / E
            const T a = a_r, U = Ops<T>::unit(r.z), Uc = (T)1 - U;
            const T den = a + Uc;
            const T ds2 = -Ops<T>::div(a, E) * Ops<T>::div(U * Uc, den * den);
            const T dsth = sth > (T)0 ? Ops<T>::div((T)2 * cth * ds2, sth) : (T)0;
            const T xx = yy * dz - yz * dy, xy = yz * dx - yx * dz, xz = yx * dy - yy * dx;
            const T sa = sth * cph, sb = sth * sph;
            // parameter gradients use the adjoint of the event's outputs
            sj += lE * (-s * Sj * ij);
            sn += g * dz * (-s * ins);
            const T rot = ldx * (-(T)2 * ds2 * dx + dsth * (cph * xx + sph * yx)) +
                          ldy * (-(T)2 * ds2 * dy + dsth * (cph * xy + sph * yy)) +
                          ldz * (-(T)2 * ds2 * dz + dsth * (cph * xz + sph * yz));
            const T nE = lE * ((T)1 + s * dl * S - s * SE) - g * dz * s * dl + rot;
            const T wx = sa * ldx - sph * lyx, wy = sa * ldy - sph * lyy, wz = sa * ldz - sph * lyz;
            const T ndx = cth * ldx + (wy * yz - wz * yy);
            const T ndy = cth * ldy + (wz * yx - wx * yz);
            const T ndz = cth * ldz + (wx * yy - wy * yx) + g * s;
            const T nyx = sb * ldx + cph * lyx + (dy * wz - dz * wy);
            const T nyy = sb * ldy + cph * lyy + (dz * wx - dx * wz);
            const T nyz = sb * ldz + cph * lyz + (dx * wy - dy * wx);
            lE = nE;
            ldx = ndx;
            ldy = ndy;
            ldz = ndz;
            lyx = nyx;
            lyy = nyy;
            lyz = nyz;
        }
    }
    A = DepthAdj<T>{lE, ldx, ldy, ldz, lyx, lyy, lyz, sj, sn};
}

// The backward pass runs only for backscattered electrons, a fraction of
// the launch: each warp owns a range of kBwdRange electrons and hands its
// backscattered ones to idle lanes in index order, so that warps stay full
// (one thread per electron left about 5 of 32 lanes active).
constexpr int kBwdRange = 256;

struct BksFeed {
    uint64_t pos, end;   // next electron of the range to scan, end of the range
    uint64_t base;       // electron of bit 0 of `found`
    unsigned found;      // backscattered electrons of [base, base + 32) not handed out yet
};

// Hands the next backscattered electrons (with a checkpointed sweep) to the
// lanes in `idle`, lowest lane first; returns this lane's electron or -1.
// Called by the whole warp with the same `idle` and `f`.
__device__ __forceinline__ int64_t bks_take(BksFeed& f, const AdjBuf& buf, unsigned idle, int lane) {
    int64_t mine = -1;
    const unsigned lt = (1u << lane) - 1u;
    while (idle) {
        if (f.found == 0u) {
            if (f.pos >= f.end) break;
            const uint64_t j = f.pos + (uint64_t)lane;
            bool b = false;
            if (j < f.end) {
                const int k = buf.kstar[j];
                b = k > 0 && (k - 1) / kSeg < buf.max_ckpt;
            }
            f.found = __ballot_sync(0xffffffffu, b);
            f.base = f.pos;
            f.pos += 32;
            continue;
        }
        const int give = min(__popc(f.found), __popc(idle));
        const int r = __popc(idle & lt);   // this lane's rank among the idle ones
        if (((idle >> lane) & 1u) && r < give) {
            unsigned m = f.found;
            for (int q = 0; q < r; ++q) m &= m - 1u;
            mine = (int64_t)(f.base + (uint64_t)(__ffs(m) - 1));
        }
        for (int q = 0; q < give; ++q) {   // the handed-out electrons and the lanes that took them
            f.found &= f.found - 1u;
            idle &= idle - 1u;
        }
    }
    return mine;
}

// d(loss)/d(exit quantity) of electron i: the soft-bin weights' derivative
// plus the sum term, in T, with gh[b] = dL/dh_b / N and gh[nbins] = dL/dsum
template <class T>
__device__ __forceinline__ T exit_adjoint(const SoftHist& sh, const AdjBuf& buf, const T* gh, uint64_t i) {
    const T q = static_cast<const T*>(buf.E_exit)[i];
    const T is2 = sizeof(T) == 8 ? (T)sh.inv_s2 : (T)sh.f_inv_s2;
    T g = gh[sh.nbins];
    soft_bins<T>(sh, q, [&](int b, T w, T d) { g += gh[b] * (-d * is2) * w; });
    return g;
}

template <class T, bool DEPTH>
__global__ void __launch_bounds__(128, 8) k_adj_bwd(const SimConst<T> cp, const SoftHist sh, const AdjBuf buf,
                                                 const double* grad_h, double inv_n, double inv_j,
                                                 double inv_ns, double* grad) {
    __shared__ SimConst<T> c;
    __shared__ double red[2];
    __shared__ T gh[MCD_HIST_E_MAX + 1];
    if (threadIdx.x == 0) {
        c = cp;
        red[0] = red[1] = 0.0;
    }
    for (int b = threadIdx.x; b <= sh.nbins; b += blockDim.x) gh[b] = (T)(b < sh.nbins ? grad_h[b] * inv_n : grad_h[b]);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t n = (uint64_t)c.num_el;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t lo = warp * (uint64_t)kBwdRange;
    BksFeed f{lo < n ? lo : n, lo + kBwdRange < n ? lo + kBwdRange : n, 0, 0u};
    const T* ck = static_cast<const T*>(buf.ckpt);
    // the lane's sums over its electrons, in T (a few electrons per lane),
    // and over the lanes and blocks in FP64
    T gj = (T)0, gn = (T)0;
    // lane state: its electron, the exit event, the segment to sweep next and
    // (exit energy) the adjoint of E and the electron's parameter sums
    int64_t cur = -1;
    int ks = 0, m = 0;
    T lam = (T)0, sj = (T)0, sn = (T)0;
    DepthAdj<T> dA{};   // depth: the adjoints carried between segments
    const T ij = (T)inv_j, ins = (T)inv_ns;
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, cur < 0);
        if (idle) {
            const int64_t e = bks_take(f, buf, idle, lane);
            if (e >= 0) {
                cur = e;
                ks = buf.kstar[e];
                m = (ks - 1) / kSeg;
                // the sweep runs in the transport precision: lambda is a
                // product of factors 1 + O(1e-2) and each step adds one term
                lam = exit_adjoint<T>(sh, buf, gh, (uint64_t)e);
                sj = sn = (T)0;
                if constexpr (DEPTH) dA = DepthAdj<T>{};
            }
        }
        if (__ballot_sync(0xffffffffu, cur >= 0) == 0u) break;
        if (cur < 0) continue;
        const uint64_t i = (uint64_t)cur;
        const uint64_t elec = c.first + i;
        if constexpr (DEPTH) {   // one segment per trip; lam holds g = dL/dZ
            depth_segment<T>(c, buf, i, elec, ks, m, lam, ij, ins, dA);
            if (--m < 0) {
                gj += dA.sj;
                gn += dA.sn;
                cur = -1;
            }
            continue;
        }
        // exit energy: one 64-event segment per trip, the last one first
        const int k0 = m * kSeg;
        const int len = min(kSeg, ks - k0);
        T Eseg[kSeg], sseg[kSeg];
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
        if (--m < 0) {
            gj += sj;
            gn += sn;
            cur = -1;
        }
    }
    double dj = (double)gj, dn = (double)gn;
    for (int o = 16; o > 0; o >>= 1) {
        dj += __shfl_down_sync(0xffffffffu, dj, o);
        dn += __shfl_down_sync(0xffffffffu, dn, o);
    }
    if (lane == 0) {
        atomicAdd(&red[0], dj);
        atomicAdd(&red[1], dn);
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
            T Ed;
            if (sh.quantity == MCD_ADJ_MAX_DEPTH) {
                // the forward's own events up to the deepest point
                Lane<T> L;
                lane_init(L, c);
                for (int k = 0; k < kstar; ++k) {
                    EventOut<T> ev;
                    cont_event<T, false>(L, c, elec, &ev);
                }
                Ed = L.z;
            } else {
                T E = c.E0;
                for (int k = 0; k < kstar; ++k) {
                    const T s = step_len<T>(c, E, elec, k);
                    E = E - Ops<T>::mul_rn(s, stopping<T>(c, E));
                }
                Ed = E;
            }
            soft_bins<T>(sh, Ed, [&](int b, T w, T) { if (w > (T)0) atomicAdd(&sh_h[b], (double)w); });
            atomicAdd(&sh_h[sh.nbins], (double)Ed);
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
    if (hist->quantity != MCD_ADJ_EXIT_E && hist->quantity != MCD_ADJ_MAX_DEPTH) return MCD_EINVAL;
    if (!(sim->J_scale >= 0) || !(sim->n_scale >= 0)) return MCD_EINVAL;
    sh->nbins = hist->nbins;
    sh->quantity = hist->quantity;
    sh->lo = hist->lo;
    sh->width = (hist->hi - hist->lo) / hist->nbins;
    sh->inv2s2 = 1.0 / (2.0 * hist->sigma * hist->sigma);
    sh->inv_s2 = 1.0 / (hist->sigma * hist->sigma);
    sh->inv_width = 1.0 / sh->width;
    sh->reach = 8.0 * hist->sigma;
    sh->f_lo = (float)sh->lo;
    sh->f_width = (float)sh->width;
    sh->f_inv_width = (float)sh->inv_width;
    sh->f_inv2s2 = (float)sh->inv2s2;
    sh->f_inv_s2 = (float)sh->inv_s2;
    sh->f_reach = (float)sh->reach;
    ab->ckpt = buf->ckpt;
    ab->kstar = buf->kstar;
    ab->E_exit = buf->E_exit;
    ab->max_ckpt = buf->max_ckpt;
    ab->queue = buf->queue;
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
    if (sim->num_el == 0) return MCD_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint32_t range = 32;
    unsigned long long grid = ((unsigned long long)sim->num_el + 255) / 256;   // one thread per electron
    if (ab.queue) {
        // a resident grid: as many blocks as fit on the GPU at once, and no
        // more than there are electrons for
        int dev = 0, sms = 0, blocks = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return MCD_ECUDA;
        const cudaError_t oc = sim->precision == MCD_FP64
                                   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_adj_fwd<double>, 256, 0)
                                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_adj_fwd<float>, 256, 0);
        if (oc != cudaSuccess) return MCD_ECUDA;
        const unsigned long long resident = (unsigned long long)(sms > 0 ? sms : 1) * (blocks > 0 ? blocks : 1);
        grid = grid < resident ? grid : resident;
        if (cudaMemsetAsync(ab.queue, 0, sizeof(unsigned long long), st) != cudaSuccess) return MCD_ECUDA;
    }
    if (grid > 0x7fffffffull) return MCD_ETOOBIG;
    if (sim->precision == MCD_FP64)
        k_adj_fwd<double><<<(unsigned)grid, 256, 0, st>>>(make_consts<double>(*sim, *mat, nullptr, nullptr), sh, ab,
                                                           range, hist_out, tally, status);
    else
        k_adj_fwd<float><<<(unsigned)grid, 256, 0, st>>>(make_consts<float>(*sim, *mat, nullptr, nullptr), sh, ab,
                                                          range, hist_out, tally, status);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}

extern "C" int mcd_adjoint(const mcd_sim* sim, const mcd_material* mat, const mcd_softhist* hist,
                           const mcd_adjoint_buf* buf, const double* grad_hist, double* grad, void* stream) {
    SoftHist sh;
    AdjBuf ab;
    int rc = adj_args(sim, mat, hist, buf, &sh, &ab);
    if (rc != MCD_OK) return rc;
    if (!grad_hist || !grad) return MCD_EINVAL;
    // one warp per kBwdRange electrons, four warps per block
    const unsigned long long grid = ((unsigned long long)sim->num_el + 4 * kBwdRange - 1) / (4 * kBwdRange);
    if (grid == 0) return MCD_OK;
    if (grid > 0x7fffffffull) return MCD_ETOOBIG;
    const double inv_n = 1.0 / (double)sim->num_el;
    const double js = 1.0 / (sim->J_scale > 0 ? sim->J_scale : 1.0);
    const double ns = 1.0 / (sim->n_scale > 0 ? sim->n_scale : 1.0);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool depth = sh.quantity == MCD_ADJ_MAX_DEPTH;
    if (sim->precision == MCD_FP64) {
        const SimConst<double> c = make_consts<double>(*sim, *mat, nullptr, nullptr);
        if (depth)
            k_adj_bwd<double, true><<<(unsigned)grid, 128, 0, st>>>(c, sh, ab, grad_hist, inv_n, js, ns, grad);
        else
            k_adj_bwd<double, false><<<(unsigned)grid, 128, 0, st>>>(c, sh, ab, grad_hist, inv_n, js, ns, grad);
    } else {
        const SimConst<float> c = make_consts<float>(*sim, *mat, nullptr, nullptr);
        if (depth)
            k_adj_bwd<float, true><<<(unsigned)grid, 128, 0, st>>>(c, sh, ab, grad_hist, inv_n, js, ns, grad);
        else
            k_adj_bwd<float, false><<<(unsigned)grid, 128, 0, st>>>(c, sh, ab, grad_hist, inv_n, js, ns, grad);
    }
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
