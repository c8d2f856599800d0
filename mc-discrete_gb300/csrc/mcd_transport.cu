// mcd_transport.cu - trajectory kernels and their C-ABI entry points.
//
//  k_plain    one thread per electron, one launch per simulation
//             (replaces multiTraj_DS/_cont, MC/tools/multiScatter.py:66-229)
//  k_batched  persistent grid over many simulations; a global queue hands
//             out electrons and a warp takes new ones as soon as `refill` of
//             its lanes are idle, so uneven trajectory lengths do not idle
//             the warp (replaces MapScatterer's pool, MC/doScatter.py:22-95)
//
// Tallies are gathered per block in shared memory and flushed once per block
// with global atomics; exit-energy/angle histograms go straight to global
// memory (one atomic per backscattered electron).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "mcd_device.cuh"

namespace mcd {

// Per-block sums; the per-event counters (events, channels) are 64-bit, as
// one persistent block can see more than 2^32 events of a channel.
struct BlockTally {
    unsigned int outcome[8];
    unsigned int double_rows, nan_events, clamped, long_path, table_range, pad_;
    unsigned long long events;
    double sum_E, sum_E2, sum_steps2;
    unsigned long long channel[MCD_MAX_CHANNELS];
};

__device__ __forceinline__ void bt_zero(BlockTally* t, int n) {
    unsigned int* p = reinterpret_cast<unsigned int*>(t);
    const int words = n * (int)(sizeof(BlockTally) / 4);
    for (int i = threadIdx.x; i < words; i += blockDim.x) p[i] = 0u;
}

__device__ __forceinline__ void add_u64(unsigned long long* p, unsigned long long v) {
    if (v) atomicAdd(p, v);
}

__device__ __forceinline__ void bt_flush(const BlockTally& t, mcd_tally* g) {
    // called by one thread per simulation
    bool any = t.events != 0;
    for (int k = 0; k < 8; ++k) any |= t.outcome[k] != 0;
    if (!any) return;
    for (int k = 0; k < 8; ++k) add_u64(&g->outcome[k], t.outcome[k]);
    add_u64(&g->events, t.events);
    add_u64(&g->double_rows, t.double_rows);
    add_u64(&g->nan_events, t.nan_events);
    add_u64(&g->clamped, t.clamped);
    add_u64(&g->long_path, t.long_path);
    add_u64(&g->table_range, t.table_range);
    for (int k = 0; k < MCD_MAX_CHANNELS; ++k) add_u64(&g->channel[k], t.channel[k]);
    if (t.sum_E != 0.0) atomicAdd(&g->sum_E_bks, t.sum_E);
    if (t.sum_E2 != 0.0) atomicAdd(&g->sum_E2_bks, t.sum_E2);
    if (t.sum_steps2 != 0.0) atomicAdd(&g->sum_steps2, t.sum_steps2);
}

struct ElOut {
    uint8_t* outcome;
    uint8_t* flags;
    void* final_E;
    void* dir;
    void* last_pos;
    void* max_z;
    int32_t* n_events;
};

template <class T, class C>
__device__ __forceinline__ uint32_t finish_electron(const C& c, const Lane<T>& L, uint64_t i, BlockTally& bt,
                                                    mcd_tally* gt, const ElOut& eo) {
    atomicAdd(&bt.outcome[L.outcome & 7], 1u);
    atomicAdd(&bt.events, (unsigned long long)L.step);
    atomicAdd(&bt.sum_steps2, (double)L.step * (double)L.step);
    if (L.flags & F_DOUBLE_ROW) atomicAdd(&bt.double_rows, 1u);
    if (L.nan_n) atomicAdd(&bt.nan_events, L.nan_n);
    if (L.clamp_n) atomicAdd(&bt.clamped, L.clamp_n);
    if (L.lpath_n) atomicAdd(&bt.long_path, L.lpath_n);
    if (L.flags & F_TABLE_RANGE) atomicAdd(&bt.table_range, 1u);
    if (L.outcome == MCD_OUT_BKS) {
        const double e = (double)L.E_row;
        atomicAdd(&bt.sum_E, e);
        atomicAdd(&bt.sum_E2, e * e);
        if (c.hE > 0) {
            const T f = L.E_row * c.invWE;
            if (f >= (T)0 && f < (T)c.hE) atomicAdd(&gt->hist_E[(int)f], 1ull);
        }
        if (c.hT > 0) {
            const T th = Ops<T>::acos_deg(-L.dz) * c.invWT;
            if (th >= (T)0 && th < (T)c.hT) atomicAdd(&gt->hist_T[(int)th], 1ull);
        }
    }
    if (eo.outcome) eo.outcome[i] = (uint8_t)L.outcome;
    if (eo.flags) eo.flags[i] = (uint8_t)(L.flags & (F_DOUBLE_ROW | F_NAN));
    const size_t n = (size_t)c.num_el;
    if (eo.final_E) static_cast<T*>(eo.final_E)[i] = L.E_row;
    if (eo.dir) {
        T* d = static_cast<T*>(eo.dir);
        d[i] = L.dx;
        d[n + i] = L.dy;
        d[2 * n + i] = L.dz;
    }
    if (eo.last_pos) {
        T* p = static_cast<T*>(eo.last_pos);
        p[i] = L.x;
        p[n + i] = L.y;
        p[2 * n + i] = L.z;
    }
    if (eo.max_z) static_cast<T*>(eo.max_z)[i] = L.max_z;
    if (eo.n_events) eo.n_events[i] = (int32_t)L.step;
    uint32_t st = 0;
    if (L.flags & F_NAN) st |= MCD_FLAG_NAN;
    if (L.flags & F_TABLE_RANGE) st |= MCD_FLAG_TABLE_RANGE;
    if (L.flags & F_CLAMPED) st |= MCD_FLAG_CLAMPED;
    if (L.flags & F_LONG_PATH) st |= MCD_FLAG_LONG_PATH;
    if (L.outcome == MCD_OUT_LONG) st |= MCD_FLAG_LONG;
    return st;
}

// Called by every thread of the block; a block smaller than a warp (plain
// launches of 1 to 16 threads) leaves lanes that never exist, so the
// reduction names the lanes present.
__device__ __forceinline__ void or_status(uint32_t* status, uint32_t st) {
    const uint32_t w = __reduce_or_sync(__activemask(), st);
    if ((threadIdx.x & 31) == 0 && w) atomicOr(status, w);
}

// ---------------------------------------------------------------------------
// plain kernel: one thread per electron
// ---------------------------------------------------------------------------
// The constant block arrives as a by-value kernel parameter and is copied to
// shared memory before use.  Reading it through a reference to the parameter
// itself made nvcc 13.0 (sm_103a, -O3) drop the loop-carried energy update of
// the lane state initialised from it; the shared-memory copy is also what the
// batched kernel reads.
template <class T, int MODE, bool REC>
__global__ void __launch_bounds__(256) k_plain(const SimConst<T> cp, mcd_tally* tally, const ElOut eo,
                                               const mcd_event_ring ring, uint32_t* status) {
    __shared__ BlockTally bt;
    __shared__ SimConst<T> c;
    if (threadIdx.x == 0) c = cp;
    bt_zero(&bt, 1);
    __syncthreads();
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t st = 0;
    if (i < (uint64_t)c.num_el) {
        Lane<T> L;
        lane_init(L, c);
        const uint64_t elec = c.first + i;
        const bool chan = (c.tally_flags & MCD_TALLY_CHANNELS) != 0;
        while (L.outcome == MCD_OUT_NONE) {
            EventOut<T> ev;
            const int ch = (MODE == MCD_MODE_DS) ? ds_event<T, REC>(L, c, elec, &ev, c.sig != nullptr)
                                                 : cont_event<T, REC>(L, c, elec, &ev);
            if (ch >= 0) {
                if (REC) st |= ring_append(ring, (uint32_t)i, L.step, ev);
                if (chan) atomicAdd(&bt.channel[ch], 1ull);
            }
        }
        st |= finish_electron(c, L, i, bt, tally, eo);
    }
    or_status(status, st);
    __syncthreads();
    if (threadIdx.x == 0) bt_flush(bt, tally);
}

// ---------------------------------------------------------------------------
// batched persistent kernel
// ---------------------------------------------------------------------------
struct BatchHeader {
    unsigned long long queue;   // next electron to hand out
    unsigned long long total;   // electrons over all simulations
    int32_t nsims;
    int32_t pad_[11];
};

constexpr int kBatchMaxSims = 256;

// Workspace layout: header | prefix[nsims+1] (u64, by queue position) |
// perm[nsims] (i32: queue position -> simulation) | pad | SimConst[nsims].
__host__ __device__ constexpr size_t batch_prefix_off() { return sizeof(BatchHeader); }
__host__ __device__ constexpr size_t batch_perm_off(int nsims) {
    return sizeof(BatchHeader) + sizeof(unsigned long long) * (size_t)(nsims + 1);
}
__host__ __device__ constexpr size_t batch_consts_off(int nsims) {
    return (batch_perm_off(nsims) + sizeof(int32_t) * (size_t)nsims + 255) & ~(size_t)255;
}
// ... | per-electron row pointers[nsims] | FP64 constants (table build only)
// | cross-section tables.  The no-alloc path copies only the core (through
// the row pointers) and has no table slots.
__host__ __device__ constexpr size_t batch_elout_off(int nsims) {
    return batch_consts_off(nsims) + sizeof(SimConst<float>) * (size_t)nsims;
}
__host__ __device__ constexpr size_t batch_core_bytes(int nsims) {
    return batch_elout_off(nsims) + sizeof(mcd_electron_out) * (size_t)nsims;
}
static_assert(sizeof(SimConst<float>) % 8 == 0, "row pointers follow the constant blocks");

// The row pointers of each simulation (zero: none), as the kernel reads them.
inline void pack_rows(const mcd_sim* sims, int nsims, uint8_t* host) {
    mcd_electron_out* eo = reinterpret_cast<mcd_electron_out*>(host + batch_elout_off(nsims));
    for (int k = 0; k < nsims; ++k) {
        if (sims[k].electrons) eo[k] = *sims[k].electrons;
        else memset(&eo[k], 0, sizeof(mcd_electron_out));
    }
}
__host__ __device__ constexpr size_t batch_dconsts_off(int nsims) {
    return (batch_core_bytes(nsims) + 255) & ~(size_t)255;
}
__host__ __device__ constexpr size_t batch_sig_off(int nsims) {
    return (batch_dconsts_off(nsims) + sizeof(SimConst<double>) * (size_t)nsims + 255) & ~(size_t)255;
}
__host__ __device__ constexpr size_t batch_sig_bytes() {   // one table slot per simulation
    return sizeof(float) * (size_t)kSigRowsMax * kSigStride;
}
__host__ __device__ constexpr size_t batch_bytes(int nsims) {
    return batch_sig_off(nsims) + batch_sig_bytes() * (size_t)nsims;
}

__host__ __device__ constexpr size_t batch_smem(int nsims) {
    return sizeof(SimConst<float>) * nsims + sizeof(unsigned long long) * (nsims + 1) +
           sizeof(int32_t) * ((nsims + 1) & ~1) + sizeof(BlockTally) * nsims;
}

// Queue order: simulations with the longest expected trajectories first, so
// that the last electrons handed out are short ones and the grid drains
// evenly.  The key is the energy to lose, less for tilted beams (which
// backscatter more).  Results do not depend on the order: every electron
// keeps its own (sim, electron, event) Philox counters.
static void batch_order(const mcd_sim* sims, int nsims, int32_t* perm) {
    for (int k = 0; k < nsims; ++k) perm[k] = k;
    auto key = [&](int k) {
        const double t = sims[k].s_tilt * kPi / 180.0;
        return (sims[k].E0 - sims[k].Emin) * cos(0.5 * t);
    };
    for (int a = 1; a < nsims; ++a) {      // stable insertion sort, descending key
        const int v = perm[a];
        const double kv = key(v);
        int b = a - 1;
        while (b >= 0 && key(perm[b]) < kv) {
            perm[b + 1] = perm[b];
            --b;
        }
        perm[b + 1] = v;
    }
}

template <bool REC>
__device__ __forceinline__ void batched_body(uint8_t* ws, mcd_tally* tallies, int refill, uint32_t* status,
                                             const mcd_event_ring& ring, int inline_sigma);

// Two register budgets of the same kernel: up to 1024 threads per block at
// 64 registers (32 warps per SM: one block of 1024), or two blocks of up to
// 576 per SM at 56 registers (36 warps, 8 bytes spilled, two copies of the
// constant blocks in shared memory): on the 64-simulation workload the
// second, in blocks of 576, is 1.2% faster (78.2 against 79.1 ms); five
// blocks of 256 at 48 registers were 26% slower.
// REC: append every event to the ring.
template <bool REC = false>
__global__ void __launch_bounds__(1024) k_batched(uint8_t* ws, mcd_tally* tallies, int refill,
                                                  uint32_t* status, const mcd_event_ring ring = mcd_event_ring{},
                                                  int inline_sigma = 0) {
    batched_body<REC>(ws, tallies, refill, status, ring, inline_sigma);
}

template <bool REC = false>
__global__ void __launch_bounds__(576, 2) k_batched_lr(uint8_t* ws, mcd_tally* tallies, int refill,
                                                       uint32_t* status, const mcd_event_ring ring = mcd_event_ring{},
                                                       int inline_sigma = 0) {
    batched_body<REC>(ws, tallies, refill, status, ring, inline_sigma);
}

template <bool REC>
__device__ __forceinline__ void batched_body(uint8_t* ws, mcd_tally* tallies, int refill, uint32_t* status,
                                             const mcd_event_ring& ring, int inline_sigma) {
    extern __shared__ __align__(16) uint8_t smem[];
    BatchHeader* hdr = reinterpret_cast<BatchHeader*>(ws);
    const int nsims = hdr->nsims;
    const unsigned long long total = hdr->total;
    SimConst<float>* s_c = reinterpret_cast<SimConst<float>*>(smem);
    unsigned long long* s_pre = reinterpret_cast<unsigned long long*>(smem + sizeof(SimConst<float>) * nsims);
    int32_t* s_perm = reinterpret_cast<int32_t*>(smem + sizeof(SimConst<float>) * nsims +
                                                 sizeof(unsigned long long) * (nsims + 1));
    BlockTally* s_t = reinterpret_cast<BlockTally*>(smem + sizeof(SimConst<float>) * nsims +
                                                    sizeof(unsigned long long) * (nsims + 1) +
                                                    sizeof(int32_t) * ((nsims + 1) & ~1));
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(ws + batch_consts_off(nsims));
        uint32_t* dst = reinterpret_cast<uint32_t*>(s_c);
        const int words = (int)(sizeof(SimConst<float>) / 4) * nsims;
        for (int k = threadIdx.x; k < words; k += blockDim.x) dst[k] = src[k];
        const unsigned long long* pre = reinterpret_cast<const unsigned long long*>(ws + batch_prefix_off());
        for (int k = threadIdx.x; k <= nsims; k += blockDim.x) s_pre[k] = pre[k];
        const int32_t* perm = reinterpret_cast<const int32_t*>(ws + batch_perm_off(nsims));
        for (int k = threadIdx.x; k < nsims; k += blockDim.x) s_perm[k] = perm[k];
        bt_zero(s_t, nsims);
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    Lane<float> L;
    int sim = 0;
    uint64_t elec = 0;
    bool have = false;
    bool exhausted = false;
    uint32_t st = 0;
    const mcd_electron_out* rows = reinterpret_cast<const mcd_electron_out*>(ws + batch_elout_off(nsims));
    while (true) {
        // the lanes without an electron; voted again only after a refill,
        // so a step with every lane busy costs one vote
        unsigned idle = __ballot_sync(0xffffffffu, !have);
        if (!exhausted && idle && (__popc(idle) >= refill || idle == 0xffffffffu)) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&hdr->queue, (unsigned long long)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (!have) {
                const unsigned long long g = base + __popc(idle & lt);
                if (g < total) {
                    int lo = 0, hi = nsims;  // s_pre[lo] <= g < s_pre[hi] (queue positions)
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (s_pre[mid] <= g) lo = mid; else hi = mid;
                    }
                    sim = s_perm[lo];
                    elec = s_c[sim].first + (g - s_pre[lo]);   // the Philox electron index
                    lane_init(L, s_c[sim]);
                    have = true;
                }
            }
            if (base + __popc(idle) >= total) exhausted = true;
            idle = __ballot_sync(0xffffffffu, !have);
        }
        if (idle == 0xffffffffu) {
            if (exhausted) break;
            continue;
        }
        if (have) {
            const SimConst<float>& c = s_c[sim];
            EventOut<float> ev;
            int ch;
            if (!(c.bits & kBitCont))
                ch = ds_event<float, REC>(L, c, elec, &ev, !inline_sigma && c.sig != nullptr);
            else
                ch = cont_event<float, REC>(L, c, elec, &ev);
            if (REC && ch >= 0) st |= ring_append(ring, (uint32_t)(elec - c.first), L.step, ev);
            if (ch >= 0 && (c.bits & kBitChan)) atomicAdd(&s_t[sim].channel[ch], 1ull);
            if (L.outcome != MCD_OUT_NONE) {
                const mcd_electron_out& r = rows[sim];
                const ElOut eo{r.outcome, r.flags, r.final_E, r.dir, r.last_pos, r.max_z, r.n_events};
                st |= finish_electron(c, L, elec - c.first, s_t[sim], tallies + sim, eo);
                have = false;
            }
        }
    }
    or_status(status, st);
    __syncthreads();
    for (int k = threadIdx.x; k < nsims; k += blockDim.x) bt_flush(s_t[k], tallies + k);
}

// Cross-section tables of a prepared batch: one thread per (table slot, grid
// point); a slot is built when its simulation leads a group sharing it.  The
// exact FP64 expressions of the inline path, stored as FP32 E * running sums
// in pick order.
// Row i of a table on the grid (l0, inv): [E total, E running sums Ruth,
// +Moller, +Gryz[k] ... (the sum through Quinn is the total)], padding
// FLT_MAX: never below a target.
__device__ __forceinline__ void sig_row(const SimConst<double>& c, float l0, float inv, int S, int i,
                                        float* row) {
    const double E = exp2((double)l0 + (double)i / (double)inv);
    const double invE = 1.0 / E;
    double cum = sig_ruth<double>(c, E);
    int col = 1;
    row[col++] = (float)(E * cum);
    cum += sig_moller<double>(c, E, invE);
    row[col++] = (float)(E * cum);
    for (int k = 0; k < c.nsh; ++k) {
        cum += sig_gryz<double>(c, E, invE, k);
        row[col++] = (float)(E * cum);
    }
    cum += sig_quinn<double>(c, E, invE);
    row[0] = (float)(E * cum);
    for (; col < S; ++col) row[col] = 3.402823466e38f;
}

__global__ void __launch_bounds__(256) k_sigtab(uint8_t* ws, int nsims) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)nsims * kSigRowsMax) return;
    const int s = (int)(gid / kSigRowsMax), i = (int)(gid % kSigRowsMax);
    const SimConst<float>& cf = reinterpret_cast<const SimConst<float>*>(ws + batch_consts_off(nsims))[s];
    const float* slot = reinterpret_cast<const float*>(ws + batch_sig_off(nsims) + batch_sig_bytes() * s);
    if (cf.sig != slot || i >= cf.sig_rows) return;
    const SimConst<double>& c = reinterpret_cast<const SimConst<double>*>(ws + batch_dconsts_off(nsims))[s];
    float* row = reinterpret_cast<float*>(ws + batch_sig_off(nsims) + batch_sig_bytes() * s) + (size_t)i * cf.sig_S;
    sig_row(c, cf.sig_l0, cf.sig_inv, cf.sig_S, i, row);
}

// The table of one simulation (mcd_build_sigma_table): one thread per row.
__global__ void __launch_bounds__(256) k_sigtab_one(const SimConst<double> c, float l0, float inv, int rows,
                                                     int S, float* table) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    sig_row(c, l0, inv, S, i, table + (size_t)i * S);
}

// The FP64 table of one simulation (mcd_build_sigma_table for FP64
// transport; layout at kSig64Cells): one thread per (octave, cell).  It
// evaluates the mean free path and the running-sum fractions at the cell's
// four nodes E_n = 2^e (1 + (i - 1 + n) / cells), n = 0..3, and stores the
// coefficients of the cubic through them in the offset f = (E - E_1) / h:
// with v_n the node values, c0 = v_1, c1 = -v_0/3 - v_1/2 + v_2 - v_3/6,
// c2 = v_0/2 - v_1 + v_2/2, c3 = (v_3 - v_0)/6 + (v_1 - v_2)/2 (the
// Lagrange cubic written in powers of f).
__global__ void __launch_bounds__(128) k_sigtab64(const SimConst<double> c, int e_lo, int blocks,
                                                   double* table) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= blocks * kSig64Cells) return;
    const int blk = gid / kSig64Cells, i = gid % kSig64Cells;
    const int K = c.nsh + 3;
    const double base = ldexp(1.0, e_lo + blk), h = base / kSig64Cells;
    double v[4][3 + MCD_MAX_SHELLS];
    for (int n = 0; n < 4; ++n) {
        const double E = base + (double)(i - 1 + n) * h;
        const double invE = 1.0 / E;
        double run[3 + MCD_MAX_SHELLS];
        double cum = sig_ruth<double>(c, E);
        run[1] = cum;
        cum += sig_moller<double>(c, E, invE);
        run[2] = cum;
        for (int k = 0; k < c.nsh; ++k) {
            cum += sig_gryz<double>(c, E, invE, k);
            run[3 + k] = cum;
        }
        cum += sig_quinn<double>(c, E, invE);
        const double inv = 1.0 / cum;
        v[n][0] = inv;
        for (int k = 1; k < K; ++k) v[n][k] = run[k] * inv;
    }
    double* rec = table + (size_t)gid * sig64_stride(K);
    const double E1 = base + (double)(i - 1) * h, E4 = E1 + 3.0 * h;
    auto in = [&](double x) { return x >= E1 && x <= E4; };
    // below 2 Wc the Moller cross section is negative and falls to -inf at
    // Wc (MC/tools/crossSections.py:183-208), which no cubic follows
    bool kink = in(c.Wc) || in(c.Epl) || E1 < 2.0 * c.Wc;
    for (int k = 0; k < c.nsh; ++k) kink |= in(c.gEs[k]);
    rec[0] = kink ? 1.0 : 0.0;
    rec[1] = 0.0;
    for (int k = 0; k < K; ++k) {
        const double a = v[0][k], b = v[1][k], d = v[2][k], e = v[3][k];
        double* q = rec + 2 + 4 * k;
        q[0] = b;
        q[1] = -a / 3.0 - b / 2.0 + d - e / 6.0;
        q[2] = a / 2.0 - b + d / 2.0;
        q[3] = (e - a) / 6.0 + (b - d) / 2.0;
    }
}

// Do two simulations have the same channel cross sections at every energy?
// (material, Wc and density enter; beam, range and Bethe settings do not)
inline bool same_sigma(const SimConst<double>& a, const SimConst<double>& b) {
    if (a.nsh != b.nsh) return false;
    if (a.cRs != b.cRs || a.aS != b.aS || a.ruth_r2 != b.ruth_r2 || a.pM != b.pM || a.Wc != b.Wc) return false;
    if (a.qK != b.qK || a.qC1 != b.qC1 || a.qInvEf != b.qInvEf || a.qB != b.qB || a.Epl != b.Epl) return false;
    for (int k = 0; k < a.nsh; ++k)
        if (a.gEs[k] != b.gEs[k] || a.gP[k] != b.gP[k] || a.gInvEs[k] != b.gInvEs[k]) return false;
    return true;
}

// Group the DS simulations of a batch by same_sigma; each group shares the
// table in its first member's slot, on a log2 grid over the union of the
// members' [Emin, E0] ranges.
inline void share_sigma_tables(const mcd_sim* sims, int nsims, const SimConst<double>* cd, SimConst<float>* cs,
                               const uint8_t* ws_dev) {
    for (int k = 0; k < nsims; ++k) {
        if (sims[k].mode != MCD_MODE_DS) continue;
        int lead = k;
        for (int j = 0; j < k; ++j)
            if (sims[j].mode == MCD_MODE_DS && cs[j].sig == reinterpret_cast<const float*>(
                                                                ws_dev + batch_sig_off(nsims) + batch_sig_bytes() * j) &&
                same_sigma(cd[j], cd[k])) {
                lead = j;
                break;
            }
        cs[k].sig = reinterpret_cast<const float*>(ws_dev + batch_sig_off(nsims) + batch_sig_bytes() * lead);
    }
    for (int k = 0; k < nsims; ++k) {
        if (sims[k].mode != MCD_MODE_DS) continue;
        const float* slot = reinterpret_cast<const float*>(ws_dev + batch_sig_off(nsims) + batch_sig_bytes() * k);
        if (cs[k].sig != slot) continue;
        double lo = sims[k].Emin, hi = sims[k].E0;
        for (int j = k + 1; j < nsims; ++j)
            if (cs[j].sig == slot) {
                lo = fmin(lo, sims[j].Emin);
                hi = fmax(hi, sims[j].E0);
            }
        float l0, inv, tmax;
        int32_t rows;
        sigma_grid(lo, hi, &l0, &inv, &tmax, &rows);
        for (int j = k; j < nsims; ++j)
            if (cs[j].sig == slot) {
                cs[j].sig_l0 = l0;
                cs[j].sig_inv = inv;
                cs[j].sig_tmax = tmax;
                cs[j].sig_rows = rows;
                cs[j].sig_off = -l0 * inv;
            }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// FP64 DS transport of a small run, one warp per two electrons.  Such a run
// lasts as long as its longest trajectory, one dependent chain of
// instructions.  The 16 lanes of each half-warp run their electron's events
// in lockstep (every lane holds the same state) and compute, 16 events
// ahead and one event per lane, what does not depend on the trajectory: the
// event's Philox block, ln U of its step uniform, the azimuth's cos and
// sin, and the uniforms of the channel pick and the polar angle (the values
// the event itself would compute); an event takes them from its lane by
// shuffles, so the chain no longer carries them.  The trajectories are
// k_plain's, bit for bit.
__global__ void __launch_bounds__(32) k_plain_lanes64(const SimConst<double> cp, mcd_tally* tally, const ElOut eo,
                                                      uint32_t* status) {
    __shared__ BlockTally bt;
    __shared__ SimConst<double> c;
    if (threadIdx.x == 0) c = cp;
    bt_zero(&bt, 1);
    __syncthreads();
    const int lane = threadIdx.x & 31, t = lane & 15, h = lane >> 4;
    const uint64_t i = (uint64_t)blockIdx.x * 2 + (uint64_t)h;
    bool active = i < (uint64_t)c.num_el;
    const uint64_t elec = c.first + i;
    const uint4 w = event_words(c);   // sim id, Philox key, event limit
    const bool chan = (c.tally_flags & MCD_TALLY_CHANNELS) != 0;
    Lane<double> L;
    lane_init(L, c);
    uint32_t base = 0, pz = 0;
    EventPre<double> mine{};
    auto ahead = [&]() {   // lane t: the event at step base + t
        const uint4 r = philox(event_counter(base + (uint32_t)t, elec, w.x), w.y, w.z);
        pz = r.z;
        mine.ln_y = ln_word(r.y);
        azimuth<double>(c, r.w, &mine.cph, &mine.sph);
        mine.ux = Ops<double>::unit(r.x);
        mine.a0u = c.a0 * Ops<double>::unit(r.z);
        mine.uzc = Ops<double>::unit_c(r.z);
    };
    ahead();
    uint32_t st = 0;
    while (__any_sync(0xffffffffu, active)) {
        if (active && L.step - base == 16u) {
            base += 16u;
            ahead();
        }
        const int src = (h << 4) | (int)((L.step - base) & 15u);
        const uint32_t rz = __shfl_sync(0xffffffffu, pz, src);   // the W tables' uniform (inelastic events)
        EventPre<double> pre;
        pre.ln_y = __shfl_sync(0xffffffffu, mine.ln_y, src);
        pre.cph = __shfl_sync(0xffffffffu, mine.cph, src);
        pre.sph = __shfl_sync(0xffffffffu, mine.sph, src);
        pre.ux = __shfl_sync(0xffffffffu, mine.ux, src);
        pre.a0u = __shfl_sync(0xffffffffu, mine.a0u, src);
        pre.uzc = __shfl_sync(0xffffffffu, mine.uzc, src);
        if (!active) continue;
        if (L.step >= w.w) {   // the 'long' check that opens every event (MC/tools/singleScatter.py:19-23)
            L.outcome = MCD_OUT_LONG;
            L.E_row = L.E;
        } else {
            L.step += 1;
            EventOut<double> ev;
            const int ch = ds_event_r<double, false>(L, c, make_uint4(0u, 0u, rz, 0u), &ev, c.sig != nullptr, &pre);
            if (chan && t == 0 && ch >= 0) atomicAdd(&bt.channel[ch], 1ull);
        }
        if (L.outcome != MCD_OUT_NONE) {
            if (t == 0) st |= finish_electron(c, L, i, bt, tally, eo);
            active = false;
        }
    }
    or_status(status, st);
    __syncthreads();
    if (threadIdx.x == 0) bt_flush(bt, tally);
}

static int launch_lanes64(const SimConst<double>& c, mcd_tally* tally, const ElOut& eo, uint32_t* status,
                          cudaStream_t st) {
    const unsigned long long grid = ((unsigned long long)c.num_el + 1) / 2;
    if (grid == 0) return MCD_OK;
    if (grid > 0x7fffffffull) return MCD_ETOOBIG;
    k_plain_lanes64<<<(unsigned)grid, 32, 0, st>>>(c, tally, eo, status);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}

template <class T, int MODE, bool REC>
static int launch_plain(const SimConst<T>& c, int block, mcd_tally* tally, const ElOut& eo,
                        const mcd_event_ring& ring, uint32_t* status, cudaStream_t st) {
    const unsigned long long grid = ((unsigned long long)c.num_el + block - 1) / block;
    if (grid == 0) return MCD_OK;
    if (grid > 0x7fffffffull) return MCD_ETOOBIG;
    k_plain<T, MODE, REC><<<(unsigned)grid, block, 0, st>>>(c, tally, eo, ring, status);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}

template <class T>
static int dispatch_plain(const SimConst<T>& c, int block, mcd_tally* tally, const ElOut& eo,
                          const mcd_event_ring& ring, bool rec, uint32_t* status, cudaStream_t st) {
    if (c.mode == MCD_MODE_DS)
        return rec ? launch_plain<T, MCD_MODE_DS, true>(c, block, tally, eo, ring, status, st)
                   : launch_plain<T, MCD_MODE_DS, false>(c, block, tally, eo, ring, status, st);
    return rec ? launch_plain<T, MCD_MODE_CONT, true>(c, block, tally, eo, ring, status, st)
               : launch_plain<T, MCD_MODE_CONT, false>(c, block, tally, eo, ring, status, st);
}

}  // namespace mcd

using namespace mcd;

extern "C" int mcd_run(const mcd_sim* sim, const mcd_material* mat, const mcd_table* moller,
                       const mcd_table* gryz, mcd_tally* tally, const mcd_electron_out* electrons,
                       const mcd_event_ring* ring, uint32_t* status, int32_t block_size, void* stream) {
    if (!sim || !mat || !tally || !status) return MCD_EINVAL;
    const int rc = check_sim(*sim, *mat, moller, gryz);
    if (rc != MCD_OK) return rc;
    const bool automatic = block_size <= 0;
    if (automatic) {
        // automatic: 128 threads, halved (down to 8) while the grid would
        // leave SMs idle, so that a small job spreads over the GPU: its
        // trajectories are latency chains, and an SM with fewer lanes runs
        // each chain faster (1000 FP32 electrons: 1.00 ms in 32 blocks of 32,
        // 0.82 ms in 125 blocks of 8).  FP64 goes further, down to 2 threads
        // while the grid stays within one warp per scheduler (4 per SM):
        // fewer lanes per warp diverge less, and the longest FP64 chain
        // shares its scheduler with no other warp (1000 FP64 electrons with
        // their table: 7.37 ms in blocks of 8, 6.69 ms in blocks of 2,
        // 8.70 ms in blocks of 1, where schedulers hold two warps)
        block_size = 128;
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return MCD_ECUDA;
        while (block_size > 8 && (sim->num_el + block_size - 1) / block_size < sms) block_size /= 2;
        if (sim->precision == MCD_FP64)
            while (block_size > 2 && 2 * ((sim->num_el + block_size - 1) / block_size) <= 4ll * sms) block_size /= 2;
    }
    if (!(block_size < 32 ? (block_size & (block_size - 1)) == 0 : block_size % 32 == 0) || block_size > 256)
        return MCD_EINVAL;
    ElOut eo{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    if (electrons) {
        eo.outcome = electrons->outcome;
        eo.flags = electrons->flags;
        eo.final_E = electrons->final_E;
        eo.dir = electrons->dir;
        eo.last_pos = electrons->last_pos;
        eo.max_z = electrons->max_z;
        eo.n_events = electrons->n_events;
    }
    mcd_event_ring rg{nullptr, 0, nullptr};
    bool rec = false;
    if (ring && ring->rec && ring->cursor && ring->capacity > 0) {
        if (ring->fields & ~(MCD_EV_ALL | MCD_EV_PACKED_HEAD)) return MCD_EINVAL;
        if ((ring->fields & MCD_EV_PACKED_HEAD) && sim->num_el > (1ll << 28)) return MCD_EINVAL;
        rg = *ring;
        rec = true;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const mcd_table* tm = sim->mode == MCD_MODE_DS ? moller : nullptr;
    const mcd_table* tg = sim->mode == MCD_MODE_DS ? gryz : nullptr;
    if (sim->precision == MCD_FP64) {
        const SimConst<double> c = make_consts<double>(*sim, *mat, tm, tg);
        // where the automatic size reached two electrons per warp, a DS run
        // without an event ring puts the warp's idle lanes to work
        if (automatic && block_size == 2 && sim->mode == MCD_MODE_DS && !rec)
            return launch_lanes64(c, tally, eo, status, st);
        return dispatch_plain<double>(c, block_size, tally, eo, rg, rec, status, st);
    }
    return dispatch_plain<float>(make_consts<float>(*sim, *mat, tm, tg), block_size, tally, eo, rg, rec, status,
                                 st);
}

extern "C" size_t mcd_sigma_table_bytes(void) { return kSigTableBytes; }

extern "C" int mcd_build_sigma_table(const mcd_sim* sim, const mcd_material* mat, void* table, void* stream) {
    if (!sim || !mat || !table) return MCD_EINVAL;
    if (sim->mode != MCD_MODE_DS) return MCD_EINVAL;
    if (sim->precision != MCD_FP32 && sim->precision != MCD_FP64) return MCD_EINVAL;
    if (sim->elastic < MCD_ELASTIC_RUTH || sim->elastic > MCD_ELASTIC_NIGRAM_WDEFL) return MCD_EINVAL;
    if (!(sim->E0 > sim->Emin) || !(sim->Emin > 0) || !(sim->Wc > 0)) return MCD_EINVAL;
    if (mat->n_shells < 0 || mat->n_shells > MCD_MAX_SHELLS || mat->atnd <= 0) return MCD_EINVAL;
    if ((reinterpret_cast<uintptr_t>(table) & 15) != 0) return MCD_EINVAL;   // rows are read as float4
    if (sim->precision == MCD_FP64 && sigma_bytes64(sim->Emin, sim->E0, mat->n_shells + 3) > kSigTableBytes)
        return MCD_ETOOBIG;
    mcd_sim s = *sim;
    s.sigma_table = table;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (sim->precision == MCD_FP64) {
        const SimConst<double> c = make_consts<double>(s, *mat, nullptr, nullptr);
        const int n = c.sig_rows * kSig64Cells;
        k_sigtab64<<<(n + 127) / 128, 128, 0, st>>>(c, (int)c.sig_l0, c.sig_rows, static_cast<double*>(table));
        return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
    }
    s.precision = MCD_FP32;
    SimConst<double> c = make_consts<double>(s, *mat, nullptr, nullptr);
    k_sigtab_one<<<(c.sig_rows + 255) / 256, 256, 0, st>>>(c, c.sig_l0, c.sig_inv, c.sig_rows, c.sig_S,
                                                            static_cast<float*>(table));
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}

extern "C" size_t mcd_batch_workspace_bytes(int32_t nsims) {
    if (nsims <= 0 || nsims > kBatchMaxSims) return 0;
    return batch_bytes(nsims);
}

extern "C" size_t mcd_batch_upload_bytes(int32_t nsims) {
    if (nsims <= 0 || nsims > kBatchMaxSims) return 0;
    return batch_sig_off(nsims);
}

extern "C" int mcd_batch_prepare(const mcd_sim* sims, int32_t nsims, const mcd_material* mats,
                                 const int32_t* sim_material, const mcd_table* tables, const int32_t* sim_moller,
                                 const int32_t* sim_gryz, void* workspace, size_t workspace_bytes, void* stream) {
    if (!sims || !mats || !sim_material || !workspace) return MCD_EINVAL;
    if (nsims <= 0) return MCD_EINVAL;
    if (nsims > kBatchMaxSims) return MCD_ETOOBIG;
    if (workspace_bytes < batch_bytes(nsims)) return MCD_EINVAL;
    if ((reinterpret_cast<uintptr_t>(workspace) & 255) != 0) return MCD_EINVAL;
    const size_t bytes = batch_sig_off(nsims);   // everything but the tables, which the GPU fills
    uint8_t* host = static_cast<uint8_t*>(calloc(1, bytes));
    if (!host) return MCD_EINVAL;
    SimConst<double>* cd = reinterpret_cast<SimConst<double>*>(host + batch_dconsts_off(nsims));
    BatchHeader* h = reinterpret_cast<BatchHeader*>(host);
    unsigned long long* pre = reinterpret_cast<unsigned long long*>(host + batch_prefix_off());
    int32_t* perm = reinterpret_cast<int32_t*>(host + batch_perm_off(nsims));
    SimConst<float>* cs = reinterpret_cast<SimConst<float>*>(host + batch_consts_off(nsims));
    int rc = MCD_OK;
    for (int k = 0; k < nsims && rc == MCD_OK; ++k) {
        const mcd_sim& s = sims[k];
        const mcd_material& m = mats[sim_material[k]];
        const mcd_table* tm = nullptr;
        const mcd_table* tg = nullptr;
        if (s.mode == MCD_MODE_DS) {
            if (!tables || !sim_moller || !sim_gryz) { rc = MCD_EINVAL; break; }
            tm = &tables[sim_moller[k]];
            tg = &tables[sim_gryz[k]];
        }
        rc = check_sim(s, m, tm, tg);
        if (rc != MCD_OK) break;
        if (s.precision != MCD_FP32) { rc = MCD_EINVAL; break; }
        cs[k] = make_consts<float>(s, m, tm, tg);
        cd[k] = make_consts<double>(s, m, tm, tg);
    }
    if (rc == MCD_OK) share_sigma_tables(sims, nsims, cd, cs, static_cast<const uint8_t*>(workspace));
    if (rc == MCD_OK) pack_rows(sims, nsims, host);
    batch_order(sims, nsims, perm);
    unsigned long long acc = 0;
    for (int q = 0; q < nsims; ++q) {
        pre[q] = acc;
        acc += (unsigned long long)sims[perm[q]].num_el;
    }
    pre[nsims] = acc;
    h->queue = 0;
    h->total = acc;
    h->nsims = nsims;
    if (rc == MCD_OK) {
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const unsigned grid = (unsigned)(((long long)nsims * kSigRowsMax + 255) / 256);
        if (cudaMemcpyAsync(workspace, host, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) rc = MCD_ECUDA;
        else {
            k_sigtab<<<grid, 256, 0, st>>>(static_cast<uint8_t*>(workspace), nsims);
            if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) rc = MCD_ECUDA;
        }
    }
    free(host);
    return rc;
}

extern "C" int mcd_run_batched(void* workspace, int32_t nsims, mcd_tally* tallies, const mcd_tune* tune,
                               uint32_t* status, void* stream) {
    if (!workspace || !tallies || !status) return MCD_EINVAL;
    if (nsims <= 0) return MCD_EINVAL;
    if (nsims > kBatchMaxSims) return MCD_ETOOBIG;
    int block = 256, per_sm = 0, refill = 1;
    if (tune) {
        if (tune->block_size > 0) block = tune->block_size;
        if (tune->blocks_per_sm > 0) per_sm = tune->blocks_per_sm;
        if (tune->refill > 0) refill = tune->refill;
    }
    if (block % 32 != 0 || block > 1024 || refill < 1 || refill > 32 || (tune && tune->reserved != 0))
        return MCD_EINVAL;
    const bool lowreg = tune && (tune->variant & 1);
    const int inline_sigma = (tune && (tune->variant & 2)) ? 1 : 0;
    if (lowreg && block > 576) return MCD_EINVAL;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCD_ECUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MCD_ECUDA;
    const size_t smem = batch_smem(nsims);
    auto kern = lowreg ? k_batched_lr<false> : k_batched<false>;
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return MCD_ECUDA;
    }
    int fit = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, block, smem) != cudaSuccess) return MCD_ECUDA;
    if (fit < 1) return MCD_ETOOBIG;
    if (per_sm <= 0 || per_sm > fit) per_sm = fit;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // reset the queue (the first word of the workspace)
    if (cudaMemsetAsync(workspace, 0, sizeof(unsigned long long), st) != cudaSuccess) return MCD_ECUDA;
    kern<<<sms * per_sm, block, smem, st>>>(static_cast<uint8_t*>(workspace), tallies, refill, status,
                                            mcd_event_ring{}, inline_sigma);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}

// Batched run that also appends every event to a device ring (the streaming
// path): the caller drains the ring between launches (mcd.stream).
extern "C" int mcd_run_batched_ring(void* workspace, int32_t nsims, mcd_tally* tallies, const mcd_tune* tune,
                                    const mcd_event_ring* ring, uint32_t* status, void* stream) {
    if (!workspace || !tallies || !status || !ring || !ring->rec || !ring->cursor || ring->capacity == 0)
        return MCD_EINVAL;
    if (ring->fields & ~(MCD_EV_ALL | MCD_EV_PACKED_HEAD)) return MCD_EINVAL;
    if (nsims <= 0) return MCD_EINVAL;
    if (nsims > kBatchMaxSims) return MCD_ETOOBIG;
    int block = 256, per_sm = 0, refill = 1;
    if (tune) {
        if (tune->block_size > 0) block = tune->block_size;
        if (tune->blocks_per_sm > 0) per_sm = tune->blocks_per_sm;
        if (tune->refill > 0) refill = tune->refill;
    }
    if (block % 32 != 0 || block > 1024 || refill < 1 || refill > 32 || (tune && tune->reserved != 0))
        return MCD_EINVAL;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCD_ECUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MCD_ECUDA;
    const size_t smem = batch_smem(nsims);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_batched<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return MCD_ECUDA;
    int fit = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_batched<true>, block, smem) != cudaSuccess)
        return MCD_ECUDA;
    if (fit < 1) return MCD_ETOOBIG;
    if (per_sm <= 0 || per_sm > fit) per_sm = fit;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(workspace, 0, sizeof(unsigned long long), st) != cudaSuccess) return MCD_ECUDA;
    const int inline_sigma = (tune && (tune->variant & 2)) ? 1 : 0;
    k_batched<true><<<sms * per_sm, block, smem, st>>>(static_cast<uint8_t*>(workspace), tallies, refill, status,
                                                          *ring, inline_sigma);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}

// ---------------------------------------------------------------------------
// Batched run that allocates nothing.
//
// Some callers cannot call cudaMalloc: an application that embeds this
// library and owns all device memory through its own arena, or a caller on a
// latency budget for which an allocation (which can synchronise the device)
// is not acceptable.  This variant keeps the batched kernel's scratch (queue
// counter, electron prefix sums and packed simulation constants) in a
// file-scope device array instead of a caller workspace.  The array holds at
// most kStaticMaxSims simulations and stays resident on every GPU that loads
// the library until the process exits.  Every call shares it and rewrites it
// in full (the queue counter starts at zero each call), so calls that overlap
// on the GPU - two streams, or two host threads - race on it and must not be
// issued concurrently.
//
// The host packs the scratch and hands it to a staging kernel as one
// by-value argument (kernel arguments may take up to 32764 bytes), which
// writes it into the array ahead of the transport launch on the same
// stream: no host buffer has to outlive the call, and nothing is copied
// from pageable memory.
// ---------------------------------------------------------------------------
#include <mutex>

namespace mcd {

constexpr int kStaticMaxSims = MCD_STATIC_MAX_SIMS;
constexpr size_t kStaticHeadBytes = batch_consts_off(kStaticMaxSims);
constexpr size_t kStaticScratchBytes = batch_core_bytes(kStaticMaxSims);
static_assert(kStaticScratchBytes % 16 == 0, "the scratch is staged as 16-byte words");

struct StaticBlock {
    uint4 w[kStaticScratchBytes / 16];
};
static_assert(sizeof(StaticBlock) + 16 <= 32764, "the packed scratch must fit the kernel argument space");

static __device__ __align__(256) uint8_t g_static_scratch[kStaticScratchBytes];

// Writes the first `words` 16-byte words of the packed block to dst.
__global__ void __launch_bounds__(256) k_static_stage(uint4* dst, const StaticBlock blk, uint32_t words) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < words; i += gridDim.x * blockDim.x)
        dst[i] = blk.w[i];
}

constexpr int kStaticMaxDevices = 64;
static std::mutex g_static_mu;
static void* g_static_ptr[kStaticMaxDevices];

// The device address of g_static_scratch on the current device, looked up
// once per device (host code may not use the symbol itself as an address).
// The address belongs to the device's primary context: a cudaDeviceReset
// makes it stale, so the library must not be used across one.
static int static_scratch(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCD_ECUDA;
    if (dev < 0 || dev >= kStaticMaxDevices) return MCD_EINVAL;
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return MCD_ECUDA;
        g_static_ptr[dev] = p;
    }
    *out = g_static_ptr[dev];
    return MCD_OK;
}

}  // namespace mcd

extern "C" int mcd_run_batched_noalloc(const mcd_sim* sims, int32_t nsims, const mcd_material* mats,
                                       const int32_t* sim_material, const mcd_table* tables,
                                       const int32_t* sim_moller, const int32_t* sim_gryz, mcd_tally* tallies,
                                       const mcd_tune* tune, uint32_t* status, void* stream) {
    if (!sims || !mats || !sim_material || !tallies || !status) return MCD_EINVAL;
    if (nsims <= 0) return MCD_EINVAL;
    if (nsims > kStaticMaxSims) return MCD_ETOOBIG;
    int block = 256, per_sm = 0, refill = 1;
    if (tune) {
        if (tune->block_size > 0) block = tune->block_size;
        if (tune->blocks_per_sm > 0) per_sm = tune->blocks_per_sm;
        if (tune->refill > 0) refill = tune->refill;
    }
    if (block % 32 != 0 || block > 1024 || refill < 1 || refill > 32 || (tune && tune->reserved != 0))
        return MCD_EINVAL;
    // the variant bits of mcd_run_batched: bit 0 the 56-register kernel,
    // bit 1 inline cross sections (a caller-built sigma_table is then not read)
    const bool lowreg = tune && (tune->variant & 1);
    const int inline_sigma = (tune && (tune->variant & 2)) ? 1 : 0;
    if (lowreg && block > 576) return MCD_EINVAL;

    // pack on the host: header (queue = 0), prefix sums, constants, row pointers
    StaticBlock blk;
    uint8_t* host = reinterpret_cast<uint8_t*>(&blk);
    memset(host, 0, kStaticHeadBytes);
    BatchHeader* h = reinterpret_cast<BatchHeader*>(host);
    unsigned long long* pre = reinterpret_cast<unsigned long long*>(host + batch_prefix_off());
    int32_t* perm = reinterpret_cast<int32_t*>(host + batch_perm_off(nsims));
    SimConst<float>* cs = reinterpret_cast<SimConst<float>*>(host + batch_consts_off(nsims));
    for (int k = 0; k < nsims; ++k) {
        const mcd_sim& s = sims[k];
        const mcd_material& m = mats[sim_material[k]];
        const mcd_table* tm = nullptr;
        const mcd_table* tg = nullptr;
        if (s.mode == MCD_MODE_DS) {
            if (!tables || !sim_moller || !sim_gryz) return MCD_EINVAL;
            tm = &tables[sim_moller[k]];
            tg = &tables[sim_gryz[k]];
        }
        const int rc = check_sim(s, m, tm, tg);
        if (rc != MCD_OK) return rc;
        if (s.precision != MCD_FP32) return MCD_EINVAL;
        cs[k] = make_consts<float>(s, m, tm, tg);
    }
    batch_order(sims, nsims, perm);
    unsigned long long acc = 0;
    for (int q = 0; q < nsims; ++q) {
        pre[q] = acc;
        acc += (unsigned long long)sims[perm[q]].num_el;
    }
    pre[nsims] = acc;
    h->queue = 0;
    h->total = acc;
    h->nsims = nsims;
    pack_rows(sims, nsims, host);
    // the core only: cross sections come from the callers' tables or are
    // evaluated inline
    const uint32_t words = (uint32_t)((batch_core_bytes(nsims) + 15) / 16);

    void* scratch = nullptr;
    int rc = static_scratch(&scratch);
    if (rc != MCD_OK) return rc;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCD_ECUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MCD_ECUDA;
    const size_t smem = batch_smem(nsims);
    auto kern = lowreg ? k_batched_lr<false> : k_batched<false>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return MCD_ECUDA;
    int fit = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, block, smem) != cudaSuccess) return MCD_ECUDA;
    if (fit < 1) return MCD_ETOOBIG;
    if (per_sm <= 0 || per_sm > fit) per_sm = fit;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_static_stage<<<(words + 255) / 256, 256, 0, st>>>(static_cast<uint4*>(scratch), blk, words);
    if (cudaGetLastError() != cudaSuccess) return MCD_ECUDA;
    kern<<<sms * per_sm, block, smem, st>>>(static_cast<uint8_t*>(scratch), tallies, refill, status,
                                            mcd_event_ring{}, inline_sigma);
    return cudaGetLastError() == cudaSuccess ? MCD_OK : MCD_ECUDA;
}
