// mcd_consts.h - per-simulation constant block shared by host and device.
//
// All cross sections are folded into inverse-mean-free-path units (1/A):
// sigma' = n * sigma * 1e-14, so that the step length is -ln(U) / sum(sigma')
// (MC/tools/scattering.py:19-36: mfp = 1e14 / (n * sum(sigma)) A) and every
// quantity stays well inside FP32 range.  The algebra below restates the
// reference formulas in forms that need fewer divisions and no cancellation:
//
//  Rutherford (MC/tools/crossSections.py:14-58), alpha = a0 / E,
//     sigma' = cR * r^2 / (E + a0),  r = (E + 511000) / (E + 1024000),
//     cR = 5.21e-21 * 1e6 * 4 pi Z^2 / a0 * n * 1e-14,  a0 = 3.4 Z^0.666667
//     (wDefl, :63-86: Z^2 -> Z (Z + 1))
//  Nigram (crossSections.py:90-147), beta* = b / E, b = 0.48 * 5.43 Z^(2/3),
//     sigma' = cN / (E + b),  cN = pi e^4 Z^2 / (4 b) * n * 1e-14
//     (wDefl: Z^2 -> Z (Z + 1)); no r^2 factor
//  diffraction (crossSections.py:329-349), sigma = 1e13 / (n xip_g) cm^2,
//     sigma' = 0.1 / xip_g, and the step of a diffraction event has mean
//     free path xip_g (scattering.py:540-548)
//  Moller (crossSections.py:183-208), E > Wc,
//     sigma' = pM / E^2 * (E/Wc - E/(E-Wc) + ln(Wc/(E-Wc))),
//     pM = n_val * pi e^4 * n * 1e-14
//  Gryzinski shell k (crossSections.py:213-242), E > Es,
//     sigma' = gP * x sqrt(x) * (1 + 2/3 (1 - Es/(2E)) ln(2.7 + sqrt((E-Es)/Es))) / E,
//     x = (E - Es)/(E + Es),  gP = ns * pi e^4 * n * 1e-14 / Es
//  Quinn (crossSections.py:247-284), E > Epl, a = E/Ef, b = Epl/Ef,
//     sigma' = qK / E * ln(qC1 * (sqrt(a) + sqrt(a - b)) / b),
//     qK = 1e-10 * Epl / (2 a_Bohr),  qC1 = sqrt(1 + b) - 1
//     (sqrt(a) - sqrt(a-b) = b / (sqrt(a) + sqrt(a-b)))
//  Bethe (MC/tools/stoppingPowers.py:112-215), eV/A,
//     classical  S = bP / E * ln(1.166 E / J)
//     JL         S = bP / E * ln(1.166 (E + k J) / J)
//     explicit   S = bX / E * (bW * ln E - bC),
//                bW = Zval + sum Zi,  bC = Zval ln Eval + sum Zi ln Ei
//     bP = 2 pi e^4 n Z 1e-14,  bX = 2 pi e^4 n 1e-14
#ifndef MCD_CONSTS_H
#define MCD_CONSTS_H

#include <stdint.h>
#include <math.h>

#include "../../include/mcd.h"

namespace mcd {

constexpr double kPiEfour = 6.51408491409531e-14;  // cm^2 eV^2 (parameters.py:7)
constexpr double kBohrR = 5.29177210544e-11;       // m (CODATA 2022)
constexpr double kPi = 3.141592653589793;

struct TableDev {
    const float* Es;
    const float* Ws;
    const float* cdf;
    float inv_dE;      // (nE - 1) / (E_last - E_first), 0 if unknown
    int32_t reserved_;
    const uint16_t* guide;
    int32_t nE;
    int32_t nW;
    float E_first, E_last;
};

template <class T>
struct __align__(16) SimConst {
    // the words every event reads first, as one 16-byte load: Philox
    // counter word 3, the key, and the events before 'long' (at most
    // 2^32 - 1, the counter word's range)
    uint32_t sim_id;
    uint32_t key0, key1;
    uint32_t max_scatt;
    // transport
    T E0, Emin, thickness;
    T d0x, d0y, d0z;
    // Rutherford: cR, a0 of the default model; the elastic total cross
    // section is sigma' = cRs * (ruth_r2 ? r^2 : 1) / (E + aS), and the polar
    // angle always uses a0
    T cR, a0, cRs, aS;
    int32_t ruth_r2;
    int32_t diff;   // diffraction channel on (DS)
    T dS, xip;      // its sigma' (1/A) and step mean free path (A)
    // Moller
    T pM, Wc;
    // Gryzinski shells
    T gEs[MCD_MAX_SHELLS];
    T gP[MCD_MAX_SHELLS];
    T gInvEs[MCD_MAX_SHELLS];
    // Quinn
    T qK, qC1, qInvEf, qB, Epl;
    // binary collision
    T Ef;
    // Bethe
    T bP, bJ, bInvJ, bkJ, bX, bW, bC;
    int32_t nsh;
    int32_t mode;
    int32_t bethe;
    uint32_t quirks;
    uint32_t tally_flags;
    uint64_t first;
    int64_t num_el;
    int32_t hE, hT;
    T invWE, invWT;  // 1/bin width (eV, degrees)
    TableDev tab[2];   // [0] Moller (valence), [1] Gryzinski (outermost shell)
    // cumulative channel cross sections tabulated on a log-E grid (FP32 DS
    // transport; nullptr = evaluate inline).  Row i (of sig_rows, sig_S
    // floats apart) holds, at E = 2^(sig_l0 + i / sig_inv), E times the
    // total, then E times the running sums over the channels in pick order
    // before the last: Ruth, Moller, Gryz[0..nsh-1] (sig_K = nsh + 3 columns;
    // padding FLT_MAX).  The total and the first sums share one 16-byte load.
    // E * sigma varies slowly in log E, so linear interpolation at 128 rows
    // per octave is within 3e-7 of the exact sums (relative to the total).
    // FP64 transport reads an FP64 table (the octave blocks of cell records
    // described at kSig64Cells) through the same pointer: sig_l0 then holds
    // the first octave's exponent and sig_rows the number of octaves; the
    // record stride is sig64_stride(sig_K) doubles.
    const void* sig;
    float sig_l0, sig_inv, sig_tmax, sig_off;   // sig_off = -sig_l0 * sig_inv
    int32_t sig_K, sig_S, sig_rows;
    // the small fields the event code tests, packed so that one load serves
    // them all: quirks (bits 0-2, the MCD_Q_* masks), kBit* flags, sig_K
    // (bits 8-11) and sig_S (bits 12-16)
    uint32_t bits;
};

// kBitFilm: a finite thickness, so that a semi-infinite sample skips the
// bottom-face test (and its shared-memory load) on every step
constexpr uint32_t kBitDiff = 1u << 3, kBitCont = 1u << 4, kBitChan = 1u << 5, kBitR2 = 1u << 6,
                   kBitFilm = 1u << 7;
template <class C>
__host__ __device__ __forceinline__ int bits_K(const C& c) { return (int)((c.bits >> 8) & 15u); }
template <class C>
__host__ __device__ __forceinline__ int bits_S(const C& c) { return (int)((c.bits >> 12) & 31u); }

constexpr int kSigRowsMax = 4096;      // grid points of a cross-section table, at most
constexpr int kSigStride = 12;         // floats per row, at most (3 + MCD_MAX_SHELLS + 1)
constexpr double kSigPerOctave = 128;  // grid density

// FP64 cross-section tables (FP64 DS transport reading mcd_sim.sigma_table):
// one block of kSig64Cells cell records per octave [2^e, 2^(e+1)) of the
// energy range, uniform in E inside the octave: cell i covers
// 2^e [1 + i / cells, 1 + (i + 1) / cells), so that the octave is the
// exponent of E, the cell the top mantissa bits and the offset f in [0, 1)
// the remaining ones (no logarithm, exact).  A record holds a flag word (1
// when a channel threshold -- a shell's binding energy, Wc, the plasmon
// energy -- lies in the span of the four nodes i - 1 .. i + 2, where the
// cross sections have a kink, or the lowest node lies below 2 Wc, where the
// Moller cross section is negative with a pole at Wc; the transport
// evaluates the cross sections there instead), a
// pad word, then for each of the sig_K columns the coefficients c0..c3 of
// the cubic c0 + f (c1 + f (c2 + f c3)) through the column's values at those
// four nodes: column 0 the mean free path 1 / sum(sigma) in A, columns
// 1 .. sig_K - 1 the running sums in pick order (Ruth, +Moller, +Gryz[k]
// ...) as fractions of the total.  The event then needs no division and no
// interpolation weights: three FMAs per column read, the channel the first
// fraction at or above U.  In the unflagged cells the cubic is within about
// 1.3e-10 of the exact mean free path (relative) and of the exact fractions
// (absolute) for Al, Si, Cu and Au over 0.1-30 keV.
constexpr int kSig64Cells = 256;
__host__ __device__ constexpr int sig64_stride(int K) { return 2 + 4 * K; }   // doubles per cell record

// Bytes of a caller's cross-section table buffer (mcd_sigma_table_bytes):
// FP32 tables take at most kSigRowsMax rows of kSigStride floats (192 KiB);
// FP64 tables take whole octaves, 920 KiB for Au from 50 eV to 30 keV.
constexpr size_t kSigTableBytes = (size_t)1 << 20;

// First octave exponent and octave count of an FP64 table over (lo, hi].
inline int sigma_octaves64(double lo, double hi, int32_t* e_lo) {
    int a = 0, b = 0;
    frexp(lo, &a);   // lo = m 2^a with m in [0.5, 1): octave a - 1
    frexp(hi, &b);
    *e_lo = a - 1;
    return b - a + 1;
}

// Bytes of the FP64 table of a simulation with K channel columns.
inline size_t sigma_bytes64(double lo, double hi, int K) {
    int32_t e0 = 0;
    return sizeof(double) * (size_t)sigma_octaves64(lo, hi, &e0) * kSig64Cells * (size_t)sig64_stride(K);
}

// The log2-E grid of a cross-section table over [lo, hi] (eV), slightly
// widened so that both ends interpolate inside it.
inline void sigma_grid(double lo, double hi, float* l0, float* inv, float* tmax, int32_t* rows) {
    const double a = log2(lo * (1.0 - 1e-6)), b = log2(hi * (1.0 + 1e-6));
    int r = (int)ceil((b - a) * kSigPerOctave) + 1;
    r = r < 2 ? 2 : (r > kSigRowsMax ? kSigRowsMax : r);
    *l0 = (float)a;
    *inv = (float)((r - 1) / (b - a));
    *tmax = (float)(r - 2) + 0.999f;
    *rows = r;
}

// Host-side builder: precompute the constant block of one simulation.
template <class T>
inline SimConst<T> make_consts(const mcd_sim& s, const mcd_material& m,
                               const mcd_table* tm, const mcd_table* tg) {
    SimConst<T> c;
    const double n = m.atnd * (s.n_scale > 0 ? s.n_scale : 1.0);
    const double Z = (double)m.Z;
    const double t = s.s_tilt * kPi / 180.0;
    c.E0 = (T)s.E0;
    c.Emin = (T)s.Emin;
    c.thickness = (T)(s.thickness > 0 ? s.thickness : 1e30);
    c.d0x = (T)(-sin(t));
    c.d0y = (T)0;
    c.d0z = (T)cos(t);
    const double a0 = 3.4 * pow(Z, 0.666667);
    c.a0 = (T)a0;
    c.cR = (T)(5.21e-21 * 1e6 * 4.0 * kPi * Z * Z / a0 * n * 1e-14);
    const bool wdefl = s.elastic == MCD_ELASTIC_RUTH_WDEFL || s.elastic == MCD_ELASTIC_NIGRAM_WDEFL;
    const double zz = wdefl ? Z * (Z + 1.0) : Z * Z;
    if (s.elastic == MCD_ELASTIC_NIGRAM || s.elastic == MCD_ELASTIC_NIGRAM_WDEFL) {
        const double b = 0.48 * 5.43 * pow(Z, 2.0 / 3.0);
        c.aS = (T)b;
        c.cRs = (T)(kPiEfour * zz / (4.0 * b) * n * 1e-14);
        c.ruth_r2 = 0;
    } else {
        c.aS = (T)a0;
        c.cRs = wdefl ? (T)(5.21e-21 * 1e6 * 4.0 * kPi * zz / a0 * n * 1e-14) : c.cR;
        c.ruth_r2 = 1;
    }
    c.diff = (s.mode == MCD_MODE_DS && s.diff_mfp) ? 1 : 0;
    c.dS = (T)(c.diff ? 0.1 / m.xip_g : 0.0);
    c.xip = (T)(c.diff ? m.xip_g : 0.0);
    c.pM = (T)(m.n_val * kPiEfour * n * 1e-14);
    c.Wc = (T)s.Wc;
    c.nsh = m.n_shells;
    for (int k = 0; k < MCD_MAX_SHELLS; ++k) {
        if (k < m.n_shells) {
            c.gEs[k] = (T)m.shell_E[k];
            c.gP[k] = (T)(m.shell_n[k] * kPiEfour * n * 1e-14 / m.shell_E[k]);
            c.gInvEs[k] = (T)(1.0 / m.shell_E[k]);
        } else {
            c.gEs[k] = (T)1e30;  // never below E: sigma' = 0
            c.gP[k] = (T)0;
            c.gInvEs[k] = (T)0;
        }
    }
    // plasmon and Fermi energies scale with the density
    const double scale = (s.n_scale > 0 ? s.n_scale : 1.0);
    const double Epl = m.plasmon_e * sqrt(scale);
    const double Ef = m.fermi_e * pow(scale, 2.0 / 3.0);
    const double b = Epl / Ef;
    c.Epl = (T)Epl;
    c.Ef = (T)Ef;
    c.qK = (T)(1e-10 * Epl / (2.0 * kBohrR));
    c.qC1 = (T)(sqrt(1.0 + b) - 1.0);
    c.qInvEf = (T)(1.0 / Ef);
    c.qB = (T)b;
    const double J = m.J * (s.J_scale > 0 ? s.J_scale : 1.0);
    c.bP = (T)(2.0 * kPiEfour * n * Z * 1e-14);
    c.bJ = (T)J;
    c.bInvJ = (T)(1.0 / J);
    c.bkJ = (T)(m.bethe_k * J);
    c.bX = (T)(2.0 * kPiEfour * n * 1e-14);
    double w = m.n_val, cc = m.n_val * log(m.E_val);
    for (int k = 0; k < m.n_shells; ++k) {
        w += m.shell_n[k];
        cc += m.shell_n[k] * log(m.shell_E[k]);
    }
    c.bW = (T)w;
    c.bC = (T)cc;
    c.mode = s.mode;
    c.bethe = s.bethe_model;
    c.quirks = s.quirks;
    c.tally_flags = s.tally_flags;
    c.sim_id = s.sim_id;
    c.key0 = (uint32_t)(s.seed & 0xffffffffull);
    c.key1 = (uint32_t)(s.seed >> 32);
    c.max_scatt = (s.max_scatt > 0 && s.max_scatt < (int64_t)UINT32_MAX) ? (uint32_t)s.max_scatt : UINT32_MAX;
    c.first = s.first_electron;
    c.num_el = s.num_el;
    c.hE = s.hist_E_bins;
    c.hT = s.hist_T_bins;
    c.invWE = (T)(s.hist_E_width > 0 ? 1.0 / s.hist_E_width : 0.0);
    c.invWT = (T)(s.hist_T_width > 0 ? 1.0 / s.hist_T_width : 0.0);
    TableDev z{nullptr, nullptr, nullptr, 0.0f, 0, nullptr, 0, 0, 0.0f, 0.0f};
    auto td = [](const mcd_table* t) {
        TableDev d{t->Es, t->Ws, t->cdf, 0.0f, 0, t->guide, t->nE, t->nW, t->E_first, t->E_last};
        if (t->E_last > t->E_first && t->nE > 1)
            d.inv_dE = (float)((double)(t->nE - 1) / ((double)t->E_last - (double)t->E_first));
        return d;
    };
    c.tab[0] = tm ? td(tm) : z;
    c.tab[1] = tg ? td(tg) : z;
    // the caller's table (mcd_run), or none until a batch shares one among
    // the simulations it fits
    c.sig = nullptr;
    c.sig_l0 = c.sig_inv = c.sig_tmax = c.sig_off = 0.0f;
    c.sig_K = m.n_shells + 3;
    c.sig_S = (c.sig_K + 3) & ~3;
    c.sig_rows = 0;
    if (s.sigma_table && s.mode == MCD_MODE_DS) {
        c.sig = s.sigma_table;
        if (s.precision == MCD_FP64) {
            int32_t e0 = 0;
            c.sig_rows = sigma_octaves64(s.Emin, s.E0, &e0);
            c.sig_l0 = (float)e0;
        } else {
            sigma_grid(s.Emin, s.E0, &c.sig_l0, &c.sig_inv, &c.sig_tmax, &c.sig_rows);
            c.sig_off = -c.sig_l0 * c.sig_inv;
        }
    }
    c.bits = (c.quirks & 7u) | (c.diff ? kBitDiff : 0u) | (c.mode == MCD_MODE_CONT ? kBitCont : 0u) |
             ((c.tally_flags & MCD_TALLY_CHANNELS) ? kBitChan : 0u) | (c.ruth_r2 ? kBitR2 : 0u) |
             ((s.thickness > 0 && s.thickness < 1e30) ? kBitFilm : 0u) |
             ((uint32_t)c.sig_K << 8) | ((uint32_t)c.sig_S << 12);
    return c;
}

// Validation shared by the entry points; returns an MCD_* code.
inline int check_sim(const mcd_sim& s, const mcd_material& m, const mcd_table* tm,
                     const mcd_table* tg) {
    if (s.mode != MCD_MODE_DS && s.mode != MCD_MODE_CONT) return MCD_EINVAL;
    if (s.mode == MCD_MODE_CONT && (s.bethe_model < 0 || s.bethe_model > 2)) return MCD_EINVAL;
    if (s.precision != MCD_FP32 && s.precision != MCD_FP64) return MCD_EINVAL;
    if (s.elastic < MCD_ELASTIC_RUTH || s.elastic > MCD_ELASTIC_NIGRAM_WDEFL) return MCD_EINVAL;
    if (s.diff_mfp && (s.mode != MCD_MODE_DS || !(m.xip_g > 0))) return MCD_EINVAL;
    if (s.sigma_table && s.mode != MCD_MODE_DS) return MCD_EINVAL;
    // an FP64 table must fit the mcd_sigma_table_bytes() a caller allocates
    if (s.sigma_table && s.precision == MCD_FP64 && m.n_shells >= 0 && m.n_shells <= MCD_MAX_SHELLS &&
        s.E0 > s.Emin && s.Emin > 0 &&
        sigma_bytes64(s.Emin, s.E0, m.n_shells + 3) > kSigTableBytes)
        return MCD_ETOOBIG;
    if (!(s.E0 > s.Emin) || !(s.Emin > 0)) return MCD_EINVAL;
    if (s.num_el < 0) return MCD_EINVAL;
    if (m.n_shells < 0 || m.n_shells > MCD_MAX_SHELLS || m.atnd <= 0) return MCD_EINVAL;
    if (s.hist_E_bins < 0 || s.hist_E_bins > MCD_HIST_E_MAX) return MCD_ETOOBIG;
    if (s.hist_T_bins < 0 || s.hist_T_bins > MCD_HIST_T_MAX) return MCD_ETOOBIG;
    if (s.mode == MCD_MODE_DS) {
        if (!tm || !tg) return MCD_EINVAL;
        if (!tm->Es || !tm->Ws || !tm->cdf || tm->nE < 1 || tm->nW < 2) return MCD_EINVAL;
        if (!tg->Es || !tg->Ws || !tg->cdf || tg->nE < 1 || tg->nW < 2) return MCD_EINVAL;
        if (!(s.Wc > 0)) return MCD_EINVAL;
    }
    return MCD_OK;
}

}  // namespace mcd

#endif  // MCD_CONSTS_H
