// mcd_device.cuh - device side of the transport: counter-based random
// numbers, cross sections, table sampling, the DS and continuous event and
// the direction update.  One template serves FP32 (throughput) and FP64
// (parity) transport.
#ifndef MCD_DEVICE_CUH
#define MCD_DEVICE_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "mcd_consts.h"

namespace mcd {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Counter = (event,
// electron lo, electron hi, sim id), key = seed: every (sim, electron, event)
// has its own block of four 32-bit words, so any electron range can be
// re-run, sharded or recomputed (the adjoint) without stored state.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        // one 32 x 32 -> 64-bit product per multiplier
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0);
    }
    return c;
}

// ---------------------------------------------------------------------------
// precision traits
// ---------------------------------------------------------------------------
template <class T>
struct Ops;

template <>
struct Ops<float> {
    // uniform in (0,1) from the top 23 bits, (u >> 9) 2^-23 + 2^-24, and its
    // exact complement 1 - U.  The 23 bits become the mantissa of a float in
    // [1, 2); subtracting 1 - 2^-24 is exact (Sterbenz), so no integer to
    // float conversion is needed.
    static __device__ __forceinline__ float unit(uint32_t u) {
        return __uint_as_float((u >> 9) | 0x3f800000u) - 0x1.fffffep-1f;
    }
    static __device__ __forceinline__ float unit_c(uint32_t u) {
        return __uint_as_float(((~u) >> 9) | 0x3f800000u) - 0x1.fffffep-1f;
    }
    static __device__ __forceinline__ float ln(float x) { return __logf(x); }
    // logarithm of the step-length draw: the special-function unit's log2,
    // absolute error <= 2^-22 for x in [1/2, 2] and 2 ulp elsewhere, i.e. a
    // step of -ln U mean free paths is off by at most about 1e-7 of one
    static __device__ __forceinline__ float ln_step_word(uint32_t w) { return __logf(unit(w)); }
    static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
    static __device__ __forceinline__ float rsqrt_(float x) { return rsqrtf(x); }
    // 1/sqrt(x) for the squared norm of a rotated unit vector
    static __device__ __forceinline__ float renorm(float x) { return rsqrtf(x); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ void sincos_pi(float u, float* s, float* c) {
        __sincosf(3.14159265358979f * u, s, c);
    }
    static __device__ __forceinline__ void sincos_pi_word(uint32_t w, float* s, float* c) { sincos_pi(unit(w), s, c); }
    static __device__ __forceinline__ float nan_() { return __int_as_float(0x7fc00000); }
    static __device__ __forceinline__ float acos_deg(float x) { return acosf(x) * 57.2957795f; }
};

// ---------------------------------------------------------------------------
// FP64 logarithm and sin/cos(pi u) of the transport's uniforms, table driven
// (the scheme of P. T. P. Tang, "Table-driven implementation of the
// logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4),
// 1990: a table at 256 breakpoints and a short series of the remainder).
// The arguments are uniforms in (0, 1) with 33 significant bits, and what a
// trajectory needs is absolute accuracy, since a step's error enters the
// position as that error times the mean free path: within one ulp, i.e.
// 2.3e-16 max(1, |ln U|) for the logarithm and 1.2e-16 for sin/cos
// (against 40-digit values in the tests).
// ---------------------------------------------------------------------------
struct F64Tabs {
    double lnm[256];    // ln(1 + j/256)
    double invm[256];   // 1 / (1 + j/256)
    double sn[256];     // sin(pi j/256)
    double cs[256];     // cos(pi j/256)
};
// The table entries are evaluated at compile time in double-double
// arithmetic (T. J. Dekker, "A floating-point technique for extending the
// available precision", Numer. Math. 18, 1971: exact sums by two-sum,
// exact products by Veltkamp's split), so that each rounds to the double
// nearest its value; series summed in plain doubles were up to 3 ulp off.
struct CxDD {
    double hi, lo;
};
constexpr CxDD cx_two_sum(double a, double b) {
    const double s = a + b, bb = s - a;
    return CxDD{s, (a - (s - bb)) + (b - bb)};
}
constexpr CxDD cx_two_prod(double a, double b) {
    const double p = a * b;
    const double ca = 134217729.0 * a, ah = ca - (ca - a), al = a - ah;   // 2^27 + 1
    const double cb = 134217729.0 * b, bh = cb - (cb - b), bl = b - bh;
    return CxDD{p, ((ah * bh - p) + ah * bl + al * bh) + al * bl};
}
constexpr CxDD cx_add(CxDD x, CxDD y) {
    const CxDD s = cx_two_sum(x.hi, y.hi);
    return cx_two_sum(s.hi, s.lo + x.lo + y.lo);
}
constexpr CxDD cx_mul(CxDD x, CxDD y) {
    const CxDD p = cx_two_prod(x.hi, y.hi);
    return cx_two_sum(p.hi, p.lo + (x.hi * y.lo + x.lo * y.hi));
}
constexpr CxDD cx_div(CxDD x, double d) {   // x / d
    const double q1 = x.hi / d;
    const CxDD p = cx_two_prod(q1, d);
    const CxDD r = cx_two_sum(x.hi, -p.hi);
    const double q2 = ((r.hi + r.lo) - p.lo + x.lo) / d;
    return cx_two_sum(q1, q2);
}
// ln(1 + j/256) = 2 atanh(y), y = j / (512 + j) < 1/3
constexpr double cx_ln_ratio(int j) {
    const CxDD y = cx_div(CxDD{(double)j, 0.0}, 512.0 + j), y2 = cx_mul(y, y);
    CxDD term = y, sum{0.0, 0.0};
    for (int k = 0; k < 36; ++k) {
        sum = cx_add(sum, cx_div(term, 2.0 * k + 1.0));
        term = cx_mul(term, y2);
    }
    return 2.0 * sum.hi + 2.0 * sum.lo;
}
struct CxPair {
    double s, c;
};
// sin(pi a/256), cos(pi a/256) by their Taylor series, 0 <= a <= 64
constexpr CxPair cx_sincos(int a) {
    const CxDD pi{3.141592653589793, 1.2246467991473532e-16};
    const CxDD x = cx_div(cx_mul(pi, CxDD{(double)a, 0.0}), 256.0);
    const CxDD mx2 = cx_mul(x, CxDD{-x.hi, -x.lo});
    CxDD ts = x, tc{1.0, 0.0}, s{0.0, 0.0}, c{0.0, 0.0};
    for (int k = 0; k < 16; ++k) {
        s = cx_add(s, ts);
        c = cx_add(c, tc);
        ts = cx_div(cx_mul(ts, mx2), (2.0 * k + 2.0) * (2.0 * k + 3.0));
        tc = cx_div(cx_mul(tc, mx2), (2.0 * k + 1.0) * (2.0 * k + 2.0));
    }
    return CxPair{s.hi + s.lo, c.hi + c.lo};
}
constexpr F64Tabs cx_f64_tabs() {
    F64Tabs t{};
    for (int j = 0; j < 256; ++j) {
        t.lnm[j] = cx_ln_ratio(j);
        t.invm[j] = 256.0 / (256.0 + j);
        // reduce to [0, pi/4]: sin(pi - x) = sin x, cos(pi - x) = -cos x;
        // sin(pi/2 - x) = cos x, cos(pi/2 - x) = sin x
        const int a = j > 128 ? 256 - j : j;
        const CxPair p = a <= 64 ? cx_sincos(a) : cx_sincos(128 - a);
        t.sn[j] = a <= 64 ? p.s : p.c;
        const double c = a <= 64 ? p.c : p.s;
        t.cs[j] = j > 128 ? -c : c;
    }
    return t;
}
static __device__ const F64Tabs kF64Tabs = cx_f64_tabs();

// ln U of the uniform U = (w + 1/2) 2^-32 = v 2^-33, v = 2w + 1 (odd, 33
// bits), from the word itself: v = m 2^p with m in [1, 2) (p from the
// leading zeros, m's mantissa bits by a shift), so U = m 2^(p - 33); the
// top 8 bits of m give the breakpoint m_j = 1 + j/256, and
// ln m = ln m_j + ln(1 + t), t = (m - m_j)/m_j in [0, 1/256), by its series
// to t^6 (the next term is below 2e-18)
__device__ __forceinline__ double ln_word(uint32_t w) {
    const unsigned long long v = 2ull * w + 1ull;
    const int p = 63 - __clzll((long long)v);                                  // 0 .. 32
    const long long mb = (long long)((v << (52 - p)) & 0x000fffffffffffffull);  // mantissa bits of m
    const int j = (int)(mb >> 44);
    const double m = __longlong_as_double(mb | 0x3ff0000000000000ll);
    const double mj = __longlong_as_double((mb & 0x000ff00000000000ll) | 0x3ff0000000000000ll);
    const double t = (m - mj) * __ldg(&kF64Tabs.invm[j]);   // m - m_j is exact
    const double q = t * fma(t, fma(t, fma(t, fma(t, fma(t, -1.0 / 6.0, 0.2), -0.25), 1.0 / 3.0), -0.5), 1.0);
    return fma((double)(p - 33), 0.6931471805599453, __ldg(&kF64Tabs.lnm[j]) + q);
}

// sin(pi u), cos(pi u) for u = j/256 + x/pi, j the breakpoint and x in
// [0, pi/256): the table at j/256 and the series of x (<= 0.0123) to x^5
// (sin) and x^6 (cos), the next terms being below 1e-17 and 2e-20
__device__ __forceinline__ void sincospi_tab(int j, double x, double* s, double* c) {
    const double x2 = x * x;
    const double sd = x * fma(x2, fma(x2, 1.0 / 120.0, -1.0 / 6.0), 1.0);
    const double cd = fma(x2, fma(x2, fma(x2, -1.0 / 720.0, 1.0 / 24.0), -0.5), 1.0);
    const double S = __ldg(&kF64Tabs.sn[j]), C = __ldg(&kF64Tabs.cs[j]);
    *s = fma(S, cd, C * sd);
    *c = fma(C, cd, -S * sd);
}

// ... of the uniform u = (w + 1/2) 2^-32 from the word: j is its top 8 bits
// and x = pi (w mod 2^24 + 1/2) 2^-32, built as the double
// 1 + (w mod 2^24 + 1/2) 2^-24 less 1 (exact) times pi/256 -- the same x,
// bit for bit, as pi (u - j/256)
__device__ __forceinline__ void sincospi_word(uint32_t w, double* s, double* c) {
    const double r = __hiloint2double(0x3ff00000 | (int)((w & 0xffffffu) >> 4), (int)((w << 28) | 0x8000000u)) - 1.0;
    sincospi_tab((int)(w >> 24), r * (3.141592653589793 / 256.0), s, c);
}

// cos(2 pi u), sin(2 pi u) of the uniform u = (w + 1/2) 2^-32 from the word:
// 2u = k/256 + x/pi with k the top 9 bits of w; for k >= 256 (u >= 1/2)
// the angle is pi more, which flips both signs; j = k mod 256 indexes the
// table and x = pi (w mod 2^23 + 1/2) 2^-31, built from the low 23 bits as
// sincospi_word builds its remainder
__device__ __forceinline__ void cossin2pi_word(uint32_t w, double* c, double* s) {
    const double r = __hiloint2double(0x3ff00000 | (int)((w & 0x7fffffu) >> 3), (int)((w << 29) | 0x10000000u)) - 1.0;
    double sv, cv;
    sincospi_tab((int)((w >> 23) & 0xffu), r * (3.141592653589793 / 256.0), &sv, &cv);
    const int flip = (int)(w & 0x80000000u);   // the sign bit, flipped in the high words
    *s = __hiloint2double(__double2hiint(sv) ^ flip, __double2loint(sv));
    *c = __hiloint2double(__double2hiint(cv) ^ flip, __double2loint(cv));
}

// 1/d for a positive normal d: the hardware approximation
// (rcp.approx.ftz.f64) refined by two steps of the third-order
// Newton-Raphson iteration r <- r (1 + e + e^2), e = 1 - d r, which cubes
// the relative error each step (from any start better than 2^-8 to below
// 2^-72), so the result is within the rounding of its last operations, two
// ulp; four FMAs instead of the correctly rounded division's sequence.
__device__ __forceinline__ double rcp_pos(double d) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
    double e = fma(-d, r, 1.0);
    r = fma(r, fma(e, e, e), r);
    e = fma(-d, r, 1.0);
    return fma(r, fma(e, e, e), r);
}

// |x| by clearing the sign bit (an integer operation, not an FP64 one)
__device__ __forceinline__ double abs_bits(double x) {
    return __hiloint2double(__double2hiint(x) & 0x7fffffff, __double2loint(x));
}

// ... of a uniform u in [0, 1) given as a double (the adjoint's stored
// azimuth uniforms): u = j/256 + d with d exact, x = pi d
__device__ __forceinline__ void sincospi_uniform(double u, double* s, double* c) {
    int j = (int)(u * 256.0);
    j = j < 0 ? 0 : (j > 255 ? 255 : j);
    sincospi_tab(j, fma((double)-j, 1.0 / 256.0, u) * 3.141592653589793, s, c);
}

template <>
struct Ops<double> {
    // (u + 1/2) 2^-32, built as the double 1 + (u + 1/2) 2^-32 (u in the top
    // 32 mantissa bits, the half below them) less 1: exact, one FP64
    // subtraction instead of a conversion, an addition and a product
    static __device__ __forceinline__ double unit(uint32_t u) {
        return __hiloint2double(0x3ff00000 | (int)(u >> 12), (int)((u << 20) | 0x80000u)) - 1.0;
    }
    static __device__ __forceinline__ double unit_c(uint32_t u) { return unit(~u); }
    static __device__ __forceinline__ double ln(double x) { return log(x); }
    // the step's uniform and the azimuth's, from their Philox words: table
    // driven (ln_word, sincospi_word above); CUDA's log and sincospi took
    // 12% and 10% of the small FP64 configuration's time
    static __device__ __forceinline__ double ln_step_word(uint32_t w) { return ln_word(w); }
    static __device__ __forceinline__ void sincos_pi_word(uint32_t w, double* s, double* c) {
        sincospi_word(w, s, c);
    }
    static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
    static __device__ __forceinline__ double rsqrt_(double x) { return rsqrt(x); }
    // 1/sqrt(x) for the squared norm x = 1 + e of a rotated unit vector: the
    // rotation keeps |e| at rounding level (about 1e-15), where one Newton
    // step from 1, 1.5 - 0.5 x = 1 - e/2, is within 3 e^2 / 8 (below 1e-30)
    // of it (CUDA's rsqrt took 5% of the small FP64 configuration's time)
    static __device__ __forceinline__ double renorm(double x) { return fma(x, -0.5, 1.5); }
    static __device__ __forceinline__ double div(double a, double b) { return a / b; }
    static __device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ void sincos_pi(double u, double* s, double* c) { sincospi_uniform(u, s, c); }
    static __device__ __forceinline__ double nan_() { return __longlong_as_double(0x7ff8000000000000ll); }
    static __device__ __forceinline__ double acos_deg(double x) { return acos(x) * 57.29577951308232; }
};

// ---------------------------------------------------------------------------
// cross sections in 1/A (see mcd_consts.h for the algebra)
// ---------------------------------------------------------------------------
template <class T, class C>
__device__ __forceinline__ T sig_ruth(const C& c, T E) {
    T f = c.cRs;
    if (c.bits & kBitR2) {
        const T r = Ops<T>::div(E + (T)511000, E + (T)1024000);
        f = c.cRs * r * r;
    }
    return Ops<T>::div(f, E + c.aS);
}

template <class T, class C>
__device__ __forceinline__ T sig_moller(const C& c, T E, T invE) {
    const T Wc = c.Wc;
    if (!(E > Wc)) return (T)0;
    const T EmW = E - Wc;
    return c.pM * invE * invE * (Ops<T>::div(E, Wc) - Ops<T>::div(E, EmW) + Ops<T>::ln(Ops<T>::div(Wc, EmW)));
}

// Branch-free: below the binding energy d = 0 makes the value 0 (x = 0), so
// lanes above and below a threshold run the same instructions.
template <class T, class C>
__device__ __forceinline__ T sig_gryz(const C& c, T E, T invE, int k) {
    const T Es = c.gEs[k];
    const T d = E > Es ? E - Es : (T)0;
    const T x = Ops<T>::div(d, E + Es);
    const T br = (T)1 + (T)(2.0 / 3.0) * ((T)1 - (T)0.5 * Es * invE) *
                            Ops<T>::ln((T)2.7 + Ops<T>::sqrt_(d * c.gInvEs[k]));
    return c.gP[k] * x * Ops<T>::sqrt_(x) * br * invE;
}

template <class T, class C>
__device__ __forceinline__ T sig_quinn(const C& c, T E, T invE) {
    if (!(E > c.Epl)) return (T)0;
    const T a = E * c.qInvEf;
    const T sa = Ops<T>::sqrt_(a), sb = Ops<T>::sqrt_(a - c.qB);
    return c.qK * invE * Ops<T>::ln(Ops<T>::div(c.qC1 * (sa + sb), c.qB));
}

template <class T, class C>
__device__ __forceinline__ T stopping(const C& c, T E) {
    if (c.bethe == MCD_BETHE_CLASSICAL)
        return Ops<T>::div(c.bP, E) * Ops<T>::ln((T)1.166 * E * c.bInvJ);
    if (c.bethe == MCD_BETHE_JL)
        return Ops<T>::div(c.bP, E) * Ops<T>::ln((T)1.166 * (E + c.bkJ) * c.bInvJ);
    return Ops<T>::div(c.bX, E) * (c.bW * Ops<T>::ln(E) - c.bC);
}

// ---------------------------------------------------------------------------
// table sampling (MC/tools/scattering.py:63-94): the first E row >= E, then
// the first CDF entry >= U in that row (masked entries, stored as 0, act as
// +inf); the loss is the lower W grid point Ws[j].
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ int table_row(const TableDev& t, T E, bool* out_of_range) {
    const int nE = t.nE;
    const bool known = t.E_last > 0.0f;
    const float e0 = known ? t.E_first : __ldg(t.Es), eL = known ? t.E_last : __ldg(t.Es + nE - 1);
    if (E > (T)eL) {
        *out_of_range = true;
        return nE - 1;
    }
    if (!(E > (T)e0)) return 0;
    // linear-grid guess, then an exact correction against the stored values
    // (computed in T: a guess only, the search below corrects it exactly)
    int g = (int)ceil((E - (T)e0) * (t.inv_dE > 0.0f ? (T)t.inv_dE : (T)(nE - 1) / (T)(eL - e0)));
    g = g < 1 ? 1 : (g > nE - 1 ? nE - 1 : g);
    int lo = 0, hi = nE - 1;  // invariant: Es[lo] < E <= Es[hi]
    {
        // both neighbours of the guess in one round trip
        const T a = (T)__ldg(t.Es + g - 1), b = (T)__ldg(t.Es + g);
        if (a < E && E <= b) return g;
        if (b < E) lo = g; else hi = g - 1;
    }
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((T)__ldg(t.Es + mid) >= E) hi = mid; else lo = mid;
    }
    return hi;
}

template <class T>
__device__ __forceinline__ T table_pick(const TableDev& t, T E, T U, bool* oor) {
    const int ncol = t.nW - 1;
    const int kq = (int)(U * (T)MCD_GUIDE);
    int i = -1, lo = 0, hi = 0;
    if (t.guide && t.E_last > 0.0f && E > (T)t.E_first && !(E > (T)t.E_last)) {
        // the row guess (from the table's inverse grid step, no division),
        // its bracketing energies and its guide entries in one round trip,
        // kept when the guess is the row (as it usually is: the E grid is a
        // float32 linspace); otherwise the search below
        const int nE = t.nE;
        int g;
        if constexpr (sizeof(T) == 4) g = __float2int_ru((E - t.E_first) * t.inv_dE);
        else g = (int)ceil((E - (T)t.E_first) * (T)t.inv_dE);
        g = g < 1 ? 1 : (g > nE - 1 ? nE - 1 : g);
        const uint16_t* gp = t.guide + (size_t)g * (MCD_GUIDE + 1) + kq;
        const T a = (T)__ldg(t.Es + g - 1), b = (T)__ldg(t.Es + g);
        const int glo = __ldg(gp), ghi = __ldg(gp + 1);
        if (a < E && E <= b) {
            i = g;
            lo = glo;
            hi = ghi;
        }
    }
    if (i < 0) {
        i = table_row(t, E, oor);
        if (t.guide) {
            const uint16_t* gp = t.guide + (size_t)i * (MCD_GUIDE + 1) + kq;
            lo = __ldg(gp);
            hi = __ldg(gp + 1);
        } else {
            lo = 0;
            hi = ncol;   // masked entries (0) act as +inf
        }
    }
    const float* row = t.cdf + (size_t)i * ncol;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const float v = __ldg(row + mid);
        if (v != 0.0f && (T)v < U) lo = mid + 1; else hi = mid;
    }
    return (T)__ldg(t.Ws + lo);
}

// ---------------------------------------------------------------------------
// electron state
// ---------------------------------------------------------------------------
enum : uint32_t { F_DOUBLE_ROW = 1u, F_NAN = 2u, F_TABLE_RANGE = 4u, F_CLAMPED = 8u, F_LONG_PATH = 16u,
                  F_DIFFRACTING = 32u };

template <class T>
struct Lane {
    T E, x, y, z, dx, dy, dz, yx, yy, yz;
    T E_row;   // energy of the first outcome row
    T max_z;
    uint32_t step;   // events so far (Philox counter word 0)
    uint32_t outcome;
    uint32_t flags;
    uint32_t nan_n, clamp_n, lpath_n;
};

template <class T, class C>
__device__ __forceinline__ void lane_init(Lane<T>& L, const C& c) {
    L.E = c.E0;
    L.x = L.y = L.z = (T)0;
    L.dx = c.d0x;
    L.dy = c.d0y;
    L.dz = c.d0z;
    L.yx = (T)0;
    L.yy = (T)1;
    L.yz = (T)0;
    L.E_row = c.E0;
    L.max_z = (T)0;
    L.step = 0;
    L.outcome = MCD_OUT_NONE;
    L.flags = 0;
    L.nan_n = L.clamp_n = L.lpath_n = 0;
}

// One event's record, filled when a ring is attached.
template <class T>
struct EventOut {
    T E, W, pathl, c2, half_phi, x, y, z;
    int ch;
    T s2, u_ang, u_phi;   // sin^2(theta/2) and the uniforms of the angles (adjoint)
};

// Position update and the exit tests (MC/tools/electron.py:64-84): leaving
// through the bottom face on a diffraction event's step is 'trdf'.
template <class T, class C>
__device__ __forceinline__ void lane_move(Lane<T>& L, const C& c, T s) {
    const T nz = L.z + s * L.dz;
    if (nz <= (T)0) {
        L.outcome = MCD_OUT_BKS;
        L.E_row = L.E;
    } else if ((c.bits & kBitFilm) && nz >= c.thickness) {
        L.outcome = (L.flags & F_DIFFRACTING) ? MCD_OUT_TRDF : MCD_OUT_TRSM;
        L.E_row = L.E;
    } else {
        L.x += s * L.dx;
        L.y += s * L.dy;
        L.z = nz;
        L.max_z = nz > L.max_z ? nz : L.max_z;
    }
}

// Energy update (MC/tools/electron.py:44-59): the 'abs' row keeps the
// pre-loss energy; after a 'bks' in the same step it is a second row.
template <class T, class C>
__device__ __forceinline__ void lane_lose(Lane<T>& L, const C& c, T W) {
    const T e = L.E - W;
    if (e <= c.Emin) {
        if (L.outcome == MCD_OUT_NONE) {
            L.outcome = MCD_OUT_ABS;
            L.E_row = L.E;
        } else if (L.outcome == MCD_OUT_BKS) {
            L.flags |= F_DOUBLE_ROW;
        }
    }
    L.E = e;
}

// Direction update (MC/tools/electron.py:87-99, MC/tools/rotation.py:41-53):
// q = q_az * q_pol with q_pol = (cos t/2, y sin t/2), q_az = (cos h, d sin h),
// applied to d and y, each renormalised.  s2 = sin^2(theta/2).  With y
// perpendicular to d (true initially and kept by every update), q_pol turns
// d about y by theta and q_az then turns both vectors about the old d by
// phi = 2h; in the frame (d, y, x = y cross d) that is
//     d' = d cos(theta) + sin(theta) (x cos(phi) + y sin(phi)),
//     y' = y cos(phi) - x sin(phi),
// the rotation q p q* written out (equal to it within rounding).
// cos(phi), sin(phi) of the event's azimuth from its Philox word: phi =
// 2 halfPhi, halfPhi = pi U (MC/tools/scattering.py:676); with the
// reference's fold cos(halfPhi) = +sqrt(1 - sin^2) (sin(halfPhi) >= 0)
// sin(phi) = 2 sin(halfPhi) |cos(halfPhi)| = |sin(2 pi U)|.  FP32 takes the
// double angle of sin/cos(pi U); FP64 reads cos/sin(2 pi U) from the table
// directly, four FP64 instructions fewer.
template <class T, class C>
__device__ __forceinline__ void azimuth(const C& c, uint32_t w_phi, T* cph, T* sph) {
    if constexpr (sizeof(T) == 8) {
        cossin2pi_word(w_phi, cph, sph);
        if (c.bits & MCD_Q_HALF_PHI_FOLD) *sph = abs_bits(*sph);
    } else {
        T sp, cp;
        Ops<T>::sincos_pi_word(w_phi, &sp, &cp);
        if (c.bits & MCD_Q_HALF_PHI_FOLD) cp = fabs(cp);
        *cph = (T)1 - (T)2 * sp * sp;
        *sph = (T)2 * sp * cp;
    }
}

template <class T>
__device__ __forceinline__ void lane_rotate_cs(Lane<T>& L, T s2, T cph, T sph) {
    // sin(theta) = 2 sin(theta/2) cos(theta/2); FP64 takes it as
    // 2 sqrt(s2 (1 - s2)), one FP64 square root instead of two, while
    // FP32 keeps the two roots (one root measured no faster there)
    T sth;
    if constexpr (sizeof(T) == 8) sth = (T)2 * Ops<T>::sqrt_(s2 * ((T)1 - s2));
    else sth = (T)2 * Ops<T>::sqrt_(s2) * Ops<T>::sqrt_((T)1 - s2);
    const T cth = (T)1 - (T)2 * s2;
    const T xx = L.yy * L.dz - L.yz * L.dy;
    const T xy = L.yz * L.dx - L.yx * L.dz;
    const T xz = L.yx * L.dy - L.yy * L.dx;
    const T a = sth * cph, b = sth * sph;
    T nd[3], ny[3];
    nd[0] = L.dx * cth + xx * a + L.yx * b;
    nd[1] = L.dy * cth + xy * a + L.yy * b;
    nd[2] = L.dz * cth + xz * a + L.yz * b;
    ny[0] = L.yx * cph - xx * sph;
    ny[1] = L.yy * cph - xy * sph;
    ny[2] = L.yz * cph - xz * sph;
    const T rd = Ops<T>::renorm(nd[0] * nd[0] + nd[1] * nd[1] + nd[2] * nd[2]);
    const T ry = Ops<T>::renorm(ny[0] * ny[0] + ny[1] * ny[1] + ny[2] * ny[2]);
    L.dx = nd[0] * rd;
    L.dy = nd[1] * rd;
    L.dz = nd[2] * rd;
    L.yx = ny[0] * ry;
    L.yy = ny[1] * ry;
    L.yz = ny[2] * ry;
}

template <class T, class C>
__device__ __forceinline__ void lane_rotate(Lane<T>& L, const C& c, T s2, uint32_t w_phi) {
    T cph, sph;
    azimuth<T>(c, w_phi, &cph, &sph);
    lane_rotate_cs(L, s2, cph, sph);
}

// ---------------------------------------------------------------------------
// DS event (MC/tools/scattering.py:440-679 in the order of
// MC/tools/singleScatter.py:15-41).  Returns the channel code.
// ---------------------------------------------------------------------------
// Channel and E times the total inverse mean free path from the tabulated
// cumulative cross sections: linear interpolation in log2(E) between two rows
// of E * (running sum); the comparison with U * E * total needs no division.
template <class C>
__device__ __forceinline__ int tab_pick(const C& c, float E, float U, float* Etot_out) {
    float t = fmaf(__log2f(E), c.sig_inv, c.sig_off);
    t = fminf(fmaxf(t, 0.0f), c.sig_tmax);
    const int i = (int)t;
    const float f = t - (float)i;
    const int S = bits_S(c);
    const float* r0 = static_cast<const float*>(c.sig) + i * S;
    const float* r1 = r0 + S;
    const int K = bits_K(c);
    // column 0 holds the total, columns 1.. the running sums before it
    const float4 x0 = __ldg(reinterpret_cast<const float4*>(r0));
    const float4 y0 = __ldg(reinterpret_cast<const float4*>(r1));
    const float tot = fmaf(f, y0.x - x0.x, x0.x);
    float all = tot;
    if (c.bits & kBitDiff) all = fmaf(E, c.dS, tot);   // + diffraction
    *Etot_out = all;
    const float target = U * all;
    if ((c.bits & kBitDiff) && target > tot) return MCD_CH_DIFF;
    // the running sums increase along the row (padding holds FLT_MAX), so
    // the channel is the number of them below the target
    int j = (fmaf(f, y0.y - x0.y, x0.y) < target) + (fmaf(f, y0.z - x0.z, x0.z) < target) +
            (fmaf(f, y0.w - x0.w, x0.w) < target);
#pragma unroll
    for (int q = 1; q < kSigStride / 4; ++q) {
        if (4 * q < S) {
            const float4 x = __ldg(reinterpret_cast<const float4*>(r0) + q);
            const float4 y = __ldg(reinterpret_cast<const float4*>(r1) + q);
            j += (fmaf(f, y.x - x.x, x.x) < target) + (fmaf(f, y.y - x.y, x.y) < target) +
                 (fmaf(f, y.z - x.z, x.z) < target) + (fmaf(f, y.w - x.w, x.w) < target);
        }
    }
    j = j < K - 1 ? j : K - 1;
    // column -> channel code: 0 Ruth, 1 Moller, 2..K-2 Gryz[k], K-1 Quinn
    if (j == 0) return MCD_CH_RUTH;
    if (j == 1) return MCD_CH_MOLLER;
    if (j == K - 1) return MCD_CH_QUINN;
    return MCD_CH_GRYZ0 + (j - 2);
}

// The channel and the mean free path from an FP64 table (FP64 transport;
// layout at kSig64Cells): the octave from the exponent bits of E, the cell
// from the top mantissa bits and its offset f from the other 44 (exact, by
// integer operations and one subtraction), then each column read is three
// FMAs.  A small FP64 run is a chain of dependent instructions in which the
// FP64 ones take longest, so the lookup is built to issue few of them: no
// logarithm, no interpolation weights, no division.  With
// diffraction (a constant cross section dS) the total grows by the factor
// g = 1 + dS lambda; the event diffracts when U g > 1, otherwise U g is
// compared with the fractions of the other channels.  Returns -1 for a cell
// whose nodes straddle a channel threshold (its flag is set): the caller
// evaluates the cross sections.
template <class C>
__device__ __forceinline__ int tab_pick64(const C& c, double E, double U, double* mfp_out) {
    const long long b = __double_as_longlong(E);   // E > 0
    int blk = (int)(b >> 52) - 1023 - (int)c.sig_l0;
    blk = blk < 0 ? 0 : (blk > c.sig_rows - 1 ? c.sig_rows - 1 : blk);
    const int i = (int)(b >> 44) & (kSig64Cells - 1);
    const double f = __longlong_as_double(((b << 8) & 0x000fffffffffff00ll) | 0x3ff0000000000000ll) - 1.0;
    const int K = bits_K(c);
    const double* r = static_cast<const double*>(c.sig) + ((size_t)blk * kSig64Cells + i) * sig64_stride(K);
    if (__ldg(reinterpret_cast<const long long*>(r)) != 0ll) return -1;
    auto at = [&](int col) {
        const double2 lo = __ldg(reinterpret_cast<const double2*>(r + 2 + 4 * col));
        const double2 hi = __ldg(reinterpret_cast<const double2*>(r + 4 + 4 * col));
        return fma(fma(fma(hi.y, f, hi.x), f, lo.y), f, lo.x);
    };
    double mfp = at(0);
    double u = U;
    if (c.bits & kBitDiff) {
        const double g = fma((double)c.dS, mfp, 1.0);
        u = U * g;
        mfp = mfp / g;
        if (u > 1.0) {
            *mfp_out = mfp;
            return MCD_CH_DIFF;
        }
    }
    *mfp_out = mfp;
    // the first running-sum fraction at or above u names the channel (most
    // events stop at the Rutherford column)
    int j = 0;
    while (j < K - 1 && at(j + 1) < u) ++j;
    if (j == 0) return MCD_CH_RUTH;
    if (j == 1) return MCD_CH_MOLLER;
    if (j == K - 1) return MCD_CH_QUINN;
    return MCD_CH_GRYZ0 + (j - 2);
}

// The trajectory-independent functions of an event's Philox words, when
// another lane has computed them ahead: ln U of the step's uniform, the
// azimuth's cos and sin (with the half-phi fold applied), the channel
// pick's uniform, and the Rutherford angle's a0 U and 1 - U.
template <class T>
struct EventPre {
    T ln_y, cph, sph, ux, a0u, uzc;
};

// Rutherford sin^2(theta/2) = a U / (a + 1 - U), a = a0 / E
// (MC/tools/scattering.py:125-152); for the DS event in FP32 with one
// division as a0 U / (a0 + E (1 - U)).
template <class T, class C>
__device__ __forceinline__ T ruth_s2(const C& c, T E, uint32_t u) {
    if constexpr (sizeof(T) == 4) {
        return Ops<T>::div(c.a0 * Ops<T>::unit(u), fmaf(E, Ops<T>::unit_c(u), c.a0));
    } else {
        return c.a0 * Ops<T>::unit(u) * rcp_pos(fma(E, Ops<T>::unit_c(u), c.a0));
    }
}

__device__ __forceinline__ uint4 event_counter(uint32_t step, uint64_t elec, uint32_t sim_id) {
    return make_uint4(step, (uint32_t)elec, (uint32_t)(elec >> 32), sim_id);
}

// One DS event from its four random words r (the step counter already
// advanced).  Returns the channel code.
template <class T, bool REC, class C>
__device__ __forceinline__ int ds_event_r(Lane<T>& L, const C& c, const uint4 r, EventOut<T>* ev,
                                          bool use_tab = false, const EventPre<T>* pre = nullptr) {
    const T E = L.E;
    int ch = MCD_CH_QUINN;
    T inv_tot;
    // FP64: the azimuth's cos/sin depend on the word alone; computed first,
    // their FP64 chain overlaps the channel pick's instead of closing the
    // event (or given, computed ahead by another lane)
    T cph = (T)0, sph = (T)0;
    if constexpr (sizeof(T) == 8) {
        if (pre) cph = pre->cph, sph = pre->sph;
        else azimuth<T>(c, r.w, &cph, &sph);
    }
    if (use_tab) {
        if constexpr (sizeof(T) == 4) {
            float Etot;
            ch = tab_pick(c, (float)E, (float)Ops<T>::unit(r.x), &Etot);
            inv_tot = Ops<T>::div(E, (T)Etot);
        } else {
            double mfp;
            ch = tab_pick64(c, E, pre ? pre->ux : Ops<T>::unit(r.x), &mfp);
            if (ch >= 0) inv_tot = mfp;
            else use_tab = false, ch = MCD_CH_QUINN;   // a threshold inside the cell
        }
    }
    if (!use_tab) {
        // --- cross sections, channel order Ruth, Moller, Gryz[k], Quinn
        const T invE = Ops<T>::div((T)1, E);
        const T sR = sig_ruth<T>(c, E);
        const T sM = sig_moller<T>(c, E, invE);
        T sG[MCD_MAX_SHELLS];
        T tot = sR + sM;
#pragma unroll
        for (int k = 0; k < MCD_MAX_SHELLS; ++k) {
            sG[k] = (k < c.nsh) ? sig_gryz<T>(c, E, invE, k) : (T)0;
            tot += sG[k];
        }
        const T sQ = sig_quinn<T>(c, E, invE);
        tot += sQ;
        const T cumQ = tot;
        if (c.bits & kBitDiff) tot += c.dS;
        // --- channel (MC/tools/scattering.py:39-59)
        const T target = (pre ? pre->ux : Ops<T>::unit(r.x)) * tot;
        T cum = sR;
        if (target <= cum) {
            ch = MCD_CH_RUTH;
        } else {
            cum += sM;
            if (target <= cum) {
                ch = MCD_CH_MOLLER;
            } else {
#pragma unroll
                for (int k = 0; k < MCD_MAX_SHELLS; ++k) {
                    cum += sG[k];
                    if (ch == MCD_CH_QUINN && k < c.nsh && target <= cum) ch = MCD_CH_GRYZ0 + k;
                }
                if ((c.bits & kBitDiff) && ch == MCD_CH_QUINN && target > cumQ) ch = MCD_CH_DIFF;
            }
        }
        inv_tot = Ops<T>::div((T)1, tot);
    }
    // --- path length (MC/tools/scattering.py:540-565): a diffraction event
    // steps with mean free path xip_g and marks the electron diffracting
    const bool diff_ev = ch == MCD_CH_DIFF;
    L.flags = diff_ev ? (L.flags | F_DIFFRACTING) : (L.flags & ~F_DIFFRACTING);
    const T s = -(pre ? pre->ln_y : Ops<T>::ln_step_word(r.y)) * (diff_ev ? c.xip : inv_tot);
    const T x0 = L.x, y0 = L.y, z0 = L.z;
    lane_move(L, c, s);
    // --- energy loss and polar angle (MC/tools/scattering.py:568-679)
    T W, s2;
    if (ch == MCD_CH_RUTH) {
        W = (T)0;
        if constexpr (sizeof(T) == 8) {
            s2 = pre ? pre->a0u * rcp_pos(fma(E, pre->uzc, c.a0)) : ruth_s2<T>(c, E, r.z);
        } else {
            s2 = ruth_s2<T>(c, E, r.z);
        }
    } else if (ch == MCD_CH_QUINN) {
        W = c.Epl;
        s2 = (T)0;
    } else if (diff_ev) {
        // no loss, no deflection (MC/tools/scattering.py:658-668)
        W = (T)0;
        s2 = (T)0;
    } else {
        bool oor = false;
        W = table_pick<T>(c.tab[ch != MCD_CH_MOLLER], E, Ops<T>::unit(r.z), &oor);
        if (oor) L.flags |= F_TABLE_RANGE;
        // binary collision (MC/tools/scattering.py:156-179)
        if (W <= (E - c.Ef) * (T)0.5) {
            const T q = Ops<T>::div(W, E);
            s2 = (T)0.5 * Ops<T>::div(q, (T)1 + Ops<T>::sqrt_((T)1 - q));
        } else {
            L.flags |= F_NAN;
            L.nan_n += 1;
            s2 = (c.bits & MCD_Q_NAN_DIRECTION) ? Ops<T>::nan_() : (T)0;
        }
    }
    const T uphi = Ops<T>::unit(r.w);
    if (REC) {
        ev->E = E;
        ev->W = W;
        ev->pathl = s;
        ev->c2 = (T)1 - s2;
        ev->half_phi = (T)3.141592653589793 * uphi;
        ev->x = x0;
        ev->y = y0;
        ev->z = z0;
        ev->ch = ch;
    }
    const bool left = L.outcome != MCD_OUT_NONE;
    // a zero loss (Rutherford, diffraction) leaves E, and with it E > Emin,
    // as it is: FP64 skips the update, an FP64 subtraction and comparison
    const bool zero_loss = sizeof(T) == 8 && (ch == MCD_CH_RUTH || diff_ev);
    if (!zero_loss && (!left || (c.bits & MCD_Q_CROSSING_STEP))) lane_lose(L, c, W);
    if (L.outcome == MCD_OUT_NONE) {
        if constexpr (sizeof(T) == 8) lane_rotate_cs(L, s2, cph, sph);
        else lane_rotate(L, c, s2, r.w);
    }
    return ch;
}

// sim_id, key0, key1, max_scatt in one load: the 'long' check that opens
// every event (MC/tools/singleScatter.py:19-23) and its Philox block
template <class C>
__device__ __forceinline__ uint4 event_words(const C& c) {
    return *reinterpret_cast<const uint4*>(&c.sim_id);
}

template <class T, bool REC, class C>
__device__ __forceinline__ int ds_event(Lane<T>& L, const C& c, uint64_t elec, EventOut<T>* ev,
                                        bool use_tab = false) {
    const uint4 w = event_words(c);
    if (L.step >= w.w) {
        L.outcome = MCD_OUT_LONG;
        L.E_row = L.E;
        return -1;
    }
    const uint4 r = philox(event_counter(L.step, elec, w.x), w.y, w.z);
    L.step += 1;
    return ds_event_r<T, REC>(L, c, r, ev, use_tab);
}

// ---------------------------------------------------------------------------
// continuous event (MC/tools/scattering.py:753-883 in the order of
// MC/tools/singleScatter.py:210-239, with the Bethe law the mode names)
// ---------------------------------------------------------------------------
template <class T, bool REC, class C>
__device__ __forceinline__ int cont_event_r(Lane<T>& L, const C& c, const uint4 r, EventOut<T>* ev) {
    const T E = L.E;
    const T sR = sig_ruth<T>(c, E);
    const T s = -Ops<T>::ln_step_word(r.y) * Ops<T>::div((T)1, sR);
    if (!(s < (T)1e4)) {
        L.flags |= F_LONG_PATH;
        L.lpath_n += 1;
    }
    const T x0 = L.x, y0 = L.y, z0 = L.z;
    lane_move(L, c, s);
    // a product that is never fused into the energy update, so that the
    // adjoint's recomputation reproduces these energies bit for bit
    T dE = Ops<T>::mul_rn(s, stopping<T>(c, E));
    if (!(dE < E)) {
        L.flags |= F_CLAMPED;
        L.clamp_n += 1;
        dE = E;
    }
    // the two-division form: in this event the single-division one of
    // ruth_s2 measured 1% slower
    const T a = Ops<T>::div(c.a0, E);
    const T s2 = Ops<T>::div(a * Ops<T>::unit(r.z), a + Ops<T>::unit_c(r.z));
    const T uphi = Ops<T>::unit(r.w);
    if (REC) {
        ev->s2 = s2;
        ev->u_ang = Ops<T>::unit(r.z);
        ev->u_phi = uphi;
        ev->E = E;
        ev->W = dE;
        ev->pathl = s;
        ev->c2 = (T)1 - s2;
        ev->half_phi = (T)3.141592653589793 * uphi;
        ev->x = x0;
        ev->y = y0;
        ev->z = z0;
        ev->ch = MCD_CH_RUTH;
    }
    const bool left = L.outcome != MCD_OUT_NONE;
    if (!left || (c.bits & MCD_Q_CROSSING_STEP)) lane_lose(L, c, dE);
    if (L.outcome == MCD_OUT_NONE) lane_rotate(L, c, s2, r.w);
    return MCD_CH_RUTH;
}

template <class T, bool REC, class C>
__device__ __forceinline__ int cont_event(Lane<T>& L, const C& c, uint64_t elec, EventOut<T>* ev) {
    const uint4 w = event_words(c);
    if (L.step >= w.w) {
        L.outcome = MCD_OUT_LONG;
        L.E_row = L.E;
        return -1;
    }
    const uint4 r = philox(event_counter(L.step, elec, w.x), w.y, w.z);
    L.step += 1;
    return cont_event_r<T, REC>(L, c, r, ev);
}

// ---------------------------------------------------------------------------
// warp-aggregated append of one record per calling lane to the event ring
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ uint32_t ring_append(const mcd_event_ring& ring, uint32_t electron, uint32_t step,
                                                const EventOut<T>& ev) {
    const bool packed = (ring.fields & MCD_EV_PACKED_HEAD) != 0;
    if (packed && electron >= (1u << 28)) return MCD_FLAG_RING_INDEX;   // reserves no slot
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    const unsigned rank = __popc(mask & ((1u << lane) - 1u));
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(ring.cursor, (unsigned long long)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    const unsigned long long slot = base + rank;
    if (slot >= ring.capacity) return 0;
    const uint32_t f = ring.fields & MCD_EV_ALL;
    if (!packed && (f == 0 || f == MCD_EV_ALL)) {
        mcd_event e;
        e.electron = electron;
        e.step_chan = ((step - 1) << 5) | (uint32_t)(ev.ch & 31);
        e.E = (float)ev.E;
        e.W = (float)ev.W;
        e.pathl = (float)ev.pathl;
        e.c2 = (float)ev.c2;
        e.half_phi = (float)ev.half_phi;
        e.x = (float)ev.x;
        e.y = (float)ev.y;
        e.z = (float)ev.z;
        static_cast<mcd_event*>(ring.rec)[slot] = e;
        return 0;
    }
    // the selected columns only, packed after the header
    const uint32_t cols = f ? f : MCD_EV_ALL;
    const int words = (packed ? 1 : 2) + __popc(cols & 0x1fu) + ((cols & MCD_EV_POS) ? 3 : 0);
    uint32_t* p = static_cast<uint32_t*>(ring.rec) + slot * (unsigned long long)words;
    int o;
    if (packed) {
        p[0] = (electron << 4) | (uint32_t)(ev.ch & 15);
        o = 1;
    } else {
        p[0] = electron;
        p[1] = ((step - 1) << 5) | (uint32_t)(ev.ch & 31);
        o = 2;
    }
    if (cols & MCD_EV_E) p[o++] = __float_as_uint((float)ev.E);
    if (cols & MCD_EV_W) p[o++] = __float_as_uint((float)ev.W);
    if (cols & MCD_EV_PATHL) p[o++] = __float_as_uint((float)ev.pathl);
    if (cols & MCD_EV_C2) p[o++] = __float_as_uint((float)ev.c2);
    if (cols & MCD_EV_PHI) p[o++] = __float_as_uint((float)ev.half_phi);
    if (cols & MCD_EV_POS) {
        p[o++] = __float_as_uint((float)ev.x);
        p[o++] = __float_as_uint((float)ev.y);
        p[o] = __float_as_uint((float)ev.z);
    }
    return 0;
}

}  // namespace mcd

#endif  // MCD_DEVICE_CUH
