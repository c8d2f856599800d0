/*
 * mcd_oracle.c - FP64 CPU oracle of the electron-trajectory Monte Carlo.
 *
 * TEST INFRASTRUCTURE ONLY: the parity reference and the CPU baseline.  It is built
 * by oracle/Makefile into oracle/_build/libmcd_oracle.so and loaded by the
 * tests and by bench.py's CPU leg; the library under mc-discrete_gb300/
 * never links or calls it.
 *
 * It is the C twin of oracle/mcd_oracle.py in its Philox mode: the same
 * reference formulas written the same way (so the two agree bit for bit),
 * run over a range of electrons with one pthread per slice.  Reference
 * functions restated (paths relative to elena-pascal/MC-discrete):
 *   crossSections.py:14-58,183-284    total cross sections
 *   stoppingPowers.py:112-215         Bethe laws
 *   scattering.py:19-36,39-59,63-94,125-179,440-679,753-883
 *   singleScatter.py:10-41,205-239    event order
 *   electron.py:44-113, rotation.py:41-53
 * The channel list is walked in the fixed order Ruth, Moller, Gryz[k],
 * Quinn (the reference re-sorts by sigma each event, which changes which
 * uniform picks which channel but not the distribution).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MCO_MAX_SHELLS 8
#define PI_EFOUR 6.51408491409531e-14
#define BOHR_R 5.29177210544e-11
#define PI_D 3.141592653589793

typedef struct {
    double Z, n_val, E_val, atnd, plasmon_e, fermi_e, J, bethe_k;
    int n_shells;
    double shell_E[MCO_MAX_SHELLS], shell_n[MCO_MAX_SHELLS];
    double xip_g;      /* extinction distance of the diffraction channel (0: none) */
} mco_mat;

typedef struct {
    const float* Es;
    const float* Ws;
    const float* cdf;
    int nE, nW;
} mco_table;

typedef struct {
    int mode;          /* 0 DS, 1 continuous                           */
    int bethe;         /* 0 classical, 1 JL, 2 explicit                */
    double E0, Emin, tilt, Wc, thickness;
    long long max_scatt;
    unsigned long long seed;
    unsigned sim_id;
    unsigned quirks;   /* bit0 crossing step, bit1 half-phi fold, bit2 NaN */
    double J_scale, n_scale;
    int elastic;       /* 0 Ruth_vanilla, 1 _vanilla_wDefl, 2 _nigram, 3 _nigram_wDefl */
    int diff;          /* diffMFP: the diffraction channel (DS)             */
} mco_sim;

typedef struct {
    unsigned char* outcome;
    unsigned char* flags;
    double* final_E;
    double* dir;       /* n x 3 */
    double* last_pos;  /* n x 3 */
    double* max_z;
    int* n_events;
    unsigned long long* channel; /* 16 counters, optional */
    unsigned long long* nan_events;
} mco_out;

enum { OUT_NONE = 0, OUT_BKS = 1, OUT_ABS = 2, OUT_TRSM = 3, OUT_TRDF = 4, OUT_LONG = 5 };
enum { CH_RUTH = 0, CH_MOLLER = 1, CH_QUINN = 2, CH_GRYZ0 = 3, CH_DIFF = 11 };

/* ---------------- Philox4x32-10 ---------------- */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    }
}

static double unit(uint32_t u) { return ((double)u + 0.5) * 0x1p-32; }

/* ---------------- cross sections (reference forms) ---------------- */
static double alpha_(double E, double Z) { return 3.4 * pow(Z, 0.666667) / E; }

static double ruther_sigma(double E, double Z) {
    double a = alpha_(E, Z);
    double Ek = E * 1e-3;
    double r = (Ek + 511.0) / (Ek + 1024.0);
    return 5.21e-21 * (Z * Z / (Ek * Ek)) * (r * r) * (4.0 * PI_D) / (a * (1.0 + a));
}

/* crossSections.py:63-86 */
static double ruther_sigma_wdefl(double E, double Z) {
    double a = alpha_(E, Z);
    double Ek = E * 1e-3;
    double r = (Ek + 511.0) / (Ek + 1024.0);
    return 5.21e-21 * (Z * (Z + 1.0) / (Ek * Ek)) * (r * r) * (4.0 * PI_D) / (a * (1.0 + a));
}

/* crossSections.py:90-147, Nigram screening 0.48 * 5.43 Z^(2/3) / E */
static double ruther_n_sigma(double E, double Z, int wdefl) {
    double b = 0.48 * (5.43 * pow(Z, 2.0 / 3.0) / E);
    double zz = wdefl ? (Z + 1.0) * Z : Z * Z;
    return PI_EFOUR * zz / (4.0 * b * (1.0 + b) * (E * E));
}

static double elastic_sigma(int model, double E, double Z) {
    switch (model) {
        case 1: return ruther_sigma_wdefl(E, Z);
        case 2: return ruther_n_sigma(E, Z, 0);
        case 3: return ruther_n_sigma(E, Z, 1);
        default: return ruther_sigma(E, Z);
    }
}

/* crossSections.py:329-349 */
static double diffr_sigma(double xip_g, double n) { return 1.0 / (n * xip_g) * 1e13; }

static double moller_sigma(double E, double Wc, double nfree) {
    if (E <= Wc) return 0.0;
    double eps = Wc * 1.0 / E;
    return nfree * PI_EFOUR * (1.0 / (E * E)) * (1.0 / eps - 1.0 / (1.0 - eps) + log(eps / (1.0 - eps)));
}

static double gryz_sigma(double E, double Esi, double nsi) {
    if (E <= Esi) return 0.0;
    double U = E * 1.0 / Esi;
    return nsi * PI_EFOUR * pow((U - 1.0) / (U + 1.0), 1.5) *
           (1.0 + (2.0 * (1.0 - (1.0 / (2.0 * U))) / 3.0 * log(2.7 + pow(U - 1.0, 0.5)))) / (E * Esi);
}

static double quinn_sigma(double E, double Epl, double Ef, double n) {
    if (E <= Epl) return 0.0;
    double E_Ef = E * 1.0 / Ef;
    double Epl_Ef = Epl * 1.0 / Ef;
    double tot = Epl * log((pow(1.0 + Epl_Ef, 0.5) - 1.0) / (pow(E_Ef, 0.5) - pow(E_Ef - Epl_Ef, 0.5))) /
                 (2.0 * BOHR_R * E);
    return tot / n * 1e4;
}

static double mfp_from_sigma(double s, double n) { return 1.0 / (n * s) * 1e14; }

static double stopping(const mco_sim* s, const mco_mat* m, double E, double n, double J) {
    double Z = m->Z;
    if (s->bethe == 0) return 2.0 * PI_EFOUR * n * (Z / E) * log(1.166 * E / J) * 1e-14;
    if (s->bethe == 1) return 2.0 * PI_EFOUR * n * (Z / E) * log(1.166 * (E + m->bethe_k * J) / J) * 1e-14;
    double pref = (2.0 * PI_EFOUR * n / E) * 1e-14;
    double sum = m->n_val * log(E * 1.0 / m->E_val);
    for (int k = 0; k < m->n_shells; ++k) sum = sum + m->shell_n[k] * log(E * 1.0 / m->shell_E[k]);
    return pref * sum;
}

/* ---------------- tables ---------------- */
static int bisect_left_f(const float* a, int n, double x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if ((double)a[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

static double table_pick(const mco_table* t, double E, double U) {
    int i = bisect_left_f(t->Es, t->nE, E);
    if (i >= t->nE) i = t->nE - 1;
    const float* row = t->cdf + (size_t)i * (t->nW - 1);
    int lo = 0, hi = t->nW - 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        float v = row[mid];
        if (v != 0.0f && (double)v < U) lo = mid + 1; else hi = mid;
    }
    return (double)t->Ws[lo];
}

/* ---------------- electron ---------------- */
typedef struct {
    double E, Emin, pos[3], dir[3], y[3];
    int outcome, first_outcome, rows;
    double row_E, row_dir[3], row_pos[3];
    double max_z;
    long long steps;
    unsigned nan_events;
    int diffracting;
} el_t;

static void save_row(el_t* e, int oc) {
    if (e->rows == 0) {
        e->first_outcome = oc;
        e->row_E = e->E;
        memcpy(e->row_dir, e->dir, sizeof e->dir);
        memcpy(e->row_pos, e->pos, sizeof e->pos);
    }
    e->rows++;
    e->outcome = oc;
}

static void update_xyz(el_t* e, double s, double maxz) {
    double p[3] = {e->pos[0] + s * e->dir[0], e->pos[1] + s * e->dir[1], e->pos[2] + s * e->dir[2]};
    if (p[2] <= 0.0) {
        save_row(e, OUT_BKS);
    } else if (p[2] >= maxz) {
        save_row(e, e->diffracting ? OUT_TRDF : OUT_TRSM);
    } else {
        memcpy(e->pos, p, sizeof p);
        if (p[2] > e->max_z) e->max_z = p[2];
    }
}

static void update_energy(el_t* e, double W) {
    double en = e->E - W;
    if (en <= e->Emin) save_row(e, OUT_ABS);
    e->E = en;
}

static void rotate(el_t* e, double c2, double half_phi, unsigned quirks) {
    double st = pow(1.0 - c2, 0.5), ct = pow(c2, 0.5);
    double sp = sin(half_phi);
    double cp = (quirks & 2u) ? pow(1.0 - sp * sp, 0.5) : cos(half_phi);
    const double* d = e->dir;
    const double* y = e->y;
    double a1 = cp, b1 = d[0] * sp, c1 = d[1] * sp, d1 = d[2] * sp;
    double a2 = ct, b2 = y[0] * st, c2_ = y[1] * st, d2 = y[2] * st;
    double w = a1 * a2 - b1 * b2 - c1 * c2_ - d1 * d2;
    double x = a1 * b2 + b1 * a2 + c1 * d2 - d1 * c2_;
    double yy = a1 * c2_ - b1 * d2 + c1 * a2 + d1 * b2;
    double z = a1 * d2 + b1 * c2_ - c1 * b2 + d1 * a2;
    double n = w * w + x * x + yy * yy + z * z;
    double m[3][3] = {
        {1.0 - 2.0 * (yy * yy + z * z) / n, 2.0 * (x * yy - z * w) / n, 2.0 * (x * z + yy * w) / n},
        {2.0 * (x * yy + z * w) / n, 1.0 - 2.0 * (x * x + z * z) / n, 2.0 * (yy * z - x * w) / n},
        {2.0 * (x * z - yy * w) / n, 2.0 * (yy * z + x * w) / n, 1.0 - 2.0 * (x * x + yy * yy) / n}};
    double out[2][3];
    const double* vs[2] = {d, y};
    for (int v = 0; v < 2; ++v) {
        double r[3];
        for (int i = 0; i < 3; ++i) r[i] = m[i][0] * vs[v][0] + m[i][1] * vs[v][1] + m[i][2] * vs[v][2];
        double nn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        for (int i = 0; i < 3; ++i) out[v][i] = r[i] / nn;
    }
    memcpy(e->dir, out[0], sizeof e->dir);
    memcpy(e->y, out[1], sizeof e->y);
}

typedef struct {
    const mco_sim* s;
    const mco_mat* m;
    const mco_table* tm;
    const mco_table* tg;
    unsigned long long first;
    long long begin, end;
    mco_out* out;
    unsigned long long channel[16];
    unsigned long long nan_events;
} job_t;

static void run_one(job_t* j, long long i) {
    const mco_sim* s = j->s;
    const mco_mat* m = j->m;
    const double n_at = m->atnd * (s->n_scale > 0 ? s->n_scale : 1.0);
    const double J = m->J * (s->J_scale > 0 ? s->J_scale : 1.0);
    const double maxz = s->thickness > 0 ? s->thickness : 1e30;
    const unsigned long long elec = j->first + (unsigned long long)i;
    const uint32_t k0 = (uint32_t)s->seed, k1 = (uint32_t)(s->seed >> 32);
    el_t e;
    memset(&e, 0, sizeof e);
    double t = s->tilt * PI_D / 180.0;
    e.E = s->E0;
    e.Emin = s->Emin;
    e.dir[0] = -sin(t);
    e.dir[1] = 0.0;
    e.dir[2] = cos(t);
    e.y[1] = 1.0;
    long long num = 0;
    while (e.outcome == OUT_NONE) {
        double Ei = e.E;
        if (num + 1 > s->max_scatt) {
            save_row(&e, OUT_LONG);
            break;
        }
        uint32_t c[4] = {(uint32_t)num, (uint32_t)elec, (uint32_t)(elec >> 32), s->sim_id};
        philox(c, k0, k1);
        num += 1;
        double W, c2, hphi, sl;
        int ch;
        if (s->mode == 0) {
            double sig[4 + MCO_MAX_SHELLS];
            int code[4 + MCO_MAX_SHELLS];
            int nch = 0;
            sig[nch] = elastic_sigma(s->elastic, Ei, m->Z); code[nch++] = CH_RUTH;
            sig[nch] = moller_sigma(Ei, s->Wc, m->n_val); code[nch++] = CH_MOLLER;
            for (int k = 0; k < m->n_shells; ++k) {
                sig[nch] = gryz_sigma(Ei, m->shell_E[k], m->shell_n[k]);
                code[nch++] = CH_GRYZ0 + k;
            }
            sig[nch] = quinn_sigma(Ei, m->plasmon_e, m->fermi_e, n_at); code[nch++] = CH_QUINN;
            if (s->diff) { sig[nch] = diffr_sigma(m->xip_g, n_at); code[nch++] = CH_DIFF; }
            double tot = 0.0;
            for (int k = 0; k < nch; ++k) tot += sig[k];
            double mfp = mfp_from_sigma(tot, n_at);
            double U = unit(c[0]);
            double cum = 0.0;
            ch = code[nch - 1];
            for (int k = 0; k < nch; ++k) {
                cum += sig[k];
                if (cum / tot >= U) { ch = code[k]; break; }
            }
            if (ch == CH_DIFF) mfp = m->xip_g;
            e.diffracting = ch == CH_DIFF;
            sl = -mfp * log(unit(c[1]));
            update_xyz(&e, sl, maxz);
            if (ch == CH_DIFF) {
                W = 0.0;
                c2 = 1.0;
            } else if (ch == CH_RUTH) {
                W = 0.0;
                double a = alpha_(Ei, m->Z), u = unit(c[2]);
                c2 = 1.0 - (a * u / (1.0 + a - u));
            } else if (ch == CH_QUINN) {
                W = m->plasmon_e;
                c2 = 1.0;
            } else {
                W = table_pick(ch == CH_MOLLER ? j->tm : j->tg, Ei, unit(c[2]));
                if (W <= (Ei - m->fermi_e) * 0.5) {
                    c2 = 0.5 * (sqrt(1.0 - W / Ei) + 1.0);
                } else {
                    c2 = (s->quirks & 4u) ? NAN : 1.0;
                    e.nan_events++;
                }
            }
        } else {
            ch = CH_RUTH;
            double mfp = mfp_from_sigma(elastic_sigma(s->elastic, Ei, m->Z), n_at);
            sl = -mfp * log(unit(c[1]));
            update_xyz(&e, sl, maxz);
            W = sl * stopping(s, m, Ei, n_at, J);
            if (!(W < Ei)) W = Ei;
            double a = alpha_(Ei, m->Z), u = unit(c[2]);
            c2 = 1.0 - (a * u / (1.0 + a - u));
        }
        hphi = PI_D * unit(c[3]);
        j->channel[ch & 15]++;
        int left = e.outcome != OUT_NONE;
        if (!left || (s->quirks & 1u)) update_energy(&e, W);
        if (e.outcome == OUT_NONE) rotate(&e, c2, hphi, s->quirks);
    }
    mco_out* o = j->out;
    if (o->outcome) o->outcome[i] = (unsigned char)e.first_outcome;
    if (o->flags) o->flags[i] = (unsigned char)((e.rows > 1 ? 1 : 0) | (e.nan_events ? 2 : 0));
    if (o->final_E) o->final_E[i] = e.row_E;
    if (o->dir) for (int k = 0; k < 3; ++k) o->dir[3 * i + k] = e.row_dir[k];
    if (o->last_pos) for (int k = 0; k < 3; ++k) o->last_pos[3 * i + k] = e.row_pos[k];
    if (o->max_z) o->max_z[i] = e.max_z;
    if (o->n_events) o->n_events[i] = (int)num;
    j->nan_events += e.nan_events;
}

static void* worker(void* arg) {
    job_t* j = (job_t*)arg;
    for (long long i = j->begin; i < j->end; ++i) run_one(j, i);
    return NULL;
}

int mco_run(const mco_sim* s, const mco_mat* m, const mco_table* tm, const mco_table* tg,
            unsigned long long first, long long n, mco_out* out, int nthreads) {
    if (!s || !m || !out || n < 0) return 1;
    if (s->mode == 0 && (!tm || !tg)) return 1;
    if (s->mode == 0 && s->diff && !(m->xip_g > 0)) return 1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    job_t* jobs = (job_t*)calloc((size_t)nthreads, sizeof(job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) return 2;
    for (int k = 0; k < nthreads; ++k) {
        jobs[k].s = s; jobs[k].m = m; jobs[k].tm = tm; jobs[k].tg = tg;
        jobs[k].first = first; jobs[k].out = out;
        jobs[k].begin = n * k / nthreads;
        jobs[k].end = n * (k + 1) / nthreads;
        pthread_create(&th[k], NULL, worker, &jobs[k]);
    }
    for (int k = 0; k < nthreads; ++k) {
        pthread_join(th[k], NULL);
        if (out->channel) for (int c = 0; c < 16; ++c) out->channel[c] += jobs[k].channel[c];
        if (out->nan_events) *out->nan_events += jobs[k].nan_events;
    }
    free(jobs);
    free(th);
    return 0;
}
