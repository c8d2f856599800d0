/*
 * mcd.h - C ABI of the GB300 electron-trajectory Monte Carlo (libmcd.so).
 *
 * Plain C types only: host structs carry device pointers, every device
 * buffer is owned by the caller, and every call that touches the GPU is
 * ordered on the stream it is given (a cudaStream_t passed as void*; NULL is
 * the legacy default stream).  Calls return an MCD_* code and never trap;
 * conditions found on the device are OR-ed into a caller-owned status word.
 *
 * Each entry point names the reference interface it replaces
 * (elena-pascal/MC-discrete, paths relative to that project).
 */
#ifndef MCD_H
#define MCD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCD_ABI_VERSION 10
#define MCD_MAX_SHELLS 8
#define MCD_MAX_CHANNELS 16
#define MCD_HIST_E_MAX 256
#define MCD_HIST_T_MAX 180
#define MCD_GUIDE 256          /* guide buckets per table row (see mcd_table) */

/* ---- return codes ------------------------------------------------------ */
enum {
    MCD_OK = 0,
    MCD_EINVAL = 1,     /* bad argument (null pointer, bad enum, bad size)    */
    MCD_ECUDA = 2,      /* a CUDA runtime call failed                          */
    MCD_ETOOBIG = 3,    /* a size is beyond a documented limit                 */
    MCD_ENOSPECIES = 4, /* unknown material name                               */
    MCD_ENODEV = 5      /* no usable CUDA device                               */
};

/* ---- device status flags (OR-ed into the caller's uint32 status word) --- */
#define MCD_FLAG_TABLE_RANGE 0x01u /* E above a table's last E row: last row used  */
#define MCD_FLAG_RING_FULL   0x02u /* event records did not fit the ring           */
#define MCD_FLAG_NAN         0x04u /* binary collision gave a NaN polar angle      */
#define MCD_FLAG_CLAMPED     0x08u /* continuous: energy loss >= E, clamped to E   */
#define MCD_FLAG_LONG_PATH   0x10u /* continuous: a step of 1e4 A or more          */
#define MCD_FLAG_LONG        0x20u /* an electron reached max_scatt                */
#define MCD_FLAG_RING_INDEX  0x40u /* packed ring header: an electron index of
                                      2^28 or more; its records were dropped   */
#define MCD_FLAG_CKPT        0x80u /* adjoint: an exiting electron had more events
                                      than checkpoint slots (no gradient)        */

/* ---- enums --------------------------------------------------------------- */
enum { MCD_OUT_NONE = 0, MCD_OUT_BKS = 1, MCD_OUT_ABS = 2, MCD_OUT_TRSM = 3,
       MCD_OUT_TRDF = 4, MCD_OUT_LONG = 5 };
/* channels: Rutherford, Moller, Quinn, then Gryzinski shell k = 3 + k in the
 * material's shell order (MC/tools/scattering.py:483-508), and diffraction
 * (diffMFP, :510-516)                                                        */
enum { MCD_CH_RUTH = 0, MCD_CH_MOLLER = 1, MCD_CH_QUINN = 2, MCD_CH_GRYZ0 = 3, MCD_CH_DIFF = 11 };
/* elastic total cross section (MC/tools/crossSections.py:37-147); the polar
 * angle is always drawn with the Rutherford screening alpha
 * (MC/tools/scattering.py:125-152, :575)                                     */
enum { MCD_ELASTIC_RUTH = 0,         /* 'Ruth_vanilla'                       */
       MCD_ELASTIC_RUTH_WDEFL = 1,   /* 'Ruth_vanilla_wDefl': Z^2 -> Z(Z+1)   */
       MCD_ELASTIC_NIGRAM = 2,       /* 'Ruth_nigram'                         */
       MCD_ELASTIC_NIGRAM_WDEFL = 3  /* 'Ruth_nigram_wDefl'                   */ };
enum { MCD_MODE_DS = 0, MCD_MODE_CONT = 1 };
enum { MCD_BETHE_CLASSICAL = 0, MCD_BETHE_JL = 1, MCD_BETHE_EXPLICIT = 2 };
enum { MCD_FP32 = 0, MCD_FP64 = 1 };
enum { MCD_TABLE_MOLLER = 0, MCD_TABLE_GRYZ = 1 };

/* Reference behaviours that can be switched off (set = reference).          */
#define MCD_Q_CROSSING_STEP 0x1u /* the step that leaves the sample still loses
                                    energy, so it can add an 'abs' row
                                    (MC/tools/singleScatter.py:35-41)        */
#define MCD_Q_HALF_PHI_FOLD 0x2u /* cos(halfPhi) = +sqrt(1-sin^2)
                                    (MC/tools/electron.py:90-91)             */
#define MCD_Q_NAN_DIRECTION 0x4u /* W > (E-Ef)/2 gives NaN cos^2(theta/2);
                                    off: no deflection for that event
                                    (MC/tools/scattering.py:177-179)         */
#define MCD_QUIRKS_REFERENCE 0x7u

/* Optional tallies (mcd_sim.tally_flags).                                     */
#define MCD_TALLY_CHANNELS 0x1u  /* per-channel event counts                  */

/* ---- material (MC/tools/material.py:117-302) ----------------------------- */
typedef struct mcd_material {
    char species[8];
    char name_val[16];
    char shell_name[MCD_MAX_SHELLS][8];
    int32_t Z;
    int32_t n_shells;
    double n_val;                    /* valence electrons                     */
    double E_val;                    /* valence binding energy, eV            */
    double density;                  /* g/cm^3                                */
    double atwt;                     /* g/mol                                 */
    double bethe_k;                  /* Joy-Luo k                             */
    double atnd;                     /* atoms per m^3                         */
    double plasmon_e;                /* eV                                    */
    double fermi_e;                  /* eV                                    */
    double J;                        /* Bethe mean ionisation energy, eV      */
    double shell_E[MCD_MAX_SHELLS];  /* binding energies, eV                  */
    double shell_n[MCD_MAX_SHELLS];  /* occupancies                           */
    double xip_g;                    /* extinction distance of the diffraction
                                        channel (0: none; Si 1360)            */
} mcd_material;

/* ---- sampled CDF table (MC/tools/probTables.py:70-162, 490-535) ---------- */
typedef struct mcd_table {
    const float* Es;         /* device, nE energies (float32 linspace)        */
    const float* Ws;         /* device, nW energy losses (float32 geomspace)  */
    const float* cdf;        /* device, nE x (nW-1); 0 marks a masked entry   */
    const int32_t* nvalid;   /* device, nE unmasked counts per row, or NULL
                                (written by mcd_build_table; the transport
                                does not read it: masked entries act as +inf) */
    const uint16_t* guide;   /* device, nE x (MCD_GUIDE+1): first CDF index
                                whose value is >= k/MCD_GUIDE, or NULL (needs
                                nW - 1 <= 65535); a draw U lies between entries
                                floor(U G) and floor(U G) + 1, so most draws
                                need no CDF read; the result is unchanged   */
    int32_t nE;
    int32_t nW;
    float E_first;           /* Es[0] and Es[nE-1] as the host holds them, so */
    float E_last;            /* the row guess needs no loads (0: read Es)     */
} mcd_table;

/* ---- one simulation (the input.file keys, MC/tools/fileTools.py:8-46) ---- */
typedef struct mcd_sim {
    int32_t mode;            /* MCD_MODE_*                                    */
    int32_t bethe_model;     /* MCD_BETHE_* (continuous mode)                 */
    int32_t precision;       /* MCD_FP32 or MCD_FP64 transport                */
    uint32_t quirks;         /* MCD_Q_* bits                                  */
    uint32_t tally_flags;    /* MCD_TALLY_* bits                              */
    uint32_t sim_id;         /* Philox counter word 3                         */
    double E0, Emin;         /* eV                                            */
    double s_tilt;           /* degrees                                       */
    double Wc;               /* Moller cut-off, eV (DS)                       */
    double thickness;        /* A; >= 1e30 means semi-infinite                */
    int64_t max_scatt;       /* events before 'long' (MC/tools/singleScatter.py:
                                19-23); <= 0 or above 2^32 - 1 means 2^32 - 1,
                                the range of the Philox event counter word   */
    int64_t num_el;
    uint64_t first_electron; /* Philox electron index of electron 0           */
    uint64_t seed;           /* Philox key                                    */
    int32_t hist_E_bins;     /* exit-energy histogram of 'bks' electrons      */
    int32_t hist_T_bins;     /* polar exit-angle histogram (from -z), degrees */
    double hist_E_width;     /* eV per bin                                    */
    double hist_T_width;     /* degrees per bin                               */
    double J_scale;          /* continuous: Bethe J multiplier (1 = reference)*/
    double n_scale;          /* density multiplier (1 = reference)            */
    int32_t elastic;         /* MCD_ELASTIC_*                                 */
    int32_t diff_mfp;        /* DS: diffraction channel of constant cross
                                section 1/(n xip_g) m^3/nm/cm^2; its step has
                                mean free path xip_g, no loss, no deflection,
                                and crossing the bottom face on that step is
                                'trdf' (MC/tools/scattering.py:510-548,658-668,
                                MC/tools/electron.py:72-79); needs xip_g > 0 */
    const void* sigma_table; /* DS: device table from mcd_build_sigma_table
                                for this simulation (built for its
                                precision: float for FP32 transport, double
                                for FP64), read by mcd_run and (FP32)
                                mcd_run_batched_noalloc instead of
                                evaluating the channel cross sections
                                (NULL: evaluate them); mcd_batch_prepare
                                builds its own tables                       */
    const struct mcd_electron_out* electrons;
                             /* mcd_batch_prepare, mcd_run_batched_noalloc:
                                this simulation's per-electron rows (device
                                arrays for num_el electrons, FP32; NULL:
                                none), read when the batch is packed; mcd_run
                                takes its rows as an argument instead       */
} mcd_sim;

/* ---- per-simulation tallies (device, caller zeroes them) ----------------- */
typedef struct mcd_tally {
    unsigned long long outcome[8];       /* first row of each electron        */
    unsigned long long events;           /* scatter events                    */
    unsigned long long double_rows;      /* 'bks' then 'abs' in one step      */
    unsigned long long nan_events;
    unsigned long long clamped;
    unsigned long long long_path;
    unsigned long long table_range;
    unsigned long long channel[MCD_MAX_CHANNELS];
    double sum_E_bks;                    /* sum of exit energies, eV          */
    double sum_E2_bks;
    double sum_steps2;                   /* sum of squared event counts       */
    double reserved;
    unsigned long long hist_E[MCD_HIST_E_MAX];
    unsigned long long hist_T[MCD_HIST_T_MAX];
} mcd_tally;

/* ---- per-electron rows (MC/tools/electron.py:105-113), all optional ----- */
typedef struct mcd_electron_out {
    uint8_t* outcome;        /* first outcome code                            */
    uint8_t* flags;          /* bit0: a second 'abs' row, bit1: NaN event     */
    void* final_E;           /* float (MCD_FP32) or double (MCD_FP64), n      */
    void* dir;               /* 3 x n, SoA (dx..., dy..., dz...)              */
    void* last_pos;          /* 3 x n, SoA                                    */
    void* max_z;             /* deepest z reached, n                          */
    int32_t* n_events;       /* events of the electron, n                     */
} mcd_electron_out;

/* ---- per-event records (MC/tools/scattering.py:527-679) ------------------ */
typedef struct mcd_event {
    uint32_t electron;       /* electron index within the simulation          */
    uint32_t step_chan;      /* event index << 5 | channel                    */
    float E;                 /* energy before the event, eV                   */
    float W;                 /* energy loss, eV                               */
    float pathl;             /* step length, A                                */
    float c2;                /* cos^2(theta/2) ('pol_angle')                  */
    float half_phi;          /* 'az_angle', rad                               */
    float x, y, z;           /* position at the start of the event, A         */
} mcd_event;                 /* 40 bytes                                      */

/* Fields of a ring record after its 8-byte header (electron,
 * event << 5 | channel), in this order, 4 bytes each (position: 12), the
 * scatter_output columns they carry in brackets (MC/tools/fileTools.py:
 * 193-242).  A column mask of 0 selects all of them: the mcd_event layout.
 * MCD_EV_PACKED_HEAD replaces the header by one word, electron << 4 |
 * channel (electron < 2^28), without the event index: the records of one
 * electron keep their order in the ring (one thread appends them, each
 * after the last one's slot was returned), so an electron's n-th record
 * is its event n.                                                          */
#define MCD_EV_E     0x01u      /* E before the event ['E']                  */
#define MCD_EV_W     0x02u      /* energy loss ['E_loss']                    */
#define MCD_EV_PATHL 0x04u      /* step length ['pathl']                     */
#define MCD_EV_C2    0x08u      /* cos^2(theta/2) ['pol_angle']              */
#define MCD_EV_PHI   0x10u      /* halfPhi ['az_angle']                      */
#define MCD_EV_POS   0x20u      /* x, y, z at the start ['position']         */
#define MCD_EV_ALL   0x3fu      /* the column bits                           */
#define MCD_EV_PACKED_HEAD 0x40u
typedef struct mcd_event_ring {
    void* rec;                       /* device, capacity records of
                                        mcd_event_bytes(fields) bytes each    */
    unsigned long long capacity;
    unsigned long long* cursor;      /* device; records reserved so far; the
                                        ones at index >= capacity are dropped */
    uint32_t fields;                 /* MCD_EV_* columns (0 = all), with
                                        MCD_EV_PACKED_HEAD or not            */
    uint32_t reserved;
} mcd_event_ring;

/* Bytes of one ring record for a field mask (host).                          */
size_t mcd_event_bytes(uint32_t fields);

/* ---- launch tuning of the batched kernel -------------------------------- */
typedef struct mcd_tune {
    int32_t block_size;      /* threads per block (multiple of 32)            */
    int32_t blocks_per_sm;   /* resident blocks per SM of the persistent grid */
    int32_t refill;          /* idle lanes a warp waits for before it takes
                                new electrons from the queue (1..32)          */
    int32_t variant;         /* bit 0: 56-register kernel (block_size <= 576,
                                two blocks per SM)
                                instead of the 64-register one; bit 1: evaluate
                                cross sections inline instead of from the
                                tables mcd_batch_prepare builds              */
    int64_t reserved;        /* must be 0                                     */
} mcd_tune;

/* ====================== host-only entry points ========================== */
int mcd_abi_version(void);
const char* mcd_strerror(int code);
size_t mcd_struct_size(const char* name);   /* layout check for bindings     */

/* Material constants for Al, Si, Cu or Au.
 * Replaces material(species) (MC/tools/material.py:117-133, 151-302).       */
int mcd_material_init(const char* species, mcd_material* out);

/* ======================= device entry points ============================ */
int mcd_device_info(int* sm_count, int* cc_major, int* cc_minor);

/* Fill one sampled CDF table in FP64 on the GPU: trapezoid steps of
 * dsigma/dW between consecutive Ws, cumulative sum, normalised by the row
 * total; intervals above Wmax(E) = (E - Ef)/2 are masked (stored as 0).
 * kind is MCD_TABLE_MOLLER (valence electrons, Wmin = Wc) or MCD_TABLE_GRYZ
 * (shell `shell` of the material).  cdf64, nvalid and guide may be NULL.
 * Replaces probTable.computeBlock/generate (MC/tools/probTables.py:415-486). */
int mcd_build_table(int kind, const mcd_material* mat, int shell,
                    int32_t nE, int32_t nW, const float* Es, const float* Ws,
                    float* cdf32, double* cdf64, int32_t* nvalid, uint16_t* guide,
                    void* stream);

/* Cross-section table of one DS simulation, for mcd_sim.sigma_table, built
 * for the simulation's precision from the FP64 evaluation of the expressions
 * of MC/tools/crossSections.py:37-284.
 * FP32: on a log2-E grid of 128 points per octave over [Emin, E0], E times the
 * total channel cross section and E times the running sums in pick order
 * (Ruth, Moller, Gryzinski shells), stored as FP32 and interpolated
 * linearly (within 3e-7 of the exact sums) -- the table the batched path
 * builds per group of simulations.
 * FP64: the mean free path and the running sums as fractions of the
 * total, as FP64 cubics in the cells of grids uniform in E inside each
 * octave of (Emin, E0] (256 cells per octave, indexed from the exponent and
 * mantissa bits of E; per cell four coefficients per column, through the
 * values at four nodes; within about 1.3e-10 of the exact values); cells
 * whose nodes straddle a channel threshold, or reach below 2 Wc (where the
 * Moller cross section turns negative towards its pole at Wc), are flagged
 * and evaluated exactly.  The octaves must fit the buffer: MCD_ETOOBIG otherwise (Au
 * from 50 eV to 30 keV fits, from 10 eV does not).
 * It depends on the material, Wc, the elastic model, n_scale, E0, Emin and
 * the precision.  table is 16-byte-aligned device memory of
 * mcd_sigma_table_bytes() bytes.                                            */
size_t mcd_sigma_table_bytes(void);
int mcd_build_sigma_table(const mcd_sim* sim, const mcd_material* mat,
                          void* table, void* stream);

/* One simulation, one GPU thread per electron, one launch.
 * Replaces multiTraj_DS / multiTraj_cont (MC/tools/multiScatter.py:66-116,
 * 171-229) and trajectory_DS / trajectory_cont_cl
 * (MC/tools/singleScatter.py:10-41, 205-239).  moller/gryz are used in DS
 * mode only (gryz = the outermost shell's table, which samples every
 * Gryzinski loss, MC/tools/scattering.py:625).  electrons and ring may be
 * NULL.  tally and status are device pointers.  block_size is 1, 2, 4, 8,
 * 16 or a multiple of 32 up to 256, or 0: 128, halved down to 8 while the
 * grid would leave SMs idle, so that a small job spreads over more SMs with
 * fewer lanes each, and for FP64 transport further down to 2 while the grid
 * stays within one warp per scheduler; there an FP64 DS run without a ring
 * puts two electrons on each warp, one per half-warp whose lanes compute
 * the coming events' random numbers and the functions of them that do not
 * depend on the trajectory (results do not depend on any of this).  A DS
 * simulation with a sigma_table reads its channel cross sections from it.  */
int mcd_run(const mcd_sim* sim, const mcd_material* mat,
            const mcd_table* moller, const mcd_table* gryz,
            mcd_tally* tally, const mcd_electron_out* electrons,
            const mcd_event_ring* ring, uint32_t* status,
            int32_t block_size, void* stream);

/* Many simulations of uneven size in one persistent launch fed by a global
 * work queue.  mcd_batch_prepare packs the simulations into a caller-owned
 * device workspace of mcd_batch_workspace_bytes(nsims) bytes (host-to-device
 * copy on `stream`; host memory may be reused when the call returns) and
 * builds there log-energy tables of E times the cumulative channel cross
 * sections (FP64 evaluation, FP32 storage, 128 points per octave, one table
 * per group of DS simulations with the same material, Wc and density) that
 * the kernel interpolates instead of evaluating 3 + n_shells formulas per
 * event (tune variant bit 1 keeps the formulas).
 * mcd_run_batched then only resets the queue and launches, so it can be
 * captured in a CUDA graph.  tallies[nsims] and status are device pointers.
 * Replaces MapScatterer.__call__ (MC/doScatter.py:54-95) with its pool of
 * multiTraj_* jobs.                                                          */
size_t mcd_batch_workspace_bytes(int32_t nsims);
/* Bytes mcd_batch_prepare copies from the host (the workspace less its
 * table slots, which the GPU fills).                                        */
size_t mcd_batch_upload_bytes(int32_t nsims);
int mcd_batch_prepare(const mcd_sim* sims, int32_t nsims,
                      const mcd_material* mats, const int32_t* sim_material,
                      const mcd_table* tables, const int32_t* sim_moller,
                      const int32_t* sim_gryz, void* workspace,
                      size_t workspace_bytes, void* stream);
int mcd_run_batched(void* workspace, int32_t nsims, mcd_tally* tallies,
                    const mcd_tune* tune, uint32_t* status, void* stream);

/* The same launch with every event appended to `ring` (device records and
 * cursor, caller-owned; records at index >= capacity are dropped and show as
 * cursor > capacity).  The streaming path of the reference's scatter_output
 * (MC/tools/scattering.py:527-679 via MC/tools/fileTools.py:193-242), which
 * replaces its per-job pickled lists and HDF5 appends (MC/doScatter.py:99-119).
 * Event records carry the electron index within its simulation.            */
int mcd_run_batched_ring(void* workspace, int32_t nsims, mcd_tally* tallies,
                         const mcd_tune* tune, const mcd_event_ring* ring,
                         uint32_t* status, void* stream);

/* ---- differentiable continuous mode ------------------------------------- */
/* Gaussian-soft exit-energy histogram of backscattered electrons:
 * h_b = (1/num_el) sum exp(-(E_exit - c_b)^2 / (2 sigma^2)),
 * c_b = lo + (b + 1/2) (hi - lo) / nbins.                                    */
enum { MCD_ADJ_EXIT_E = 0,      /* exit energy of 'bks' electrons, eV        */
       MCD_ADJ_MAX_DEPTH = 1    /* deepest z reached by 'bks' electrons, A   */ };
typedef struct mcd_softhist {
    int32_t nbins;           /* <= MCD_HIST_E_MAX                             */
    int32_t quantity;        /* MCD_ADJ_*: what is binned                     */
    double lo, hi, sigma;    /* in the quantity's unit                        */
} mcd_softhist;

/* Per-electron adjoint state (device, caller-owned).                         */
typedef struct mcd_adjoint_buf {
    void* ckpt;              /* T [max_ckpt][num_el] (exit energy: E every 64
                                events) or T [max_ckpt][8][num_el] (depth: E,
                                z, direction and local y axis every 64 events) */
    int32_t* kstar;          /* [num_el], 'bks' electrons, else -1: the exit
                                event (exit energy) or the number of events
                                up to the deepest point (depth)              */
    void* E_exit;            /* T [num_el]: the binned quantity (exit energy
                                of the first outcome row, or deepest z)     */
    int32_t max_ckpt;
    int32_t reserved;
    unsigned long long* queue;
                             /* one device word (or NULL): the forward pass
                                zeroes it on its stream and runs a resident
                                grid whose lanes take the next electron from
                                it as they finish; NULL runs one thread per
                                electron instead                            */
} mcd_adjoint_buf;

/* Continuous-mode forward pass that also stores the adjoint checkpoints.
 * hist_out[nbins + 2] (device, zeroed by the caller) receives the unnormalised
 * soft bins of hist->quantity, its sum and the number of 'bks' electrons; tally
 * (may be NULL) the outcome and event counts.  sim->J_scale and sim->n_scale
 * scale the Bethe J and the density.  Replaces multiTraj_cont + trajectory_cont_cl
 * (MC/tools/multiScatter.py:171-229, MC/tools/singleScatter.py:205-239) with
 * gradients in mind; the reference has no derivative of its own.            */
int mcd_adjoint_forward(const mcd_sim* sim, const mcd_material* mat, const mcd_softhist* hist,
                        const mcd_adjoint_buf* buf, double* hist_out, mcd_tally* tally,
                        uint32_t* status, void* stream);

/* Reverse sweep: grad_hist[nbins + 1] holds dL/dh_b and dL/d(sum of the
 * quantity); grad[2] (device, zeroed by the caller) receives dL/dJ_scale and
 * dL/dn_scale, the pathwise derivatives with random numbers and event
 * sequence (for depth also the deepest event) frozen.  Each 64-event segment
 * is recomputed from its checkpoint and the Philox counters; for depth the
 * sweep carries the adjoints of the energy, the direction and the local y
 * axis through the Rutherford deflections.  No counterpart in the reference. */
int mcd_adjoint(const mcd_sim* sim, const mcd_material* mat, const mcd_softhist* hist,
                const mcd_adjoint_buf* buf, const double* grad_hist, double* grad, void* stream);

/* The binned quantity along the frozen event sequence of the last forward
 * pass, at this call's J_scale / n_scale, as soft bins (for finite-difference
 * checks of mcd_adjoint).  No counterpart in the reference.                  */
int mcd_adjoint_chain(const mcd_sim* sim, const mcd_material* mat, const mcd_softhist* hist,
                      const mcd_adjoint_buf* buf, double* hist_out, void* stream);

/* The batched run above without any device allocation, for callers that
 * cannot call cudaMalloc (an embedding application that owns all device
 * memory through its own arena; a caller for which an allocation, which can
 * synchronise the device, would break its latency budget).  No counterpart
 * in the reference.  Its scratch is a static device array sized for
 * MCD_STATIC_MAX_SIMS simulations (31.5 KiB), resident on every GPU that
 * loads the library until exit; more simulations return MCD_ETOOBIG.  The
 * first call on a device looks up that array's address and keeps it for
 * the life of the device's primary context: do not use the library across
 * a cudaDeviceReset.  Calls share
 * the array: calls that overlap on the GPU race.  The simulations are
 * packed on the host and handed to a staging kernel on `stream` as one
 * kernel argument, so no host memory has to outlive the call;
 * tallies[nsims] (zeroed by the caller) and status are device pointers.
 * tune is read as by mcd_run_batched (variant bit 0: the 56-register
 * kernel; bit 1: inline cross sections).  Without bit 1 a simulation that
 * carries a caller-built sigma_table reads it; the others evaluate their
 * cross sections inline (there is no room for tables in the array).       */
#define MCD_STATIC_MAX_SIMS 64
int mcd_run_batched_noalloc(const mcd_sim* sims, int32_t nsims,
                            const mcd_material* mats, const int32_t* sim_material,
                            const mcd_table* tables, const int32_t* sim_moller,
                            const int32_t* sim_gryz, mcd_tally* tallies,
                            const mcd_tune* tune, uint32_t* status, void* stream);

/* Exit directions -> detector coordinates, replacing projOnDetector
 * (MC/tools/rotation.py:78-102) with the detector geometry of
 * MC/tools/parameters.py:22-33 supplied by the caller.  dir holds n
 * directions as three planes dx[n], dy[n], dz[n] (the mcd_electron_out.dir
 * layout); xy receives x[n], y[n]:
 *     x = dx - x_pc,  y = R_x(-alpha)[1] . d - y_pc,
 * the rotation taken from the conjugate of q = (cos(alpha/2), sin(alpha/2),
 * 0, 0) as the reference does; L (the z translation) does not reach x, y.
 * precision is MCD_FP32 (float planes, FP32 arithmetic) or MCD_FP64.
 * Device pointers, stream-ordered; n == 0 launches nothing.              */
int mcd_project_detector(const void* dir, int64_t n, int32_t precision, double alpha_deg,
                         double x_pc, double y_pc, double L, void* xy, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MCD_H */
