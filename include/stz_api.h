/*
 * stz_api.h -- C ABI of the GB300 shear-transformation-zone (STZ) kinetic Monte
 * Carlo engine.
 *
 * Plain C types only: no CUDA, no C++ and no framework types cross this
 * boundary. Every entry point returns an int status (STZ_OK == 0) and never
 * aborts the process. The device owns all simulation state; host copies are
 * produced only on request (stz_get_field / stz_get_scalars / stz_get_events).
 *
 * Reference interfaces replaced (paths inside the reference project
 * "Mesoscale simulation STZ model/"):
 *   stz_params_from_input_file  <- ReadInput(FILE*) + Init()        io.c:4-101, init.c:6-75
 *   stz_create                  <- FFT_MPI_Init, Rand_Init, Alloc, Grad,
 *                                  Energy_Init, DStrain, initial solve
 *                                  init.c:77-206, init.c:225-479, elastic.c:6-142,
 *                                  bmg.c:117-124
 *   stz_run / stz_step          <- the driver loop body                bmg.c:138-411
 *                                  (SofteningFactor init.c:711-739, ActEnergy
 *                                  init.c:561-690, Q<0 test bmg.c:148-157,
 *                                  athermal_plasticity evolution.c:47-100,
 *                                  KMC evolution.c:102-363)
 *   stz_solve                   <- InhomogeneousStressSolver / HomogeneousStressSolver
 *                                  elastic.c:977-1066, elastic.c:779-903
 *   stz_elastic_energy          <- ElasticEnergy()                     elastic.c:533-547
 *   stz_destroy                 <- Free()                              init.c:482-559
 * The reference-named entry points themselves (KMC, ActEnergy, ...,
 * WriteScalarMPI) are defined in metallic_glasses_gb300/refapi/refapi.c on
 * top of this interface; the reference's own bmg.h declares them, so that
 * file is compiled against the user's bmg.h, my_fft.h and bmgFlags.h.
 */
#ifndef STZ_API_H
#define STZ_API_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STZ_API_VERSION 1
#define STZ_MODES 20           /* candidate modes per site (reference MODES, bmg.h:29) */

/* ---- status codes -------------------------------------------------------- */
enum {
  STZ_OK = 0,
  STZ_ERR_INVALID = 1,      /* bad argument or parameter combination */
  STZ_ERR_CUDA = 2,         /* CUDA runtime error (message in stz_last_error) */
  STZ_ERR_NAN = 3,          /* non-finite value met in a field or in the total rate */
  STZ_ERR_NO_EVENT = 4,     /* selection located no event (evolution.c:229-234) */
  STZ_ERR_UNSUPPORTED = 5,  /* a flag combination this engine does not implement */
  STZ_ERR_TIMEOUT = 6,      /* a bounded device wait gave up */
  STZ_ERR_IO = 7,           /* input file could not be read / parsed */
  STZ_ERR_NOMEM = 8         /* device or host allocation failed */
};

/* ---- model, loading, precision ------------------------------------------ */
enum {
  STZ_MODEL_REF2D = 0,      /* the reference's own 2D model: per-site per-mode
                               barriers and eigenstrains, re-drawn after each
                               transformation (elastic.c:126-130, 508-512) */
  STZ_MODEL_GLOBAL3D = 1    /* 3D: one table of STZ_MODES traceless modes shared
                               by all sites, per-site barrier dF */
};

enum {                      /* bmgFlags.h:7-9 plus a stress-controlled mode */
  STZ_LOAD_TENSION = 0,
  STZ_LOAD_SHEAR = 1,
  STZ_LOAD_COMPRESSION = 2,
  STZ_LOAD_STRESS = 3       /* constant applied mean stress (applied_stress[]) */
};

enum {                      /* direction-softening schemes, bmgFlags.h:30-35 */
  STZ_SF_LINEAR_FWD = 0,
  STZ_SF_LINEAR_BWD = 1,
  STZ_SF_EVEN = 2,
  STZ_SF_SQUARE_FWD = 3,
  STZ_SF_CUBIC_FWD = 4,
  STZ_SF_GAUSS_FWD = 5
};

enum {
  STZ_PREC_FP64 = 0,        /* "plain": FP64 throughout */
  STZ_PREC_MIXED = 1        /* FP32 stress field, contraction and rates; selection
                               exact in distribution over the FP32 rates (64-bit
                               fixed point, integer sums, rejection of the rare
                               draw beyond a line's exact site sum); FP64 clock,
                               eigenstrain and mean strain; periodic full re-solve
                               (FP64 with resolve_fp64, else FP32 pairs) */
};

enum {
  STZ_SOLVER_FFT = 0,       /* full Green's-function re-solve by FFT after every
                               transformation (the reference's method) */
  STZ_SOLVER_KERNEL = 1,    /* incremental: add the precomputed real-space
                               response of one transformed voxel (the mixed form's
                               FP32 table; in the FP64 forms an FP64 table of the
                               unit responses of each strain component, avalanches
                               and prints still re-solving by FFT; homogeneous
                               moduli only) */
  STZ_SOLVER_AUTO = 2       /* pick per grid size from the tuning table */
};

enum {                      /* barrier (dF) generators for STZ_MODEL_GLOBAL3D */
  STZ_DF_TRUNC_NORMAL = 0,  /* iid Normal(q0_mean, q0_sd) truncated at +-q0_trunc sd */
  STZ_DF_CORRELATED = 1     /* Gaussian random field, Gaussian covariance of
                               length q0_corr_len voxels, clipped at +-q0_trunc sd */
};

/* Voigt component order. 3D: xx yy zz yz xz xy. 2D: xx yy xy (reference DE=3).
 * x runs along the fastest grid axis n[2] (reference index j), y along n[1]
 * (reference index i) and z along n[0] (1 in 2D). */
enum { STZ_XX = 0, STZ_YY = 1, STZ_ZZ = 2, STZ_YZ = 3, STZ_XZ = 4, STZ_XY = 5 };

typedef struct stz_params {
  int32_t model;             /* STZ_MODEL_* */
  int32_t n[3];              /* grid extents, slowest first; 2D: n[0] == 1 */
  /* elastic medium (GPa) */
  double  lambda, mu;        /* Lame constants of the homogeneous medium */
  double  young, poisson;    /* E and nu as used by the loading formulas
                                (reference: E from input, nu after LOW_T, init.c:26) */
  /* kinetics */
  double  temperature;       /* K */
  double  trial_frequency;   /* s^-1 (reference TRIAL_FREQUENCY, bmg.h:42) */
  double  voxel_volume;      /* nm^3 (reference VOXEL0, bmg.h:90) */
  /* barriers and modes */
  int32_t df_kind;           /* STZ_DF_* (GLOBAL3D) */
  double  q0_mean, q0_sd, q0_trunc, q0_corr_len;
  double  gamma0;            /* mode magnitude (reference GAMMA0 = 0.14, bmg.h:94) */
  /* loading (evolution.c:262-358) */
  int32_t loading;           /* STZ_LOAD_* */
  double  strain_rate;       /* rate of the loaded tensor component, s^-1 */
  double  strain_increment;  /* elastic-step increment; dt = increment / rate */
  double  end_strain;        /* stop when |loaded mean strain| exceeds this */
  double  applied_stress[6]; /* GPa, STZ_LOAD_STRESS only */
  int32_t no_subtract_error; /* bmgFlags.h NO_SUBTRACT_ERROR */
  int32_t shear_elastic_quirk; /* 1: elastic step adds strain_rate*1 to the mean
                                  shear strain, as evolution.c:350 does */
  /* softening / memory (init.c:59-68, 711-739; elastic.c:366-397) */
  int32_t softening;         /* input "Softening Flag" */
  int32_t sf_scheme;         /* STZ_SF_* */
  double  perm_soft, temp_soft, perm_soft_cap, t_temp;
  /* crystal-like MRO sites of STZ_MODEL_REF2D (init.c:345-437, elastic.c:61-137 and
   * 361-520, ActEnergy under NO_SF_XTAL_MRO init.c:645-660) */
  double  xmro_frac;         /* init_mro 0: share of six-fold sites ("Volume fraction of
                                crystal-like MRO") */
  double  xq0amp;            /* barrier of a crystal-like site after it transforms */
  double  random_ratio;      /* "Random ratio of fluctuation in energy barrier" */
  int32_t init_mro;          /* 0: the map is drawn; 1: the map is mro_type/mro_theta
                                (the reference's MROstructure.ms) */
  int32_t no_sf_xtal_mro;    /* bmgFlags.h NO_SF_XTAL_MRO (on as shipped): the barriers of a
                                crystal-like site soften less (init.c:645-660) */
  double  perm_soft_mro, temp_soft_mro; /* a six-fold site's PermSoftmro, TempSoftmro
                                (init.c:61-63) */
  const int32_t* mro_type;   /* init_mro 1: host array of N types (0 glass, 1 six-fold,
                                2 two-fold, 3 ten-fold) in site order, read by stz_create
                                only; NULL otherwise */
  const double*  mro_theta;  /* init_mro 1: host array of N angles (MROthe0), as above */
  /* bookkeeping */
  int32_t print_period;      /* reference "Print period" */
  uint64_t seed;             /* MT19937 seed; 0 maps to 4357 as GSL does */
  /* engine controls */
  int32_t precision;         /* STZ_PREC_* */
  int32_t solver;            /* STZ_SOLVER_* */
  int32_t resolve_period;    /* mixed: full re-solve every this many events (0 = never) */
  int32_t device;            /* CUDA device ordinal */
  int32_t log_capacity;      /* device event-ring entries (0: 1 << 20) */
  int32_t mode_seed_set;     /* GLOBAL3D: 1 = the 20 modes come from their own MT19937
                                stream seeded with mode_seed (replicas sharing one mode
                                set, each with its own barrier field from seed); 0 = the
                                modes are the first draws of the seed's stream */
  int32_t mode_seed;
  int32_t resolve_fp64;      /* mixed: 1 = the field solves (start, periodic re-solves, prints,
                                avalanches) in FP64; 0 = in FP32 pairs (unevaluated sums of two
                                floats, about 48 bits, at the FP32 issue rate) */
  int32_t sel_slack_shift;   /* mixed, for tests and analysis: the selection's per-line upper
                                bound exceeds the FP32 line sum by 2^-sel_slack_shift of it
                                (0: the smallest slack the line sum's rounding allows, chosen
                                per grid); smaller values make rejected draws frequent */
  int32_t main_pass_general; /* mixed, for tests: 1 = the per-event pass runs its general
                                code for every line length instead of the bodies
                                specialised to lines of 32, 64, 96, 128 and 256 sites */
  int32_t reserved[2];
} stz_params;

/* kinds of stz_event */
enum { STZ_EV_THERMAL = 0, STZ_EV_ATHERMAL = 1, STZ_EV_ELASTIC = 2 };

typedef struct stz_event {
  int64_t step;              /* driver-loop iteration, 1-based (reference 'step') */
  int64_t site;              /* linear site index (i0*n1 + i1)*n2 + i2, -1 for elastic */
  int32_t kind;              /* STZ_EV_* */
  int32_t mode;              /* 0..STZ_MODES-1, -1 for elastic */
  double  time;              /* simulation clock after the step, s */
  double  dt;                /* clock advance of the step, s */
  double  q;                 /* activation energy of the chosen (site, mode), eV */
  double  total_rate;        /* summed rate over all (mode, site), s^-1 */
  double  margin;            /* thermal: distance of the dice from the nearer edge of the
                                chosen (site, mode)'s cumulative-rate interval, as a
                                fraction of the total rate (how far a rate error must move
                                a boundary to change the selection) */
  int32_t draws;             /* thermal: generator words the selection took (1 unless
                                the mixed form rejected a draw, see stz_scalars.rejections) */
  int32_t reserved_ev;
} stz_event;

/* scalars returned by stz_get_scalars */
typedef struct stz_scalars {
  double  time;              /* totime */
  double  eps_avg[6];        /* mean strain EpsAvg (Voigt, tensor shear) */
  double  stress[6];         /* mean stress Stress */
  double  eps0_avg[6];       /* mean eigenstrain */
  int64_t step, kstep, astep, estep;  /* bmg.h:350-354 counters */
  int64_t n_print;
  int64_t n_events_logged;
  int32_t stopped;           /* 1: end strain reached, 2: unstable (bmg.c:382-409) */
  int32_t status;            /* sticky device error status */
  double  stress_err_max;    /* mixed, last full re-solve: max |ds| / max |s| of the
                                deviatoric stress s against the re-solve */
  double  stress_err_rms;    /* mixed, last full re-solve: |ds|_2 / |s|_2 */
  int64_t near_ties;         /* selections whose margin was below the form's rate
                                precision: 1e-12 of R (FP64 forms), 2^-24 of R (mixed) */
  int64_t log_dropped;       /* events not logged (ring full) */
  int64_t n_resolves;        /* periodic full re-solves done */
  double  stress_err_rms_worst;  /* worst of stress_err_rms over all re-solves */
  double  stress_err_max_worst;
  int64_t rejections;        /* mixed: draws rejected because the dice fell in a line's
                                slack above the exact sum of its sites (each is redrawn) */
  int64_t reserved[1];
} stz_scalars;

/* field selectors for stz_get_field / stz_set_field */
enum {
  STZ_FIELD_SIGMA = 0,       /* stress, comp 0..5 (0..2 in 2D) */
  STZ_FIELD_EPS0 = 1,        /* accumulated eigenstrain */
  STZ_FIELD_DF = 2,          /* barrier: GLOBAL3D dF (comp 0); REF2D Q0[mode] (comp = mode) */
  STZ_FIELD_DEPS = 3,        /* REF2D mode eigenstrain: comp = mode*3 + voigt */
  STZ_FIELD_TLAST = 4,
  STZ_FIELD_PERM_SOFT = 5,
  STZ_FIELD_TEMP_SOFT = 6,
  STZ_FIELD_PREV_DEPS = 7,   /* eigenstrain increment of the site's last transformation */
  STZ_FIELD_Q = 8,           /* activation energy Q[mode] for the current stress */
  STZ_FIELD_SDEV = 9,        /* mixed form: the stored FP32 deviatoric stress,
                                coordinate comp 0..4 of the orthonormal basis
                                (xx-yy)/sqrt2, (2zz-xx-yy)/sqrt6, sqrt2 yz,
                                sqrt2 xz, sqrt2 xy (pending update applied first) */
  STZ_FIELD_LAMBDA = 10,     /* plain forms: the Lame moduli of each site (Lambda, Mu of   */
  STZ_FIELD_MU = 11,         /* init.c:456-465; the params' lambda, mu until set). Once either
                                varies, every stress solve is the reference's polarisation
                                fixed point (InhomogeneousStressSolver, elastic.c:977-1066)
                                with the params' moduli as the reference medium */
  STZ_FIELD_MRO = 12         /* REF2D crystal-like MRO map (read only): comp 0 the type of
                                each site (0 glass, 1 six-fold, 2 two-fold, 3 ten-fold),
                                comp 1 its angle MROthe0 */
};

typedef struct stz_ctx stz_ctx;

/* ---- parameters ---------------------------------------------------------- */
/* Fill defaults for a model (reference constants for REF2D, the 3D study
 * constants for GLOBAL3D). */
int stz_params_default(stz_params* p, int32_t model);

/* Parse the reference's labelled 'input' file (io.c:4-101) and derive the
 * moduli, clock and softening constants exactly as Init() does (init.c:6-75).
 * Grid extents are left unchanged (the reference fixes them at compile time). */
int stz_params_from_input_file(stz_params* p, const char* path);

/* ---- lifecycle ----------------------------------------------------------- */
int  stz_create(const stz_params* p, stz_ctx** out);
void stz_destroy(stz_ctx* ctx);
const char* stz_last_error(void);   /* thread-local message of the last failure */

/* ---- stepping ------------------------------------------------------------ */
/* Run driver-loop iterations until max_steps iterations or max_events thermal
 * events have been done, or the run stops (end strain / instability). The
 * event log keeps every thermal, athermal and elastic step of the run. */
int stz_run(stz_ctx* ctx, int64_t max_steps, int64_t max_events);

/* ---- batches of independent replicas (mixed form, 3D) ---------------------
 * Every replica keeps its own state, seed, grid, temperature and loading; one
 * round advances every replica that is not done by one driver step, with one
 * grid-wide launch over all replicas' sites and one selection block per
 * replica. Rounds are captured in CUDA graphs. */
typedef struct stz_batch stz_batch;
int  stz_batch_create(const stz_params* params, int32_t count, stz_batch** out);
void stz_batch_destroy(stz_batch* b);
/* Advance every replica by up to `events` thermal events (fewer when it stops). */
int  stz_batch_run(stz_batch* b, int64_t events);
int  stz_batch_size(stz_batch* b);
/* The context of replica i (for stz_get_scalars / stz_get_events / stz_get_field).
 * It stays owned by the batch. */
stz_ctx* stz_batch_replica(stz_batch* b, int32_t i);

/* Re-solve the stress field from the accumulated eigenstrain in FP64 (the
 * reference's elastic solve). */
int stz_solve(stz_ctx* ctx);

/* The same solve without any device allocation, for callers that cannot call
 * cudaMalloc (code running inside another framework's memory pool or budget,
 * or in a process whose allocator someone else owns). No counterpart in the
 * reference.
 * The caller passes device buffers eps0_dev [nc][N] and sigma_dev [nc][N]
 * (nc = 3 for dim 2 with n0 == 1, 6 for dim 3), the mean strain eps_avg
 * (nc host doubles) and a cudaStream_t (or NULL); sigma = C:(eps - eps*)
 * with <eps> = eps_avg. Scratch is one fixed device array (about 13 MB, held
 * by every GPU that loads the library until exit) that fits at most six
 * components of 64^3 (2D up to 512^2); larger grids return STZ_ERR_INVALID.
 * The first call on a device looks up the array's device address. All calls
 * share the array: calls
 * that overlap on the GPU race. Each call copies its twiddle tables and the
 * mean strain from host memory to the array and synchronises the stream
 * before returning. */
int stz_solve_noalloc(int32_t dim, int32_t n0, int32_t n1, int32_t n2, double lambda, double mu,
                      const double* eps0_dev, const double* eps_avg, double* sigma_dev, void* stream);

int stz_get_scalars(stz_ctx* ctx, stz_scalars* out);
/* Copy out log entries [first, first+cap) ; *n receives the number copied. */
int stz_get_events(stz_ctx* ctx, int64_t first, stz_event* out, int64_t cap, int64_t* n);
int stz_get_field(stz_ctx* ctx, int32_t which, int32_t comp, double* host, int64_t count);
/* The displacement field u of the current eigenstrain's elastic solution (periodic, zero
 * mean): dim x N doubles component-major (dim = 2 in REF2D, axis order (j, i) of g in Grad,
 * init.c:112-140; dim = 3 in GLOBAL3D). Replaces the displacement part of
 * HomogeneousStressSolver(..., uflag 2) (elastic.c:873-900) and DispField (io.c:137-240); the
 * supercell position (i (1 + EpsAvg[0]) LX + j EpsAvg[2] LY, ...) is the caller's, as there. */
int stz_get_displacement(stz_ctx* ctx, double* host, int64_t count);
int stz_set_field(stz_ctx* ctx, int32_t which, int32_t comp, const double* host, int64_t count);
/* The FFT schedule the context runs (FFT_MPI_Init's plans, init.c:77-110, are
 * replaced by passes whose tiles and radix order are timed per grid shape):
 * tiles[4] = lines per block of the x, y and outer-axis passes and the number
 * of candidate schedules rejected for differing from the default's result;
 * radices[36] = the radix order of the half-length x transform, of axis 1 and
 * of axis 0, 12 entries each, zero-terminated. Either pointer may be null. */
int stz_fft_schedule(stz_ctx* ctx, int32_t* tiles, int32_t* radices);
/* Sets the mean strain EpsAvg (Voigt order, tensor shear; the first 3 in 2D)
 * that the next solve applies: the host assignment of EpsAvg before the first
 * solve of bmg.c:114, passed to the device. */
int stz_set_mean_strain(stz_ctx* ctx, const double* eps_avg);
int stz_elastic_energy(stz_ctx* ctx, double* out);

/* ---- timing and accounting (for benchmarks) ------------------------------ */
int stz_sync(stz_ctx* ctx);
int stz_timer_start(stz_ctx* ctx);
int stz_timer_stop(stz_ctx* ctx, float* ms);       /* CUDA events on the ctx stream */
int stz_flush_l2(stz_ctx* ctx);                      /* writes a buffer larger than L2 */
int64_t stz_kernel_launches(stz_ctx* ctx);           /* kernels launched by this ctx so far */
/* Bytes copied host->device and device->host by this ctx so far. */
int stz_transfer_bytes(stz_ctx* ctx, int64_t* h2d, int64_t* d2h);
/* Mixed form: average device-clock time per event from the start of the
 * stress-update/rate pass to the start of the selection tail (the pass and the
 * plane sums), and of the tail (total rate, search, commit; one block), since
 * the context was created. */
int stz_phase_times(stz_ctx* ctx, double* main_us, double* tail_us, int64_t* n);
/* Self-test of the kernels' bounded device waits, without a fault: one block
 * waits with `tries` attempts on a barrier armed for bytes that never arrive,
 * as the per-event pass waits on its staged lines, and gives up.
 * *status = STZ_ERR_TIMEOUT when the wait ran out (the expected result),
 * *ms = the kernel's duration, *kernel_tries = the limit the per-event kernels
 * use (their wait lasts about ms * kernel_tries / tries). The device stays
 * usable afterwards. */
int stz_selftest_wait(int32_t device, int32_t tries, int32_t* status, double* ms, int32_t* kernel_tries);
/* sizeof the ABI structs, for bindings: 0 stz_params, 1 stz_event, 2 stz_scalars */
int64_t stz_sizeof(int32_t which);
/* Timed with CUDA events on the ctx stream over *launches events launched
 * one by one. Mixed form: which = 0 the grid-wide stress-update/rate kernel,
 * 2 the whole event (that kernel and the selection kernel: one block per plane
 * for the plane sums, the last of them running the tail), 1 the update-only
 * variant (the stress-field streaming floor). FP64 forms: which = 0 the rate
 * kernel of *launches driver steps (rates, sums, selection and commit).
 * In the mixed form a 40 us one-warp hold kernel runs before each timed
 * launch, so the start event is not stamped ahead of the host's launch.
 * Returns the average ms; *launches receives the number of launches timed. */
int stz_kernel_time(stz_ctx* ctx, int32_t which, double* ms_avg, int64_t* launches);

#ifdef __cplusplus
}
#endif
#endif /* STZ_API_H */
