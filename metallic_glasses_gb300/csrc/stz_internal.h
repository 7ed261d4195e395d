// stz_internal.h -- engine internals shared by the host and device sources.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <vector>

#include "../../include/stz_api.h"
#include "mt19937.cuh"

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
#include <vector_types.h>
typedef struct CUstream_st* cudaStream_t;
typedef struct CUevent_st* cudaEvent_t;
typedef struct CUgraphExec_st* cudaGraphExec_t;
#endif

namespace stz {

void set_error(const char* fmt, ...);

// Physical constants of the reference (bmg.h:71-77).
constexpr double kEvInJ = 1.60217733e-19;
constexpr double kJInEv = 1 / kEvInJ;
constexpr double kBoltz = 1.380658e-23;
constexpr double kEpsilon = 1e-17;

enum StepKind { kThermal = 0, kAthermal = 1, kElastic = 2, kNone = -1 };

enum HaltReason {
  kHaltNone = 0,
  kHaltAthermal = 1,   // mixed path: an avalanche needs the FFT path
  kHaltResolve = 2,    // mixed path: periodic FP64 re-solve due
  kHaltPrint = 3,      // mixed path: print re-solve due
  kHaltStop = 4,       // end strain / instability
  kHaltError = 5,
  kHaltTarget = 6      // requested number of events / steps reached
};

// Device-resident control block: every scalar of the simulation state plus
// the per-step flags that steer the kernels of a step. One per context.
// What the mixed-form main pass reads at its start, prepared by the kernel
// that last changed the pending state: the deviatoric coordinates of the
// uniform change U in FP32 and the pending transformation (site coordinates
// and mode), so that pass does no FP64 arithmetic and no dependent loads.
struct __align__(16) MixHead {  // read as three 16-byte words; keep the order
  float Ud[5];
  int has_pend;
  int p0, p1, p2, pend_mode;
  int pad[2];
};
static_assert(sizeof(MixHead) == 48, "MixHead is three 16-byte words");

struct Ctl {
  MixHead head;
  double totime;
  double eps_avg[6];         // EpsAvg
  double eps_avg_applied[6]; // mean strain the stored field was solved with
  double stress[6];          // Stress
  double u[6];               // uniform stress added to the field since its solve
  double eps0_sum[6];        // sum over sites of the eigenstrain
  double last_print_strain;
  double t_kmc;              // clock advance of the current thermal event
  double U[6];               // incremental path: pending uniform stress change
  double stress_err_max, stress_err_rms;
  double total_rate;         // R of the last selection
  double sel_q;              // Q of the last selected (site, mode)
  long long step, kstep, astep, estep, n_print;
  long long nlog, nlog_dropped, near_ties;
  long long log_base;        // first log entry not yet copied to the host
  long long max_kstep, max_step;  // halt targets (absolute), < 0 = none
  long long next_resolve;    // mixed: kstep at which the periodic re-solve is due
  unsigned long long neg_count;   // (mode, site) pairs with Q < 0 this step
  int step_kind;
  int solve_req;             // an FFT solve of the current phase is requested
  int print_done;            // the print of this step re-solved the field
  int stopped;
  int status;                // sticky STZ_* error
  int halt, halt_reason;
  int has_pend;              // incremental path: a transformation is pending
  int pend_mode;
  long long pend_site;
  int incr_req;              // FP64 incremental form: the thermal event's update is due
  double pend_deps[6];       // FP64 forms: eigenstrain increment of the last transformation
  double ebar_solved[6];     // FP64 forms: mean strain of the stored field's last solve
  unsigned int ticket;       // last-block-done counter of the rate kernels
  int sel_mode;
  long long sel_site;
  int ath_count;
  unsigned int line_emax;    // mixed: largest biased FP32 exponent of this event's line sums
                             // (atomic maximum of the main pass; 0xff: a non-finite sum)
  long long rejections;      // mixed: selection draws rejected (dice in a line's slack)
  // device-clock phase times of the mixed-form kernel (globaltimer, ns)
  unsigned long long prof_t0, prof_main_ns, prof_tail_ns, prof_n;
  unsigned long long prof_part_ns[8];  // tail: copy-in+sums, twist+decision, search, commit,
                                       // search levels (mode, plane), line, site
  MT rng;
};

// Device fields. Layout: component-major structure of arrays, site index
// s = (i0 * n1 + i1) * n2 + i2 (i2 fastest), 8-byte aligned rows.
struct Fields {
  double* eps0 = nullptr;    // [nc][N] accumulated eigenstrain (FP64 always)
  double* sig = nullptr;     // [nc][N] stress (FP64 forms)
  float* sdev = nullptr;     // [5][N] deviatoric stress coordinates (mixed form)
  double* dF = nullptr;      // [N] barrier (GLOBAL3D)
  float* dF32 = nullptr;     // [N] barrier (mixed form)
  double* Q0 = nullptr;      // [MODES][N] (REF2D)
  double* deps = nullptr;    // [MODES][3][N] (REF2D)
  double* dnorm = nullptr;   // [MODES][N] 1 / (|deps| + eps) of each mode (REF2D), kept with deps
  double* rtab64 = nullptr;  // [nc][nc][N] FP64 incremental form: stress component c of the
                             // solve of a unit eigenstrain component k at site 0, ebar = 0
  int8_t* mro = nullptr;     // [N] crystal-like MRO type 0..3 (REF2D); null for an all-glass map
  double* Q1 = nullptr;      // [MODES][N] the initial Q0, restored at every print (bmg.c:214-221);
                             // only with crystal-like sites (glass sites never change Q0)
  double* prev_deps = nullptr;  // [nc][N]
  double* perm_soft = nullptr;
  double* temp_soft = nullptr;
  double* tlast = nullptr;
  signed char* amark = nullptr; // [N] athermal marks (mode+1, 0 = none)
  double* part = nullptr;    // [MODES][nblk] per (mode, block) rate sums
  double* gsum = nullptr;    // [MODES][ngroups] per (mode, group of blocks) sums
  unsigned* gticket = nullptr;  // [ngroups] last-block counters of the groups
  float* lsum = nullptr;     // mixed: [n0 n1][MODES] per-line rate sums
  long long* lbnd = nullptr; // mixed: [n0][MODES][n1] the lines' selection bounds in the event's
                             // fixed point, written by the plane sums (mode-major per plane,
                             // so the search reads one contiguous run)
  long long* psum = nullptr; // mixed: [MODES + 1][n0] per-(mode, plane) sums of the line
                             // bounds in the event's fixed point; row MODES: each plane's
                             // fixed-point sum of its line sums over all modes (the clock)
  void* spec = nullptr;      // [nc][Nk] complex FP64 spectrum
  float* ktab = nullptr;     // mixed: [kt0][kt1][kt2][16] response table (15 used)
  stz_event* log = nullptr;  // event ring
  Ctl* ctl = nullptr;
  double* scratch = nullptr;  // small scratch (error statistics nobody reads)
  double* msum = nullptr;     // [nc][c2r_blocks] block sums of the solved field
  // spatially varying moduli (plain forms; allocated when first set)
  double* lam_site = nullptr;  // [N] Lambda
  double* mu_site = nullptr;   // [N] Mu
  double* inh_tau0 = nullptr;  // [nc][N] C(x):eps*  of the polarisation fixed point
  double* inh_eeff = nullptr;  // [nc][N] effective eigenstrain of the reference medium
  double* inh_last = nullptr;  // [nc][N] its previous iterate
  double* inh_part = nullptr;  // [blocks] partial sums of the iterate's squared change
};

// Constant parameters of one context, passed to kernels by value.
struct KParams {
  int model, nc, n0, n1, n2, nh;
  long long N, Nk;
  int nblk, bsites;          // rate kernel: blocks and sites per block
  int ngroups;               // groups of kGroup blocks
  int mx_c1, mx_units;       // mixed form: d1 chunks per d0, units (kt0 * mx_c1)
  unsigned c1_magic;         // ceil(2^32 / mx_c1), for the division of unit indices
  int adv_q2, adv_r2;        // kRateThreads sites = adv_q2 rows of n2 plus adv_r2 sites
  int fast_inv;              // mixed form: precomputed compliance coefficients
  double inv_2mu, inv_lam_coef, invN, inv_a_scale;
  int loading, softening, sf_scheme, no_subtract_error, shear_quirk, no_sf_xtal_mro;
  int incr64;                      // FP64 forms: thermal events by the incremental update
  double lambda, mu, young, poisson;
  double kT, vt, V0, dt, gamma0;
  double inv_kT;                   // 1/kT rounded to nearest (rate quotients, over_kT)
  double w_scale;                  // V0 1e-18 J / (2 kT): work to rate argument (FP64 forms)
  double perm_soft, temp_soft, perm_soft_cap, t_temp;
  double perm_soft_mro, temp_soft_mro, xq0amp, random_ratio;  // crystal-like MRO sites (REF2D)
  double end_strain, strain_rate, strain_increment, print_thr;
  double applied[6];
  double modes[STZ_MODES][6];      // GLOBAL3D mode table (Voigt, tensor shear)
  // mixed form
  float mdev[STZ_MODES][5];        // mode deviatoric coords * (c/2) * log2(e) (c: eV per GPa
                                   // and unit strain); the rate argument is
                                   // a + sum_k (s_k * inv_kt) mdev[m][k]
  float2 mdev2[STZ_MODES / 2][5];  // the same, modes paired (2j, 2j+1) for packed FMA
  float inv_kt;                    // 1 / kT (eV): the replica's scale of the stress coordinates
  float a_scale;                   // log2(e)/kT
  float q_ref;                     // reference barrier of the scaled rates
  double rate_scale;               // vt * exp(-q_ref/kT): true rate per scaled unit
  float mdev_raw[STZ_MODES][5];    // mode deviatoric coords (unscaled)
  int kt0, kt1, kt2;               // response-table extents (n/2+1)
  int sel_slack;                   // a line's selection bound exceeds its fixed-point FP32 sum
                                   // by 2^-sel_slack of it (plus 3 quanta)
  int general_pass;                // the per-event pass runs its general code for every n2
  long long log_cap;
  int resolve_period;
  int c2r_blocks;                  // blocks of the FFT's C2R pass (msum row length)
};

// One replica of a batch as the batched kernels see it.
// The mode matrices of the mixed form, for a batch whose replicas share them.
struct ModeSet {
  float2 mdev2[STZ_MODES / 2][5];
  float mdev_raw[STZ_MODES][5];
};

struct BatchDesc {
  KParams kp;
  Fields f;
};

// Per-replica summary written by the batched selection kernel.
struct BatchStatus {
  int halt, halt_reason, stopped, status;
  long long kstep;
  long long pad;
};

}  // namespace stz

struct stz_ctx {
  stz_params p{};
  stz::KParams kp{};
  stz::Fields f{};
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t kev0 = nullptr, kev1 = nullptr;
  void* fft = nullptr;               // FFT plan (fft.cu)
  int64_t launches = 0;
  std::vector<stz_event> host_log;   // drained events
  long long drained = 0;
  stz::Ctl host_ctl{};
  double ktime_ms = 0;
  int64_t ktime_n = 0;
  int use_graph = 1;
  int inhom = 0;                      // some site's moduli differ from the params' (plain forms)
  std::vector<double> lam_h, mu_h;    // host copies of the site moduli (empty until set)
  std::vector<int8_t> mro_h;          // REF2D crystal-like MRO map (types) and its angles
  std::vector<double> mro_theta_h;
  cudaGraphExec_t graph = nullptr;
  int graph_batch = 0;
  int64_t graph_launches = 0;        // kernels per graph launch
  void* l2buf = nullptr;
  size_t l2flush_bytes = 0;
  double* qbuf = nullptr;            // [N] activation energies of one mode (stz_get_field)
  int fft_tuned[4] = {0, 0, 0, 0};   // FFT tiles chosen (L_x, L_y, L_g) and candidates rejected
  double* err_dev = nullptr;         // [4] error sums of the periodic re-solve
  double err_max = 0, err_rms = 0;   // last periodic re-solve
  double err_max_worst = 0, err_rms_worst = 0;
  int64_t n_resolves = 0;
  int64_t h2d_bytes = 0, d2h_bytes = 0;  // host<->device copies made by stepping and getters
};
