// kmc.cu -- the STZ kinetic Monte Carlo step on the device.
//
// One driver-loop iteration (bmg.c:139-178) of the FP64 forms is
//   k_rate64     SofteningFactor + ActEnergy + KMC rates for every (mode, site)
//                (init.c:561-739, evolution.c:120-128), per-(mode, block) FP64
//                sums; the last block to finish reduces them, decides athermal
//                / thermal / elastic, draws the dice, finds the event with a
//                hierarchical search in the reference's mode-major order
//                (evolution.c:136-193) and commits it (elastic.c:361-520)
//   k_ath_mark, k_ath_commit   athermal avalanche (evolution.c:47-100)
//   FFT solve    fft.cu
//   k_post_a     loading, clock and print check (evolution.c:262-358, bmg.c:181-187)
//   FFT solve    print re-solve (bmg.c:292-295), skipped unless printing
//   k_post_b     stop conditions (bmg.c:382-410) and run targets
// Kernels after the first read their work flags from the control block and
// return at once when the step does not need them.
//
// The mixed form replaces the per-event FFT by the response of one voxel
// (linearity of the Green's operator): k_mixed adds the pending
// transformation's response to the FP32 deviatoric stress field, evaluates
// the rates in FP32, sums them in FP64 and selects/commits in its last block.
#include <cfloat>
#include <cmath>
#include <cstddef>

#include "kmc.cuh"

namespace stz {
namespace {

constexpr int TH = kRateThreads;
constexpr unsigned FULL = 0xffffffffu;

// ------------------------------------------------------------ scalar state
__device__ __forceinline__ int ndiag(int nc) { return nc == 3 ? 2 : 3; }

__device__ void apply_C(const KParams& kp, const double* e, double* s) {
  const int nd = ndiag(kp.nc);
  double tr = 0;
  for (int c = 0; c < nd; c++) tr += e[c];
  for (int c = 0; c < kp.nc; c++) s[c] = (c < nd ? kp.lambda * tr : 0.0) + 2.0 * kp.mu * e[c];
}

// isotropicinv (elastic.c:522-531) in DIM dimensions. The mixed form uses
// precomputed coefficients (no divisions on the one-thread commit path); the
// FP64 forms keep the reference's operation order.
__device__ void iso_inv(const KParams& kp, const double* s, double* e) {
  const double lam = kp.lambda, mu = kp.mu;
  if (kp.fast_inv) {
    const int nd = ndiag(kp.nc);
    double tr = 0;
    for (int c = 0; c < nd; c++) tr += s[c];
    const double t = -kp.inv_lam_coef * tr;
    for (int c = 0; c < kp.nc; c++) e[c] = (c < nd ? t : 0.0) + s[c] * kp.inv_2mu;
    return;
  }
  if (kp.nc == 3) {
    double tra = -lam / 2 / mu / (2 * lam + 2 * mu) * (s[0] + s[1]);
    e[0] = tra + s[0] / 2 / mu;
    e[1] = tra + s[1] / 2 / mu;
    e[2] = s[2] / 2 / mu;
  } else {
    double tra = -lam / 2 / mu / (3 * lam + 2 * mu) * (s[0] + s[1] + s[2]);
    for (int c = 0; c < 3; c++) e[c] = tra + s[c] / 2 / mu;
    for (int c = 3; c < 6; c++) e[c] = s[c] / 2 / mu;
  }
}

// AvgStress (elastic.c:733-752): mean of the solved field, from the per-block
// sums the C2R pass left in msum (fixed summation order)
// Mean stress of the solved field from the C2R pass's block sums, by the
// whole block: strided partial sums per thread, then a fixed shuffle tree and
// the warps in order (a dependent chain of FP64 additions in one thread took
// about 1 ms at 128^3: GB300 runs FP64 at 1/64 of the FP32 rate). Thread 0
// writes out; every thread of the block must call it.
__device__ void field_mean_stress(const KParams& kp, const Fields& f, double* out) {
  __shared__ double red[TH / 32][6];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int c = 0; c < kp.nc; c++)
    for (int b = threadIdx.x; b < kp.c2r_blocks; b += blockDim.x) s[c] += f.msum[(long long)c * kp.c2r_blocks + b];
  for (int c = 0; c < kp.nc; c++) {
    for (int off = 16; off > 0; off >>= 1) s[c] += __shfl_xor_sync(FULL, s[c], off);
    if (lane == 0) red[w][c] = s[c];
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int c = 0; c < kp.nc; c++) {
      double t = 0;
      for (int k = 0; k < nw; k++) t += red[k][c];
      out[c] = t / (double)kp.N;
    }
  __syncthreads();
}

__device__ void solved_mean_stress(const KParams& kp, const Ctl* ctl, const double* ebar, double* out) {
  double e[6];
  for (int c = 0; c < kp.nc; c++) e[c] = ebar[c] - ctl->eps0_sum[c] * kp.invN;
  apply_C(kp, e, out);
}

__device__ __forceinline__ int shear_comp(const KParams& kp) { return kp.nc == 3 ? 2 : STZ_XY; }
__device__ __forceinline__ int loaded_comp(const KParams& kp) {
  return kp.loading == STZ_LOAD_SHEAR ? shear_comp(kp) : 0;
}

// eps_avg correction from the mean stress of the solved field
// (evolution.c:92-97, 263-300)
__device__ void subtract_error(const KParams& kp, const Ctl* ctl, int athermal, double* tmpStrain) {
  double ts[6] = {0, 0, 0, 0, 0, 0};
  if (!kp.no_subtract_error) {
    for (int c = 0; c < kp.nc; c++) ts[c] = ctl->stress[c];
    const int zc = (athermal && kp.nc == 3) ? 0 : loaded_comp(kp);
    ts[zc] = 0.0;
  }
  iso_inv(kp, ts, tmpStrain);
}

__device__ void hold_stress(const KParams& kp, Ctl* ctl) {
  double d[6] = {0, 0, 0, 0, 0, 0}, de[6];
  for (int c = 0; c < kp.nc; c++) d[c] = kp.applied[c] - ctl->stress[c];
  iso_inv(kp, d, de);
  for (int c = 0; c < kp.nc; c++) {
    ctl->eps_avg[c] += de[c];
    ctl->u[c] += d[c];
    ctl->stress[c] = kp.applied[c];
  }
}

// loading after a thermal event (evolution.c:262-317); ctl->stress holds the
// mean stress of the field solved right after the transformation
__device__ void load_after_event(const KParams& kp, Ctl* ctl, double t_kmc) {
  double ts[6];
  const double rate = kp.strain_rate, nu = kp.poisson, E = kp.young, mu = kp.mu;
  const bool d2 = kp.nc == 3;
  switch (kp.loading) {
    case STZ_LOAD_TENSION:
      subtract_error(kp, ctl, 0, ts);
      ctl->eps_avg[0] += (rate * t_kmc * 1 - ts[0]);
      ctl->eps_avg[1] += (rate * t_kmc * (-nu) - ts[1]);
      if (d2) {
        ctl->eps_avg[2] += (-ts[2]);
      } else {
        ctl->eps_avg[2] += (rate * t_kmc * (-nu) - ts[2]);
        for (int c = 3; c < 6; c++) ctl->eps_avg[c] += (-ts[c]);
      }
      ctl->stress[0] += E * rate * t_kmc;
      ctl->u[0] += E * rate * t_kmc;
      break;
    case STZ_LOAD_COMPRESSION:
      subtract_error(kp, ctl, 0, ts);
      ctl->eps_avg[0] += (-rate * t_kmc * 1);
      ctl->eps_avg[1] += (rate * t_kmc * (nu));
      ctl->eps_avg[0] += (-rate * t_kmc * 1 - ts[0]);
      ctl->eps_avg[1] += (rate * t_kmc * (nu) - ts[1]);
      for (int c = 2; c < kp.nc; c++) ctl->eps_avg[c] += (-ts[c]);
      ctl->stress[0] += -E * rate * t_kmc;
      ctl->u[0] += -E * rate * t_kmc;
      break;
    case STZ_LOAD_SHEAR: {
      const int sc = shear_comp(kp);
      subtract_error(kp, ctl, 0, ts);
      for (int c = 0; c < kp.nc; c++)
        if (c != sc) ctl->eps_avg[c] += -ts[c];
      ctl->eps_avg[sc] += rate * t_kmc;
      ctl->stress[sc] += 2 * mu * rate * t_kmc;
      ctl->u[sc] += 2 * mu * rate * t_kmc;
      break;
    }
    case STZ_LOAD_STRESS:
      hold_stress(kp, ctl);
      break;
  }
}

// pure elastic step (evolution.c:321-358)
__device__ void elastic_step(const KParams& kp, Ctl* ctl) {
  const double inc = kp.strain_increment, nu = kp.poisson, E = kp.young, mu = kp.mu;
  const bool d2 = kp.nc == 3;
  switch (kp.loading) {
    case STZ_LOAD_TENSION:
      ctl->eps_avg[0] += (inc * 1);
      ctl->eps_avg[1] += (inc * (-nu));
      ctl->eps_avg[2] += d2 ? (inc * 0.0) : (inc * (-nu));
      ctl->stress[0] += E * inc;
      ctl->u[0] += E * inc;
      break;
    case STZ_LOAD_COMPRESSION:
      ctl->eps_avg[0] += (inc * (-1));
      ctl->eps_avg[1] += (inc * (nu));
      ctl->eps_avg[2] += d2 ? (inc * 0.0) : (inc * (nu));
      ctl->stress[0] += -E * inc;
      ctl->u[0] += -E * inc;
      break;
    case STZ_LOAD_SHEAR: {
      const int sc = shear_comp(kp);
      if (kp.shear_quirk) ctl->eps_avg[sc] += kp.strain_rate * 1;
      else ctl->eps_avg[sc] += inc;
      ctl->stress[sc] += 2 * mu * inc;
      ctl->u[sc] += 2 * mu * inc;
      break;
    }
    default:
      break;
  }
}

// print test (bmg.c:181-187); returns 1 when the step prints (and re-solves)
__device__ int print_check(const KParams& kp, Ctl* ctl) {
  if (kp.loading == STZ_LOAD_STRESS) return 0;
  const int lc = loaded_comp(kp);
  if (fabs(ctl->eps_avg[lc] - ctl->last_print_strain) >= kp.print_thr) {
    ctl->n_print++;
    ctl->last_print_strain = ctl->eps_avg[lc];
    return 1;
  }
  return 0;
}

// stop conditions (bmg.c:382-410) and run targets; sets halt
__device__ void stop_check(const KParams& kp, Ctl* ctl) {
  if (kp.loading != STZ_LOAD_STRESS) {
    const int lc = loaded_comp(kp);
    if (fabs(ctl->eps_avg[lc]) > kp.end_strain) ctl->stopped = 1;
    else if (kp.loading == STZ_LOAD_TENSION && ctl->stress[0] < -0.5) ctl->stopped = 2;
    else if (kp.loading == STZ_LOAD_SHEAR && fabs(ctl->stress[lc]) < kEpsilon) ctl->stopped = 2;
  }
  if (ctl->stopped) { ctl->halt = 1; ctl->halt_reason = kHaltStop; return; }
  if ((ctl->max_kstep >= 0 && ctl->kstep >= ctl->max_kstep) || (ctl->max_step >= 0 && ctl->step >= ctl->max_step)) {
    ctl->halt = 1;
    ctl->halt_reason = kHaltTarget;
  }
}

// margin: a thermal event's distance of the dice from the nearer edge of the
// chosen element's cumulative interval, as a fraction of the total rate;
// draws: the generator words its selection took.
__device__ void log_event(const KParams& kp, const Fields& f, Ctl* ctl, int kind, long long site, int mode,
                          double time, double dt, double q, double R, double margin = 0.0, int draws = 0) {
  const long long i = ctl->nlog;
  if (i - ctl->log_base >= kp.log_cap) {
    ctl->nlog_dropped++;
    return;
  }
  stz_event e;
  e.step = ctl->step;
  e.site = site;
  e.kind = kind;
  e.mode = mode;
  e.time = time;
  e.dt = dt;
  e.q = q;
  e.total_rate = R;
  e.margin = margin;
  e.draws = draws;
  e.reserved_ev = 0;
  f.log[i % kp.log_cap] = e;
  ctl->nlog = i + 1;
}

// ------------------------------------------------------- per-site physics
// Unpack a site index into grid coordinates (32-bit: grids hold < 2^31 sites).
__device__ __forceinline__ void site_coords(const KParams& kp, long long s, int* i0, int* i1, int* i2) {
  const unsigned u = (unsigned)s;
  const unsigned r = u / (unsigned)kp.n2;
  *i2 = (int)(u - r * (unsigned)kp.n2);
  const unsigned q = r / (unsigned)kp.n1;
  *i1 = (int)(r - q * (unsigned)kp.n1);
  *i0 = (int)q;
}

// The same header from warp 0: lane k < 5 forms coordinate k, lane 5 the
// pending transformation (the FP64 steps of the five coordinates run side by
// side instead of one after another).
__device__ void set_mixed_head_warp(const KParams& kp, Ctl* c) {
  const int k = threadIdx.x & 31;
  MixHead& h = c->head;
  const double* U = c->U;
  const double r2 = 0.70710678118654752440, r6 = 0.40824829046386301637, q2 = 1.41421356237309504880;
  if (k == 0) h.Ud[0] = (float)((U[0] - U[1]) * r2);
  else if (k == 1) h.Ud[1] = (float)((2.0 * U[2] - U[0] - U[1]) * r6);
  else if (k < 5) h.Ud[k] = (float)(q2 * U[k + 1]);
  else if (k == 5) {
    h.has_pend = c->has_pend;
    h.pend_mode = c->has_pend ? c->pend_mode : 0;
    if (c->has_pend) site_coords(kp, c->pend_site, &h.p0, &h.p1, &h.p2);
    else h.p0 = h.p1 = h.p2 = 0;
  }
  __syncwarp();
}

// The mixed-form main pass's header from U, has_pend, pend_site and
// pend_mode (one thread; FP64 here, FP32 for the pass).
__device__ void set_mixed_head(const KParams& kp, Ctl* c) {
  MixHead& h = c->head;
  const double* U = c->U;
  const double r2 = 0.70710678118654752440, r6 = 0.40824829046386301637, q2 = 1.41421356237309504880;
  h.Ud[0] = (float)((U[0] - U[1]) * r2);
  h.Ud[1] = (float)((2.0 * U[2] - U[0] - U[1]) * r6);
  h.Ud[2] = (float)(q2 * U[3]);
  h.Ud[3] = (float)(q2 * U[4]);
  h.Ud[4] = (float)(q2 * U[5]);
  h.has_pend = c->has_pend;
  h.pend_mode = c->has_pend ? c->pend_mode : 0;
  if (c->has_pend) site_coords(kp, c->pend_site, &h.p0, &h.p1, &h.p2);
  else h.p0 = h.p1 = h.p2 = 0;
}

// Direction modifier of the softening schemes (init.c:590-642)
// The direction modifier from DM = dot / (n1 + eps) / (n2 + eps), here formed
// as dot * r1 * r2 with the reciprocals r = 1 / (n + eps) (the mode's stored,
// the site's once per site): two multiplications in place of two divisions,
// within a few ulps of the quotients.
__device__ __forceinline__ double dire_modifier(int scheme, double dot, double r1, double r2) {
  const double DM = dot * r1 * r2;
  switch (scheme) {
    case STZ_SF_LINEAR_FWD: return (DM + 1) / 2;
    case STZ_SF_LINEAR_BWD: return (-DM + 1) / 2;
    case STZ_SF_EVEN: return 0.5;
    case STZ_SF_SQUARE_FWD: return (1 + DM) * (1 + DM) / 4;
    case STZ_SF_CUBIC_FWD: return (DM + 1) * (DM + 1) * (DM + 1) / 8;
    default: return exp(-DM * DM * 9 / 2);
  }
}

// ---------------------------------------------------------- FP64 rates
// exp(x) of the FP64 rate kernels by Tang's table-driven method (P. T. P. Tang,
// "Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15(2), 1989): x = (256 m + j) ln2/256 + r
// with |r| <= ln2/512, exp(x) = 2^m 2^(j/256) e^r; ln2/256 in a 32-bit head (k
// times it is exact for |k| < 2^21) and a tail; e^r - 1 by its Taylor
// polynomial of degree 4 (truncation below 2^-54 relative); 2^(j/256) from
// exp_table.h (generated by exp_table.py) as hi + lo, read through L1 since
// each lane takes its own entry. Within 1 ulp of the C library's exp (checked
// for 5 10^7 arguments). Arguments outside (-700, 700), and NaN, take the
// library routine. As written the FP64 pipe (the bound of the rate kernels)
// does the arithmetic only: the range test compares the bit pattern of |x|,
// 2^m enters as an integer add to the exponent field, and hi + lo rounds to hi
// (|lo| is below half an ulp of hi), so S(J) of Tang's reconstruction is hi.
#define STZ_EXP_TABLE_STORAGE __device__ const
#include "exp_table.h"
#undef STZ_EXP_TABLE_STORAGE

__device__ __forceinline__ double exp_tang(double x) {
  if (!((__double_as_longlong(x) & 0x7fffffffffffffffLL) < 0x4085e00000000000LL)) return exp(x);  // |x| < 700
  const double kd = rint(x * STZ_EXP_INV_STEP);
  const int k = (int)kd;
  const double r1 = __fma_rn(-kd, STZ_EXP_STEP_HEAD, x);
  const double r2 = -kd * STZ_EXP_STEP_TAIL;
  const double r = r1 + r2;
  const double c = __fma_rn(r, __fma_rn(r, 1.0 / 24, 1.0 / 6), 0.5);
  const double p = r1 + __fma_rn(r * r, c, r2);
  const int j = k & 255, m = (k - j) / 256;
  const double hi = __ldg(&kExp2Hi[j]), lo = __ldg(&kExp2Lo[j]);
  return __longlong_as_double(__double_as_longlong(hi + __fma_rn(hi, p, lo)) + ((long long)m << 52));
}

// Q/kT correctly rounded: Markstein's refinement of Q times the rounded
// reciprocal of kT (one correction of the product by its exact residual;
// checked against the division for 2 10^7 barriers at three temperatures)
__device__ __forceinline__ double over_kT(const KParams& kp, double Q) {
  const double q0 = Q * kp.inv_kT;
  return isfinite(q0) ? __fma_rn(__fma_rn(-q0, kp.kT, Q), kp.inv_kT, q0) : Q / kp.kT;
}

// x > 0 for a rate argument (Q < 0, the avalanche trigger), on the integer
// pipe: the bit patterns of +min subnormal .. +inf, which leaves out NaN
__device__ __forceinline__ bool arg_positive(double x) {
  return (unsigned long long)(__double_as_longlong(x) - 1) < 0x7ff0000000000000ULL;
}

// REF2D: site data shared by the 20 modes; ft is the factor NO_SF_XTAL_MRO
// applies at a crystal-like site (init.c:645-660), 0 at a glass site
struct R2Site {
  double sg[3], pd[3], r2, soft, ft;  // r2: 1 / (|last increment| + eps)
  double sw[3];                       // the stresses times V0 1e-18 J / (2 kT), shear weight 2
};

// the factor of MRO type 1 (six-fold), 2 (two-fold), 3 (ten-fold)
__device__ __forceinline__ double mro_factor(int t) { return t == 1 ? 0.1 : (t == 2 ? 0.01 : 0.9); }

__device__ __forceinline__ R2Site r2_load(const KParams& kp, const Fields& f, const double* u, double totime,
                                          long long s) {
  R2Site d;
  const long long N = kp.N;
  for (int c = 0; c < 3; c++) {
    d.sg[c] = f.sig[c * N + s] + u[c];
    d.pd[c] = f.prev_deps[c * N + s];
    d.sw[c] = ((c == 2 ? 2.0 : 1.0) * d.sg[c]) * kp.w_scale;
  }
  d.r2 = 1.0 / (sqrt(d.pd[0] * d.pd[0] + d.pd[1] * d.pd[1] + 2 * d.pd[2] * d.pd[2]) + kEpsilon);
  // a site without temporary softening skips the decay's exponential: its
  // term is 0 times a finite positive factor, +0 exactly
  const double ts = kp.softening ? f.temp_soft[s] : 0.0;
  d.soft = kp.softening ? (ts != 0.0 ? f.perm_soft[s] + ts * exp_tang((f.tlast[s] - totime) / kp.t_temp)
                                     : f.perm_soft[s])
                        : 0.0;
  const int t = (f.mro && kp.no_sf_xtal_mro) ? f.mro[s] : 0;
  d.ft = t ? mro_factor(t) : 0.0;
  return d;
}

// Norm of a 2D mode increment, sqrt(de_xx^2 + de_yy^2 + 2 de_xy^2)
// (init.c:600-603), every operation rounded on its own as the reference's C
// evaluates it, and the reciprocal 1 / (norm + eps) of the direction
// modifier. The reciprocal is stored per mode and site whenever the modes are
// drawn, so the rate passes load it instead of taking a square root and a
// division per mode.
__device__ __forceinline__ double mode_norm(double d0, double d1, double d2) {
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(__dmul_rn(2.0, d2), d2)));
}
__device__ __forceinline__ double mode_rnorm(double d0, double d1, double d2) {
  return 1.0 / (mode_norm(d0, d1, d2) + kEpsilon);
}

// ActEnergy for one (mode, site) of the reference model (init.c:585-686)
// The softened barrier Q0 exp(-DM soft) of a softened site (init.c:612-684)
__device__ __forceinline__ double r2_soft_q0(const KParams& kp, const Fields& f, const R2Site& d, long long s, int m,
                                             double d0, double d1, double d2) {
  const long long N = kp.N;
  const double dot = d.pd[0] * d0 + d.pd[1] * d1 + 2 * d.pd[2] * d2;
  const double r1 = f.dnorm[(long long)m * N + s];
  double DM = dire_modifier(kp.sf_scheme, dot, r1, d.r2);
  double soft = d.soft;
  if (d.ft != 0.0) {
    // a crystal-like site: the reference scales the direction modifier and,
    // in place, the site's softening by the factor for every mode in turn,
    // so mode m sees the softening times the factor m + 1 times
    DM = __dmul_rn(DM, d.ft);
    for (int k = 0; k <= m; k++) soft = __dmul_rn(soft, d.ft);
  }
  return f.Q0[(long long)m * N + s] * exp_tang(-DM * soft);
}

__device__ __forceinline__ double r2_Q(const KParams& kp, const Fields& f, const R2Site& d, long long s, int m) {
  const long long N = kp.N;
  const double* dd = f.deps + (long long)m * 3 * N;
  const double d0 = dd[s], d1 = dd[N + s], d2 = dd[2 * N + s];
  const double DWork = (d.sg[0] * d0 + d.sg[1] * d1 + 2 * d.sg[2] * d2) * kp.V0 * 1e-18 * kJInEv;
  // an unsoftened site (every site before its first transformation): the
  // direction modifier is finite (its norms carry kEpsilon), so the factor
  // exp(-DM * 0) is exactly 1 and the barrier is Q0 - W/2 to the bit; the
  // square root, two divisions and an exponential per mode are skipped
  if (d.soft == 0.0) return f.Q0[(long long)m * N + s] - DWork / 2;
  return r2_soft_q0(kp, f, d, s, m, d0, d1, d2) - DWork / 2;
}

// The rate argument x = -Q/kT = W V0 1e-18 J / (2 kT) - Q0 e / kT of the rate
// pass (e the softening factor, 1 at an unsoftened site), the work from the
// site's stresses scaled once by V0 1e-18 J / (2 kT) (r2_load): three FMAs and
// the quotient of Q0 e by kT per mode in place of the work sum, its scale
// factors, the difference and the quotient of Q. Within a few ulps of -Q/kT;
// x > 0 exactly when Q < 0 unless |Q| is within a few ulps of zero (the
// avalanche's marking keeps r2_Q).
__device__ __forceinline__ double r2_arg(const KParams& kp, const Fields& f, const R2Site& d, long long s, int m) {
  const long long N = kp.N;
  const double* dd = f.deps + (long long)m * 3 * N;
  const double d0 = dd[s], d1 = dd[N + s], d2 = dd[2 * N + s];
  const double hw = __fma_rn(d.sw[2], d2, __fma_rn(d.sw[1], d1, d.sw[0] * d0));
  const double q = d.soft == 0.0 ? f.Q0[(long long)m * N + s] : r2_soft_q0(kp, f, d, s, m, d0, d1, d2);
  return hw - over_kT(kp, q);
}

// GLOBAL3D FP64: Q = dF - W/2 with W = sigma:deps_m
__device__ __forceinline__ double g3_Q(const KParams& kp, const double* sg, double dF, int m) {
  double w = 0;
  for (int c = 0; c < 6; c++) w += (c >= 3 ? 2.0 : 1.0) * sg[c] * kp.modes[m][c];
  return dF - w * kp.V0 * 1e-18 * kJInEv / 2;
}

__device__ __forceinline__ void g3_load(const KParams& kp, const Fields& f, const double* u, long long s, double* sg) {
  for (int c = 0; c < 6; c++) sg[c] = f.sig[c * kp.N + s] + u[c];
}

// GLOBAL3D FP64 rate arguments x_m = -Q_m/kT = W_m V0 1e-18 J / (2 kT) - dF/kT,
// from the site's stresses scaled once by V0 1e-18 J / (2 kT) (Voigt shear
// weights included): six FMAs per mode in place of the work sum, its four
// scale factors, the difference and the quotient of -Q/kT, which x matches to
// a few ulps. x > 0 exactly when Q < 0 (the avalanche trigger) unless |Q| is
// within a few ulps of zero; the avalanche's own marking keeps g3_Q.
struct G3Arg {
  double ws[6], x0;
};
__device__ __forceinline__ G3Arg g3_arg_site(const KParams& kp, const double* sg, double dF) {
  G3Arg a;
  for (int c = 0; c < 6; c++) a.ws[c] = ((c >= 3 ? 2.0 : 1.0) * sg[c]) * kp.w_scale;
  a.x0 = -over_kT(kp, dF);
  return a;
}
__device__ __forceinline__ double g3_arg(const KParams& kp, const G3Arg& a, int m) {
  double x = a.x0;
  for (int c = 0; c < 6; c++) x = __fma_rn(a.ws[c], kp.modes[m][c], x);
  return x;
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Programmatic dependent launch: wait until the preceding kernel of the
// stream has completed and its writes are visible (a no-op when the kernel
// was launched without the attribute), and let the following kernel be
// scheduled early (it still waits for this one before touching memory).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// 2^x with the hardware approximation (PTX ex2.approx.ftz.f32: one MUFU
// operation, relative error below 2^-22; results under 2^-126 flush to 0).
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Mixed: scaled log2-rate x = log2(e)/kT (q_ref - Q) = a + sum_k (s_k/kT) mdev[m][k]
// with temperature-free mode coordinates; identical code in the main pass and
// in the rescan so both see the same bits.
__device__ __forceinline__ float mx_x(const KParams& kp, const float* sv, float a, int m) {
  float x = a;
#pragma unroll
  for (int k = 0; k < 5; k++) x = __fmaf_rn(__fmul_rn(sv[k], kp.inv_kt), kp.mdev[m][k], x);
  return x;
}

// The stored FP32 coordinates of site s (the mixed form's rates see them).
__device__ __forceinline__ void mx_site(const KParams& kp, const Fields& f, long long s, float* sv) {
#pragma unroll
  for (int k = 0; k < 5; k++) sv[k] = f.sdev[(long long)k * kp.N + s];
}

// ---------------------------------------------------- block-level helpers
// Inclusive scan of one double per thread over a 256-thread block; returns the
// inclusive value and leaves every thread's inclusive value in sh_inc.
__device__ double block_incl_scan(double v, double* sh_inc) {
  __shared__ double wsum[TH / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double y = __shfl_up_sync(FULL, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    double t = lane < TH / 32 ? wsum[lane] : 0.0;
#pragma unroll
    for (int off = 1; off < TH / 32; off <<= 1) {
      const double y = __shfl_up_sync(FULL, t, off);
      if (lane >= off) t += y;
    }
    if (lane < TH / 32) wsum[lane] = t;
  }
  __syncthreads();
  const double incl = (w > 0 ? wsum[w - 1] : 0.0) + x;
  sh_inc[threadIdx.x] = incl;
  __syncthreads();
  return incl;
}

// Sum of STZ_MODES per-thread accumulators over the block, written to
// part[m * nblk + b] by threads 0..STZ_MODES-1 in a fixed order.
__device__ void block_mode_sums(const double* acc, double* part, int nblk, int b) {
  __shared__ double red[TH / 32][STZ_MODES];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < STZ_MODES; m++) {
    double v = acc[m];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL, v, off);
    if (lane == 0) red[w][m] = v;
  }
  __syncthreads();
  if (threadIdx.x < STZ_MODES) {
    double s = 0;
    for (int k = 0; k < TH / 32; k++) s += red[k][threadIdx.x];
    part[(long long)threadIdx.x * nblk + b] = s;
  }
}

__device__ unsigned block_sum_u(unsigned v) {
  __shared__ unsigned red[TH / 32];
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL, v, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned t = 0;
  for (int k = 0; k < TH / 32; k++) t += red[k];
  return t;
}

// Block-wide sum of v and maximum of mx (every thread of the block calls it).
__device__ void block_sum_max_u(unsigned v, unsigned mx, unsigned* sum, unsigned* vmax) {
  __shared__ unsigned red[2][TH / 32];
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL, v, off);
  mx = __reduce_max_sync(FULL, mx);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = v;
    red[1][threadIdx.x >> 5] = mx;
  }
  __syncthreads();
  unsigned t = 0, m = 0;
  for (int k = 0; k < TH / 32; k++) {
    t += red[0][k];
    m = max(m, red[1][k]);
  }
  *sum = t;
  *vmax = m;
}

// Last-block detection (threadfence reduction pattern). Returns true in the
// block that finished last; that block then sees every block's writes.
__device__ bool last_block(Ctl* ctl, int nblk) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(&ctl->ticket, 1u);
    is_last = (t == (unsigned)nblk - 1);
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}

// ------------------------------------------------------------------ RNG
// Whole block: when the generator is exhausted, refill its 624 words with the
// MT19937 recurrence in four phases, each of which only reads words that no
// thread of the same phase writes (old words k, k+1 and either old k+397 or
// new k-227). Bit-identical to the sequential twist.
__device__ void block_twist(MT* g);
__device__ void block_twist_if_needed(MT* g) {
  __shared__ int need;
  __syncthreads();
  if (threadIdx.x == 0) need = g->mti >= 624;
  __syncthreads();
  if (need) block_twist(g);
}

// The refill itself (whole block, unconditional).
__device__ void block_twist(MT* g) {
  const uint32_t UP = 0x80000000u, LO = 0x7fffffffu, A = 0x9908b0dfu;
  uint32_t* mt = g->mt;
  const int k0[4] = {0, 227, 454, 623}, k1[4] = {227, 454, 623, 624};
  for (int ph = 0; ph < 4; ph++) {
    const int k = k0[ph] + (int)threadIdx.x;
    uint32_t v = 0;
    const bool mine = k < k1[ph];
    if (mine) {
      const uint32_t y = (mt[k] & UP) | (mt[k == 623 ? 0 : k + 1] & LO);
      const uint32_t src = k < 227 ? mt[k + 397] : mt[k - 227];
      v = src ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
    }
    __syncthreads();
    if (mine) mt[k] = v;
    __syncthreads();
  }
  if (threadIdx.x == 0) g->mti = 0;
  __syncthreads();
}

// Second level of the rate sums: the last block of each group of kGroup
// blocks reduces the group's per-(mode, block) sums to per-(mode, group) sums
// with a fixed warp butterfly (every lane ends with the same bits). Returns
// true in that block.
__device__ bool group_reduce(const KParams& kp, const Fields& f, int b) {
  __shared__ bool is_last;
  const int g = b / kGroup;
  const int g0 = g * kGroup, g1 = min(g0 + kGroup, kp.nblk);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(&f.gticket[g], 1u);
    is_last = (t == (unsigned)(g1 - g0 - 1));
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int m = w; m < STZ_MODES; m += TH / 32) {
    double v = (g0 + lane < g1) ? f.part[(long long)m * kp.nblk + g0 + lane] : 0.0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL, v, off);
    if (lane == 0) f.gsum[(long long)m * kp.ngroups + g] = v;
  }
  if (threadIdx.x == 0) f.gticket[g] = 0;
  return true;
}

// ----------------------------------------------------------- selection
// Rate of (site, mode) exactly as the main pass computed it (raw units).
template <int MODEL>
__device__ __forceinline__ double site_rate(const KParams& kp, const Fields& f, const double* u, double totime,
                                            long long s, int m) {
  if (MODEL == 0) {
    const R2Site d = r2_load(kp, f, u, totime, s);
    return kp.vt * exp_tang(r2_arg(kp, f, d, s, m));
  } else if (MODEL == 1) {
    double sg[6];
    g3_load(kp, f, u, s, sg);
    return kp.vt * exp_tang(g3_arg(kp, g3_arg_site(kp, sg, f.dF[s]), m));
  } else {
    float sv[5];
    mx_site(kp, f, s, sv);
    const float a = (kp.q_ref - f.dF32[s]) * kp.a_scale;
    return (double)ex2_approx(mx_x(kp, sv, a, m));
  }
}

// Q of (site, mode) for the log (FP64 from the stored field).
template <int MODEL>
__device__ double site_Q(const KParams& kp, const Fields& f, const double* u, double totime, long long s, int m) {
  if (MODEL == 0) {
    const R2Site d = r2_load(kp, f, u, totime, s);
    return r2_Q(kp, f, d, s, m);
  } else if (MODEL == 1) {
    double sg[6];
    g3_load(kp, f, u, s, sg);
    return g3_Q(kp, sg, f.dF[s], m);
  } else {
    float sv[5];
    mx_site(kp, f, s, sv);
    const float a = (kp.q_ref - f.dF32[s]) * kp.a_scale;
    return (double)kp.q_ref - (double)mx_x(kp, sv, a, m) / (double)kp.a_scale;
  }
}

// Hierarchical search of the (mode, site) whose cumulative rate, in the
// reference's mode-major order m*N + s, first reaches T. Level 1: the
// per-(mode, block) sums, one contiguous chunk per thread, whose inclusive
// scan the caller left in sh_inc; level 2: the rates of the chosen mode in the
// chosen block, recomputed into registers and scanned. Whole block.
template <int MODEL>
__device__ void search_event(const KParams& kp, const Fields& f, const double* u, double totime, double T,
                             const double* sh_inc, long long* site_out, int* mode_out, double* margin_out) {
  __shared__ double sh_inc2[TH];
  __shared__ long long sh_p;
  __shared__ double sh_cb;
  __shared__ long long sh_site;
  __shared__ double sh_margin;
  const int t = threadIdx.x;
  const long long P = (long long)STZ_MODES * kp.ngroups;
  const long long ch = (P + TH - 1) / TH;
  const long long p0 = t * ch, p1 = min(p0 + ch, P);
  if (t == 0) { sh_p = -1; sh_site = -1; sh_margin = 0; }
  __syncthreads();
  const double I = sh_inc[t];
  const double E = t > 0 ? sh_inc[t - 1] : 0.0;
  const double Ttot = sh_inc[TH - 1];
  double Tq = T;
  if (Tq > Ttot) Tq = Ttot;
  if (E < Tq && Tq <= I) {
    double run = E;
    long long hit = -1, lastpos = -1;
    double hb = E, lastbefore = E;
    for (long long q = p0; q < p1; q++) {
      const double v = f.gsum[q];
      const double before = run;
      run += v;
      const bool pos = v > 0;
      if (pos) { lastpos = q; lastbefore = before; }
      if (hit < 0 && pos && run >= Tq) { hit = q; hb = before; }
    }
    if (hit < 0) { hit = lastpos; hb = lastbefore; }
    sh_p = hit;
    sh_cb = hb;
  }
  __syncthreads();
  const long long pg = sh_p;
  if (pg < 0) {
    if (t == 0) { *site_out = -1; *mode_out = -1; }
    return;
  }
  const int m = (int)(pg / kp.ngroups);
  const int g = (int)(pg - (long long)m * kp.ngroups);
  // level 1.5: the blocks of group g for mode m, one warp
  if (t < 32) {
    const int g0 = g * kGroup, g1 = min(g0 + kGroup, kp.nblk);
    const double v = (g0 + t < g1) ? f.part[(long long)m * kp.nblk + g0 + t] : 0.0;
    double x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const double y = __shfl_up_sync(FULL, x, off);
      if (t >= off) x += y;
    }
    const double before = __shfl_up_sync(FULL, x, 1);
    const double ex = t > 0 ? before : 0.0;
    const double Tg = Tq - sh_cb;
    const unsigned ok = __ballot_sync(FULL, v > 0 && x >= Tg);
    const unsigned posb = __ballot_sync(FULL, v > 0);
    int lane = ok ? __ffs(ok) - 1 : (posb ? 31 - __clz(posb) : -1);
    if (lane >= 0) {
      const double exl = __shfl_sync(FULL, ex, lane);
      if (t == 0) {
        sh_p = g0 + lane;
        sh_cb = sh_cb + exl;
      }
    } else if (t == 0) {
      sh_p = -1;
    }
  }
  __syncthreads();
  if (sh_p < 0) {
    if (t == 0) { *site_out = -1; *mode_out = -1; }
    return;
  }
  const int b = (int)sh_p;
  double T2 = Tq - sh_cb;
  const long long s0 = (long long)b * kp.bsites;
  const long long s1 = min(s0 + (long long)kp.bsites, kp.N);
  const long long per = (s1 - s0 + TH - 1) / TH;
  const long long a0 = s0 + t * per;
  constexpr int kMaxPer = kSptFp64;  // sites per thread
  double rr[kMaxPer];
  double loc = 0;
#pragma unroll
  for (int k = 0; k < kMaxPer; k++) {
    const long long s = a0 + k;
    rr[k] = (k < per && s < s1) ? site_rate<MODEL>(kp, f, u, totime, s, m) : 0.0;
    loc += rr[k];
  }
  const double I2 = block_incl_scan(loc, sh_inc2);
  const double E2 = t > 0 ? sh_inc2[t - 1] : 0.0;
  const double tot2 = sh_inc2[TH - 1];
  if (T2 > tot2) T2 = tot2;
  if (!(T2 > 0)) T2 = DBL_MIN;
  if (E2 < T2 && T2 <= I2) {
    double run = E2;
    int hit = -1, lastk = -1;
    double hb = E2, ha = E2, lb = E2, la = E2;
#pragma unroll
    for (int k = 0; k < kMaxPer; k++) {
      const double before = run;
      run += rr[k];
      const bool pos = rr[k] > 0;
      if (pos) { lastk = k; lb = before; la = run; }
      if (hit < 0 && pos && run >= T2) { hit = k; hb = before; ha = run; }
    }
    if (hit < 0) { hit = lastk; hb = lb; ha = la; }
    sh_site = hit < 0 ? -1 : a0 + hit;
    sh_margin = fmin(T2 - hb, ha - T2);
  }
  __syncthreads();
  if (t == 0) {
    *site_out = sh_site;
    *mode_out = m;
    *margin_out = sh_margin;
  }
}

// ------------------------------------------------------------ commits
// VoxelShearTransform (elastic.c:361-520) for the FP64 models; thread 0 only.
template <int MODEL>
__device__ void transform(const KParams& kp, const Fields& f, Ctl* ctl, int mm, long long s, MT* rng) {
  const long long N = kp.N;
  double d[6];
  if (MODEL == 0) {
    const double* dd = f.deps + (long long)mm * 3 * N;
    d[0] = dd[s]; d[1] = dd[N + s]; d[2] = dd[2 * N + s];
  } else {
    for (int c = 0; c < 6; c++) d[c] = kp.modes[mm][c];
  }
  for (int c = 0; c < kp.nc; c++) {
    f.prev_deps[c * N + s] = d[c];
    f.eps0[c * N + s] += d[c];
    ctl->eps0_sum[c] += d[c];
    ctl->pend_deps[c] = d[c];
  }
  if (MODEL == 0) {
    const int ty = f.mro ? f.mro[s] : 0;
    const double ds = d[0] * d[0] + d[1] * d[1] + 2 * d[2] * d[2];
    double ps = f.perm_soft[s] + ds * (ty == 1 ? kp.perm_soft_mro : kp.perm_soft);
    if (ps > kp.perm_soft_cap) ps = kp.perm_soft_cap;
    f.perm_soft[s] = ps;
    f.temp_soft[s] = ds * (ty == 1 ? kp.temp_soft_mro : kp.temp_soft);
    f.tlast[s] = ctl->totime;
    if (ty) {
      // a crystal-like site keeps its modes and draws new barriers
      // xQ0amp (1 - RandomRatio + RandomRatio u) (elastic.c:451-500)
      for (int i = 0; i < STZ_MODES; i++) {
        const double u = mt_uniform(rng);
        f.Q0[(long long)i * N + s] =
            __dmul_rn(kp.xq0amp, __dadd_rn(1.0 - kp.random_ratio, __dmul_rn(kp.random_ratio, u)));
      }
      return;
    }
    // re-draw the site's modes, glass branch (elastic.c:508-512)
    for (int i = 0; i < STZ_MODES; i++) {
      double* dd = f.deps + (long long)i * 3 * N;
      const double a = 0.5 * kp.gamma0 * mt_gaussian(rng, 1.0);
      const double c2 = 0.5 * kp.gamma0 * mt_gaussian(rng, 1.0);
      dd[s] = a;
      dd[N + s] = -a;
      dd[2 * N + s] = c2;
      f.dnorm[(long long)i * N + s] = mode_rnorm(a, -a, c2);
    }
  }
}

// Block copy of the control block between global and shared memory: the
// last block does its sequential bookkeeping on the shared copy (the global
// one would cost an L2 round trip per field access).
__device__ __forceinline__ void ctl_copy(Ctl* dst, const Ctl* src) {
  const uint32_t* a = reinterpret_cast<const uint32_t*>(src);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(Ctl) / 4); i += blockDim.x) d[i] = a[i];
}

// Last block of a rate kernel: total rate, step kind, dice, event search and
// commit. MODEL 0 REF2D FP64, 1 GLOBAL3D FP64.
template <int MODEL>
__device__ void finish_step(const KParams& kp, const Fields& f) {
  __shared__ Ctl sc;
  __shared__ double sh_inc[TH];
  __shared__ int sh_kind;
  __shared__ double sh_T, sh_R;
  __shared__ double sh_u[6];
  __shared__ double sh_tot;
  __shared__ long long sh_site;
  __shared__ int sh_mode;
  __shared__ double sh_margin;
  const unsigned long long t_tail = gtimer();
  Ctl* const g = f.ctl;
  ctl_copy(&sc, g);
  // per-thread contiguous chunks of the per-(mode, group) sums, fixed order
  const long long P = (long long)STZ_MODES * kp.ngroups;
  const long long ch = (P + TH - 1) / TH;
  const long long p0 = threadIdx.x * ch, p1 = min(p0 + ch, P);
  double S = 0;
  for (long long p = p0; p < p1; p++) S += f.gsum[p];
  block_incl_scan(S, sh_inc);  // also orders the copy above
  const unsigned long long t_sums = gtimer();
  if (MODEL != 0) block_twist_if_needed(&sc.rng);
  Ctl* c = &sc;
  if (threadIdx.x == 0) {
    c->ticket = 0;
    c->step++;
    const double Rraw = sh_inc[TH - 1];
    const double R = Rraw;
    sh_R = Rraw;
    for (int k = 0; k < 6; k++) sh_u[k] = c->u[k];
    sh_tot = c->totime;
    c->total_rate = R;
    int kind;
    if (c->neg_count > 0) {
      kind = kAthermal;
    } else if (!(R > 0) || !isfinite(R)) {
      kind = kNone;
      c->status = STZ_ERR_NAN;
      c->halt = 1;
      c->halt_reason = kHaltError;
    } else {
      const double t_kmc = 1 / R;
      if (t_kmc < kp.dt) {
        kind = kThermal;
        c->kstep++;
        const double dice = mt_uniform(&c->rng);
        sh_T = dice * Rraw;
        c->t_kmc = t_kmc;
        if (!(dice > 0)) {
          kind = kNone;
          c->status = STZ_ERR_NO_EVENT;
          c->halt = 1;
          c->halt_reason = kHaltError;
        }
      } else {
        kind = kElastic;
      }
    }
    c->neg_count = 0;
    c->step_kind = kind;
    sh_kind = kind;
  }
  __syncthreads();
  const unsigned long long t_dec = gtimer();
  const int kind = sh_kind;
  if (kind == kThermal) {
    search_event<MODEL>(kp, f, sh_u, sh_tot, sh_T, sh_inc, &sh_site, &sh_mode, &sh_margin);
    __syncthreads();
  }
  const unsigned long long t_search = gtimer();
  if (threadIdx.x == 0) {
    const double Rtrue = sh_R;
    if (kind == kThermal) {
      const long long s = sh_site;
      const int m = sh_mode;
      if (s < 0) {
        c->status = STZ_ERR_NO_EVENT;
        c->halt = 1;
        c->halt_reason = kHaltError;
        c->step_kind = kNone;
      } else {
        if (sh_margin < 1e-12 * sh_R) c->near_ties++;
        const double q = site_Q<MODEL>(kp, f, sh_u, sh_tot, s, m);
        c->sel_site = s;
        c->sel_mode = m;
        c->sel_q = q;
        transform<MODEL>(kp, f, c, m, s, &c->rng);
        if (kp.incr64) {
          c->incr_req = 1;  // the incremental update instead of the re-solve
          c->pend_site = s;
        } else {
          c->solve_req = 1;
        }
        log_event(kp, f, c, STZ_EV_THERMAL, s, m, c->totime + c->t_kmc, c->t_kmc, q, Rtrue, sh_margin / sh_R, 1);
      }
    } else if (kind == kElastic) {
      c->estep++;
      c->totime += kp.dt;
      elastic_step(kp, c);
      c->solve_req = 0;
      log_event(kp, f, c, STZ_EV_ELASTIC, -1, -1, c->totime, kp.dt, 0.0, Rtrue);
    } else if (kind == kAthermal) {
      c->solve_req = 0;  // the athermal commit requests the solve
    }
  }
  __syncthreads();
  ctl_copy(g, &sc);
}

// ------------------------------------------------------------ FP64 rates
template <int MODEL>
__global__ void __launch_bounds__(TH) k_rate64(KParams kp, Fields f) {
  Ctl* ctl = f.ctl;
  if (ctl->halt) return;
  const int b = blockIdx.x;
  const long long s0 = (long long)b * kp.bsites;
  const long long s1 = min(s0 + (long long)kp.bsites, kp.N);
  double u[6];
  for (int c = 0; c < 6; c++) u[c] = ctl->u[c];
  const double totime = ctl->totime;
  double acc[STZ_MODES];
#pragma unroll
  for (int m = 0; m < STZ_MODES; m++) acc[m] = 0;
  unsigned neg = 0;
  for (long long s = s0 + threadIdx.x; s < s1; s += TH) {
    if (MODEL == 0) {
      const R2Site d = r2_load(kp, f, u, totime, s);
#pragma unroll 4
      for (int m = 0; m < STZ_MODES; m++) {
        const double x = r2_arg(kp, f, d, s, m);
        neg += arg_positive(x);
        acc[m] += kp.vt * exp_tang(x);
      }
    } else {
      double sg[6];
      g3_load(kp, f, u, s, sg);
      const G3Arg a = g3_arg_site(kp, sg, f.dF[s]);
#pragma unroll 4
      for (int m = 0; m < STZ_MODES; m++) {
        const double x = g3_arg(kp, a, m);
        neg += arg_positive(x);
        acc[m] += kp.vt * exp_tang(x);
      }
    }
  }
  block_mode_sums(acc, f.part, kp.nblk, b);
  const unsigned nb = block_sum_u(neg);
  if (threadIdx.x == 0 && nb) atomicAdd(&ctl->neg_count, (unsigned long long)nb);
  if (!group_reduce(kp, f, b)) return;
  if (!last_block(ctl, kp.ngroups)) return;
  finish_step<MODEL>(kp, f);
}

// ------------------------------------------------------------ athermal
// Mark every site whose lowest-barrier mode has Q < 0 or |Q| < 0.33
// (evolution.c:55-65). mixed: Q from the FP32 deviatoric field.
__global__ void k_ath_mark(KParams kp, Fields f, int mixed) {
  Ctl* ctl = f.ctl;
  if (ctl->step_kind != kAthermal) return;
  double u[6];
  for (int c = 0; c < 6; c++) u[c] = ctl->u[c];
  const double totime = ctl->totime;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < kp.N; s += (long long)gridDim.x * blockDim.x) {
    int mm = 0;
    double minQ = 0;
    for (int m = 0; m < STZ_MODES; m++) {
      double Q;
      if (kp.model == STZ_MODEL_REF2D) Q = site_Q<0>(kp, f, u, totime, s, m);
      else if (mixed) Q = site_Q<2>(kp, f, u, totime, s, m);
      else Q = site_Q<1>(kp, f, u, totime, s, m);
      if (m == 0 || minQ > Q) { mm = m; minQ = Q; }
    }
    f.amark[s] = (minQ < 0 || fabs(minQ) < 0.33) ? (signed char)(mm + 1) : (signed char)0;
  }
}

// Transform the marked sites in index order (the RNG stream order of the
// reference's space_loop); one block, thread 0 commits.
__global__ void k_ath_commit(KParams kp, Fields f, int mixed) {
  Ctl* ctl = f.ctl;
  if (ctl->step_kind != kAthermal) return;
  __shared__ unsigned ballot[TH / 32];
  __shared__ MT srng;
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&ctl->rng);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&srng);
    for (int i = threadIdx.x; i < (int)(sizeof(MT) / 4); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  double u[6];
  for (int c = 0; c < 6; c++) u[c] = ctl->u[c];
  const double totime = ctl->totime;
  if (threadIdx.x == 0) ctl->astep++;
  for (long long base = 0; base < kp.N; base += TH) {
    const long long s = base + threadIdx.x;
    const bool mk = s < kp.N && f.amark[s] != 0;
    const unsigned bal = __ballot_sync(FULL, mk);
    if ((threadIdx.x & 31) == 0) ballot[threadIdx.x >> 5] = bal;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 0; w < TH / 32; w++) {
        unsigned bb = ballot[w];
        while (bb) {
          const int lane = __ffs(bb) - 1;
          bb &= bb - 1;
          const long long site = base + w * 32 + lane;
          const int mm = f.amark[site] - 1;
          double q;
          if (kp.model == STZ_MODEL_REF2D) q = site_Q<0>(kp, f, u, totime, site, mm);
          else if (mixed) q = site_Q<2>(kp, f, u, totime, site, mm);
          else q = site_Q<1>(kp, f, u, totime, site, mm);
          if (kp.model == STZ_MODEL_REF2D) transform<0>(kp, f, ctl, mm, site, &srng);
          else transform<1>(kp, f, ctl, mm, site, &srng);
          log_event(kp, f, ctl, STZ_EV_ATHERMAL, site, mm, ctl->totime, 0.0, q, 0.0);
        }
      }
    }
    __syncthreads();
  }
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&srng);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&ctl->rng);
    for (int i = threadIdx.x; i < (int)(sizeof(MT) / 4); i += blockDim.x) dst[i] = src[i];
  }
  if (threadIdx.x == 0) ctl->solve_req = 1;
}

// ------------------------------------------------------------ post steps
// One block of TH threads: the field mean by the block, the rest by thread 0.
__global__ void k_post_a(KParams kp, Fields f) {
  Ctl* ctl = f.ctl;
  if (ctl->halt && ctl->step_kind == kNone) return;
  const int kind = ctl->step_kind;
  // the mean of the solved field; after an incremental update, C:(ebar - <eps*>)
  // of the same linear solve
  const bool fieldmean = f.msum != nullptr && !(kp.incr64 && kind == kThermal);
  if ((kind == kThermal || kind == kAthermal) && fieldmean) field_mean_stress(kp, f, ctl->stress);
  if (threadIdx.x != 0) return;
  if (kind == kThermal) {
    if (!fieldmean) solved_mean_stress(kp, ctl, ctl->eps_avg, ctl->stress);
    for (int c = 0; c < 6; c++) ctl->u[c] = 0;
    load_after_event(kp, ctl, ctl->t_kmc);
    ctl->totime += ctl->t_kmc;
  } else if (kind == kAthermal) {
    if (!fieldmean) solved_mean_stress(kp, ctl, ctl->eps_avg, ctl->stress);
    for (int c = 0; c < 6; c++) ctl->u[c] = 0;
    if (kp.loading == STZ_LOAD_STRESS) {
      hold_stress(kp, ctl);
    } else {
      double ts[6];
      subtract_error(kp, ctl, 1, ts);
      for (int c = 0; c < kp.nc; c++) ctl->eps_avg[c] -= ts[c];
    }
  } else {
    ctl->solve_req = 0;
    return;
  }
  ctl->print_done = 0;
  ctl->solve_req = 0;
}

// FP64 incremental form, after a thermal event: the field the re-solve would
// give, from its linearity in the eigenstrain and the mean strain. Each site r
// gains sum_k d_k R_k(r - s) over the strain components k of the site's
// increment d (the unit responses of rtab64, shifted to the transformed site
// s) and C:(ebar - ebar_solved), the mean strain's change since the stored
// field was solved.
__global__ void k_incr64(KParams kp, Fields f) {
  const Ctl* ctl = f.ctl;
  if (!ctl->incr_req) return;
  const int nc = kp.nc, nd = nc == 3 ? 2 : 3;
  const long long N = kp.N;
  double d[6], dU[6], dE[6];
  for (int c = 0; c < nc; c++) {
    d[c] = ctl->pend_deps[c];
    dE[c] = ctl->eps_avg[c] - ctl->ebar_solved[c];
  }
  double tr = 0;
  for (int c = 0; c < nd; c++) tr += dE[c];
  for (int c = 0; c < nc; c++) dU[c] = (c < nd ? kp.lambda * tr : 0.0) + 2.0 * kp.mu * dE[c];
  const long long sp = ctl->pend_site;
  const int a2 = (int)(sp % kp.n2), a1 = (int)((sp / kp.n2) % kp.n1), a0 = (int)(sp / ((long long)kp.n2 * kp.n1));
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (long long)gridDim.x * blockDim.x) {
    const int r2 = (int)(r % kp.n2), r1 = (int)((r / kp.n2) % kp.n1), r0 = (int)(r / ((long long)kp.n2 * kp.n1));
    int o0 = r0 - a0, o1 = r1 - a1, o2 = r2 - a2;
    o0 += o0 < 0 ? kp.n0 : 0;
    o1 += o1 < 0 ? kp.n1 : 0;
    o2 += o2 < 0 ? kp.n2 : 0;
    const long long o = ((long long)o0 * kp.n1 + o1) * kp.n2 + o2;
    for (int c = 0; c < nc; c++) {
      double acc = dU[c];
      for (int k = 0; k < nc; k++) acc = __fma_rn(d[k], __ldg(&f.rtab64[((long long)k * nc + c) * N + o]), acc);
      f.sig[c * N + r] += acc;
    }
  }
}

// the update is in the field: it now holds the solve at the current mean strain
__global__ void k_incr64_done(Fields f) {
  Ctl* ctl = f.ctl;
  if (!ctl->incr_req) return;
  for (int c = 0; c < 6; c++) ctl->ebar_solved[c] = ctl->eps_avg[c];
  ctl->incr_req = 0;
}

// an FFT solve (when its gate was set) leaves the field at the mean strain ebar
__global__ void k_note_solve(Fields f, const int* gate, const double* ebar) {
  if (gate && !*gate) return;
  for (int c = 0; c < 6; c++) f.ctl->ebar_solved[c] = ebar[c];
}

// print check after every step kind; requests the print re-solve
__global__ void k_post_print(KParams kp, Fields f) {
  Ctl* ctl = f.ctl;
  if (ctl->step_kind == kNone) return;
  ctl->print_done = print_check(kp, ctl);
  ctl->solve_req = ctl->print_done;
}

// The print's reset of the barriers to their initial copy (bmg.c:214-221),
// when this step printed. Only REF2D grids with crystal-like sites have Q1.
__global__ void k_q0_reset(KParams kp, Fields f) {
  if (!f.ctl->print_done || f.ctl->step_kind == kNone) return;
  const long long total = (long long)STZ_MODES * kp.N;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    f.Q0[i] = f.Q1[i];
}

// One block of TH threads, as k_post_a.
__global__ void k_post_b(KParams kp, Fields f) {
  Ctl* ctl = f.ctl;
  if (ctl->step_kind == kNone) return;
  if (ctl->print_done && f.msum) field_mean_stress(kp, f, ctl->stress);
  if (threadIdx.x != 0) return;
  if (ctl->print_done) {
    if (!f.msum) solved_mean_stress(kp, ctl, ctl->eps_avg, ctl->stress);
    for (int c = 0; c < 6; c++) ctl->u[c] = 0;
  }
  ctl->print_done = 0;
  ctl->solve_req = 0;
  ctl->step_kind = kNone;
  stop_check(kp, ctl);
  (void)f;
}

// ------------------------------------------------------------ mixed form
__device__ __forceinline__ int fold(int d, int n, int* flip) {
  if (d < 0) d += n;
  if (2 * d > n) { *flip = 1; return n - d; }
  *flip = 0;
  return d;
}

// ---------------------------------------------------- mixed-form main pass
// Work decomposition. A line of the grid is (i0, i1) with its n2 contiguous
// sites; one warp owns one line, lane l its sites i2 = l, l + 32, ... Lines
// are grouped by their folded distance (d0, d1) to the transformed site p:
// the lines (p0 +- d0, p1 +- d1) read the same row (d0, d1, *) of the response
// table, and each record of a row twice along a line, so a unit of up to eight
// lines (one d0, d1 in {2c, 2c + 1}, both signs of each) fetches each record
// of its two rows from L2 once and serves the other reads from L1. Unit
// u = d0 * mx_c1 + c; warp w of the unit takes sign0 = w & 1, d1 = 2c + (w >> 1
// & 1), sign1 = w >> 2, and idles where that line coincides with another one
// (d = 0 or d = n/2) or d1 is past the table. Every line belongs to exactly
// one (unit, warp).
struct LineOf {
  int i0, i1, valid;
};

// The per-replica constants and field pointers of the main pass, copied to
// registers at the block's start: read through the KParams / Fields in shared
// memory of the batched kernel, every use would be a reload after each
// shared-memory store of the loop.
struct MixK {
  int n0, n1, n2, kt1, kt2, mx_c1, mx_units, nblk;
  unsigned c1_magic;  // ceil(2^32 / mx_c1): u / mx_c1 = umulhi(u, c1_magic) for u < 2^22
  long long N;
  float q_ref, a_scale, inv_kt;
  float* sdev;
  const float* dF32;
  const float* ktab;
  float* lsum;
};

__device__ __forceinline__ int wrap1(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

__device__ __forceinline__ LineOf unit_line(const MixK& kp, int u, int w, int p0, int p1) {
  const int d0 = (int)__umulhi((unsigned)u, kp.c1_magic), c = u - d0 * kp.mx_c1;
  const int s0 = w & 1, s1 = w >> 2;
  const int d1 = 2 * c + ((w >> 1) & 1);
  LineOf L;
  L.valid = d1 < kp.kt1 && (!s0 || (d0 != 0 && 2 * d0 != kp.n0)) && (!s1 || (d1 != 0 && 2 * d1 != kp.n1));
  L.i0 = wrap1(s0 ? p0 - d0 : p0 + d0, kp.n0);
  L.i1 = wrap1(s1 ? p1 - d1 : p1 + d1, kp.n1);
  return L;
}

// Stress update of one site (sv holds its coordinates): the pending
// transformation's response S K(|x - p|) S de (S the reflection signs, K the
// folded table record whose chunks are rec[0], rec[kt2], rec[2 kt2],
// rec[3 kt2]) plus the uniform change Ud; stores the new
// coordinates and leaves them in sv. dl holds
// de (5), then the sign of coordinate 2 (y z) and the z and y flips that,
// times the site's x flip sx, give the signs of coordinates 3 (x z) and 4 (x y).
__device__ __forceinline__ void mixed_update(float* sdev, int N32, int s, int hp, const float4* rec, int kt2,
                                             float sx, const float* dl, const float* Ud, float* sv) {
  if (hp) {
    const float4 q0 = __ldg(rec), q1 = __ldg(rec + kt2), q2 = __ldg(rec + 2 * kt2), q3 = __ldg(rec + 3 * kt2);
    const float K[16] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w,
                         q2.x, q2.y, q2.z, q2.w, q3.x, q3.y, q3.z, q3.w};
    const float g2 = dl[5], g3 = dl[6] * sx, g4 = dl[7] * sx;
    const float e[5] = {dl[0], dl[1], dl[2] * g2, dl[3] * g3, dl[4] * g4};
    // symmetric 5x5 from the packed upper triangle (row-major, a <= b)
    const float y0 = K[0] * e[0] + K[1] * e[1] + K[2] * e[2] + K[3] * e[3] + K[4] * e[4];
    const float y1 = K[1] * e[0] + K[5] * e[1] + K[6] * e[2] + K[7] * e[3] + K[8] * e[4];
    const float y2 = K[2] * e[0] + K[6] * e[1] + K[9] * e[2] + K[10] * e[3] + K[11] * e[4];
    const float y3 = K[3] * e[0] + K[7] * e[1] + K[10] * e[2] + K[12] * e[3] + K[13] * e[4];
    const float y4 = K[4] * e[0] + K[8] * e[1] + K[11] * e[2] + K[13] * e[3] + K[14] * e[4];
    // the small increments are added together first, so the field takes one
    // rounding per event
    sv[0] += y0 + Ud[0];
    sv[1] += y1 + Ud[1];
    sv[2] += __fmaf_rn(g2, y2, Ud[2]);
    sv[3] += __fmaf_rn(g3, y3, Ud[3]);
    sv[4] += __fmaf_rn(g4, y4, Ud[4]);
  } else {
#pragma unroll
    for (int k = 0; k < 5; k++) sv[k] += Ud[k];
  }
#pragma unroll
  for (int k = 0; k < 5; k++) sdev[k * N32 + s] = sv[k];
}

// The 20 rates of one site (a lane whose pair partner is past the line).
// TRACK: also the largest argument in *xma.
template <int TRACK>
__device__ __forceinline__ void mixed_rates1(const float* sa, float aa, float ct, const float2* md, float2* acc2,
                                             float* xma) {
  float mx = -INFINITY;
  float ta[5];
#pragma unroll
  for (int k = 0; k < 5; k++) ta[k] = __fmul_rn(sa[k], ct);
#pragma unroll
  for (int j = 0; j < STZ_MODES / 2; j++) {
    float2 xa = make_float2(aa, aa);
#pragma unroll
    for (int k = 0; k < 5; k++) xa = __ffma2_rn(make_float2(ta[k], ta[k]), md[5 * j + k], xa);
    acc2[j] = __fadd2_rn(acc2[j], make_float2(ex2_approx(xa.x), ex2_approx(xa.y)));
    if (TRACK) mx = fmaxf(mx, fmaxf(xa.x, xa.y));
  }
  if (TRACK) *xma = mx;
}

// The 20 rates of two sites (b may be absent), packed two modes per FP32x2
// FMA after scaling the stress coordinates by ct = 1/kT; each lane of a pair
// is the scalar chain of mx_x, so the search sees the same bits. One load of
// each mode coefficient serves both sites. TRACK: also the largest argument
// of site a in *xma and of site b in *xmb (an argument above q_ref a_scale is
// a negative barrier, the athermal trigger).
template <int TRACK>
__device__ __forceinline__ void mixed_rates2(const float* sa, float aa, const float* sb, float ab, bool hb, float ct,
                                             const float2* md, float2* acc2, float* xma, float* xmb) {
  float2 mx = make_float2(-INFINITY, -INFINITY);
  float ta[5], tb[5];
#pragma unroll
  for (int k = 0; k < 5; k++) {
    ta[k] = __fmul_rn(sa[k], ct);
    tb[k] = __fmul_rn(sb[k], ct);
  }
#pragma unroll
  for (int j = 0; j < STZ_MODES / 2; j++) {
    float2 xa = make_float2(aa, aa), xb = make_float2(ab, ab);
#pragma unroll
    for (int k = 0; k < 5; k++) {
      const float2 c = md[5 * j + k];
      xa = __ffma2_rn(make_float2(ta[k], ta[k]), c, xa);
      xb = __ffma2_rn(make_float2(tb[k], tb[k]), c, xb);
    }
    acc2[j] = __fadd2_rn(acc2[j], make_float2(ex2_approx(xa.x), ex2_approx(xa.y)));
    if (hb) acc2[j] = __fadd2_rn(acc2[j], make_float2(ex2_approx(xb.x), ex2_approx(xb.y)));
    if (TRACK) {
      mx.x = fmaxf(mx.x, fmaxf(xa.x, xa.y));
      mx.y = fmaxf(mx.y, fmaxf(xb.x, xb.y));
    }
  }
  if (TRACK) {
    *xma = mx.x;
    *xmb = mx.y;
  }
}

// The 20 rates of Q sites of a lane (all inside the line), one coefficient
// pair load per Q FP32x2 FMAs; each site's lane of a pair is the scalar chain
// of mx_x, and the sums take sites 0 .. Q-1 in order.
template <int Q>
__device__ __forceinline__ void mixed_rates_q(const float (*t)[5], const float* a, const float2* md, float2* acc2) {
#pragma unroll
  for (int j = 0; j < STZ_MODES / 2; j++) {
    float2 x[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) x[q] = make_float2(a[q], a[q]);
#pragma unroll
    for (int k = 0; k < 5; k++) {
      const float2 c = md[5 * j + k];
#pragma unroll
      for (int q = 0; q < Q; q++) x[q] = __ffma2_rn(make_float2(t[q][k], t[q][k]), c, x[q]);
    }
#pragma unroll
    for (int q = 0; q < Q; q++) acc2[j] = __fadd2_rn(acc2[j], make_float2(ex2_approx(x[q].x), ex2_approx(x[q].y)));
  }
}

// Exact athermal test of one line by its warp, for the lines whose mode sums
// reach half of 2^thr (see line_sums): every site's 20 arguments recomputed
// with the chain of mixed_rates1/2 from the stored (updated) stress; true in
// a lane when one of its sites has an argument above thr. Rare: only lines
// holding a barrier within a few kT of zero get here.
__device__ __forceinline__ bool line_negative(const float* sdev, const float* dF32, int N32, int base, int n2,
                                              float q_ref, float a_scale, float ct, const float2* md, float thr) {
  bool neg = false;
#pragma unroll 1
  for (int i2 = threadIdx.x & 31; i2 < n2; i2 += 32) {
    float t[5];
#pragma unroll
    for (int k = 0; k < 5; k++) t[k] = __fmul_rn(sdev[k * N32 + base + i2], ct);
    const float a = (q_ref - dF32[base + i2]) * a_scale;
#pragma unroll 1
    for (int j = 0; j < STZ_MODES / 2; j++) {
      float x0 = a, x1 = a;
#pragma unroll
      for (int k = 0; k < 5; k++) {
        const float2 c = md[5 * j + k];
        x0 = __fmaf_rn(t[k], c.x, x0);
        x1 = __fmaf_rn(t[k], c.y, x1);
      }
      neg |= x0 > thr || x1 > thr;
    }
  }
  return neg;
}

// ------------------------------------------ bulk-copy staging of a line
// One lane of each warp copies the next line's five stress components and
// barrier (contiguous runs of n2 floats) into the warp's other stage with
// cp.async.bulk, tracked by that stage's mbarrier (expected bytes), while the
// warp computes the current line from shared memory. The copies need 16-byte
// aligned runs: n2 is a multiple of 4 for the mixed form.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait (each try_wait suspends for a hardware-chosen interval, about
// 4 us on GB300); false after `tries` attempts. kMbarTries, the kernels'
// limit, is about a second: a staged line lands within microseconds.
constexpr int kMbarTries = 1 << 18;
__device__ __forceinline__ bool mbar_wait_n(unsigned long long* bar, unsigned parity, int tries) {
  for (int it = 0; it < tries; it++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  return mbar_wait_n(bar, parity, kMbarTries);
}

// Self-test of the bounded wait: thread 0 arms an mbarrier for 16 bytes that
// no copy will deliver and waits on it with `tries` attempts, as the main
// pass waits on its staged lines; the wait runs out and the status says so.
// Nothing is in flight on the barrier, so the block may leave at once.
__global__ void k_wait_selftest(int tries, int* out) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  mbar_expect_tx(&bar, 16u);
  *out = mbar_wait_n(&bar, 0u, tries) ? STZ_OK : STZ_ERR_TIMEOUT;
}
// L2 prefetch of a contiguous run (16-byte aligned, a multiple of 16 bytes)
// by the bulk-copy unit; no completion to wait for.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Floats of one stage: 6 runs of n2 (stress, barrier); at least 32 x 20 so
// the stage just consumed can hold the line-sum transpose.
__host__ __device__ __forceinline__ int mix_stage_floats(int n2) {
  const int a = 6 * n2, r = 32 * STZ_MODES;
  return a > r ? a : r;
}
// Dynamic shared memory of a mixed-form main block: 8 warps x 2 stages.
__host__ __device__ __forceinline__ size_t mix_smem_bytes(int n2) {
  return (size_t)(TH / 32) * 2 * mix_stage_floats(n2) * sizeof(float);
}
// Run length of the single-grid main pass's stages: lines of 256 sites are
// staged and computed in two pieces of 128 (a block's stages then stay at
// 49 KB, three blocks to an SM); other lines whole.
__host__ __device__ constexpr int mix_piece(int n2) { return n2 == 256 ? 128 : n2; }
// Dynamic shared memory of a single-grid main block: the stages of its
// pieces, and for lines in pieces each thread's 20 rate sums parked between
// pieces (20 KB).
__host__ __device__ __forceinline__ size_t mix_smem_main_bytes(int n2) {
  return mix_smem_bytes(mix_piece(n2)) + (mix_piece(n2) != n2 ? (size_t)TH * STZ_MODES * sizeof(float) : 0);
}

// Stage the sites off .. off + len - 1 of line (i0, i1).
template <int UPDATE_ONLY>
__device__ __forceinline__ void issue_line(const MixK& kp, int i0, int i1, int off, int len, float* stage,
                                           unsigned long long* bar) {
  const long long base = ((long long)i0 * kp.n1 + i1) * kp.n2 + off;
  const unsigned bytes = (unsigned)len * 4u;
  // the generic-proxy reads and writes of this stage are done (syncwarp by
  // the caller); order them before the asynchronous writes
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect_tx(bar, (UPDATE_ONLY ? 5u : 6u) * bytes);
#pragma unroll
  for (int k = 0; k < 5; k++) bulk_g2s(stage + k * len, kp.sdev + (long long)k * kp.N + base, bytes, bar);
  if (!UPDATE_ONLY) bulk_g2s(stage + 5 * len, kp.dF32 + base, bytes, bar);
}

// One line (i0, i1), or its piece h of mix_piece(N2) sites, by one warp from
// its staged inputs: update every site, and (unless UPDATE_ONLY) accumulate
// the lane's 20 rate sums in acc2. Unless LINEVOTE (the athermal test is then
// made per line from the mode sums), set neg when a site's largest argument
// exceeds thr_neg.
template <int UPDATE_ONLY, int LINEVOTE, int N2>
__device__ __forceinline__ void mixed_line(const MixK& kp, int N32, int hp, int i0, int i1, int h,
                                           int p0, int p1, int p2, const float* de, const float* Ud,
                                           const float2* md, const float* stage, float2* acc2, unsigned& neg,
                                           float thr_neg) {
  const int lane = threadIdx.x & 31;
  const int n2 = N2 > 0 ? N2 : kp.n2;
  int fz, fy;
  const int d0 = fold(i0 - p0, kp.n0, &fz);
  const int d1 = fold(i1 - p1, kp.n1, &fy);
  const float4* row = reinterpret_cast<const float4*>(kp.ktab) + 4LL * ((d0 * kp.kt1 + d1) * kp.kt2);
  // per-line signs: coordinate 2 takes y z, 3 takes x z, 4 takes x y; the x
  // flip varies along the line and is applied per site
  const float sy = fy ? -1.f : 1.f, sz = fz ? -1.f : 1.f;
  float dl[8];
#pragma unroll
  for (int k = 0; k < 5; k++) dl[k] = de[k];
  dl[5] = sy * sz;
  dl[6] = sz;
  dl[7] = sy;
  const int base = (i0 * kp.n1 + i1) * n2;
  if constexpr (N2 > 0 && LINEVOTE && !UPDATE_ONLY) {
    // each lane's sites lane + 32 q of the piece in one pass; offsets are
    // immediates
    constexpr int kKt2 = N2 / 2 + 1, kP = mix_piece(N2), kQ = kP / 32;
    float t[kQ][5], a[kQ];
#pragma unroll
    for (int q = 0; q < kQ; q++) {
      const int si = lane + 32 * q, i2 = si + kP * h;
      int fx;
      const int d2 = fold(i2 - p2, N2, &fx);
      float sv[5];
#pragma unroll
      for (int k = 0; k < 5; k++) sv[k] = stage[k * kP + si];
      mixed_update(kp.sdev, N32, base + i2, hp, row + d2, kKt2, fx ? -1.f : 1.f, dl, Ud, sv);
#pragma unroll
      for (int k = 0; k < 5; k++) t[q][k] = __fmul_rn(sv[k], kp.inv_kt);
      a[q] = (kp.q_ref - stage[5 * kP + si]) * kp.a_scale;
    }
    mixed_rates_q<kQ>(t, a, md, acc2);
    return;
  }
  for (int i2 = lane; i2 < n2; i2 += 64) {
    const int i2b = i2 + 32;
    const bool hb = i2b < n2;
    float sa[5], sb[5];
    {
      int fx;
      const int d2 = fold(i2 - p2, n2, &fx);
#pragma unroll
      for (int k = 0; k < 5; k++) sa[k] = stage[k * n2 + i2];
      mixed_update(kp.sdev, N32, base + i2, hp, row + d2, kp.kt2, fx ? -1.f : 1.f, dl, Ud, sa);
    }
    if (hb) {
      int fx;
      const int d2 = fold(i2b - p2, n2, &fx);
#pragma unroll
      for (int k = 0; k < 5; k++) sb[k] = stage[k * n2 + i2b];
      mixed_update(kp.sdev, N32, base + i2b, hp, row + d2, kp.kt2, fx ? -1.f : 1.f, dl, Ud, sb);
    } else {
#pragma unroll
      for (int k = 0; k < 5; k++) sb[k] = sa[k];
    }
    if (!UPDATE_ONLY) {
      const float dFa = stage[5 * n2 + i2];
      const float dFb = hb ? stage[5 * n2 + i2b] : dFa;
      const float aa = (kp.q_ref - dFa) * kp.a_scale, ab = (kp.q_ref - dFb) * kp.a_scale;
      float xma = -INFINITY, xmb = -INFINITY;
      // lines of 32 and the last third of 96: no lane has a partner. The vote
      // is among the lanes executing here (lines shorter than 32 leave some
      // outside the loop); a lane takes the single-site path only when no
      // lane of its group has a partner, so the result is the same either way.
      if (__any_sync(__activemask(), hb)) mixed_rates2<!LINEVOTE>(sa, aa, sb, ab, hb, kp.inv_kt, md, acc2, &xma, &xmb);
      else mixed_rates1<!LINEVOTE>(sa, aa, kp.inv_kt, md, acc2, &xma);
      if (!LINEVOTE) neg |= (xma > thr_neg || (hb && xmb > thr_neg)) ? 1u : 0u;
    }
  }
}

// Per-line sums: each lane parks its 20 sums in shared memory and lanes
// 0..19 add one mode each over the 32 lanes (a fixed order), written to
// lsum[line][m]; emx (lanes 0..19) keeps the largest biased exponent of the
// sums written so far (0xff for a non-finite sum), from which the selection
// takes the event's fixed-point scale.
//
// With LINEVOTE, also the line's athermal vote: a site argument above thr
// gives a term of at least 2^thr (1 - 2^-22) in its mode's line sum, and FP32
// sums of non-negative terms never fall below their largest term, so a line
// whose 20 sums all stay below 2^(thr - 1) holds no trigger; true when one
// does not (or is NaN), for an exact test of the line.
template <int LINEVOTE>
__device__ __forceinline__ bool line_sums(const float2* acc2, float (*red)[STZ_MODES], float* lsum_line,
                                          float thr, unsigned& emx) {
  const int lane = threadIdx.x & 31;
  float4* my = reinterpret_cast<float4*>(red[lane]);
#pragma unroll
  for (int j = 0; j < STZ_MODES / 4; j++)
    my[j] = make_float4(acc2[2 * j].x, acc2[2 * j].y, acc2[2 * j + 1].x, acc2[2 * j + 1].y);
  __syncwarp();
  bool hot = false;
  if (lane < STZ_MODES) {
    float t = 0.f;
#pragma unroll 8
    for (int r = 0; r < 32; r++) t += red[r][lane];
    lsum_line[lane] = t;
    emx = max(emx, (__float_as_uint(t) >> 23) & 0xffu);
    if (LINEVOTE) hot = !(t < exp2f(thr - 1.0f));
  }
  if (LINEVOTE) return __any_sync(FULL, hot);
  __syncwarp();
  return false;
}

// ------------------------------------------------ fixed-point selection
// The selection of the mixed form is exact in distribution over the FP32
// site rates the main pass computed. Every quantity it compares is an integer
// in one 64-bit fixed point per event (value v held as floor(v 2^e)), so sums
// are exact and do not depend on their order:
//   site    r = floor(rate 2^e), the rate recomputed with the main pass's
//           exact instruction chain;
//   line    B = floor(L 2^e) + (floor(L 2^e) >> slack) + 3 for its FP32 sum
//           L > 0 (else 0), an upper bound of the exact sum of its sites'
//           r: L is within gamma_D of the exact sum of the same FP32 rates
//           (D the depth of its summation tree) and 2^-slack >= gamma_D;
//   plane   the exact sum of its lines' B; total the exact sum of the planes.
// A target T uniform on [0, total) selects the plane and the line whose
// intervals hold it, exactly; within the line, the site whose interval of
// r holds the rest, or, when the rest falls beyond the sites' exact sum (in
// the slack of the bound, a few per million draws), the draw is rejected and
// a new target drawn. Accepted selections therefore take (site, mode) with
// probability r / sum of all r: no level is clamped and no rounding mass is
// moved to a neighbour. The clock uses the exact fixed-point sum of the FP32
// line sums (not of the bounds).
constexpr long long kFixMax = 1LL << 62;
__device__ __forceinline__ long long fix_f(float v, int e) {
  const unsigned b = __float_as_uint(v);
  const int ex = (int)(b >> 23) & 0xff;
  if (ex == 0 || (b >> 31)) return 0;
  const unsigned long long mant = (unsigned long long)((b & 0x7fffffu) | 0x800000u);
  const int sh = ex - 150 + e;
  if (sh >= 38) return kFixMax;
  if (sh <= -24) return 0;
  return (long long)(sh >= 0 ? mant << sh : mant >> -sh);
}
// ceil(log2(n)) for n >= 1
__device__ __forceinline__ int clog2(long long n) { return n <= 1 ? 0 : 64 - __clzll(n - 1); }

// The event's scale e from the largest biased exponent emax of its line sums:
// every line sum is below 2^(emax - 126), so floor(L 2^e) < 2^(61 - c) with
// c = ceil(log2(n0 n1 MODES)), and the bounds of all lines and modes (each
// below (1 + 2^-slack) 2^(61 - c) + 3) add up to less than 2^62. The quantum
// is 2^-(42 + ...) of the largest line sum (2^-42 at 128^3).
__device__ __forceinline__ int fix_scale(const KParams& kp, unsigned emax) {
  return 187 - clog2((long long)kp.n0 * kp.n1 * STZ_MODES) - (int)emax;
}
// A line's selection bound from its FP32 sum L and v = floor(L 2^e).
__device__ __forceinline__ long long line_bound(float L, long long v, int slack) {
  return L > 0.f ? v + (v >> slack) + 3 : 0;
}

__device__ __forceinline__ long long shfl_xor_i64(long long v, int off) {
  return (long long)__shfl_xor_sync(FULL, (unsigned long long)v, off);
}

// Plane i0's sums by one block, in the event's fixed point (scale from the
// main pass's largest line-sum exponent): psum[m][i0] = the sum of the line
// bounds of mode m over the plane's lines, and psum[MODES][i0] = the sum over
// modes and lines of floor(L 2^e) (the clock); each line's bound also goes to
// lbnd[i0][m][i1] for the search. 8 threads per mode take lines g, g + 8, ...;
// integer sums, so the result does not depend on the order.
// halted: the event does not run (the loads are issued anyway, next to the
// halt flag's, so that the flag's round trip is not paid before them).
__device__ __forceinline__ void plane_sums(const KParams& kp, const float* lsum, long long* psum, long long* lbnd,
                                           int i0, unsigned emax, int halted) {
  constexpr int kG = 8;       // threads per mode
  constexpr int kBatch = 16;  // loads in flight per thread
  __shared__ long long wv[TH / 32];
  const int n0 = kp.n0, n1 = kp.n1;
  const int e = fix_scale(kp, emax), slack = kp.sel_slack;
  const int m = threadIdx.x / kG, g = threadIdx.x % kG;
  const float* ls = lsum + (long long)i0 * n1 * STZ_MODES + m;
  long long* lb = lbnd + ((long long)i0 * STZ_MODES + m) * n1;
  long long bs = 0, vs = 0;
  float x[kBatch];
  int i1 = g;
  if (m < STZ_MODES) {
#pragma unroll
    for (int q = 0; q < kBatch; q++) x[q] = i1 + q * kG < n1 ? ls[(i1 + q * kG) * STZ_MODES] : 0.f;
  }
  if (halted) return;  // the same in every thread of the block, before any barrier
  if (m < STZ_MODES) {
    for (;;) {
#pragma unroll
      for (int q = 0; q < kBatch; q++) {
        const long long v = fix_f(x[q], e);
        const long long b = line_bound(x[q], v, slack);
        vs += v;
        bs += b;
        if (i1 + q * kG < n1) lb[i1 + q * kG] = b;
      }
      i1 += kG * kBatch;
      if (i1 >= n1) break;
#pragma unroll
      for (int q = 0; q < kBatch; q++) x[q] = i1 + q * kG < n1 ? ls[(i1 + q * kG) * STZ_MODES] : 0.f;
    }
  }
  // the 8 threads of a mode are consecutive lanes of one warp
#pragma unroll
  for (int off = 1; off < kG; off <<= 1) {
    bs += shfl_xor_i64(bs, off);
    vs += shfl_xor_i64(vs, off);
  }
  if (m < STZ_MODES && g == 0) psum[(long long)m * n0 + i0] = bs;
#pragma unroll
  for (int off = kG; off < 32; off <<= 1) vs += shfl_xor_i64(vs, off);  // the warp's modes
  if ((threadIdx.x & 31) == 0) wv[threadIdx.x >> 5] = vs;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t = 0;
#pragma unroll
    for (int k = 0; k < TH / 32; k++) t += wv[k];
    psum[(long long)STZ_MODES * n0 + i0] = t;
  }
}

// Body of the grid-wide mixed-form kernel for block b of one replica (kp may
// live in kernel parameters or, for batches, in shared memory); the block
// takes units b, b + nblk, ... and its warps run through them independently.
template <int UPDATE_ONLY, int LINEVOTE, int N2 = 0>
__device__ __forceinline__ void mixed_main_body(const KParams& kp, const Fields& f, int b, const float2* md,
                                                const float (*mraw)[5], float* mix_smem) {
  __shared__ __align__(8) unsigned long long mbar[TH / 32][2];
  Ctl* ctl = f.ctl;
  // the header and the halt flag in independent loads
  const int4* hq = reinterpret_cast<const int4*>(&ctl->head);
  const int4 h0 = hq[0], h1 = hq[1], h2 = hq[2];
  const int halted = ctl->halt;
  if (halted && !UPDATE_ONLY) return;
  if (!UPDATE_ONLY && b == 0 && threadIdx.x == 0) ctl->prof_t0 = gtimer();
  // pending transformation and uniform change
  const float Ud[5] = {__int_as_float(h0.x), __int_as_float(h0.y), __int_as_float(h0.z), __int_as_float(h0.w),
                       __int_as_float(h1.x)};
  const int hp = h1.y;
  const int p0 = h1.z, p1 = h1.w;
  const int p2 = h2.x, pm = h2.y;  // MixHead: Ud[5], has_pend, p0, p1, p2, pend_mode
  float de[5] = {0, 0, 0, 0, 0};
  if (hp) {
#pragma unroll
    for (int k = 0; k < 5; k++) de[k] = mraw[pm][k];
  }
  const MixK k = {kp.n0, kp.n1,    kp.n2,      kp.kt1,    kp.kt2, kp.mx_c1, kp.mx_units, kp.nblk, kp.c1_magic,
                  kp.N,  kp.q_ref, kp.a_scale, kp.inv_kt, f.sdev, f.dF32,   f.ktab,      f.lsum};
  const float thr_neg = k.q_ref * k.a_scale;
  unsigned neg = 0, emx = 0;
  const int N32 = (int)k.N;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // pieces per line and their length (whole lines but for the 256-site pass)
  constexpr int kPieces = (N2 > 0 && LINEVOTE && !UPDATE_ONLY) ? N2 / mix_piece(N2) : 1;
  const int plen = kPieces > 1 ? mix_piece(N2) : k.n2;
  const int sf = mix_stage_floats(plen);
  float* stages = mix_smem + (size_t)w * 2 * sf;
  float4* park = reinterpret_cast<float4*>(mix_smem + (size_t)(TH / 32) * 2 * sf) + threadIdx.x * (STZ_MODES / 4);
  unsigned long long* bar = &mbar[w][0];
  if (lane == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  // this warp's lines: units b, b + nblk, ... (skipping the ones where the
  // warp idles), each in kPieces pieces; piece j of the warp lives in stage
  // j & 1, and the next piece's copy is in flight while a piece is computed.
  // The next line is found before the line's first piece; between the pieces
  // of a line the rate sums wait in shared memory (the registers are at the
  // three-block limit).
  // Response tables larger than a share of L2 (grids above ~190^3) come from
  // HBM: warps 0 and 2, whose lines take the unit's two table rows (d0, 2c)
  // and (d0, 2c + 1) and are valid whenever the row exists, prefetch the rows
  // of their next unit into L2 (8 KB each, one bulk prefetch) a line ahead.
  // (compiled into the passes that meet such grids: 256-site lines and the
  // general pass)
  constexpr bool kRowPrefetch = !UPDATE_ONLY && (N2 == 0 || N2 == 256);
  const bool pf_rows = kRowPrefetch && (w == 0 || w == 2) &&
                       (long long)(k.n0 / 2 + 1) * k.kt1 * k.kt2 * 64 > (48ll << 20);
  int u = b;
  LineOf L{0, 0, 0};
  for (; u < k.mx_units; u += k.nblk)
    if ((L = unit_line(k, u, w, p0, p1)).valid) break;
  if (u < k.mx_units && lane == 0) issue_line<UPDATE_ONLY>(k, L.i0, L.i1, 0, plen, stages, &bar[0]);
  unsigned pending = u < k.mx_units ? 1u : 0u;  // stages with a copy in flight
  unsigned ppar = 0;                                // bit k: parity the copy of stage k completes
  bool timed_out = false;
  for (int j = 0; u < k.mx_units;) {
    int un = u + k.nblk;
    LineOf Ln{0, 0, 0};
    for (; un < k.mx_units; un += k.nblk)
      if ((Ln = unit_line(k, un, w, p0, p1)).valid) break;
    float2 acc2[STZ_MODES / 2];
#pragma unroll
    for (int q = 0; q < STZ_MODES / 2; q++) acc2[q] = make_float2(0.f, 0.f);
    float* cur = stages;
#pragma unroll 1
    for (int h = 0; h < kPieces; h++, j++) {
      const bool last = h == kPieces - 1;
      cur = stages + (j & 1) * sf;
      float* nxt = stages + ((j + 1) & 1) * sf;
      __syncwarp();
      if (!last || un < k.mx_units) {
        if (lane == 0) {
          issue_line<UPDATE_ONLY>(k, last ? Ln.i0 : L.i0, last ? Ln.i1 : L.i1, last ? 0 : (h + 1) * plen, plen, nxt,
                                  &bar[(j + 1) & 1]);
          if (kRowPrefetch && pf_rows && last) {
            const int d0 = (int)__umulhi((unsigned)un, k.c1_magic);
            const int d1 = 2 * (un - d0 * k.mx_c1) + ((w >> 1) & 1);
            bulk_prefetch_l2(reinterpret_cast<const float4*>(k.ktab) + 4LL * ((d0 * k.kt1 + d1) * k.kt2),
                             (unsigned)k.kt2 * 64u);
          }
        }
        pending |= 1u << ((j + 1) & 1);
        ppar = (ppar & ~(1u << ((j + 1) & 1))) | ((((unsigned)(j + 1) >> 1) & 1u) << ((j + 1) & 1));
      }
      if (!mbar_wait(&bar[j & 1], (unsigned)(j >> 1) & 1u)) {
        pending &= ~(1u << (j & 1));  // waited for already, to the limit
        timed_out = true;
        break;
      }
      pending &= ~(1u << (j & 1));
      if (kPieces > 1 && h > 0) {
#pragma unroll
        for (int q = 0; q < STZ_MODES / 4; q++) {
          const float4 v = park[q];
          acc2[2 * q] = make_float2(v.x, v.y);
          acc2[2 * q + 1] = make_float2(v.z, v.w);
        }
      }
      mixed_line<UPDATE_ONLY, LINEVOTE, N2>(k, N32, hp, L.i0, L.i1, h, p0, p1, p2, de, Ud, md, cur, acc2, neg,
                                            thr_neg);
      if (kPieces > 1 && !last) {
#pragma unroll
        for (int q = 0; q < STZ_MODES / 4; q++)
          park[q] = make_float4(acc2[2 * q].x, acc2[2 * q].y, acc2[2 * q + 1].x, acc2[2 * q + 1].y);
      }
    }
    if (timed_out) break;
    if (!UPDATE_ONLY) {
      // the consumed stage holds the transpose
      __syncwarp();
      const int base = (L.i0 * k.n1 + L.i1) * k.n2;
      if (line_sums<LINEVOTE>(acc2, reinterpret_cast<float(*)[STZ_MODES]>(cur),
                              k.lsum + ((long long)L.i0 * k.n1 + L.i1) * STZ_MODES, thr_neg, emx))
        neg |= line_negative(k.sdev, k.dF32, N32, base, k.n2, k.q_ref, k.a_scale, k.inv_kt, md, thr_neg) ? 1u : 0u;
    }
    u = un;
    L = Ln;
  }
  if (timed_out) {
    // record the error and wait (bounded) for this warp's copies in flight,
    // so no copy lands in shared memory after the block has left
    if (lane == 0) {
      f.ctl->status = STZ_ERR_TIMEOUT;
      f.ctl->halt_reason = kHaltError;
      f.ctl->halt = 1;
    }
    for (int k = 0; k < 2; k++)
      if (pending & (1u << k)) (void)mbar_wait(&bar[k], (ppar >> k) & 1u);
  }
  if (UPDATE_ONLY) return;
  pdl_release();
  unsigned nb, eb;
  block_sum_max_u(neg, emx, &nb, &eb);
  if (threadIdx.x == 0) {
    if (nb) atomicAdd(&ctl->neg_count, (unsigned long long)nb);
    if (eb) atomicMax(&ctl->line_emax, eb);
  }
}

template <int UPDATE_ONLY, int N2 = 0>
__global__ void __launch_bounds__(TH, 3) k_mixed(KParams kp, Fields f) {
  extern __shared__ __align__(128) float mix_smem[];
  pdl_wait();
  mixed_main_body<UPDATE_ONLY, 1, N2>(kp, f, blockIdx.x, &kp.mdev2[0][0], kp.mdev_raw, mix_smem);
}


// ------------------------------------------------------- mixed-form tail
// Lane-parallel scalar algebra on the shared control block: lane k of warp 0
// owns Voigt component k (k < 6); the traces come from warp shuffles. Lanes
// >= 6 take part in the shuffles only.
__device__ __forceinline__ double lane_trace(double v, int k) {
  double t = k < 3 ? v : 0.0;
  t += __shfl_xor_sync(FULL, t, 1);
  t += __shfl_xor_sync(FULL, t, 2);
  t += __shfl_xor_sync(FULL, t, 4);  // lanes 0..7 now hold the sum of lanes 0..2
  return __shfl_sync(FULL, t, 0);
}
// C:e for component k
__device__ __forceinline__ double lane_C(const KParams& kp, double e, int k) {
  const double tr = lane_trace(e, k);
  return (k < 3 ? kp.lambda * tr : 0.0) + 2.0 * kp.mu * e;
}
// C^-1:s for component k (3D isotropic compliance)
__device__ __forceinline__ double lane_Cinv(const KParams& kp, double s, int k) {
  const double tr = lane_trace(s, k);
  return (k < 3 ? -kp.inv_lam_coef * tr : 0.0) + s * kp.inv_2mu;
}

// Thermal event of the mixed form: eigenstrain update, the incremental
// "solve" (pending response + uniform change U) and the loading of
// evolution.c:262-317, lane-parallel over the six components.
// The site's part of the commit (lanes 0..5 of a warp): its eigenstrain and
// last strain increment in global memory.
__device__ void mixed_commit_site_lanes(const KParams& kp, const Fields& f, long long s, int m) {
  const int k = threadIdx.x & 31;
  if (k < 6) {
    const long long N = kp.N;
    const double mk = kp.modes[m][k];
    f.prev_deps[k * N + s] = mk;
    f.eps0[k * N + s] += mk;
  }
}

// The rest of the commit, which needs only the mode and the clock advance
// c->t_kmc (so it runs while another warp searches the site): the sum of the
// eigenstrain, the uniform stress change U of the loading, the mean strains
// and the stress.
__device__ void mixed_commit_lanes(const KParams& kp, Ctl* c, int m) {
  const int k = threadIdx.x & 31;
  const bool own = k < 6;
  const double mk = own ? kp.modes[m][k] : 0.0;
  if (own) c->eps0_sum[k] += mk;
  __syncwarp();
  const double ebar = own ? c->eps_avg[k] : 0.0;
  const double dA = own ? ebar - c->eps_avg_applied[k] : 0.0;
  const double CdA = lane_C(kp, dA, k);
  const double u_old = own ? c->u[k] : 0.0;
  // mean stress of the field solved with ebar: C:(ebar - <eps*>)
  const double em = own ? ebar - c->eps0_sum[k] * kp.invN : 0.0;
  double stress = lane_C(kp, em, k);
  // subtract_error (evolution.c:263-300): loaded component masked
  const int lc = kp.loading == STZ_LOAD_SHEAR ? STZ_XY : 0;
  const double ts = (kp.no_subtract_error || k == lc || !own) ? 0.0 : stress;
  const double te = lane_Cinv(kp, ts, k);
  const double t = c->t_kmc, rate = kp.strain_rate, nu = kp.poisson, E = kp.young, mu = kp.mu;
  double de = 0.0, u_new = 0.0;
  switch (kp.loading) {
    case STZ_LOAD_TENSION:
      de = (k == 0 ? rate * t * 1 : (k == 1 || k == 2) ? rate * t * (-nu) : 0.0) - te;
      if (k == 0) { stress += E * rate * t; u_new = E * rate * t; }
      break;
    case STZ_LOAD_COMPRESSION:
      de = (k == 0 ? -rate * t * 2 : k == 1 ? rate * t * nu * 2 : 0.0) - te;
      if (k == 0) { stress += -E * rate * t; u_new = -E * rate * t; }
      break;
    case STZ_LOAD_SHEAR:
      de = k == STZ_XY ? rate * t : -te;
      if (k == STZ_XY) { stress += 2 * mu * rate * t; u_new = 2 * mu * rate * t; }
      break;
    case STZ_LOAD_STRESS: {
      const double d = own ? kp.applied[k] - stress : 0.0;
      de = lane_Cinv(kp, d, k);
      u_new = d;
      stress = own ? kp.applied[k] : 0.0;
      break;
    }
  }
  if (own) {
    c->U[k] = CdA - u_old + u_new;
    c->eps_avg_applied[k] = ebar;
    c->eps_avg[k] = ebar + de;
    c->u[k] = u_new;
    c->stress[k] = stress;
  }
  __syncwarp();
}

__device__ __forceinline__ long long shfl_up_i64(long long v, int off) {
  return (long long)__shfl_up_sync(FULL, (unsigned long long)v, off);
}

// Inclusive scan of one value per thread over the 256-thread block; returns
// the inclusive value and leaves every thread's in sh_inc.
__device__ long long block_incl_scan_i64(long long v, long long* sh_inc) {
  __shared__ long long wsum[TH / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const long long y = shfl_up_i64(x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    long long t = lane < TH / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int off = 1; off < TH / 32; off <<= 1) {
      const long long y = shfl_up_i64(t, off);
      if (lane >= off) t += y;
    }
    if (lane < TH / 32) wsum[lane] = t;
  }
  __syncthreads();
  const long long incl = (w > 0 ? wsum[w - 1] : 0) + x;
  sh_inc[threadIdx.x] = incl;
  __syncthreads();
  return incl;
}

// Warp search over per-lane contiguous chunks with sums v: the lane whose
// interval [excl, excl + v) holds T (at most one does), its exclusive prefix
// in *excl; -1 when T is not below the warp's total.
__device__ __forceinline__ int warp_find_i64(long long v, long long T, long long* excl) {
  const int lane = threadIdx.x & 31;
  long long x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const long long y = shfl_up_i64(x, off);
    if (lane >= off) x += y;
  }
  const long long Eu = shfl_up_i64(x, 1);  // every lane takes part in the shuffle
  const long long El = lane ? Eu : 0;
  const unsigned hit = __ballot_sync(FULL, El <= T && T < x);
  const int L = hit ? __ffs(hit) - 1 : -1;
  *excl = (long long)__shfl_sync(FULL, (unsigned long long)El, L < 0 ? 0 : L);
  return L;
}

// Within one lane's chunk of K values (registers, unrolled) starting at E:
// the entry whose interval holds T (T < E + sum of v), and the running sum
// before it in *before.
template <int K>
__device__ __forceinline__ int chunk_find(const long long* v, long long E, long long T, long long* before) {
  long long run = E, hb = E;
  int hit = -1;
#pragma unroll
  for (int k = 0; k < K; k++) {
    if (hit < 0 && T < run + v[k]) {
      hit = k;
      hb = run;
    }
    run += v[k];
  }
  *before = hb;
  return hit;
}

// Levels 2 and 3 of the mixed-form search, by warp 0 alone: the lines of
// plane i0 for mode m by their bounds, then the sites of the chosen line with
// their rates recomputed exactly as the main pass computed them, all in the
// fixed point of scale e. T (in [0, the plane's bound sum)) is the target
// left within (m, i0). Returns the site in every lane, or kRejected when the
// target left within the line lies beyond its sites' exact sum; *margin
// receives the distance of the target from the nearer edge of the chosen
// site's interval and *x_sel the chosen (site, mode)'s scaled log2-rate
// argument (the chain of mx_x).
constexpr long long kRejected = -2;
constexpr int kLaneChunk = 20;  // plane sums per thread held in registers (20 n0 over TH threads: n0 <= 256)
// KL: the lines or sites a lane holds (n1, n2 <= 32 KL)
template <int KL>
__device__ long long search_line_site(const KParams& kp, const Fields& f, int m, int i0, long long T, int e,
                                      long long* margin, unsigned long long* t_lines, float* x_sel) {
  const int lane = threadIdx.x & 31;
  // level 2: lines, by their bounds
  const int n1 = kp.n1;
  const int c2 = (n1 + 31) / 32;
  const int a1 = lane * c2;
  const long long* lp = f.lbnd + ((long long)i0 * STZ_MODES + m) * n1;
  long long lv[KL];
  long long S1 = 0;
#pragma unroll
  for (int q = 0; q < KL; q++) {
    lv[q] = (q < c2 && a1 + q < n1) ? lp[a1 + q] : 0;
    S1 += lv[q];
  }
  long long E1;
  const int L1 = warp_find_i64(S1, T, &E1);
  if (lane == 0) *t_lines = gtimer();
  if (L1 < 0) return -1;  // not reached: the plane's sum is the sum of these bounds
  int i1 = -1;
  long long rem2 = 0;
  if (lane == L1) {
    long long hb;
    const int h = chunk_find<KL>(lv, E1, T, &hb);
    i1 = a1 + h;
    rem2 = T - hb;
  }
  i1 = __shfl_sync(FULL, i1, L1);
  rem2 = (long long)__shfl_sync(FULL, (unsigned long long)rem2, L1);
  // level 3: sites of line (i0, i1), rates recomputed with the main pass's chain
  const int n2 = kp.n2;
  const long long base = ((long long)i0 * n1 + i1) * n2;
  const int c3 = (n2 + 31) / 32;
  const int a2 = lane * c3;
  long long rv[KL];
  float xv[KL];
  long long S2 = 0;
#pragma unroll
  for (int q = 0; q < KL; q++) {
    xv[q] = 0.f;
    rv[q] = 0;
    if (q < c3 && a2 + q < n2) {
      const long long s = base + a2 + q;
      float sv[5];
      mx_site(kp, f, s, sv);
      xv[q] = mx_x(kp, sv, (kp.q_ref - f.dF32[s]) * kp.a_scale, m);
      rv[q] = fix_f(ex2_approx(xv[q]), e);
    }
    S2 += rv[q];
  }
  long long E2;
  const int L2 = warp_find_i64(S2, rem2, &E2);
  if (L2 < 0) return kRejected;  // in the slack of the line's bound
  long long site = -1, mg = 0;
  float xs = 0.f;
  if (lane == L2) {
    long long hb;
    const int h = chunk_find<KL>(rv, E2, rem2, &hb);
    long long ha = hb;
#pragma unroll
    for (int q = 0; q < KL; q++)
      if (q == h) {
        xs = xv[q];
        ha = hb + rv[q];
      }
    site = base + a2 + h;
    mg = min(rem2 - hb, ha - rem2);
  }
  site = (long long)__shfl_sync(FULL, (unsigned long long)site, L2);
  *margin = (long long)__shfl_sync(FULL, (unsigned long long)mg, L2);
  *x_sel = __shfl_sync(FULL, xs, L2);
  return site;
}

// The scalar part of the control block (everything before the generator).
constexpr int kCtlScalarWords = (int)(offsetof(Ctl, rng) / 4);

// One block after the grid of k_mixed: total rate, step kind, dice, search,
// commit, log and the halt conditions of the mixed form.
// check_halt: read the halt flag first (the selection kernel's blocks have
// read it already; nothing sets it between their read and the tail).
__device__ __forceinline__ void mixed_tail_body(const KParams& kp, const Fields& f, int update_only,
                                                int check_halt = 1) {
  Ctl* const g = f.ctl;
  if (update_only) {
    if (threadIdx.x == 0) {
      for (int k = 0; k < 6; k++) g->U[k] = 0;
      g->has_pend = 0;
      set_mixed_head(kp, g);
    }
    return;
  }
  if (check_halt && g->halt) return;
  const unsigned long long t_tail = gtimer();
  __shared__ Ctl sc;
  __shared__ int sh_kind;
  __shared__ long long sh_site;
  __shared__ int sh_mode;
  __shared__ long long sh_margin;
  __shared__ float sh_x;
  __shared__ long long sh_p1, sh_rem1, sh_T, sh_RB;
  __shared__ int sh_draws, sh_twist;
  __shared__ long long sh_inc_i[TH];
  __shared__ long long sh_wclk[TH / 32];
  __shared__ unsigned long long sh_tl[2];  // search clock: level 1 done, level 2 done
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // the plane bounds q = m n0 + i0 in per-thread contiguous chunks (loaded
  // before the control-block copy so that the two overlap), and the clock row
  const long long P = (long long)STZ_MODES * kp.n0;
  const int ch = (int)((P + TH - 1) / TH);
  const long long q0 = (long long)threadIdx.x * ch, q1 = min(q0 + ch, P);
  long long iv[kLaneChunk];
#pragma unroll
  for (int k = 0; k < kLaneChunk; k++) iv[k] = (q0 + k < q1) ? f.psum[q0 + k] : 0;
  long long vc = 0;
  for (int i = threadIdx.x; i < kp.n0; i += TH) vc += f.psum[P + i];
  // the generator word the dice will take, unless the state is refilled first
  int mti0 = 624;
  uint32_t w0 = 0;
  if (threadIdx.x == 0) {
    mti0 = g->rng.mti;
    if (mti0 < 624) w0 = g->rng.mt[mti0];
  }
  {
    const uint32_t* a = reinterpret_cast<const uint32_t*>(g);
    uint32_t* d = reinterpret_cast<uint32_t*>(&sc);
    for (int i = threadIdx.x; i < kCtlScalarWords; i += blockDim.x) d[i] = a[i];
  }
  if (threadIdx.x == 0) {
    sh_p1 = -1; sh_site = -1; sh_margin = 0; sh_mode = -1; sh_draws = 1;
    sh_twist = mti0 >= 624;  // the generator needs a refill before the dice
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) vc += shfl_xor_i64(vc, off);
  if (lane == 0) sh_wclk[wid] = vc;
  __syncthreads();
  // the event's fixed point, from the largest line-sum exponent the main pass
  // gathered (0xff: a non-finite sum)
  const int emax = (int)sc.line_emax;
  const int e = fix_scale(kp, emax);
  long long S = 0;
#pragma unroll
  for (int k = 0; k < kLaneChunk; k++) S += iv[k];
  for (long long q = q0 + kLaneChunk; q < q1; q++) S += f.psum[q];
  const long long Iq = block_incl_scan_i64(S, sh_inc_i);
  const unsigned long long t_sums = gtimer();
  if (sh_twist) block_twist(&g->rng);  // (every thread read sh_twist after the scan's barriers)
  Ctl* c = &sc;
  if (threadIdx.x == 0) {
    c->step++;
    c->line_emax = 0;  // read by every thread before the scan's barriers
    c->has_pend = 0;
    for (int k = 0; k < 6; k++) c->U[k] = 0;
    long long RL = 0;  // the exact sum of the quantised FP32 line sums
    for (int k = 0; k < TH / 32; k++) RL += sh_wclk[k];
    const long long RB = sh_inc_i[TH - 1];
    sh_RB = RB;
    const double R = ldexp((double)RL, -e) * kp.rate_scale;
    c->total_rate = R;
    int kind;
    if (c->neg_count > 0) {
      kind = kAthermal;
      c->halt = 1;
      c->halt_reason = kHaltAthermal;
    } else if (emax == 0xff || RL <= 0 || RB <= 0) {
      kind = kNone;
      c->status = STZ_ERR_NAN;
      c->halt = 1;
      c->halt_reason = kHaltError;
    } else if (R * kp.dt > 1.0) {  // 1/R < dt without the division
      kind = kThermal;
      c->kstep++;
      // one draw: the word at mti, tempered (the block refilled the state above)
      const int i = mti0 < 624 ? mti0 : g->rng.mti;
      uint32_t y = mti0 < 624 ? w0 : g->rng.mt[i];
      g->rng.mti = i + 1;
      y = mt_temper(y);
      // T = dice RB with dice = y / 2^32: uniform on [0, RB) at the dice's resolution
      sh_T = (long long)__umul64hi((unsigned long long)RB, (unsigned long long)y << 32);
      if (y == 0) {  // dice 0 locates no event in the reference (evolution.c:171-224)
        kind = kNone;
        c->status = STZ_ERR_NO_EVENT;
        c->halt = 1;
        c->halt_reason = kHaltError;
      }
    } else {
      kind = kElastic;
    }
    c->neg_count = 0;
    c->step_kind = kind;
    sh_kind = kind;
  }
  __syncthreads();
  const unsigned long long t_dec = gtimer();
  const int kind = sh_kind;
  if (kind == kThermal) {
    // warp 1's lanes 0..5 keep the components the mode-only commit changes
    // (in shared memory, not registers), to put them back when a draw is
    // rejected
    __shared__ double sh_keep[6][6];
    if (wid == 1 && lane < 6) {
      sh_keep[0][lane] = c->eps0_sum[lane];
      sh_keep[1][lane] = c->eps_avg[lane];
      sh_keep[2][lane] = c->eps_avg_applied[lane];
      sh_keep[3][lane] = c->u[lane];
      sh_keep[4][lane] = c->stress[lane];
      sh_keep[5][lane] = c->U[lane];
    }
    // level 1 of the first draw: (mode, plane), by the thread whose chunk
    // holds the target, from the sums it holds in registers (dead after this:
    // a redraw walks its chunk in memory)
    {
      const long long T = sh_T;
      const long long E = threadIdx.x > 0 ? sh_inc_i[threadIdx.x - 1] : 0;
      if (E <= T && T < Iq && q0 + kLaneChunk >= q1) {
        long long hb = E;
        const int h = chunk_find<kLaneChunk>(iv, E, T, &hb);
        sh_p1 = q0 + h;
        sh_rem1 = T - hb;
      }
    }
    for (int draw = 0;; draw++) {
      // level 1 from memory: redraws, and chunks of more than kLaneChunk planes
      {
        const long long T = sh_T;
        const long long E = threadIdx.x > 0 ? sh_inc_i[threadIdx.x - 1] : 0;
        if (E <= T && T < Iq && (draw > 0 || q0 + kLaneChunk < q1)) {
          long long run = E, hb = E;
          int h = -1;
          for (long long q = q0; q < q1 && h < 0; q++) {
            const long long v = f.psum[q];
            if (T < run + v) {
              h = (int)(q - q0);
              hb = run;
            }
            run += v;
          }
          sh_p1 = q0 + h;
          sh_rem1 = T - hb;
        }
      }
      __syncthreads();
      if (wid == 0) {
        // levels 2 and 3: warp 0
        const long long pg = sh_p1;
        long long site = -1, mg = 0;
        float xs = 0.f;
        int m = -1;
        if (lane == 0) sh_tl[0] = gtimer();
        if (pg >= 0) {
          m = (int)(pg / kp.n0);
          const int i0 = (int)(pg - (long long)m * kp.n0);
          const int nl = max(kp.n1, kp.n2);
          if (nl <= 128) site = search_line_site<4>(kp, f, m, i0, sh_rem1, e, &mg, &sh_tl[1], &xs);
          else if (nl <= 256) site = search_line_site<8>(kp, f, m, i0, sh_rem1, e, &mg, &sh_tl[1], &xs);
          else site = search_line_site<16>(kp, f, m, i0, sh_rem1, e, &mg, &sh_tl[1], &xs);
        }
        if (lane == 0) {
          sh_site = site;
          sh_mode = m;
          sh_margin = mg;
          sh_x = xs;
        }
      } else if (wid == 1) {
        // warp 1, while warp 0 searches: the clock advance and the parts of the
        // commit that need only the mode (level 1 chose it). If the search then
        // finds no site the step ends in an error and this state is not used.
        const long long pg = sh_p1;
        if (pg >= 0) {
          if (lane == 0) c->t_kmc = 1.0 / c->total_rate;
          __syncwarp();
          mixed_commit_lanes(kp, c, (int)(pg / kp.n0));
        }
      }
      __syncthreads();
      if (sh_site != kRejected) break;
      // rejected: undo warp 1's commit and draw a new target
      if (wid == 1 && lane < 6) {
        c->eps0_sum[lane] = sh_keep[0][lane];
        c->eps_avg[lane] = sh_keep[1][lane];
        c->eps_avg_applied[lane] = sh_keep[2][lane];
        c->u[lane] = sh_keep[3][lane];
        c->stress[lane] = sh_keep[4][lane];
        c->U[lane] = sh_keep[5][lane];
      }
      block_twist_if_needed(&g->rng);
      if (threadIdx.x == 0) {
        c->rejections++;
        sh_draws++;
        const int i = g->rng.mti;
        const uint32_t y = mt_temper(g->rng.mt[i]);
        g->rng.mti = i + 1;
        sh_T = (long long)__umul64hi((unsigned long long)sh_RB, (unsigned long long)y << 32);
        sh_p1 = -1;
        sh_site = -1;
      }
      __syncthreads();
    }
  }
  const unsigned long long t_search = gtimer();
  if (wid == 2) {
    // warp 2: the site's eigenstrain, while thread 0 logs the event
    if (kind == kThermal && sh_site >= 0) mixed_commit_site_lanes(kp, f, sh_site, sh_mode);
  } else if (wid == 0) {
    const long long s = sh_site;
    const int m = sh_mode;
    if (threadIdx.x == 0) {
      const double Rtrue = c->total_rate;
      if (kind == kThermal) {
        if (s < 0) {
          c->status = STZ_ERR_NO_EVENT;
          c->halt = 1;
          c->halt_reason = kHaltError;
          c->step_kind = kNone;
        } else {
          if (sh_margin < (sh_RB >> 24)) c->near_ties++;  // within 2^-24 R of an edge
          // Q of the chosen (site, mode) from the argument the search computed
          const double q = (double)kp.q_ref - (double)sh_x * kp.inv_a_scale;
          c->sel_site = s;
          c->sel_mode = m;
          c->sel_q = q;
          c->has_pend = 1;
          c->pend_site = s;
          c->pend_mode = m;
          c->totime += c->t_kmc;
          log_event(kp, f, c, STZ_EV_THERMAL, s, m, c->totime, c->t_kmc, q, Rtrue,
                    (double)sh_margin / (double)sh_RB, sh_draws);
          if (kp.resolve_period > 0 && c->kstep >= c->next_resolve) {
            c->halt = 1;
            c->halt_reason = kHaltResolve;
          }
        }
      } else if (kind == kElastic) {
        c->estep++;
        c->totime += kp.dt;
        double u0[6];
        for (int k = 0; k < 6; k++) u0[k] = c->u[k];
        elastic_step(kp, c);
        for (int k = 0; k < 6; k++) c->U[k] = c->u[k] - u0[k];
        log_event(kp, f, c, STZ_EV_ELASTIC, -1, -1, c->totime, kp.dt, 0.0, Rtrue);
      }
      if ((kind == kThermal || kind == kElastic) && c->step_kind != kNone) {
        if (print_check(kp, c)) {
          c->print_done = 1;
          c->halt = 1;
          c->halt_reason = kHaltPrint;
        } else {
          if (!c->halt) stop_check(kp, c);
          c->step_kind = kNone;
        }
      }
      const unsigned long long t_end = gtimer();
      c->prof_main_ns += t_tail - c->prof_t0;
      c->prof_tail_ns += t_end - t_tail;
      c->prof_part_ns[0] += t_sums - t_tail;
      c->prof_part_ns[1] += t_dec - t_sums;
      c->prof_part_ns[2] += t_search - t_dec;
      c->prof_part_ns[3] += t_end - t_search;
      if (kind == kThermal) {
        c->prof_part_ns[4] += sh_tl[0] - t_dec;      // level 1 (mode, plane)
        c->prof_part_ns[5] += sh_tl[1] - sh_tl[0];   // level 2 (line)
        c->prof_part_ns[6] += t_search - sh_tl[1];   // level 3 (site)
      }
      c->prof_n++;
    }
  }
  if (wid == 0) {
    __syncwarp();
    set_mixed_head_warp(kp, c);
  }
  __syncthreads();
  {
    const uint32_t* a = reinterpret_cast<const uint32_t*>(&sc);
    uint32_t* d = reinterpret_cast<uint32_t*>(g);
    for (int i = threadIdx.x; i < kCtlScalarWords; i += blockDim.x) d[i] = a[i];
  }
}

__global__ void __launch_bounds__(TH) k_mixed_tail(KParams kp, Fields f, int update_only) {
  pdl_wait();
  pdl_release();
  mixed_tail_body(kp, f, update_only);
}

// Last of `count` blocks to pass (threadfence pattern; the counter returns to
// zero for the next launch). That block then sees every block's writes.
__device__ bool last_of(unsigned* counter, unsigned count) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    is_last = atomicAdd(counter, 1u) == count - 1;
    if (is_last) *counter = 0;
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}

// One block per plane forms that plane's sums; the last block to finish runs
// the selection, commit and loading of the event (one launch after the main
// pass instead of two).
__global__ void __launch_bounds__(TH) k_mixed_select(KParams kp, Fields f) {
  pdl_wait();
  pdl_release();
  const int halted = f.ctl->halt;
  plane_sums(kp, f.lsum, f.psum, f.lbnd, blockIdx.x, f.ctl->line_emax, halted);
  if (halted) return;
  if (!last_of(&f.ctl->ticket, gridDim.x)) return;
  mixed_tail_body(kp, f, 0, 0);
}

// ------------------------------------------------------------ batches
// Replicas of a batch: grid-wide kernel over every replica's blocks (block ->
// replica map), then one tail block per replica. Each block copies its
// replica's constants to shared memory.
__device__ __forceinline__ void load_desc(const BatchDesc* d, int r, KParams* skp, Fields* sf) {
  const uint32_t* a = reinterpret_cast<const uint32_t*>(&d[r]);
  uint32_t* k = reinterpret_cast<uint32_t*>(skp);
  for (int i = threadIdx.x; i < (int)(sizeof(KParams) / 4); i += blockDim.x) k[i] = a[i];
  const uint32_t* a2 = reinterpret_cast<const uint32_t*>(&d[r].f);
  uint32_t* k2 = reinterpret_cast<uint32_t*>(sf);
  for (int i = threadIdx.x; i < (int)(sizeof(Fields) / 4); i += blockDim.x) k2[i] = a2[i];
  __syncthreads();
}

// SHARED: every replica has the same modes, passed as kernel parameters
// (constant-bank operands) instead of being read from each block's copy of
// its replica's constants in shared memory.
// N2: the line length of every replica of this launch (0: any); blk_off:
// the first block of this launch in blk_rep.
template <int SHARED, int N2>
__global__ void __launch_bounds__(TH, 3) k_mixed_batched(const BatchDesc* __restrict__ d,
                                                          const int* __restrict__ blk_rep,
                                                          const int* __restrict__ rep_first, int blk_off,
                                                          ModeSet ms) {
  __shared__ KParams skp;
  __shared__ Fields sf;
  pdl_wait();
  const int blk = blockIdx.x + blk_off;
  const int r = blk_rep[blk];
  if (d[r].f.ctl->halt) return;  // a halted replica's blocks skip the copy
  load_desc(d, r, &skp, &sf);
  extern __shared__ __align__(128) float mix_smem[];
  // lines of a known length: the pass specialised to it, with the athermal
  // test per line; otherwise the general pass with the per-site maximum
  constexpr int LV = N2 > 0 ? 1 : 0;
  if (SHARED)
    mixed_main_body<0, LV, N2>(skp, sf, blk - rep_first[r], &ms.mdev2[0][0], ms.mdev_raw, mix_smem);
  else
    mixed_main_body<0, LV, N2>(skp, sf, blk - rep_first[r], &skp.mdev2[0][0], skp.mdev_raw, mix_smem);
}

// Plane sums of a batch: block (x, r) sums plane x of replica r. A kernel of
// its own (about 40 registers, six blocks per SM) so that the thousands of
// plane blocks of a batch are not held to the tail's register count.
__global__ void __launch_bounds__(TH, 6) k_plane_sums_batched(const BatchDesc* __restrict__ d) {
  pdl_wait();
  pdl_release();
  const int r = blockIdx.y;
  const BatchDesc& e = d[r];
  if ((int)blockIdx.x >= e.kp.n0) return;
  Ctl* ctl = e.f.ctl;
  const int halted = ctl->halt;
  plane_sums(e.kp, e.f.lsum, e.f.psum, e.f.lbnd, blockIdx.x, ctl->line_emax, halted);
}

// The tail of each replica of a batch (block r, after every plane sum of the
// round), which then reports the replica's state.
__global__ void __launch_bounds__(TH) k_mixed_tail_batched(const BatchDesc* __restrict__ d,
                                                           BatchStatus* __restrict__ st) {
  __shared__ KParams skp;
  __shared__ Fields sf;
  const int r = blockIdx.x;
  load_desc(d, r, &skp, &sf);
  mixed_tail_body(skp, sf, 0, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    const Ctl* c = sf.ctl;
    st[r].halt = c->halt;
    st[r].halt_reason = c->halt_reason;
    st[r].stopped = c->stopped;
    st[r].status = c->status;
    st[r].kstep = c->kstep;
  }
}

// After a full re-solve into sdev (mixed form).
__global__ void k_mixed_after_resolve(KParams kp, Fields f, int kind) {
  Ctl* ctl = f.ctl;
  ctl->has_pend = 0;
  for (int c = 0; c < 6; c++) ctl->U[c] = 0;
  set_mixed_head(kp, ctl);
  if (kind == 0) {
    for (int c = 0; c < 6; c++) {
      ctl->eps_avg_applied[c] = ctl->eps_avg[c];
      ctl->u[c] = 0;
    }
  }
}

// ------------------------------------------------------------ misc
__global__ void k_q_mode(KParams kp, Fields f, int mode, double* out, int model) {
  Ctl* ctl = f.ctl;
  double u[6];
  for (int c = 0; c < 6; c++) u[c] = ctl->u[c];
  const double totime = ctl->totime;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < kp.N; s += (long long)gridDim.x * blockDim.x) {
    if (model == 0) out[s] = site_Q<0>(kp, f, u, totime, s, mode);
    else if (model == 1) out[s] = site_Q<1>(kp, f, u, totime, s, mode);
    else out[s] = site_Q<2>(kp, f, u, totime, s, mode);
  }
}

__device__ __forceinline__ void dev5(const double* s, double* d) {
  const double r2 = 0.70710678118654752440, r6 = 0.40824829046386301637, q2 = 1.41421356237309504880;
  d[0] = (s[0] - s[1]) * r2;
  d[1] = (2.0 * s[2] - s[0] - s[1]) * r6;
  d[2] = q2 * s[3];
  d[3] = q2 * s[4];
  d[4] = q2 * s[5];
}

__global__ void k_dev_from_sig(KParams kp, const double* sig, float* sdev) {
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < kp.N; s += (long long)gridDim.x * blockDim.x) {
    double v[6], d[5];
    for (int c = 0; c < 6; c++) v[c] = sig[c * kp.N + s];
    dev5(v, d);
    for (int k = 0; k < 5; k++) sdev[k * kp.N + s] = (float)d[k];
  }
}

// Column b of the response table: K[a][b](d) = e_a : sigma^(b)(d) for d in
// the octant 0 <= d_i <= n_i/2, stored in the packed upper triangle (15 of a
// record's 16 floats). A row (d0, d1) holds its kt2 records chunk-major: the
// 16-byte chunk q of record d2 at float4 index (row * 4 + q) * kt2 + d2, so
// the lanes of a warp reading consecutive records read contiguous bytes.
__global__ void k_ktab_column(KParams kp, const double* sig, float* ktab, int b) {
  const long long ts = (long long)kp.kt1 * kp.kt2, tn = (long long)kp.kt0 * ts;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tn; t += (long long)gridDim.x * blockDim.x) {
    const int d2 = (int)(t % kp.kt2);
    const int d1 = (int)((t / kp.kt2) % kp.kt1);
    const int d0 = (int)(t / ts);
    const long long s = ((long long)d0 * kp.n1 + d1) * kp.n2 + d2;
    double v[6], d[5];
    for (int c = 0; c < 6; c++) v[c] = sig[c * kp.N + s];
    dev5(v, d);
    for (int a = 0; a <= b; a++) {
      // packed index of (a, b), a <= b, row-major upper triangle
      const int idx = a * 5 - a * (a - 1) / 2 + (b - a);
      ktab[((t / kp.kt2 * 4 + (idx >> 2)) * kp.kt2 + d2) * 4 + (idx & 3)] = (float)d[a];
    }
  }
}

// ------------------------------------------- spatially varying moduli
// The polarisation fixed point of InhomogeneousStressSolver (elastic.c:977-
// 1066) per site: C(x):e with the site's Lambda, Mu (IsotropicMul_RF,
// elastic.c:905-920) and (C0 - C(x)):e (IsotropicMul_RF_D, elastic.c:922-938).
__device__ __forceinline__ void site_C(int nc, double lam, double mu, const double* e, double* s) {
  const int nd = ndiag(nc);
  double tr = 0;
  for (int c = 0; c < nd; c++) tr += e[c];
  const double tra = lam * tr;
  for (int c = 0; c < nc; c++) s[c] = (c < nd ? tra : 0.0) + 2 * mu * e[c];
}

// Start (elastic.c:993-1009): tau0 = C(x):eps*, and the reference medium's
// effective eigenstrain eeff = C0^-1:(tau0 + (C0 - C(x)):(eps* + ebar)).
__global__ void k_inhom_init(KParams kp, const double* __restrict__ eps0, const double* __restrict__ ebar,
                             const double* __restrict__ lam_s, const double* __restrict__ mu_s,
                             double* __restrict__ tau0, double* __restrict__ eeff) {
  const int nc = kp.nc;
  double eb[6];
  for (int c = 0; c < nc; c++) eb[c] = ebar[c];
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < kp.N; s += (long long)gridDim.x * blockDim.x) {
    double e0[6], e1[6], t0[6], t1[6], T[6], ee[6];
    for (int c = 0; c < nc; c++) {
      e0[c] = eps0[c * kp.N + s];
      e1[c] = e0[c] + eb[c];
    }
    site_C(nc, lam_s[s], mu_s[s], e0, t0);
    site_C(nc, kp.lambda - lam_s[s], kp.mu - mu_s[s], e1, t1);
    for (int c = 0; c < nc; c++) T[c] = t0[c] + t1[c];
    iso_inv(kp, T, ee);
    for (int c = 0; c < nc; c++) {
      tau0[c * kp.N + s] = t0[c];
      eeff[c * kp.N + s] = ee[c];
    }
  }
}

// One iteration after the homogeneous solve of the reference medium with
// eigenstrain `last` (elastic.c:1027-1049): total strain e = C0^-1:sigma +
// last, tau = tau0 + (C0 - C(x)):e, eeff = (C0^-1:tau + last) / 2 (mix 0.5),
// and this block's sum of (eeff - last)^2 in part[blockIdx.x] (AvgChange,
// elastic.c:957-975; a fixed tree, so the sum does not depend on timing).
__global__ void k_inhom_update(KParams kp, const double* __restrict__ sig, const double* __restrict__ last,
                               const double* __restrict__ lam_s, const double* __restrict__ mu_s,
                               const double* __restrict__ tau0, double* __restrict__ eeff,
                               double* __restrict__ part) {
  const int nc = kp.nc;
  double acc = 0;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < kp.N; s += (long long)gridDim.x * blockDim.x) {
    double sg[6], el[6], et[6], t1[6], T[6], en[6];
    for (int c = 0; c < nc; c++) sg[c] = sig[c * kp.N + s];
    iso_inv(kp, sg, el);
    for (int c = 0; c < nc; c++) et[c] = el[c] + last[c * kp.N + s];
    site_C(nc, kp.lambda - lam_s[s], kp.mu - mu_s[s], et, t1);
    for (int c = 0; c < nc; c++) T[c] = tau0[c * kp.N + s] + t1[c];
    iso_inv(kp, T, en);
    for (int c = 0; c < nc; c++) {
      const double lv = last[c * kp.N + s];
      const double v = 0.5 * en[c] + (1 - 0.5) * lv;
      eeff[c * kp.N + s] = v;
      acc += (v - lv) * (v - lv);
    }
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(FULL, acc, off);
  __shared__ double red[TH / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += red[k];
    part[blockIdx.x] = t;
  }
}

__global__ void k_fill_f32(const double* in, float* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

__global__ void k_l2_flush(uint4* buf, long long n, unsigned v) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    buf[i] = make_uint4(v, v + 1, v + 2, (unsigned)i);
}

// Keeps the stream busy for about `ns` nanoseconds of the global timer: the
// host has queued the launches behind it by the time it ends, so an event
// recorded after it stamps the next kernel's start rather than the host's
// launch latency. The loop is bounded by an iteration limit as well.
__global__ void k_hold(unsigned long long ns) {
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (int i = 0; i < (1 << 20); i++) {
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 >= ns) break;
    __nanosleep(256);
  }
}

}  // namespace

void launch_rate_fp64(const KParams& kp, const Fields& f, cudaStream_t st) {
  if (kp.model == STZ_MODEL_REF2D) k_rate64<0><<<kp.nblk, TH, 0, st>>>(kp, f);
  else k_rate64<1><<<kp.nblk, TH, 0, st>>>(kp, f);
}

// The staged lines of the mixed-form main kernels are dynamic shared memory,
// above the 48 KB default for long lines: raise their limit once per device
// to what the device allows next to their static shared memory.
static void mixed_smem_init() {
  static bool done_dev[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (done_dev[dev & 63]) return;
  done_dev[dev & 63] = true;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) optin = 48 * 1024;
  auto raise = [&](const void* k) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, k) != cudaSuccess) { (void)cudaGetLastError(); return; }
    const int bytes = optin - (int)fa.sharedSizeBytes;
    if (bytes > 0 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
      (void)cudaGetLastError();
  };
  raise((const void*)k_mixed<0>);
  raise((const void*)k_mixed<0, 128>);
  raise((const void*)k_mixed<0, 256>);
  raise((const void*)k_mixed<1>);
  raise((const void*)k_mixed<0, 32>);
  raise((const void*)k_mixed<0, 64>);
  raise((const void*)k_mixed<0, 96>);
  raise((const void*)k_mixed_batched<0, 0>);
  raise((const void*)k_mixed_batched<1, 0>);
  raise((const void*)k_mixed_batched<0, 32>);
  raise((const void*)k_mixed_batched<1, 32>);
  raise((const void*)k_mixed_batched<0, 64>);
  raise((const void*)k_mixed_batched<1, 64>);
  raise((const void*)k_mixed_batched<0, 96>);
  raise((const void*)k_mixed_batched<1, 96>);
  raise((const void*)k_mixed_batched<0, 128>);
  raise((const void*)k_mixed_batched<1, 128>);
}

size_t mixed_smem(int n2) { return mix_smem_bytes(n2); }

int mixed_blocks_per_sm(int n2) {
  mixed_smem_init();
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mixed<0>, TH, mix_smem_main_bytes(n2)) != cudaSuccess ||
      occ < 1) {
    (void)cudaGetLastError();
    occ = 1;
  }
  return occ;
}

namespace {
// Launch with the programmatic-stream-serialization attribute: the kernel may
// be scheduled while the previous kernel of the stream finishes; it waits for
// it with griddepcontrol.wait.
template <typename... A>
void launch_pdl(void (*kern)(A...), dim3 grid, size_t smem, cudaStream_t st, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(TH);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, args...);
}
}  // namespace

int batch_class(int n2) {
  for (int c = 0; c < kBatchClasses - 1; c++)
    if (kBatchClassN2[c] == n2) return c;
  return kBatchClasses - 1;
}

namespace {
template <int N2>
void launch_batched_class(const BatchDesc* d, const int* blk_rep, const int* rep_first, int start, int count,
                          int max_n2, const ModeSet* shared, cudaStream_t s) {
  const size_t smem = mix_smem_bytes(max_n2);
  if (shared) k_mixed_batched<1, N2><<<count, TH, smem, s>>>(d, blk_rep, rep_first, start, *shared);
  else k_mixed_batched<0, N2><<<count, TH, smem, s>>>(d, blk_rep, rep_first, start, ModeSet{});
}
}  // namespace

void launch_mixed_batched(const BatchDesc* d, const int* blk_rep, const int* rep_first, const BatchLaunch& bl,
                          BatchStatus* status, int nrep, int max_n0, const ModeSet* shared, cudaStream_t st) {
  mixed_smem_init();
  // the classes run side by side: the first on st, the others on side
  // streams that fork from st and join it before the selection
  int first = -1;
  cudaEventRecord(bl.fork, st);
  for (int c = 0; c < kBatchClasses; c++) {
    if (bl.count[c] <= 0) continue;
    cudaStream_t s = st;
    if (first < 0) {
      first = c;
    } else {
      s = bl.side[c];
      cudaStreamWaitEvent(s, bl.fork, 0);
    }
    switch (kBatchClassN2[c]) {
      case 32: launch_batched_class<32>(d, blk_rep, rep_first, bl.start[c], bl.count[c], bl.max_n2[c], shared, s); break;
      case 64: launch_batched_class<64>(d, blk_rep, rep_first, bl.start[c], bl.count[c], bl.max_n2[c], shared, s); break;
      case 96: launch_batched_class<96>(d, blk_rep, rep_first, bl.start[c], bl.count[c], bl.max_n2[c], shared, s); break;
      case 128:
        launch_batched_class<128>(d, blk_rep, rep_first, bl.start[c], bl.count[c], bl.max_n2[c], shared, s);
        break;
      default: launch_batched_class<0>(d, blk_rep, rep_first, bl.start[c], bl.count[c], bl.max_n2[c], shared, s);
    }
    if (s != st) {
      cudaEventRecord(bl.join[c], s);
      cudaStreamWaitEvent(st, bl.join[c], 0);
    }
  }
  k_plane_sums_batched<<<dim3(max_n0, nrep), TH, 0, st>>>(d);
  k_mixed_tail_batched<<<nrep, TH, 0, st>>>(d, status);
}

void launch_mixed_main(const KParams& kp, const Fields& f, int update_only, cudaStream_t st) {
  mixed_smem_init();
  if (update_only) k_mixed<1><<<kp.nblk, TH, mix_smem_bytes(kp.n2), st>>>(kp, f);
  else if (kp.general_pass) launch_pdl(k_mixed<0>, dim3(kp.nblk), mix_smem_bytes(kp.n2), st, kp, f);
  else if (kp.n2 == 256) launch_pdl(k_mixed<0, 256>, dim3(kp.nblk), mix_smem_main_bytes(256), st, kp, f);
  else if (kp.n2 == 128) launch_pdl(k_mixed<0, 128>, dim3(kp.nblk), mix_smem_bytes(kp.n2), st, kp, f);
  else if (kp.n2 == 96) launch_pdl(k_mixed<0, 96>, dim3(kp.nblk), mix_smem_bytes(kp.n2), st, kp, f);
  else if (kp.n2 == 64) launch_pdl(k_mixed<0, 64>, dim3(kp.nblk), mix_smem_bytes(kp.n2), st, kp, f);
  else if (kp.n2 == 32) launch_pdl(k_mixed<0, 32>, dim3(kp.nblk), mix_smem_bytes(kp.n2), st, kp, f);
  else launch_pdl(k_mixed<0>, dim3(kp.nblk), mix_smem_bytes(kp.n2), st, kp, f);
}

void launch_mixed_tail(const KParams& kp, const Fields& f, int update_only, cudaStream_t st) {
  if (update_only) k_mixed_tail<<<1, TH, 0, st>>>(kp, f, update_only);
  else launch_pdl(k_mixed_select, dim3(kp.n0), 0, st, kp, f);
}

// The stored mode norms of every (mode, site) from the mode increments.
__global__ void k_mode_norms(KParams kp, Fields f) {
  const long long N = kp.N, total = (long long)STZ_MODES * N;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long m = i / N, s = i - m * N;
    const double* dd = f.deps + m * 3 * N;
    f.dnorm[i] = mode_rnorm(dd[s], dd[N + s], dd[2 * N + s]);
  }
}

void launch_mode_norms(const KParams& kp, const Fields& f, cudaStream_t st) {
  const long long total = (long long)STZ_MODES * kp.N;
  const unsigned nb = (unsigned)std::min<long long>((total + TH - 1) / TH, 152LL * 16);
  k_mode_norms<<<nb, TH, 0, st>>>(kp, f);
}

int wait_selftest(int tries, int* status_dev, int* kmax, cudaStream_t st) {
  *kmax = kMbarTries;
  k_wait_selftest<<<1, 32, 0, st>>>(tries, status_dev);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

void launch_mixed(const KParams& kp, const Fields& f, int update_only, cudaStream_t st) {
  launch_mixed_main(kp, f, update_only, st);
  launch_mixed_tail(kp, f, update_only, st);
}

void launch_athermal(const KParams& kp, const Fields& f, int mixed, cudaStream_t st) {
  const long long nb = std::min<long long>((kp.N + TH - 1) / TH, 152LL * 8);
  k_ath_mark<<<(unsigned)nb, TH, 0, st>>>(kp, f, mixed);
  k_ath_commit<<<1, TH, 0, st>>>(kp, f, mixed);
}

void launch_post_a(const KParams& kp, const Fields& f, cudaStream_t st) {
  k_post_a<<<1, TH, 0, st>>>(kp, f);
  k_post_print<<<1, 1, 0, st>>>(kp, f);
}

void launch_post_b(const KParams& kp, const Fields& f, cudaStream_t st) { k_post_b<<<1, TH, 0, st>>>(kp, f); }

void launch_incr64(const KParams& kp, const Fields& f, cudaStream_t st) {
  const unsigned nb = (unsigned)std::min<long long>((kp.N + TH - 1) / TH, 152LL * 8);
  k_incr64<<<nb, TH, 0, st>>>(kp, f);
  k_incr64_done<<<1, 1, 0, st>>>(f);
}

void launch_note_solve(const Fields& f, const int* gate, const double* ebar, cudaStream_t st) {
  k_note_solve<<<1, 1, 0, st>>>(f, gate, ebar);
}

void launch_q0_reset(const KParams& kp, const Fields& f, cudaStream_t st) {
  const long long total = (long long)STZ_MODES * kp.N;
  const unsigned nb = (unsigned)std::min<long long>((total + TH - 1) / TH, 152LL * 8);
  k_q0_reset<<<nb, TH, 0, st>>>(kp, f);
}

void launch_mixed_after_resolve(const KParams& kp, const Fields& f, int kind, cudaStream_t st) {
  k_mixed_after_resolve<<<1, 1, 0, st>>>(kp, f, kind);
}

void launch_q_mode(const KParams& kp, const Fields& f, int mode, double* out, cudaStream_t st) {
  const int model = kp.model == STZ_MODEL_REF2D ? 0 : (f.sdev ? 2 : 1);
  const long long nb = std::min<long long>((kp.N + 255) / 256, 4096);
  k_q_mode<<<(unsigned)nb, 256, 0, st>>>(kp, f, mode, out, model);
}

void launch_dev_from_sig(const KParams& kp, const double* sig, float* sdev, cudaStream_t st) {
  const long long nb = std::min<long long>((kp.N + 255) / 256, 4096);
  k_dev_from_sig<<<(unsigned)nb, 256, 0, st>>>(kp, sig, sdev);
}

void launch_ktab_column(const KParams& kp, const double* sig, float* ktab, int b, cudaStream_t st) {
  const long long tn = (long long)kp.kt0 * kp.kt1 * kp.kt2;
  const long long nb = std::min<long long>((tn + 255) / 256, 4096);
  k_ktab_column<<<(unsigned)nb, 256, 0, st>>>(kp, sig, ktab, b);
}

void launch_inhom_init(const KParams& kp, const Fields& f, const double* ebar, cudaStream_t st) {
  k_inhom_init<<<kInhomBlocks, TH, 0, st>>>(kp, f.eps0, ebar, f.lam_site, f.mu_site, f.inh_tau0, f.inh_eeff);
}

void launch_inhom_update(const KParams& kp, const Fields& f, cudaStream_t st) {
  k_inhom_update<<<kInhomBlocks, TH, 0, st>>>(kp, f.sig, f.inh_last, f.lam_site, f.mu_site, f.inh_tau0, f.inh_eeff,
                                              f.inh_part);
}

void launch_fill_f32(const double* in, float* out, long long n, cudaStream_t st) {
  const long long nb = std::min<long long>((n + 255) / 256, 4096);
  k_fill_f32<<<(unsigned)nb, 256, 0, st>>>(in, out, n);
}

void launch_hold(unsigned long long ns, cudaStream_t st) { k_hold<<<1, 32, 0, st>>>(ns); }

void launch_l2_flush(void* buf, size_t bytes, cudaStream_t st) {
  const long long n = (long long)(bytes / sizeof(uint4));
  static unsigned v = 1;
  k_l2_flush<<<152 * 4, 256, 0, st>>>(reinterpret_cast<uint4*>(buf), n, v++);
}

}  // namespace stz
