/*
 * stz_oracle.c -- TEST INFRASTRUCTURE ONLY: the CPU oracle for the STZ kinetic
 * Monte Carlo step. See stz_oracle.h for what pins it.
 *
 * Citations are to files of the reference project directory
 * "Mesoscale simulation STZ model/". Compile with -ffp-contract=off so that
 * results are identical on x86-64 and aarch64 hosts.
 */
#define _GNU_SOURCE
#include "stz_oracle.h"

#include <math.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ===================================================================== RNG */
/* GSL mt19937 (rng/mt.c): Matsumoto & Nishimura 1998 with the 1812433253
 * seeding recurrence; seed 0 is replaced by 4357. Used by Rand_Init
 * (init.c:142-150) through gsl_rng_default. */
void or_rng_seed(or_rng* r, unsigned long s) {
  if (s == 0) s = 4357;
  r->mt[0] = (uint32_t)(s & 0xffffffffUL);
  for (int i = 1; i < 624; i++)
    r->mt[i] = (uint32_t)(1812433253UL * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (unsigned long)i);
  r->mti = 624;
}

uint32_t or_rng_get(or_rng* r) {
  const uint32_t UPPER = 0x80000000u, LOWER = 0x7fffffffu, MATRIX_A = 0x9908b0dfu;
  if (r->mti >= 624) {
    int k;
    for (k = 0; k < 624 - 397; k++) {
      uint32_t y = (r->mt[k] & UPPER) | (r->mt[k + 1] & LOWER);
      r->mt[k] = r->mt[k + 397] ^ (y >> 1) ^ ((y & 1u) ? MATRIX_A : 0u);
    }
    for (; k < 623; k++) {
      uint32_t y = (r->mt[k] & UPPER) | (r->mt[k + 1] & LOWER);
      r->mt[k] = r->mt[k + 397 - 624] ^ (y >> 1) ^ ((y & 1u) ? MATRIX_A : 0u);
    }
    uint32_t y = (r->mt[623] & UPPER) | (r->mt[0] & LOWER);
    r->mt[623] = r->mt[396] ^ (y >> 1) ^ ((y & 1u) ? MATRIX_A : 0u);
    r->mti = 0;
  }
  uint32_t k = r->mt[r->mti++];
  k ^= (k >> 11);
  k ^= (k << 7) & 0x9d2c5680u;
  k ^= (k << 15) & 0xefc60000u;
  k ^= (k >> 18);
  return k;
}

double or_rng_uniform(or_rng* r) { return or_rng_get(r) / 4294967296.0; }

double or_rng_uniform_pos(or_rng* r) {
  double x;
  do { x = or_rng_uniform(r); } while (x == 0);
  return x;
}

/* Polar Box-Muller, exactly as the reference restates gsl_ran_gaussian at
 * init.c:207-223 (including the order of the two uniform draws). */
double or_ran_gaussian(or_rng* r, double sigma) {
  double x, y, r2;
  do {
    x = -1 + 2 * or_rng_uniform_pos(r);
    y = -1 + 2 * or_rng_uniform_pos(r);
    r2 = x * x + y * y;
  } while (r2 > 1.0 || r2 == 0);
  return sigma * y * sqrt(-2.0 * log(r2) / r2);
}

/* ===================================================================== FFT */
/* Mixed radix (2, 3, 4) Stockham autosort DFT of one contiguous line. */
static int fft_factor(int n, int* f) {
  int k = 0;
  while (n % 4 == 0) { f[k++] = 4; n /= 4; }
  while (n % 2 == 0) { f[k++] = 2; n /= 2; }
  while (n % 3 == 0) { f[k++] = 3; n /= 3; }
  return n == 1 ? k : -1;
}

static void fft_line(int n, double* a, double* b, int sign, const double* tw) {
  /* a: input/output (interleaved), b: scratch of the same size,
   * tw[2k], tw[2k+1] = cos, sin of 2 pi k / n */
  if (n == 1) return;
  int f[40];
  int nf = fft_factor(n, f);
  double* src = a;
  double* dst = b;
  int ns = 1;
  for (int s = 0; s < nf; s++) {
    int R = f[s];
    int m = n / R;
    int step = n / (ns * R);
    for (int j = 0; j < m; j++) {
      int jm = j % ns;
      double vr[4], vi[4];
      for (int r = 0; r < R; r++) {
        double xr = src[2 * (j + r * m)], xi = src[2 * (j + r * m) + 1];
        if (r > 0 && jm != 0) {
          int t = (jm * r * step) % n;
          double c = tw[2 * t], sn = sign * tw[2 * t + 1];
          double tr = xr * c - xi * sn;
          double ti = xr * sn + xi * c;
          xr = tr; xi = ti;
        }
        vr[r] = xr; vi[r] = xi;
      }
      if (R == 2) {
        double t0r = vr[0] + vr[1], t0i = vi[0] + vi[1];
        double t1r = vr[0] - vr[1], t1i = vi[0] - vi[1];
        vr[0] = t0r; vi[0] = t0i; vr[1] = t1r; vi[1] = t1i;
      } else if (R == 4) {
        double a0r = vr[0] + vr[2], a0i = vi[0] + vi[2];
        double a1r = vr[0] - vr[2], a1i = vi[0] - vi[2];
        double a2r = vr[1] + vr[3], a2i = vi[1] + vi[3];
        double a3r = vr[1] - vr[3], a3i = vi[1] - vi[3];
        /* multiply a3 by sign*i */
        double b3r = -sign * a3i, b3i = sign * a3r;
        vr[0] = a0r + a2r; vi[0] = a0i + a2i;
        vr[2] = a0r - a2r; vi[2] = a0i - a2i;
        vr[1] = a1r + b3r; vi[1] = a1i + b3i;
        vr[3] = a1r - b3r; vi[3] = a1i - b3i;
      } else { /* R == 3 */
        double c1 = -0.5, s1 = sign * (sqrt(3.0) / 2.0);
        double tr = vr[1] + vr[2], ti = vi[1] + vi[2];
        double ur = vr[1] - vr[2], ui = vi[1] - vi[2];
        double y0r = vr[0] + tr, y0i = vi[0] + ti;
        double mr = vr[0] + c1 * tr, mi = vi[0] + c1 * ti;
        /* s1 * i * u */
        double qr = -s1 * ui, qi = s1 * ur;
        vr[0] = y0r; vi[0] = y0i;
        vr[1] = mr + qr; vi[1] = mi + qi;
        vr[2] = mr - qr; vi[2] = mi - qi;
      }
      int base = (j / ns) * ns * R + jm;
      for (int r = 0; r < R; r++) {
        dst[2 * (base + r * ns)] = vr[r];
        dst[2 * (base + r * ns) + 1] = vi[r];
      }
    }
    double* t = src; src = dst; dst = t;
    ns *= R;
  }
  if (src != a) memcpy(a, src, sizeof(double) * 2 * (size_t)n);
}

int or_fft3(int n0, int n1, int n2, double* data, int sign) {
  int dims[3] = {n0, n1, n2};
  int f[40];
  for (int d = 0; d < 3; d++)
    if (dims[d] > 1 && fft_factor(dims[d], f) < 0) return STZ_ERR_INVALID;
  /* strides in complex elements */
  long st[3] = {(long)n1 * n2, n2, 1};
  for (int d = 0; d < 3; d++) {
    int n = dims[d];
    if (n == 1) continue;
    long nlines = (long)n0 * n1 * n2 / n;
    double* tw = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    for (int k = 0; k < n; k++) {
      tw[2 * k] = cos(2.0 * M_PI * (double)k / (double)n);
      tw[2 * k + 1] = sin(2.0 * M_PI * (double)k / (double)n);
    }
#pragma omp parallel
    {
      double* buf = (double*)malloc(sizeof(double) * 4 * (size_t)n);
#pragma omp for schedule(static)
      for (long l = 0; l < nlines; l++) {
        /* decompose line index over the two other axes */
        long rem = l, base = 0;
        for (int e = 2; e >= 0; e--) {
          if (e == d) continue;
          long idx = rem % dims[e];
          rem /= dims[e];
          base += idx * st[e];
        }
        for (int i = 0; i < n; i++) {
          buf[2 * i] = data[2 * (base + i * st[d])];
          buf[2 * i + 1] = data[2 * (base + i * st[d]) + 1];
        }
        fft_line(n, buf, buf + 2 * n, sign, tw);
        for (int i = 0; i < n; i++) {
          data[2 * (base + i * st[d])] = buf[2 * i];
          data[2 * (base + i * st[d]) + 1] = buf[2 * i + 1];
        }
      }
      free(buf);
    }
    free(tw);
  }
  return STZ_OK;
}

void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int or_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* =================================================================== model */
/* Physical constants of bmg.h:71-90 */
#define OR_EV_IN_J 1.60217733e-19
#define OR_J_IN_EV (1 / OR_EV_IN_J)
#define OR_EPSILON 1e-17
#define OR_BOLZ 1.380658e-23

struct or_model {
  stz_params p;
  int dim, nc;           /* 2 -> 3 Voigt comps (xx yy xy); 3 -> 6 */
  int n0, n1, n2;
  long N;
  double kT, dt, vt;     /* kT (eV), elastic step dt, V0 * nu0 */
  or_rng rng;
  /* fields */
  double* eps0[6];
  double* sigma[6];
  double* Q;             /* [MODES][N] activation energies of the current step */
  /* REF2D */
  double* Q0;            /* [MODES][N] */
  double* Q1;            /* [MODES][N] initial copy (bmg.c:221 reset) */
  double* deps;          /* [MODES][3][N] */
  int8_t* mro;           /* [N] crystal-like MRO type 0..3, NULL for an all-glass map */
  double* mro_theta;     /* [N] MROthe0 */
  /* GLOBAL3D */
  double* dF;            /* [N] */
  double modes[STZ_MODES][6];
  /* memory / softening */
  double* prev_deps[6];  /* increment of the last transformation at each site */
  double* perm_soft;
  double* temp_soft;
  double* tlast;
  double* softening;
  /* scalars */
  double eps_avg[6], stress[6], totime;
  int64_t step, kstep, astep, estep, n_print;
  double last_print_strain;
  int stopped;
  /* work */
  double* rate;          /* [MODES*N] */
  double* work;          /* complex buffers for the solver: nc * N * 2 */
  /* log */
  stz_event* log;
  int64_t nlog, caplog;
  /* forced path (or_force_path): the thermal events to take instead of the
   * oracle's own choices, and what the oracle would have chosen */
  int64_t* force_site;
  int32_t* force_mode;
  int32_t* force_draws;
  int64_t force_n, force_i;
  double* force_check;   /* [force_n][7]: own site, own mode, dice, forced element's
                            cumulative interval (lower, upper), total rate, own draws */
  int sel_slack;         /* 0: the reference's selection; > 0: the line-bound rule
                            (or_set_bounded_selection) */
  double* line_cb;       /* bounded rule: cumulative line bounds */
};

static int is2d(const or_model* m) { return m->dim == 2; }

/* Voigt helpers. 2D comps: 0 xx, 1 yy, 2 xy. 3D: xx yy zz yz xz xy. */
static int shear_comp(const or_model* m) { return is2d(m) ? 2 : STZ_XY; }
static double voigt_weight(const or_model* m, int c) {
  if (is2d(m)) return c == 2 ? 2.0 : 1.0;
  return c >= 3 ? 2.0 : 1.0;
}

static void log_event(or_model* m, int kind, long site, int mode, double dt, double q, double R, double margin,
                      int draws) {
  if (m->nlog == m->caplog) {
    m->caplog = m->caplog ? m->caplog * 2 : 1024;
    m->log = (stz_event*)realloc(m->log, sizeof(stz_event) * (size_t)m->caplog);
  }
  stz_event* e = &m->log[m->nlog++];
  memset(e, 0, sizeof(*e));
  e->step = m->step; e->site = site; e->kind = kind; e->mode = mode;
  e->time = m->totime; e->dt = dt; e->q = q; e->total_rate = R;
  e->margin = margin; e->draws = draws;
}

/* isotropicinv (elastic.c:522-531) generalised to DIM dimensions:
 * e = s/(2mu) - lambda/(2mu (DIM lambda + 2mu)) tr(s) I. In 2D the operation
 * order is the reference's. */
static void iso_inv(const or_model* m, const double* s, double* e) {
  double lam = m->p.lambda, mu = m->p.mu;
  if (is2d(m)) {
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

/* ------------------------------------------------------------- initialise */
/* Crystal-like MRO types: 0 glass, 1 six-fold, 2 two-fold, 3 ten-fold. Per
 * type: the amplitude of mode 0 in units of gamma0 (elastic.c:68-112), the
 * number of slip modes (XMODES_SIX/TWO/TEN, bmg.h:30-32; the other modes have
 * no eigenstrain) and the factor NO_SF_XTAL_MRO applies to the direction
 * modifier and to the softening in ActEnergy (init.c:645-660). */
static const double kMroAmp[4] = {0.0, 0.5, 0.8, 0.5};
static const int kMroModes[4] = {0, 6, 2, 12};
static const double kMroFactor[4] = {1.0, 0.1, 0.01, 0.9};
#define OR_PI 3.14159265359 /* the reference's PI, bmg.h:74 */

/* a factor 1 + 0.2 (2u - 1) of the MRO mode rotation (elastic.c:72-79) */
static double mro_jitter(or_model* m) { return 1. + 0.2 * (2 * or_rng_uniform(&m->rng) - 1.); }

static int init_ref2d(or_model* m) {
  long N = m->N;
  /* Alloc(): the MRO map (init.c:350-437). InitMRO 0: one uniform per site;
   * a site at or below xMROFrac is six-fold with an angle uniform on
   * [-PI/2, PI/2) (a second uniform). InitMRO 1: the types and angles of a
   * structure file, then one uniform per ten-fold site, below 0.5 making it
   * two-fold. */
  int any_mro = 0;
  int8_t* t = (int8_t*)calloc((size_t)N, 1);
  double* th = (double*)calloc((size_t)N, sizeof(double));
  if (m->p.init_mro == 0) {
    for (long s = 0; s < N; s++) {
      double tmp = or_rng_uniform(&m->rng);
      if (tmp <= m->p.xmro_frac) {
        any_mro = 1;
        t[s] = 1;
        th[s] = or_rng_uniform(&m->rng) * OR_PI - OR_PI / 2.0;
      }
    }
  } else if (m->p.init_mro == 1) {
    if (!m->p.mro_type || !m->p.mro_theta) { free(t); free(th); return STZ_ERR_INVALID; }
    for (long s = 0; s < N; s++) {
      int32_t v = m->p.mro_type[s];
      if (v < 0 || v > 3) { free(t); free(th); return STZ_ERR_INVALID; }
      t[s] = (int8_t)v;
      th[s] = m->p.mro_theta[s];
      any_mro |= v != 0;
    }
    for (long s = 0; s < N; s++)
      if (t[s] == 3) {
        double tmp = or_rng_uniform(&m->rng);
        if (tmp < 0.5) t[s] = 2;
      }
  } else {
    free(t); free(th);
    return STZ_ERR_INVALID;
  }
  m->mro_theta = th;
  if (any_mro) m->mro = t;
  else free(t);
  /* Energy_Init (init.c:181-198): Q0 = N(0, 0.25) + Q0amp, mode-major, every
   * site (its MRO branch is commented out in the reference). */
  for (int mo = 0; mo < STZ_MODES; mo++)
    for (long s = 0; s < N; s++) {
      double q = or_ran_gaussian(&m->rng, m->p.q0_sd) + m->p.q0_mean;
      m->Q0[mo * N + s] = q;
      m->Q1[mo * N + s] = q;
    }
  /* DStrain (elastic.c:61-137), mode-major. Glass: two normal draws. MRO:
   * mode 0 along the site's angle; modes 1..X-1 that increment rotated by
   * m 2PI/X, angle and the two terms of each component jittered by
   * 1 + 0.2 (2u - 1) (five uniforms, taken in the order the reference's
   * expressions evaluate them when built with gcc: left term first); the
   * other modes zero. */
  for (int mo = 0; mo < STZ_MODES; mo++)
    for (long s = 0; s < N; s++) {
      double* d = m->deps + (size_t)mo * 3 * N;
      int ty = m->mro ? m->mro[s] : 0;
      if (ty == 0) {
        d[0 * N + s] = 0.5 * m->p.gamma0 * or_ran_gaussian(&m->rng, 1.0);
        d[1 * N + s] = -d[0 * N + s];
        d[2 * N + s] = 0.5 * m->p.gamma0 * or_ran_gaussian(&m->rng, 1.0);
      } else if (mo == 0) {
        d[0 * N + s] = kMroAmp[ty] * m->p.gamma0 * cos(th[s]);
        d[1 * N + s] = -d[0 * N + s];
        d[2 * N + s] = kMroAmp[ty] * m->p.gamma0 * sin(th[s]);
      } else if (mo < kMroModes[ty]) {
        const double a0 = m->deps[s], a2 = m->deps[2 * N + s];  /* mode 0 of the site */
        double tt = mo * 2. * OR_PI / kMroModes[ty] * mro_jitter(m);
        double j1 = mro_jitter(m), j2 = mro_jitter(m);
        d[0 * N + s] = a0 * j1 * cos(2 * tt) + a2 * j2 * sin(2 * tt);
        d[1 * N + s] = -d[0 * N + s];
        double j3 = mro_jitter(m), j4 = mro_jitter(m);
        d[2 * N + s] = -a0 * j3 * sin(2 * tt) + a2 * j4 * cos(2 * tt);
      } else {
        d[0 * N + s] = 0.0;
        d[1 * N + s] = 0.0;
        d[2 * N + s] = 0.0;
      }
    }
  return STZ_OK;
}

/* Uniform random rotation from a point uniform on S^3 (Marsaglia 1972: two
 * points uniform in the unit disk). Needs only +,*,/ and sqrt, so it is
 * bit-identical on every IEEE host. */
static void random_rotation(or_rng* r, double R[3][3]) {
  double x1, x2, s1, x3, x4, s2;
  do {
    x1 = 2 * or_rng_uniform(r) - 1;
    x2 = 2 * or_rng_uniform(r) - 1;
    s1 = x1 * x1 + x2 * x2;
  } while (s1 >= 1.0);
  do {
    x3 = 2 * or_rng_uniform(r) - 1;
    x4 = 2 * or_rng_uniform(r) - 1;
    s2 = x3 * x3 + x4 * x4;
  } while (s2 >= 1.0 || s2 == 0.0);
  double t = sqrt((1 - s1) / s2);
  double w = x1, x = x2, y = x3 * t, z = x4 * t;
  R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - z * w);     R[0][2] = 2 * (x * z + y * w);
  R[1][0] = 2 * (x * y + z * w);     R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - x * w);
  R[2][0] = 2 * (x * z - y * w);     R[2][1] = 2 * (y * z + x * w);     R[2][2] = 1 - 2 * (x * x + y * y);
}

static int gen_dF(or_model* m);

static int init_global3d(or_model* m) {
  /* 20 global modes: eps* = gamma0/2 (a b^T + b a^T), a = R e_x, b = R e_y,
   * from the main stream or from their own stream (mode_seed_set) */
  or_rng mrng;
  if (m->p.mode_seed_set) or_rng_seed(&mrng, (unsigned long)(uint32_t)m->p.mode_seed);
  or_rng* const modes_rng = m->p.mode_seed_set ? &mrng : &m->rng;
  for (int mo = 0; mo < STZ_MODES; mo++) {
    double R[3][3];
    random_rotation(modes_rng, R);
    double a[3] = {R[0][0], R[1][0], R[2][0]};
    double b[3] = {R[0][1], R[1][1], R[2][1]};
    double g = 0.5 * m->p.gamma0;
    m->modes[mo][STZ_XX] = g * (2 * a[0] * b[0]);
    m->modes[mo][STZ_YY] = g * (2 * a[1] * b[1]);
    m->modes[mo][STZ_ZZ] = g * (2 * a[2] * b[2]);
    m->modes[mo][STZ_YZ] = g * (a[1] * b[2] + a[2] * b[1]);
    m->modes[mo][STZ_XZ] = g * (a[0] * b[2] + a[2] * b[0]);
    m->modes[mo][STZ_XY] = g * (a[0] * b[1] + a[1] * b[0]);
  }
  return gen_dF(m);
}

/* Barrier field dF for GLOBAL3D. Truncated normal: per site, in index order,
 * redraw z until |z| <= trunc. Correlated: white N(0,1) per site, filtered by
 * the square root of a Gaussian covariance spectrum, renormalised to unit
 * variance, clipped at +-trunc. */
static int gen_dF(or_model* m) {
  long N = m->N;
  double tr = m->p.q0_trunc;
  if (m->p.df_kind == STZ_DF_TRUNC_NORMAL) {
    for (long s = 0; s < N; s++) {
      double z;
      do { z = or_ran_gaussian(&m->rng, 1.0); } while (tr > 0 && fabs(z) > tr);
      m->dF[s] = m->p.q0_mean + m->p.q0_sd * z;
    }
    return STZ_OK;
  }
  if (m->p.df_kind != STZ_DF_CORRELATED) return STZ_ERR_INVALID;
  double* c = (double*)calloc((size_t)N * 2, sizeof(double));
  if (!c) return STZ_ERR_NOMEM;
  for (long s = 0; s < N; s++) c[2 * s] = or_ran_gaussian(&m->rng, 1.0);
  or_fft3(m->n0, m->n1, m->n2, c, -1);
  double l = m->p.q0_corr_len;
  for (int i0 = 0; i0 < m->n0; i0++)
    for (int i1 = 0; i1 < m->n1; i1++)
      for (int i2 = 0; i2 < m->n2; i2++) {
        double f0 = (double)i0 / m->n0; f0 -= round(f0);
        double f1 = (double)i1 / m->n1; f1 -= round(f1);
        double f2 = (double)i2 / m->n2; f2 -= round(f2);
        double k2 = 4 * M_PI * M_PI * (f0 * f0 + f1 * f1 + f2 * f2);
        /* covariance exp(-r^2/(2 l^2)) has spectrum ~ exp(-k^2 l^2 / 2);
           the filter is its square root */
        double w = exp(-0.25 * k2 * l * l);
        long s = ((long)i0 * m->n1 + i1) * m->n2 + i2;
        c[2 * s] *= w; c[2 * s + 1] *= w;
      }
  c[0] = 0; c[1] = 0; /* zero mean */
  or_fft3(m->n0, m->n1, m->n2, c, +1);
  double ss = 0;
  for (long s = 0; s < N; s++) ss += c[2 * s] * c[2 * s];
  double sd = sqrt(ss / N);
  for (long s = 0; s < N; s++) {
    double z = c[2 * s] / sd;
    if (tr > 0) { if (z > tr) z = tr; if (z < -tr) z = -tr; }
    m->dF[s] = m->p.q0_mean + m->p.q0_sd * z;
  }
  free(c);
  return STZ_OK;
}

/* --------------------------------------------------------------- solver */
/* HomogeneousStressSolver with uflag 0 (elastic.c:779-828) generalised to 3D:
 * eps*_hat = FFT(eps*); tau = C:eps*_hat; F_i = tau_ij g_j; G = g.F;
 * eps_hat_ij = (F_i g_j + F_j g_i)/(2 mu) - (alpha/mu) G g_i g_j with
 * alpha = (lambda+mu)/(lambda+2mu) and g the unit wave vector of Grad()
 * (init.c:112-140, zero at k = 0); eps = Re IFFT(eps_hat)/N + eps_avg;
 * sigma = C:(eps - eps*); Stress = <sigma> (AvgStress, elastic.c:733-752). */
static void homogeneous_solve(or_model* m, double* const* eps_in) {
  long N = m->N;
  int nc = m->nc, D = m->dim;
  double lam = m->p.lambda, mu = m->p.mu;
  double alpha = (lam + mu) / (lam + 2.0 * mu);
  double* W = m->work;
  for (int c = 0; c < nc; c++) {
    double* w = W + (size_t)c * 2 * N;
    for (long s = 0; s < N; s++) { w[2 * s] = eps_in[c][s]; w[2 * s + 1] = 0.; }
    or_fft3(m->n0, m->n1, m->n2, w, -1);
  }
  /* component index pairs */
  int ci[6], cj[6];
  if (D == 2) { ci[0] = 0; cj[0] = 0; ci[1] = 1; cj[1] = 1; ci[2] = 0; cj[2] = 1; }
  else {
    int a[6] = {0, 1, 2, 1, 0, 0}, b[6] = {0, 1, 2, 2, 2, 1};
    for (int c = 0; c < 6; c++) { ci[c] = a[c]; cj[c] = b[c]; }
  }
#pragma omp parallel for schedule(static)
  for (long s = 0; s < N; s++) {
    int i2 = (int)(s % m->n2);
    int i1 = (int)((s / m->n2) % m->n1);
    int i0 = (int)(s / ((long)m->n1 * m->n2));
    /* Grad(): s1 from the fast index, s2 from the slow one; wrap s - round(s).
     * Cartesian x <- axis 2, y <- axis 1, z <- axis 0. */
    double g[3];
    double s1 = (double)i2 * (1.0 / m->n2);
    double s2 = (double)i1 * (1.0 / m->n1);
    double s3 = (double)i0 * (1.0 / m->n0);
    g[0] = (s1 - round(s1)) * (2 * 3.14159265359);
    g[1] = (s2 - round(s2)) * (2 * 3.14159265359);
    g[2] = (s3 - round(s3)) * (2 * 3.14159265359);
    double g2 = sqrt(g[0] * g[0] + g[1] * g[1] + (D == 3 ? g[2] * g[2] : 0.0));
    if (s == 0) g2 = 1.0;
    g[0] /= g2; g[1] /= g2; g[2] /= g2;
    if (D == 2) g[2] = 0;
    /* 3D only: at wave vectors with Nyquist components the operator is
     * averaged over the signs of those components (all 2^k choices), which
     * keeps the discrete Green's function symmetric under reflections of each
     * axis. The 2D path keeps the reference's operator unchanged. */
    int nyq[3] = {0, 0, 0};
    if (D == 3) {
      nyq[0] = (m->n2 % 2 == 0) && (2 * i2 == m->n2);
      nyq[1] = (m->n1 % 2 == 0) && (2 * i1 == m->n1);
      nyq[2] = (m->n0 % 2 == 0) && (2 * i0 == m->n0);
    }
    double er[6], ei[6], tr_r = 0, tr_i = 0;
    for (int c = 0; c < nc; c++) {
      er[c] = W[(size_t)c * 2 * N + 2 * s];
      ei[c] = W[(size_t)c * 2 * N + 2 * s + 1];
    }
    for (int c = 0; c < D; c++) { tr_r += er[c]; tr_i += ei[c]; }
    /* tau = C:eps* (IsotropicMul_C, elastic.c:652-670) as a symmetric matrix */
    double tr[3][3] = {{0}}, ti[3][3] = {{0}};
    for (int c = 0; c < nc; c++) {
      double vr = 2 * mu * er[c], vi = 2 * mu * ei[c];
      if (ci[c] == cj[c]) { vr += lam * tr_r; vi += lam * tr_i; }
      tr[ci[c]][cj[c]] = vr; tr[cj[c]][ci[c]] = vr;
      ti[ci[c]][cj[c]] = vi; ti[cj[c]][ci[c]] = vi;
    }
    double accr[6] = {0}, acci[6] = {0};
    int nvar = 0;
    for (int sgn = 0; sgn < 8; sgn++) {
      if (((sgn & 1) && !nyq[0]) || ((sgn & 2) && !nyq[1]) || ((sgn & 4) && !nyq[2])) continue;
      double gv[3] = {(sgn & 1) ? -g[0] : g[0], (sgn & 2) ? -g[1] : g[1], (sgn & 4) ? -g[2] : g[2]};
      double Fr[3], Fi[3], Gr = 0, Gi = 0;
      for (int a = 0; a < 3; a++) {
        Fr[a] = 0; Fi[a] = 0;
        for (int b = 0; b < 3; b++) { Fr[a] += tr[a][b] * gv[b]; Fi[a] += ti[a][b] * gv[b]; }
      }
      for (int a = 0; a < 3; a++) { Gr += gv[a] * Fr[a]; Gi += gv[a] * Fi[a]; }
      for (int c = 0; c < nc; c++) {
        int a = ci[c], b = cj[c];
        accr[c] += (0.5 / mu) * (Fr[a] * gv[b] + Fr[b] * gv[a]) + (-1.0 * alpha / mu) * (Gr * (gv[a] * gv[b]));
        acci[c] += (0.5 / mu) * (Fi[a] * gv[b] + Fi[b] * gv[a]) + (-1.0 * alpha / mu) * (Gi * (gv[a] * gv[b]));
      }
      nvar++;
    }
    for (int c = 0; c < nc; c++) {
      W[(size_t)c * 2 * N + 2 * s] = nvar == 1 ? accr[c] : accr[c] / nvar;
      W[(size_t)c * 2 * N + 2 * s + 1] = nvar == 1 ? acci[c] : acci[c] / nvar;
    }
  }
  double sum[6] = {0};
  for (int c = 0; c < nc; c++) {
    double* w = W + (size_t)c * 2 * N;
    or_fft3(m->n0, m->n1, m->n2, w, +1);
  }
  /* eps = Re/N + eps_avg ; sigma = C:(eps - eps*) (IsotropicMul_R2, elastic.c:703-718) */
  for (long s = 0; s < N; s++) {
    double e[6], tr = 0;
    for (int c = 0; c < nc; c++) {
      double tot = W[(size_t)c * 2 * N + 2 * s] / N + m->eps_avg[c];
      e[c] = tot - eps_in[c][s];
    }
    for (int c = 0; c < D; c++) tr += e[c];
    tr *= lam;
    for (int c = 0; c < nc; c++) {
      int diag = is2d(m) ? (c < 2) : (c < 3);
      m->sigma[c][s] = diag ? tr + 2.0 * mu * e[c] : 2.0 * mu * e[c];
    }
  }
  for (int c = 0; c < nc; c++) {
    double acc = 0;
    for (long s = 0; s < N; s++) acc += m->sigma[c][s];
    sum[c] = acc;
    m->stress[c] = sum[c] / N;
  }
}

/* InhomogeneousStressSolver (elastic.c:977-1066) for homogeneous moduli
 * (Lambda = lambda, Mu = mu, init.c:462): it converges after one homogeneous
 * solve whose eigenstrain is the round trip C^-1:(C:eps*) (elastic.c:999-1009,
 * 1025-1026). In 3D the eigenstrain is used directly. */
int or_solve(or_model* m) {
  long N = m->N;
  if (is2d(m)) {
    double* rt[3];
    for (int c = 0; c < 3; c++) rt[c] = m->rate + (size_t)c * N; /* scratch */
    double lam = m->p.lambda, mu = m->p.mu;
    for (long s = 0; s < N; s++) {
      double e0 = m->eps0[0][s], e1 = m->eps0[1][s], e2 = m->eps0[2][s];
      double tra = lam * (e0 + e1);
      double t[3] = {tra + 2 * mu * e0, tra + 2 * mu * e1, 2 * mu * e2};
      double tra2 = -1.0 * lam / 2.0 / mu / (2.0 * lam + 2.0 * mu) * (t[0] + t[1]);
      rt[0][s] = tra2 + t[0] / 2.0 / mu;
      rt[1][s] = tra2 + t[1] / 2.0 / mu;
      rt[2][s] = t[2] / 2.0 / mu;
    }
    homogeneous_solve(m, rt);
  } else {
    homogeneous_solve(m, m->eps0);
  }
  return STZ_OK;
}

/* ------------------------------------------------------ activation energy */
/* Direction modifier of the softening schemes (init.c:590-642). */
static double dire_modifier(int scheme, double dot, double n1, double n2) {
  double DM;
  switch (scheme) {
    case STZ_SF_LINEAR_FWD:
      DM = dot / (n1 + OR_EPSILON) / (n2 + OR_EPSILON); return (DM + 1) / 2;
    case STZ_SF_LINEAR_BWD:
      DM = dot / (n1 + OR_EPSILON) / (n2 + OR_EPSILON); return (-DM + 1) / 2;
    case STZ_SF_EVEN: return 0.5;
    case STZ_SF_SQUARE_FWD:
      DM = dot / (n1 + OR_EPSILON) / (n2 + OR_EPSILON); return (1 + DM) * (1 + DM) / 4;
    case STZ_SF_CUBIC_FWD:
      DM = dot / (n1 + OR_EPSILON) / (n2 + OR_EPSILON); return (DM + 1) * (DM + 1) * (DM + 1) / 8;
    default:
      DM = dot / (n1 + OR_EPSILON) / (n2 + OR_EPSILON); return exp(-DM * DM * 9 / 2);
  }
}

/* SofteningFactor (init.c:711-739, default branch) and ActEnergy
 * (init.c:561-690) with MICRO_MEMORY and NO_SF_XTAL_MRO. At a crystal-like
 * site the reference multiplies the direction modifier and, in place, the
 * site's Softening by the type's factor for every mode in turn, so mode m sees
 * the softening times the factor m + 1 times (each product rounded).
 * PreDEps0[PreSelectMode[s]][:][s] is kept as prev_deps[:][s]: VoxelShearTransform
 * copies every mode's DEps0 into PreDEps0 (elastic.c:369-374) and KMC then sets
 * PreSelectMode to the transformed mode (evolution.c:208), so ActEnergy only
 * ever reads the increment of the site's last transformation. */
static long act_energy(or_model* m) {
  long N = m->N;
  int nc = m->nc;
  double V0 = m->p.voxel_volume;
  if (m->p.softening) {
    for (long s = 0; s < N; s++)
      m->softening[s] = m->perm_soft[s] + m->temp_soft[s] * exp((m->tlast[s] - m->totime) / m->p.t_temp);
  }
  long flag = 0;
#pragma omp parallel for schedule(static) reduction(+ : flag)
  for (long s = 0; s < N; s++) {
    double sg[6], pd[6];
    for (int c = 0; c < nc; c++) { sg[c] = m->sigma[c][s]; pd[c] = m->prev_deps[c][s]; }
    double n2 = 0;
    if (is2d(m)) n2 = sqrt(pd[0] * pd[0] + pd[1] * pd[1] + 2 * pd[2] * pd[2]);
    const int ty = (m->mro && m->p.no_sf_xtal_mro) ? m->mro[s] : 0;
    double soft = m->softening[s];
    for (int mo = 0; mo < STZ_MODES; mo++) {
      double d[6], q0;
      if (is2d(m)) {
        const double* dd = m->deps + (size_t)mo * 3 * N;
        d[0] = dd[s]; d[1] = dd[N + s]; d[2] = dd[2 * N + s];
        q0 = m->Q0[(size_t)mo * N + s];
      } else {
        for (int c = 0; c < 6; c++) d[c] = m->modes[mo][c];
        q0 = m->dF[s];
      }
      double DWork, Q;
      if (is2d(m)) {
        DWork = (sg[0] * d[0] + sg[1] * d[1] + 2 * sg[2] * d[2]) * V0 * 1e-18 * OR_J_IN_EV;
        double dot = pd[0] * d[0] + pd[1] * d[1] + 2 * pd[2] * d[2];
        double n1 = sqrt(d[0] * d[0] + d[1] * d[1] + 2 * d[2] * d[2]);
        double DM = dire_modifier(m->p.sf_scheme, dot, n1, n2);
        if (ty) {
          DM *= kMroFactor[ty];
          soft *= kMroFactor[ty];
        }
        Q = q0 * exp(-DM * soft) - DWork / 2;
      } else {
        double w = 0;
        for (int c = 0; c < 6; c++) w += voigt_weight(m, c) * sg[c] * d[c];
        DWork = w * V0 * 1e-18 * OR_J_IN_EV;
        Q = q0 - DWork / 2;
      }
      m->Q[(size_t)mo * N + s] = Q;
      if (Q < 0) flag++;
    }
  }
  return flag;
}

/* --------------------------------------------------------- transformation */
/* VoxelShearTransform (elastic.c:361-520). Glass sites draw new mode
 * eigenstrains; crystal-like sites keep theirs and draw new barriers
 * xQ0amp (1 - RandomRatio + RandomRatio u), and a six-fold site softens with
 * PermSoftmro and TempSoftmro. */
static void voxel_transform(or_model* m, int mm, long s) {
  long N = m->N;
  int nc = m->nc;
  double d[6];
  if (is2d(m)) {
    const double* dd = m->deps + (size_t)mm * 3 * N;
    d[0] = dd[s]; d[1] = dd[N + s]; d[2] = dd[2 * N + s];
  } else {
    for (int c = 0; c < 6; c++) d[c] = m->modes[mm][c];
  }
  for (int c = 0; c < nc; c++) {
    m->prev_deps[c][s] = d[c];
    m->eps0[c][s] += d[c];
  }
  double ds = 0;
  for (int c = 0; c < nc; c++) ds += voigt_weight(m, c) * d[c] * d[c];
  if (is2d(m)) ds = d[0] * d[0] + d[1] * d[1] + 2 * d[2] * d[2];
  const int ty = m->mro ? m->mro[s] : 0;
  m->perm_soft[s] += ds * (ty == 1 ? m->p.perm_soft_mro : m->p.perm_soft);
  if (m->perm_soft[s] > m->p.perm_soft_cap) m->perm_soft[s] = m->p.perm_soft_cap;
  m->temp_soft[s] = ds * (ty == 1 ? m->p.temp_soft_mro : m->p.temp_soft);
  m->tlast[s] = m->totime;
  if (ty) {
    for (int i = 0; i < STZ_MODES; i++)
      m->Q0[(size_t)i * N + s] = m->p.xq0amp * (1 - m->p.random_ratio + m->p.random_ratio * or_rng_uniform(&m->rng));
  } else if (is2d(m)) {
    for (int i = 0; i < STZ_MODES; i++) {
      double* dd = m->deps + (size_t)i * 3 * N;
      dd[s] = 0.5 * m->p.gamma0 * or_ran_gaussian(&m->rng, 1.0);
      dd[N + s] = -dd[s];
      dd[2 * N + s] = 0.5 * m->p.gamma0 * or_ran_gaussian(&m->rng, 1.0);
    }
  }
}

/* ------------------------------------------------------ loading helpers */
static int loaded_comp(const or_model* m) {
  if (m->p.loading == STZ_LOAD_SHEAR) return shear_comp(m);
  return 0;
}

/* Mean-stress correction after a solve: tmpStress = Stress with the loaded
 * component zeroed (evolution.c:264,283,300), eps_avg -= C^-1 tmpStress.
 * 'athermal' selects the mask of evolution.c:92 (first comp zeroed) in 2D. */
static void subtract_error(or_model* m, int athermal, double* tmpStrain) {
  double ts[6] = {0};
  int nc = m->nc;
  if (!m->p.no_subtract_error) {
    for (int c = 0; c < nc; c++) ts[c] = m->stress[c];
    int zc = (athermal && is2d(m)) ? 0 : loaded_comp(m);
    ts[zc] = 0.0;
  }
  iso_inv(m, ts, tmpStrain);
}

static void uniform_sigma_add(or_model* m, int c, double v) {
  for (long s = 0; s < m->N; s++) m->sigma[c][s] += v;
}

/* STZ_LOAD_STRESS: hold <sigma> at applied_stress by shifting the mean strain
 * and the stress field together. */
static void hold_stress(or_model* m) {
  double d[6] = {0}, de[6];
  for (int c = 0; c < m->nc; c++) d[c] = m->p.applied_stress[c] - m->stress[c];
  iso_inv(m, d, de);
  for (int c = 0; c < m->nc; c++) {
    m->eps_avg[c] += de[c];
    uniform_sigma_add(m, c, d[c]);
    m->stress[c] = m->p.applied_stress[c];
  }
}

/* Loading after a thermal event (evolution.c:262-317). */
static void load_after_event(or_model* m, double t_kmc) {
  double ts[6];
  double rate = m->p.strain_rate, nu = m->p.poisson, E = m->p.young, mu = m->p.mu;
  int nc = m->nc;
  switch (m->p.loading) {
    case STZ_LOAD_TENSION:
      subtract_error(m, 0, ts);
      m->eps_avg[0] += (rate * t_kmc * 1 - ts[0]);
      m->eps_avg[1] += (rate * t_kmc * (-nu) - ts[1]);
      if (is2d(m)) m->eps_avg[2] += (-ts[2]);
      else {
        m->eps_avg[2] += (rate * t_kmc * (-nu) - ts[2]);
        for (int c = 3; c < 6; c++) m->eps_avg[c] += (-ts[c]);
      }
      m->stress[0] += E * rate * t_kmc;
      uniform_sigma_add(m, 0, E * rate * t_kmc);
      break;
    case STZ_LOAD_COMPRESSION:
      /* evolution.c:262-280, including the doubled increments of 268-269 */
      subtract_error(m, 0, ts);
      m->eps_avg[0] += (-rate * t_kmc * 1);
      m->eps_avg[1] += (rate * t_kmc * (nu));
      m->eps_avg[0] += (-rate * t_kmc * 1 - ts[0]);
      m->eps_avg[1] += (rate * t_kmc * (nu) - ts[1]);
      for (int c = 2; c < nc; c++) m->eps_avg[c] += (-ts[c]);
      m->stress[0] += -E * rate * t_kmc;
      uniform_sigma_add(m, 0, -E * rate * t_kmc);
      break;
    case STZ_LOAD_SHEAR: {
      int sc = shear_comp(m);
      subtract_error(m, 0, ts);
      for (int c = 0; c < nc; c++) if (c != sc) m->eps_avg[c] += -ts[c];
      m->eps_avg[sc] += rate * t_kmc;
      m->stress[sc] += 2 * mu * rate * t_kmc;
      uniform_sigma_add(m, sc, 2 * mu * rate * t_kmc);
      break;
    }
    case STZ_LOAD_STRESS:
      hold_stress(m);
      break;
  }
}

/* Pure elastic step (evolution.c:321-358). */
static void elastic_step(or_model* m) {
  double inc = m->p.strain_increment, nu = m->p.poisson, E = m->p.young, mu = m->p.mu;
  switch (m->p.loading) {
    case STZ_LOAD_TENSION:
      m->eps_avg[0] += (inc * 1);
      m->eps_avg[1] += (inc * (-nu));
      if (is2d(m)) m->eps_avg[2] += (inc * 0.0);
      else m->eps_avg[2] += (inc * (-nu));
      m->stress[0] += E * inc;
      uniform_sigma_add(m, 0, E * inc);
      break;
    case STZ_LOAD_COMPRESSION:
      m->eps_avg[0] += (inc * (-1));
      m->eps_avg[1] += (inc * (nu));
      if (is2d(m)) m->eps_avg[2] += (inc * 0.0);
      else m->eps_avg[2] += (inc * (nu));
      m->stress[0] += -E * inc;
      uniform_sigma_add(m, 0, -E * inc);
      break;
    case STZ_LOAD_SHEAR: {
      int sc = shear_comp(m);
      if (m->p.shear_elastic_quirk) m->eps_avg[sc] += m->p.strain_rate * 1;
      else m->eps_avg[sc] += inc;
      m->stress[sc] += 2 * mu * inc;
      uniform_sigma_add(m, sc, 2 * mu * inc);
      break;
    }
    case STZ_LOAD_STRESS:
      break;
  }
}

/* --------------------------------------------------------------- athermal */
static int athermal(or_model* m) {
  long N = m->N;
  m->astep++;
  for (long s = 0; s < N; s++) {
    int mm = 0;
    double minQ = m->Q[s];
    for (int mo = 0; mo < STZ_MODES; mo++)
      if (minQ > m->Q[(size_t)mo * N + s]) { mm = mo; minQ = m->Q[(size_t)mo * N + s]; }
    if (minQ < 0 || fabs(minQ) < 0.33) {
      voxel_transform(m, mm, s);
      log_event(m, STZ_EV_ATHERMAL, s, mm, 0.0, minQ, 0.0, 0.0, 0);
    }
  }
  or_solve(m);
  if (m->p.loading == STZ_LOAD_STRESS) { hold_stress(m); return STZ_OK; }
  double ts[6];
  subtract_error(m, 1, ts);
  for (int c = 0; c < m->nc; c++) m->eps_avg[c] -= ts[c];
  return STZ_OK;
}

/* -------------------------------------------------------------------- KMC */
/* The bounded selection rule (or_set_bounded_selection), for checking another
 * implementation's rejection path: the normalised cumulative rates c[] of the
 * mode-major elements, grouped in lines of n2 consecutive elements; each line
 * j gets the bound B_j = L_j (1 + 2^-slack) of its sum L_j; a dice u picks
 * the line whose bound interval holds T = u sum(B); the rest of T within the
 * line picks the element by the cumulative rates, unless it lies beyond L_j,
 * when the draw is rejected and the next generator word is drawn. Returns
 * the element and the words used in *draws, drawn from g (a copy of the
 * generator as it was before the event's first word). */
static long bounded_select(or_model* m, const double* c, long M, or_rng g, double* dice_used, int* draws) {
  const long n2 = m->n2, nl = M / n2;
  const double f = 1.0 + ldexp(1.0, -m->sel_slack);
  double* cb = m->line_cb;
  double run = 0;
  for (long j = 0; j < nl; j++) {
    const double base = j ? c[j * n2 - 1] : 0.0;
    cb[j] = run;
    run += (c[(j + 1) * n2 - 1] - base) * f;
  }
  const double RB = run;
  for (int d = 1; d < 1000; d++) {
    const double u = or_rng_uniform(&g);
    const double T = u * RB;
    long lo = 0, hi = nl - 1;  /* last line with cb <= T */
    while (lo < hi) {
      long mid = lo + (hi - lo + 1) / 2;
      if (cb[mid] <= T) lo = mid; else hi = mid - 1;
    }
    const long j = lo;
    const double base = j ? c[j * n2 - 1] : 0.0;
    const double rem = T - cb[j];
    if (rem >= c[(j + 1) * n2 - 1] - base) continue;  /* in the line's slack */
    long i = j * n2;
    while (i < (j + 1) * n2 - 1 && c[i] - base <= rem) i++;
    *draws = d;
    *dice_used = u;
    return i;
  }
  *draws = 0;
  return -1;
}

static int kmc(or_model* m) {
  long N = m->N, M = (long)STZ_MODES * N;
  double t_kmc = 0;
  double* rate = m->rate;
  /* rates, mode-major index m*N + s (evolution.c:120-128) */
#pragma omp parallel for schedule(static)
  for (long i = 0; i < M; i++) rate[i] = m->vt * exp(-m->Q[i] / m->kT);
  for (long i = 0; i < M; i++) t_kmc += rate[i];
  double R = t_kmc;
  if (!isfinite(R) || !(R > 0)) return STZ_ERR_NAN;
  t_kmc = 1 / t_kmc;
  if (t_kmc < m->dt) {
    m->kstep++;
    const int forced = m->force_i < m->force_n;
    const int draws = forced ? m->force_draws[m->force_i] : 1;
    const or_rng g0 = m->rng;  /* before this event's words */
    for (int k = 1; k < draws; k++) (void)or_rng_get(&m->rng);  /* draws the forced path rejected */
    double dice = or_rng_uniform(&m->rng);
    for (long i = 0; i < M; i++) rate[i] *= t_kmc;
    for (long i = 1; i < M; i++) rate[i] += rate[i - 1];
    long event = -1;
    /* first index whose cumulative value reaches dice (evolution.c:171-224) */
    if (rate[M - 1] >= dice && rate[0] < dice) {
      long lo = 1, hi = M - 1;
      while (lo < hi) {
        long mid = lo + (hi - lo) / 2;
        if (rate[mid] >= dice) hi = mid; else lo = mid + 1;
      }
      event = lo;
    } else if (dice > 0 && dice <= rate[0]) {
      event = 0;
    }
    if (event < 0) return STZ_ERR_NO_EVENT;
    int own_draws = 1;
    if (m->sel_slack > 0) {
      /* the bounded rule: own choice from the same words (a copy of the
       * generator from before this event's draws) */
      double u;
      const long e2 = bounded_select(m, rate, M, g0, &u, &own_draws);
      if (e2 < 0) return STZ_ERR_NO_EVENT;
      event = e2;
      if (!forced)
        for (int k = 1; k < own_draws; k++) (void)or_rng_get(&m->rng);  /* the rejected words */
    }
    if (forced) {
      /* take the forced element; record the oracle's own choice and where the
       * dice lies against the forced element's cumulative interval */
      const long fe = (long)m->force_mode[m->force_i] * N + m->force_site[m->force_i];
      double* ck = m->force_check + 7 * m->force_i;
      ck[0] = (double)(event - (event / N) * N);
      ck[1] = (double)(event / N);
      ck[2] = dice;
      ck[3] = fe > 0 ? rate[fe - 1] : 0.0;
      ck[4] = rate[fe];
      ck[5] = R;
      ck[6] = (double)own_draws;
      m->force_i++;
      event = fe;
    }
    int mo = (int)(event / N);
    long s = event - (long)mo * N;
    double q = m->Q[event];
    const double lo = event > 0 ? rate[event - 1] : 0.0, hi = rate[event];
    const double margin = fmin(dice - lo, hi - dice);
    voxel_transform(m, mo, s);
    or_solve(m);
    load_after_event(m, t_kmc);
    m->totime += t_kmc;
    log_event(m, STZ_EV_THERMAL, s, mo, t_kmc, q, R, margin, forced ? draws : own_draws);
  } else {
    m->estep++;
    m->totime += m->dt;
    elastic_step(m);
    log_event(m, STZ_EV_ELASTIC, -1, -1, m->dt, 0.0, R, 0.0, 0);
  }
  return STZ_OK;
}

/* ------------------------------------------------------------ driver loop */
static int print_and_stop(or_model* m) {
  if (m->p.loading == STZ_LOAD_STRESS) return 0;
  int lc = loaded_comp(m);
  /* print check (bmg.c:181-187); the print re-solves the field (bmg.c:292-295) */
  if (fabs(m->eps_avg[lc] - m->last_print_strain) >= (m->p.print_period * m->p.strain_increment * 0.99)) {
    m->n_print++;
    m->last_print_strain = m->eps_avg[lc];
    if (is2d(m)) memcpy(m->Q0, m->Q1, sizeof(double) * STZ_MODES * (size_t)m->N);
    or_solve(m);
  }
  /* stop conditions (bmg.c:382-410) */
  if (fabs(m->eps_avg[lc]) > m->p.end_strain) { m->stopped = 1; return 1; }
  if (m->p.loading == STZ_LOAD_TENSION && m->stress[0] < -0.5) { m->stopped = 2; return 1; }
  if (m->p.loading == STZ_LOAD_SHEAR && fabs(m->stress[lc]) < OR_EPSILON) { m->stopped = 2; return 1; }
  return 0;
}

int or_run(or_model* m, int64_t max_steps, int64_t max_events) {
  int64_t s0 = m->step, k0 = m->kstep;
  while (!m->stopped && (max_steps <= 0 || m->step - s0 < max_steps) &&
         (max_events <= 0 || m->kstep - k0 < max_events)) {
    m->step++;
    long flag = act_energy(m);
    int st;
    if (flag > 0) st = athermal(m);
    else st = kmc(m);
    if (st != STZ_OK) return st;
    print_and_stop(m);
  }
  return STZ_OK;
}

/* ------------------------------------------------------------ lifecycle */
static void* xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

or_model* or_create(const stz_params* p, int* status) {
  int st = STZ_OK;
  or_model* m = (or_model*)calloc(1, sizeof(or_model));
  m->p = *p;
  m->n0 = p->n[0]; m->n1 = p->n[1]; m->n2 = p->n[2];
  m->dim = p->model == STZ_MODEL_REF2D ? 2 : 3;
  m->nc = m->dim == 2 ? 3 : 6;
  if ((m->dim == 2 && m->n0 != 1) || m->n1 < 1 || m->n2 < 2 || m->n0 < 1) { st = STZ_ERR_INVALID; goto fail; }
  if (m->dim == 3 && p->softening) { st = STZ_ERR_UNSUPPORTED; goto fail; }
  m->N = (long)m->n0 * m->n1 * m->n2;
  m->kT = p->temperature * OR_BOLZ * OR_J_IN_EV;
  m->vt = p->voxel_volume * p->trial_frequency;
  m->dt = p->strain_rate > 0 ? p->strain_increment / p->strain_rate : INFINITY;
  {
    long N = m->N;
    for (int c = 0; c < m->nc; c++) {
      m->eps0[c] = (double*)xcalloc((size_t)N, sizeof(double));
      m->sigma[c] = (double*)xcalloc((size_t)N, sizeof(double));
      m->prev_deps[c] = (double*)xcalloc((size_t)N, sizeof(double));
    }
    m->Q = (double*)xcalloc((size_t)STZ_MODES * N, sizeof(double));
    m->rate = (double*)xcalloc((size_t)STZ_MODES * N, sizeof(double));
    m->work = (double*)xcalloc((size_t)m->nc * 2 * N, sizeof(double));
    m->perm_soft = (double*)xcalloc((size_t)N, sizeof(double));
    m->temp_soft = (double*)xcalloc((size_t)N, sizeof(double));
    m->softening = (double*)xcalloc((size_t)N, sizeof(double));
    m->tlast = (double*)xcalloc((size_t)N, sizeof(double));
    for (long s = 0; s < N; s++) m->tlast[s] = -100 * p->t_temp;
    or_rng_seed(&m->rng, (unsigned long)p->seed);
    if (m->dim == 2) {
      m->Q0 = (double*)xcalloc((size_t)STZ_MODES * N, sizeof(double));
      m->Q1 = (double*)xcalloc((size_t)STZ_MODES * N, sizeof(double));
      m->deps = (double*)xcalloc((size_t)STZ_MODES * 3 * N, sizeof(double));
      st = init_ref2d(m);
    } else {
      m->dF = (double*)xcalloc((size_t)N, sizeof(double));
      st = init_global3d(m);
    }
    if (st != STZ_OK) goto fail;
  }
  /* initial state: EpsAvg = 0 (bmg.c:117) or the applied stress, then solve */
  memset(m->eps_avg, 0, sizeof(m->eps_avg));
  if (p->loading == STZ_LOAD_STRESS) iso_inv(m, p->applied_stress, m->eps_avg);
  or_solve(m);
  if (status) *status = STZ_OK;
  return m;
fail:
  if (status) *status = st;
  or_destroy(m);
  return NULL;
}

void or_destroy(or_model* m) {
  if (!m) return;
  for (int c = 0; c < 6; c++) { free(m->eps0[c]); free(m->sigma[c]); free(m->prev_deps[c]); }
  free(m->Q); free(m->rate); free(m->work); free(m->perm_soft); free(m->temp_soft);
  free(m->softening); free(m->tlast); free(m->Q0); free(m->Q1); free(m->deps); free(m->dF);
  free(m->mro); free(m->mro_theta);
  free(m->log);
  free(m->force_site); free(m->force_mode); free(m->force_draws); free(m->force_check);
  free(m->line_cb);
  free(m);
}

/* Selection by line bounds with rejection (see bounded_select); slack 0
 * restores the reference's rule. The generator must stay in step with the
 * implementation under test: use it with or_force_path, whose draws give the
 * words each event takes. */
int or_set_bounded_selection(or_model* m, int slack) {
  if (slack < 0 || slack > 60) return STZ_ERR_INVALID;
  m->sel_slack = slack;
  free(m->line_cb);
  m->line_cb = slack ? (double*)xcalloc((size_t)(STZ_MODES * m->N / m->n2 + 1), sizeof(double)) : NULL;
  return STZ_OK;
}

/* The next n thermal events take the given (site, mode) instead of the
 * oracle's own choice, after discarding draws[k] - 1 generator words (the
 * draws another implementation rejected); each records in or_get_checks what
 * the oracle would have chosen with the same dice. The rest of the step (the
 * FP64 rates, clock, solve and loading) is the oracle's own. */
int or_force_path(or_model* m, const int64_t* sites, const int32_t* modes, const int32_t* draws, int64_t n) {
  free(m->force_site); free(m->force_mode); free(m->force_draws); free(m->force_check);
  m->force_site = (int64_t*)xcalloc((size_t)n, sizeof(int64_t));
  m->force_mode = (int32_t*)xcalloc((size_t)n, sizeof(int32_t));
  m->force_draws = (int32_t*)xcalloc((size_t)n, sizeof(int32_t));
  m->force_check = (double*)xcalloc((size_t)n * 7, sizeof(double));
  for (int64_t k = 0; k < n; k++) {
    if (sites[k] < 0 || sites[k] >= m->N || modes[k] < 0 || modes[k] >= STZ_MODES || draws[k] < 1)
      return STZ_ERR_INVALID;
    m->force_site[k] = sites[k];
    m->force_mode[k] = modes[k];
    m->force_draws[k] = draws[k];
  }
  m->force_n = n;
  m->force_i = 0;
  return STZ_OK;
}

/* Checks of the forced events taken so far: [k][7] = own site, own mode,
 * dice, the forced element's cumulative interval [lower, upper] (fractions of
 * the total rate), the total rate and the words the own choice took. Returns
 * the number of records. */
int64_t or_get_checks(or_model* m, double* out, int64_t cap) {
  int64_t k = m->force_i < cap ? m->force_i : cap;
  memcpy(out, m->force_check, sizeof(double) * 7 * (size_t)k);
  return k;
}

int or_get_scalars(or_model* m, stz_scalars* o) {
  memset(o, 0, sizeof(*o));
  o->time = m->totime;
  for (int c = 0; c < 6; c++) { o->eps_avg[c] = m->eps_avg[c]; o->stress[c] = m->stress[c]; }
  for (int c = 0; c < m->nc; c++) {
    double a = 0;
    for (long s = 0; s < m->N; s++) a += m->eps0[c][s];
    o->eps0_avg[c] = a / m->N;
  }
  o->step = m->step; o->kstep = m->kstep; o->astep = m->astep; o->estep = m->estep;
  o->n_print = m->n_print; o->n_events_logged = m->nlog; o->stopped = m->stopped;
  return STZ_OK;
}

int64_t or_num_events(or_model* m) { return m->nlog; }

int or_get_events(or_model* m, int64_t first, stz_event* out, int64_t cap, int64_t* n) {
  int64_t k = 0;
  for (int64_t i = first; i < m->nlog && k < cap; i++) out[k++] = m->log[i];
  if (n) *n = k;
  return STZ_OK;
}

static double* field_ptr(or_model* m, int which, int comp) {
  long N = m->N;
  switch (which) {
    case STZ_FIELD_SIGMA: return comp < m->nc ? m->sigma[comp] : NULL;
    case STZ_FIELD_EPS0: return comp < m->nc ? m->eps0[comp] : NULL;
    case STZ_FIELD_DF:
      if (is2d(m)) return comp < STZ_MODES ? m->Q0 + (size_t)comp * N : NULL;
      return comp == 0 ? m->dF : NULL;
    case STZ_FIELD_DEPS: return (is2d(m) && comp < 3 * STZ_MODES) ? m->deps + (size_t)comp * N : NULL;
    case STZ_FIELD_TLAST: return m->tlast;
    case STZ_FIELD_PERM_SOFT: return m->perm_soft;
    case STZ_FIELD_TEMP_SOFT: return m->temp_soft;
    case STZ_FIELD_PREV_DEPS: return comp < m->nc ? m->prev_deps[comp] : NULL;
    case STZ_FIELD_Q: return comp < STZ_MODES ? m->Q + (size_t)comp * N : NULL;
  }
  return NULL;
}

int or_get_field(or_model* m, int which, int comp, double* out, int64_t count) {
  if (which == STZ_FIELD_MRO) {
    if (!is2d(m) || comp < 0 || comp > 1 || count != m->N) return STZ_ERR_INVALID;
    for (long s = 0; s < m->N; s++)
      out[s] = comp == 0 ? (m->mro ? (double)m->mro[s] : 0.0) : m->mro_theta[s];
    return STZ_OK;
  }
  if (which == STZ_FIELD_Q) act_energy(m);
  double* f = field_ptr(m, which, comp);
  if (!f || count != m->N) return STZ_ERR_INVALID;
  memcpy(out, f, sizeof(double) * (size_t)m->N);
  return STZ_OK;
}

int or_set_field(or_model* m, int which, int comp, const double* in, int64_t count) {
  double* f = field_ptr(m, which, comp);
  if (!f || count != m->N || which == STZ_FIELD_Q) return STZ_ERR_INVALID;
  memcpy(f, in, sizeof(double) * (size_t)m->N);
  return STZ_OK;
}

/* ElasticEnergy (elastic.c:533-547) */
int or_elastic_energy(or_model* m, double* out) {
  double e = 0;
  for (long s = 0; s < m->N; s++) {
    double sg[6] = {0}, el[6];
    for (int c = 0; c < m->nc; c++) sg[c] = m->sigma[c][s];
    iso_inv(m, sg, el);
    double acc = 0;
    for (int c = 0; c < m->nc; c++) acc += voigt_weight(m, c) * sg[c] * el[c];
    e += 0.5 * acc;
  }
  *out = e;
  return STZ_OK;
}

/* Mean strain EpsAvg that the next or_solve applies (the host assignment of
 * EpsAvg before the solve of bmg.c:114-124). */
int or_set_mean_strain(or_model* m, const double* eps_avg) {
  for (int c = 0; c < m->nc; c++) m->eps_avg[c] = eps_avg[c];
  return STZ_OK;
}

/* ============================================================ parameters */
/* The oracle's own derivation of a run's parameters, so that CPU runs of the
 * oracle need nothing from the engine library. */
static double or_kt(double T) { return T * OR_BOLZ * OR_J_IN_EV; }

/* tTemp of Init() (init.c:60): the relaxation time of the temporary softening */
static double or_t_temp(const stz_params* p) {
  return 1 / (p->trial_frequency * exp(-0.37 / or_kt(p->temperature)));
}

int or_params_default(stz_params* p, int model) {
  if (!p || (model != STZ_MODEL_REF2D && model != STZ_MODEL_GLOBAL3D)) return STZ_ERR_INVALID;
  memset(p, 0, sizeof(*p));
  p->model = model;
  p->trial_frequency = 1e13;               /* TRIAL_FREQUENCY, bmg.h:42 */
  p->precision = STZ_PREC_FP64;
  p->solver = STZ_SOLVER_FFT;
  p->resolve_period = 1000;
  p->sf_scheme = STZ_SF_SQUARE_FWD;        /* bmgFlags.h as shipped */
  p->perm_soft = 13;                       /* PermSoft, TempSoft, cap: init.c:62-68 */
  p->temp_soft = 39;
  p->perm_soft_cap = -log(0.6);
  p->perm_soft_mro = 20;                   /* PermSoftmro, TempSoftmro: init.c:61-63 */
  p->temp_soft_mro = 60;
  p->no_sf_xtal_mro = 1;                   /* bmgFlags.h as shipped */
  p->print_period = 5;
  if (model == STZ_MODEL_REF2D) {
    /* bmg.h:23-94 and the shipped input file, through Init() under LOW_T */
    double E = 69.46, nu = 2 * 0.365;
    p->n[0] = 1;
    p->n[1] = p->n[2] = 512;
    p->temperature = 300;
    p->voxel_volume = 0.7 * 0.7 * 1.0;
    p->gamma0 = 0.14;
    p->q0_mean = 2.0;
    p->q0_sd = 0.25;
    p->loading = STZ_LOAD_TENSION;
    p->shear_elastic_quirk = 1;
    p->young = E;
    p->poisson = nu;
    p->mu = E / (2 + 2 * nu);
    p->lambda = E * nu / (1 - nu * nu);
    p->strain_rate = 1e-4;
    p->strain_increment = 1e-4;
    p->end_strain = 0.06;
    p->softening = 1;
    p->seed = 123;
    p->random_ratio = 0.2;
    p->xq0amp = 2.0;
  } else {
    /* the 3D study: mu = 35 GPa, nu = 0.35, 455 K, Omega0 = 1 nm^3 */
    double mu = 35.0, nu = 0.35;
    p->n[0] = p->n[1] = p->n[2] = 64;
    p->mu = mu;
    p->poisson = nu;
    p->lambda = 2 * mu * nu / (1 - 2 * nu);
    p->young = 2 * mu * (1 + nu);
    p->temperature = 455;
    p->voxel_volume = 1.0;
    p->gamma0 = 0.1;
    p->df_kind = STZ_DF_TRUNC_NORMAL;
    p->q0_mean = 1.2;
    p->q0_sd = 0.1;
    p->q0_trunc = 3.0;
    p->q0_corr_len = 4.0;
    p->loading = STZ_LOAD_SHEAR;
    p->strain_rate = 0.5e-4;
    p->strain_increment = 1e-4;
    p->end_strain = 0.025;
  }
  p->t_temp = or_t_temp(p);
  return STZ_OK;
}

/* One labelled entry of the reference's input file (io.c:4-101): the label
 * on its own line, its value(s) on the next line, then a blank line. */
typedef struct or_entry { const char* label; const char* fmt; int want; void* a; void* b; } or_entry;

static int or_next_line(FILE* f, char* buf, int cap) {
  while (fgets(buf, cap, f)) {
    size_t n = strlen(buf);
    while (n && (buf[n - 1] == '\n' || buf[n - 1] == '\r')) buf[--n] = 0;
    if (n) return 1;                       /* blank lines separate entries */
  }
  return 0;
}

int or_params_from_input_file(stz_params* p, const char* path) {
  FILE* f = path ? fopen(path, "r") : NULL;
  if (!p || !f) return f ? (fclose(f), STZ_ERR_INVALID) : STZ_ERR_IO;
  double E = 0, nu = 0, q0 = 0, rate = 0, inc = 0, rr = 0, end = 0, relx = 0, xs = 0, xq = 0, resi = 0,
         xfrac = 0, xq0 = 0;
  int seed = 0, period = 0, soft = 0, initmro = 0;
  char resfile[256];
  or_entry e[] = {
      {"Moduli(E, nu):", "%lf %lf", 2, &E, &nu},
      {"Stress-free energy barrier:", "%lf", 1, &q0, NULL},
      {"Applied strain rate:", "%lf", 1, &rate, NULL},
      {"Strain increment:", "%lf", 1, &inc, NULL},
      {"Random seed:", "%d", 1, &seed, NULL},
      {"Random ratio of fluctuation in energy barrier:", "%lf", 1, &rr, NULL},
      {"Print period:", "%d", 1, &period, NULL},
      {"End Strain:", "%lf", 1, &end, NULL},
      {"Softening Flag:", "%d", 1, &soft, NULL},
      {"Relaxation Time:", "%lf", 1, &relx, NULL},
      {"Characteristic Xtal shear:", "%lf", 1, &xs, NULL},
      {"Barrier for Xtal shear:", "%lf", 1, &xq, NULL},
      {"Ratio for generating residual stress:", "%lf", 1, &resi, NULL},
      {"Residual stress data file:", "%255s", 1, resfile, NULL},
      {"Volume fraction of crystal-like MRO:", "%lf", 1, &xfrac, NULL},
      {"Initialization condition for MRO:", "%d", 1, &initmro, NULL},
      {"Stress-free energy barrier for crystal-like MRO:", "%lf", 1, &xq0, NULL},
  };
  const int ne = (int)(sizeof(e) / sizeof(e[0]));
  int matched = 0;
  char line[512];
  for (int i = 0; i < ne; i++) {
    if (!or_next_line(f, line, sizeof line)) break;
    if (strcmp(line, e[i].label) != 0) continue;
    if (!or_next_line(f, line, sizeof line)) break;
    if (sscanf(line, e[i].fmt, e[i].a, e[i].b) == e[i].want) matched++;
  }
  fclose(f);
  if (matched == 0) return STZ_ERR_IO;
  /* Init() with LOW_T (init.c:26-27, 44) */
  nu *= 2;
  p->young = E;
  p->poisson = nu;
  p->mu = E / (2 + 2 * nu);
  p->lambda = E * nu / (1 - nu * nu);
  p->q0_mean = q0;
  p->strain_rate = rate;
  p->strain_increment = inc;
  p->seed = (uint64_t)(uint32_t)seed;
  p->random_ratio = rr;
  p->print_period = period;
  p->end_strain = end;
  p->softening = soft;
  p->xmro_frac = xfrac;
  p->init_mro = initmro;
  p->xq0amp = xq0;
  p->t_temp = or_t_temp(p);
  (void)relx; (void)xs; (void)xq; (void)resi;
  return STZ_OK;
}
