// engine.cu -- context lifecycle, initial state, step orchestration, C ABI.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fft.cuh"
#include "kmc.cuh"
#include "stz_internal.h"

namespace stz {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                __LINE__);                                                         \
      return STZ_ERR_CUDA;                                                         \
    }                                                                              \
  } while (0)

namespace {

FFTPlan* plan_of(stz_ctx* c) { return reinterpret_cast<FFTPlan*>(c->fft); }

template <typename T>
int dalloc(T** p, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
  if (e != cudaSuccess) {
    set_error("cudaMalloc of %zu bytes failed: %s", sizeof(T) * count, cudaGetErrorString(e));
    return STZ_ERR_NOMEM;
  }
  // zero on the legacy stream and wait: the engine's own stream does not
  // order itself after the legacy stream
  cudaMemset(*p, 0, sizeof(T) * count);
  cudaDeviceSynchronize();
  return STZ_OK;
}

bool good_len(int n) {
  if (n < 1) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  return n == 1;
}

// Uniform random rotation from a point uniform on S^3 (Marsaglia 1972, two
// points uniform in the unit disk): only +, *, / and sqrt, so every IEEE
// host produces the same bits.
void random_rotation(MT* r, double R[3][3]) {
  double x1, x2, s1, x3, x4, s2;
  do {
    x1 = 2 * mt_uniform(r) - 1;
    x2 = 2 * mt_uniform(r) - 1;
    s1 = x1 * x1 + x2 * x2;
  } while (s1 >= 1.0);
  do {
    x3 = 2 * mt_uniform(r) - 1;
    x4 = 2 * mt_uniform(r) - 1;
    s2 = x3 * x3 + x4 * x4;
  } while (s2 >= 1.0 || s2 == 0.0);
  const double t = std::sqrt((1 - s1) / s2);
  const double w = x1, x = x2, y = x3 * t, z = x4 * t;
  R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - z * w);     R[0][2] = 2 * (x * z + y * w);
  R[1][0] = 2 * (x * y + z * w);     R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - x * w);
  R[2][0] = 2 * (x * z - y * w);     R[2][1] = 2 * (y * z + x * w);     R[2][2] = 1 - 2 * (x * x + y * y);
}

void dev_coords(const double* s, double* d) {
  const double r2 = 0.70710678118654752440, r6 = 0.40824829046386301637, q2 = 1.41421356237309504880;
  d[0] = (s[0] - s[1]) * r2;
  d[1] = (2.0 * s[2] - s[0] - s[1]) * r6;
  d[2] = q2 * s[3];
  d[3] = q2 * s[4];
  d[4] = q2 * s[5];
}

void host_iso_inv(const KParams& kp, const double* s, double* e) {
  const double lam = kp.lambda, mu = kp.mu;
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

int upload(void* d, const void* h, size_t bytes, cudaStream_t st) {
  CK(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st));
  return STZ_OK;
}

// ------------------------------------------------------------- initial state
// Crystal-like MRO types 0 glass, 1 six-fold, 2 two-fold, 3 ten-fold: the
// amplitude of mode 0 in units of gamma0 (elastic.c:68-112) and the number of
// slip modes (XMODES_SIX/TWO/TEN, bmg.h:30-32; the site's other modes carry no
// eigenstrain). The reference's PI (bmg.h:74) sets the angles.
constexpr double kMroAmp[4] = {0.0, 0.5, 0.8, 0.5};
constexpr int kMroModes[4] = {0, 6, 2, 12};
constexpr double kRefPi = 3.14159265359;

// the rotation jitter 1 + 0.2 (2u - 1) of a crystal-like site's modes
double mro_jitter(MT* rng) { return 1. + 0.2 * (2 * mt_uniform(rng) - 1.); }

int init_ref2d(stz_ctx* c, MT* rng) {
  const stz_params& p = c->p;
  const long long N = c->kp.N;
  // Alloc(): the MRO map (init.c:350-437). InitMRO 0: one uniform per site,
  // at or below xMROFrac a six-fold site with a second uniform for its angle
  // in [-PI/2, PI/2). InitMRO 1: the caller's types and angles (the
  // structure file), then one uniform per ten-fold site, below 0.5 making it
  // two-fold. Then Energy_Init (init.c:181-198) and DStrain (elastic.c:61-137);
  // the draw order is the reference's.
  std::vector<int8_t> ty((size_t)N, 0);
  std::vector<double> th((size_t)N, 0.0);
  bool any_mro = false;
  if (p.init_mro == 0) {
    for (long long s = 0; s < N; s++) {
      const double tmp = mt_uniform(rng);
      if (tmp <= p.xmro_frac) {
        any_mro = true;
        ty[s] = 1;
        th[s] = mt_uniform(rng) * kRefPi - kRefPi / 2.0;
      }
    }
  } else if (p.init_mro == 1) {
    if (!p.mro_type || !p.mro_theta) {
      set_error("init_mro 1 needs the map (mro_type, mro_theta)");
      return STZ_ERR_INVALID;
    }
    for (long long s = 0; s < N; s++) {
      const int32_t v = p.mro_type[s];
      if (v < 0 || v > 3) {
        set_error("MRO type %d at site %lld (only 0..3 are allowed)", (int)v, s);
        return STZ_ERR_INVALID;
      }
      ty[s] = (int8_t)v;
      th[s] = p.mro_theta[s];
      any_mro = any_mro || v != 0;
    }
    for (long long s = 0; s < N; s++)
      if (ty[s] == 3) {
        const double tmp = mt_uniform(rng);
        if (tmp < 0.5) ty[s] = 2;
      }
  } else {
    set_error("init_mro %d (0: drawn map, 1: given map)", (int)p.init_mro);
    return STZ_ERR_INVALID;
  }
  std::vector<double> Q0((size_t)STZ_MODES * N), deps((size_t)STZ_MODES * 3 * N);
  for (int m = 0; m < STZ_MODES; m++)
    for (long long s = 0; s < N; s++) Q0[(size_t)m * N + s] = mt_gaussian(rng, p.q0_sd) + p.q0_mean;
  for (int m = 0; m < STZ_MODES; m++)
    for (long long s = 0; s < N; s++) {
      double* d = deps.data() + (size_t)m * 3 * N;
      const int t = ty[s];
      if (t == 0) {
        d[s] = 0.5 * p.gamma0 * mt_gaussian(rng, 1.0);
        d[N + s] = -d[s];
        d[2 * N + s] = 0.5 * p.gamma0 * mt_gaussian(rng, 1.0);
      } else if (m == 0) {
        d[s] = kMroAmp[t] * p.gamma0 * std::cos(th[s]);
        d[N + s] = -d[s];
        d[2 * N + s] = kMroAmp[t] * p.gamma0 * std::sin(th[s]);
      } else if (m < kMroModes[t]) {
        // mode 0 rotated by m 2PI/X; angle and the two terms of each
        // component jittered, the left term's draw first
        const double a0 = deps[s], a2 = deps[2 * N + s];
        const double tt = m * 2. * kRefPi / kMroModes[t] * mro_jitter(rng);
        const double j1 = mro_jitter(rng), j2 = mro_jitter(rng);
        d[s] = a0 * j1 * std::cos(2 * tt) + a2 * j2 * std::sin(2 * tt);
        d[N + s] = -d[s];
        const double j3 = mro_jitter(rng), j4 = mro_jitter(rng);
        d[2 * N + s] = -a0 * j3 * std::sin(2 * tt) + a2 * j4 * std::cos(2 * tt);
      } else {
        d[s] = d[N + s] = d[2 * N + s] = 0.0;
      }
    }
  int st;
  c->mro_h = ty;
  c->mro_theta_h = th;
  if (any_mro) {
    if ((st = dalloc(&c->f.mro, (size_t)N))) return st;
    if ((st = upload(c->f.mro, ty.data(), (size_t)N, c->stream))) return st;
    // crystal-like sites draw new barriers when they transform; each print
    // restores the initial ones
    if ((st = dalloc(&c->f.Q1, Q0.size()))) return st;
    if ((st = upload(c->f.Q1, Q0.data(), sizeof(double) * Q0.size(), c->stream))) return st;
  }
  if ((st = upload(c->f.Q0, Q0.data(), sizeof(double) * Q0.size(), c->stream))) return st;
  if ((st = upload(c->f.deps, deps.data(), sizeof(double) * deps.size(), c->stream))) return st;
  launch_mode_norms(c->kp, c->f, c->stream);
  CK(cudaGetLastError());
  std::vector<double> tl((size_t)N, -100 * p.t_temp);
  if ((st = upload(c->f.tlast, tl.data(), sizeof(double) * N, c->stream))) return st;
  CK(cudaStreamSynchronize(c->stream));
  return STZ_OK;
}

int init_global3d(stz_ctx* c, MT* rng) {
  const stz_params& p = c->p;
  KParams& kp = c->kp;
  const long long N = kp.N;
  MT mrng;
  if (p.mode_seed_set) mt_seed(&mrng, (unsigned long)(uint32_t)p.mode_seed);
  MT* const modes_rng = p.mode_seed_set ? &mrng : rng;
  for (int m = 0; m < STZ_MODES; m++) {
    double R[3][3];
    random_rotation(modes_rng, R);
    const double a[3] = {R[0][0], R[1][0], R[2][0]};
    const double b[3] = {R[0][1], R[1][1], R[2][1]};
    const double g = 0.5 * p.gamma0;
    kp.modes[m][STZ_XX] = g * (2 * a[0] * b[0]);
    kp.modes[m][STZ_YY] = g * (2 * a[1] * b[1]);
    kp.modes[m][STZ_ZZ] = g * (2 * a[2] * b[2]);
    kp.modes[m][STZ_YZ] = g * (a[1] * b[2] + a[2] * b[1]);
    kp.modes[m][STZ_XZ] = g * (a[0] * b[2] + a[2] * b[0]);
    kp.modes[m][STZ_XY] = g * (a[0] * b[1] + a[1] * b[0]);
  }
  std::vector<double> dF((size_t)N);
  const double tr = p.q0_trunc;
  if (p.df_kind == STZ_DF_TRUNC_NORMAL) {
    for (long long s = 0; s < N; s++) {
      double z;
      do { z = mt_gaussian(rng, 1.0); } while (tr > 0 && std::fabs(z) > tr);
      dF[s] = p.q0_mean + p.q0_sd * z;
    }
  } else if (p.df_kind == STZ_DF_CORRELATED) {
    for (long long s = 0; s < N; s++) dF[s] = mt_gaussian(rng, 1.0);
    int st;
    if ((st = upload(c->f.dF, dF.data(), sizeof(double) * N, c->stream))) return st;
    fft_filter_gaussian(*plan_of(c), c->f.dF, p.q0_corr_len, c->f.spec, c->stream);
    CK(cudaMemcpyAsync(dF.data(), c->f.dF, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double ss = 0;
    for (long long s = 0; s < N; s++) ss += dF[s] * dF[s];
    const double sd = std::sqrt(ss / (double)N);
    for (long long s = 0; s < N; s++) {
      double z = dF[s] / sd;
      if (tr > 0) z = std::min(tr, std::max(-tr, z));
      dF[s] = p.q0_mean + p.q0_sd * z;
    }
  } else {
    set_error("unknown barrier generator %d", p.df_kind);
    return STZ_ERR_INVALID;
  }
  int st;
  if ((st = upload(c->f.dF, dF.data(), sizeof(double) * N, c->stream))) return st;
  if (c->f.dF32) launch_fill_f32(c->f.dF, c->f.dF32, N, c->stream);
  CK(cudaStreamSynchronize(c->stream));
  return STZ_OK;
}

// Slack exponent of the mixed form's per-line selection bounds. A line sum
// of the main pass adds its sites' FP32 rates in a tree of depth at most
// D = ceil(n2 / 32) + 31 (each lane's sites in order, then the 32 lanes in
// order), so it is within gamma_D = D u / (1 - D u) (u = 2^-24) of the exact
// sum of the same rates; a bound of the line sum plus 2^-slack of it plus 3
// quanta holds the exact fixed-point sum of its sites when 2^-slack >=
// gamma_D. The largest such slack is taken (18 for n2 <= 1024). `req` > 0
// overrides it (tests of the rejection path).
int selection_slack(int n2, int req) {
  if (req > 0) return std::min(req, 40);
  const double u = std::ldexp(1.0, -24), D = (double)((n2 + 31) / 32 + 31);
  const double g = D * u / (1.0 - D * u);
  int slack = 1;
  while (slack < 40 && std::ldexp(1.0, -(slack + 1)) >= g) slack++;
  return slack;
}

// Mixed-form constants: deviatoric mode coordinates and rate scaling.
void mixed_constants(stz_ctx* c) {
  KParams& kp = c->kp;
  const double cW = kp.V0 * 1e-18 * kJInEv;   // eV per (GPa * unit strain)
  const double l2e = 1.4426950408889634074;
  kp.q_ref = (float)c->p.q0_mean;
  kp.a_scale = (float)(l2e / kp.kT);
  kp.inv_a_scale = 1.0 / (double)kp.a_scale;
  kp.rate_scale = kp.vt * std::exp(-(double)kp.q_ref / kp.kT);
  // temperature-free mode coordinates (shared by replicas of one mode set at
  // different temperatures); the stress coordinates carry 1/kT
  for (int m = 0; m < STZ_MODES; m++) {
    double d[5];
    dev_coords(kp.modes[m], d);
    for (int k = 0; k < 5; k++) {
      kp.mdev_raw[m][k] = (float)d[k];
      kp.mdev[m][k] = (float)(d[k] * cW * 0.5 * l2e);
    }
  }
  for (int j = 0; j < STZ_MODES / 2; j++)
    for (int k = 0; k < 5; k++) kp.mdev2[j][k] = make_float2(kp.mdev[2 * j][k], kp.mdev[2 * j + 1][k]);
  kp.inv_kt = (float)(1.0 / kp.kT);
}

// ------------------------------------------------------------- solves
int solve_inhom(stz_ctx* c, const int* gate, const double* ebar);

int solve_plain(stz_ctx* c, const int* gate, const double* ebar) {
  if (c->inhom) return solve_inhom(c, gate, ebar);
  SolveArgs a{};
  a.eps = c->f.eps0;
  a.ebar = ebar;
  a.lambda = c->kp.lambda;
  a.mu = c->kp.mu;
  a.gate = gate;
  a.out = kOutSig64;
  a.sig64 = c->f.sig;
  a.msum = c->f.msum;
  a.spec = c->f.spec;
  a.fp32 = 0;
  const int st = fft_solve(*plan_of(c), a, c->stream, &c->launches);
  if (!st && c->kp.incr64) {
    // the incremental updates start from the mean strain of this solve
    launch_note_solve(c->f, gate, ebar, c->stream);
    c->launches += 1;
  }
  return st;
}

// FP64 incremental form: the solve of a unit eigenstrain component k at site
// 0 with zero mean strain, for each k, as the stress table rtab64 [k][c][N].
// The solve is linear in the eigenstrain and the mean strain, so a transformed
// voxel's increment d and a mean-strain change adds sum_k d_k R_k (shifted to
// the voxel) plus C:(change) to the field.
int build_response_table64(stz_ctx* c) {
  const KParams& kp = c->kp;
  const long long N = kp.N;
  const int nc = kp.nc;
  int st;
  if ((st = dalloc(&c->f.rtab64, (size_t)nc * nc * N))) return st;
  double *eps = nullptr, *zero = nullptr;
  if ((st = dalloc(&eps, (size_t)nc * N))) return st;
  if ((st = dalloc(&zero, 6))) { cudaFree(eps); return st; }
  const double one = 1.0;
  for (int k = 0; k < nc && !st; k++) {
    if (cudaMemsetAsync(eps, 0, sizeof(double) * nc * N, c->stream) != cudaSuccess ||
        cudaMemcpyAsync(eps + (size_t)k * N, &one, sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
      set_error("response table: %s", cudaGetErrorString(cudaGetLastError()));
      st = STZ_ERR_CUDA;
      break;
    }
    SolveArgs a{};
    a.eps = eps;
    a.ebar = zero;
    a.lambda = kp.lambda;
    a.mu = kp.mu;
    a.out = kOutSig64;
    a.sig64 = c->f.rtab64 + (size_t)k * nc * N;
    a.msum = c->f.msum;
    a.spec = c->f.spec;
    if ((st = fft_solve(*plan_of(c), a, c->stream, &c->launches))) break;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
      set_error("response table: %s", cudaGetErrorString(cudaGetLastError()));
      st = STZ_ERR_CUDA;
    }
  }
  cudaFree(eps);
  cudaFree(zero);
  return st;
}

// A spatially varying medium (InhomogeneousStressSolver, elastic.c:977-1066):
// the polarisation fixed point around the reference medium of the params'
// moduli. Each iteration is one homogeneous FP64 solve of the effective
// eigenstrain (into sig and msum, as solve_plain) and one update; the host
// reads the change (AvgChange) and stops as the reference does: below 1e-3
// of the mean strain's norm, or at once when that norm is below 1e-4, or after
// 101 iterations. sig and msum hold the last solve. Runs outside CUDA graphs
// (the gate, when given, is read first).
int solve_inhom(stz_ctx* c, const int* gate, const double* ebar) {
  const KParams& kp = c->kp;
  Fields& f = c->f;
  const long long N = kp.N;
  const int nc = kp.nc;
  if (gate) {
    int g = 0;
    CK(cudaMemcpyAsync(&g, gate, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (!g) return STZ_OK;
  }
  double eb[6] = {0, 0, 0, 0, 0, 0};
  if (ebar) CK(cudaMemcpyAsync(eb, ebar, sizeof(double) * nc, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  // the reference's norm of EpsAvg (its three 2D components; all six in 3D)
  double nrm = 0;
  for (int k = 0; k < nc; k++) nrm += eb[k] * eb[k];
  nrm = std::sqrt(nrm);
  double* d_ebar = ebar ? const_cast<double*>(ebar) : c->f.scratch;
  if (!ebar) CK(cudaMemsetAsync(c->f.scratch, 0, sizeof(double) * 6, c->stream));
  launch_inhom_init(kp, f, d_ebar, c->stream);
  std::vector<double> part(kInhomBlocks);
  for (int step = 1;; step++) {
    CK(cudaMemcpyAsync(f.inh_last, f.inh_eeff, sizeof(double) * nc * N, cudaMemcpyDeviceToDevice, c->stream));
    SolveArgs a{};
    a.eps = f.inh_last;
    a.ebar = ebar;
    a.lambda = kp.lambda;
    a.mu = kp.mu;
    a.out = kOutSig64;
    a.sig64 = f.sig;
    a.msum = f.msum;
    a.spec = f.spec;
    int st = fft_solve(*plan_of(c), a, c->stream, &c->launches);
    if (st) return st;
    launch_inhom_update(kp, f, c->stream);
    c->launches += 1;
    CK(cudaMemcpyAsync(part.data(), f.inh_part, sizeof(double) * kInhomBlocks, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double sum = 0;
    for (double v : part) sum += v;
    const double convg = std::sqrt(sum / (double)N);
    if (convg < 1e-3 * nrm || nrm < 1e-4) break;
    if (step > 100) break;
  }
  return STZ_OK;
}

// Full re-solve into the FP32 deviatoric field (mixed form), in FP32 pairs
// unless the parameters ask for FP64.
int solve_dev(stz_ctx* c, const double* ebar, const double* uadd, double* err) {
  SolveArgs a{};
  a.pair = c->p.resolve_fp64 ? 0 : 1;
  a.eps = c->f.eps0;
  a.ebar = ebar;
  a.uadd = uadd;
  a.lambda = c->kp.lambda;
  a.mu = c->kp.mu;
  a.out = kOutDev32;
  a.sdev = c->f.sdev;
  a.err = err;
  a.spec = c->f.spec;
  return fft_solve(*plan_of(c), a, c->stream, &c->launches);
}


// The response of one voxel: five FP64 solves with a unit deviatoric
// eigenstrain at the origin, projected on the deviatoric basis.
int build_response_table(stz_ctx* c) {
  KParams& kp = c->kp;
  const long long N = kp.N;
  const long long tn = (long long)kp.kt0 * kp.kt1 * kp.kt2;
  int st;
  if ((st = dalloc(&c->f.ktab, (size_t)16 * tn))) return st;
  double *eps = nullptr, *sig = nullptr;
  if ((st = dalloc(&eps, (size_t)6 * N))) return st;
  if ((st = dalloc(&sig, (size_t)6 * N))) { cudaFree(eps); return st; }
  const double r2 = 0.70710678118654752440, r6 = 0.40824829046386301637;
  const double basis[5][6] = {{r2, -r2, 0, 0, 0, 0},
                              {-r6, -r6, 2 * r6, 0, 0, 0},
                              {0, 0, 0, r2, 0, 0},
                              {0, 0, 0, 0, r2, 0},
                              {0, 0, 0, 0, 0, r2}};
  for (int b = 0; b < 5; b++) {
    for (int comp = 0; comp < 6; comp++)
      CK(cudaMemcpyAsync(eps + (size_t)comp * N, &basis[b][comp], sizeof(double), cudaMemcpyHostToDevice, c->stream));
    SolveArgs a{};
    a.eps = eps;
    a.ebar = nullptr;
    a.lambda = kp.lambda;
    a.mu = kp.mu;
    a.out = kOutSig64;
    a.sig64 = sig;
    a.spec = c->f.spec;
    fft_solve(*plan_of(c), a, c->stream, &c->launches);
    launch_ktab_column(kp, sig, c->f.ktab, b, c->stream);
  }
  CK(cudaStreamSynchronize(c->stream));
  cudaFree(eps);
  cudaFree(sig);
  return STZ_OK;
}

// ------------------------------------------------------------- stepping
// One driver-loop iteration of the FP64 forms, as a fixed kernel sequence.
// One driver step of the FP64 forms; t0/t1 (optional) are recorded around the
// rate kernel.
void enqueue_plain_step(stz_ctx* c, cudaEvent_t t0 = nullptr, cudaEvent_t t1 = nullptr) {
  const KParams& kp = c->kp;
  const Fields& f = c->f;
  const int* gate = &f.ctl->solve_req;
  const double* ebar = f.ctl->eps_avg;
  if (t0) cudaEventRecord(t0, c->stream);
  launch_rate_fp64(kp, f, c->stream);
  if (t1) cudaEventRecord(t1, c->stream);
  launch_athermal(kp, f, 0, c->stream);
  solve_plain(c, gate, ebar);
  if (kp.incr64) {
    launch_incr64(kp, f, c->stream);
    c->launches += 2;
  }
  launch_post_a(kp, f, c->stream);
  solve_plain(c, gate, ebar);
  if (f.Q1) {
    launch_q0_reset(kp, f, c->stream);
    c->launches += 1;
  }
  launch_post_b(kp, f, c->stream);
  c->launches += 1 + 2 + 2 + 1;
}

int sync_ctl(stz_ctx* c) {
  // a failed launch (configuration or resources) leaves an error here
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&c->host_ctl, c->f.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->d2h_bytes += sizeof(Ctl);
  return STZ_OK;
}

int drain_log(stz_ctx* c) {
  Ctl& h = c->host_ctl;
  const long long cap = c->kp.log_cap;
  long long from = h.log_base, to = h.nlog;
  if (to > from) {
    const size_t old = c->host_log.size();
    c->host_log.resize(old + (size_t)(to - from));
    long long i = from;
    while (i < to) {
      const long long slot = i % cap;
      const long long n = std::min(to - i, cap - slot);
      CK(cudaMemcpyAsync(c->host_log.data() + old + (i - from), c->f.log + slot, sizeof(stz_event) * n,
                         cudaMemcpyDeviceToHost, c->stream));
      c->d2h_bytes += (int64_t)sizeof(stz_event) * n;
      i += n;
    }
    h.log_base = to;
    CK(cudaMemcpyAsync(&c->f.ctl->log_base, &h.log_base, sizeof(long long), cudaMemcpyHostToDevice, c->stream));
    c->h2d_bytes += sizeof(long long);
    CK(cudaStreamSynchronize(c->stream));
  }
  return STZ_OK;
}

int set_targets(stz_ctx* c, long long max_kstep, long long max_step) {
  Ctl& h = c->host_ctl;
  h.max_kstep = max_kstep;
  h.max_step = max_step;
  h.halt = h.stopped ? 1 : 0;
  h.halt_reason = h.stopped ? kHaltStop : kHaltNone;
  CK(cudaMemcpyAsync(&c->f.ctl->max_kstep, &h.max_kstep, sizeof(long long) * 2, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(&c->f.ctl->halt, &h.halt, sizeof(int) * 2, cudaMemcpyHostToDevice, c->stream));
  c->h2d_bytes += sizeof(long long) * 2 + sizeof(int) * 2;
  return STZ_OK;
}

int capture_plain_graph(stz_ctx* c, int steps) {
  if (c->graph && c->graph_batch == steps) return STZ_OK;
  if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  cudaGraph_t g;
  const int64_t l0 = c->launches;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  for (int i = 0; i < steps; i++) {
    if (c->kp.nc == 6 && c->f.sdev) {
      launch_mixed(c->kp, c->f, 0, c->stream);
      c->launches += kMixedLaunches;
    } else {
      enqueue_plain_step(c);
    }
  }
  CK(cudaStreamEndCapture(c->stream, &g));
  c->graph_launches = c->launches - l0;
  c->launches = l0;
  CK(cudaGraphInstantiate(&c->graph, g, 0));
  cudaGraphDestroy(g);
  c->graph_batch = steps;
  return STZ_OK;
}

// Handle a halt of the mixed form between batches. Returns 1 when the run
// must stop (target, stop condition or error).
int mixed_service(stz_ctx* c, int* done) {
  Ctl& h = c->host_ctl;
  const KParams& kp = c->kp;
  const Fields& f = c->f;
  *done = 0;
  if (h.status) { *done = 1; return STZ_OK; }
  if (h.step_kind == kAthermal) {
    // the avalanche, the reference's re-solve with the current mean strain,
    // the athermal correction and the print check, then the stop checks
    launch_athermal(kp, f, 1, c->stream);
    solve_dev(c, f.ctl->eps_avg, nullptr, f.scratch);
    launch_mixed_after_resolve(kp, f, 0, c->stream);
    launch_post_a(kp, f, c->stream);
    int st = sync_ctl(c);
    if (st) return st;
    if (h.print_done) {
      solve_dev(c, f.ctl->eps_avg, nullptr, f.scratch);
      launch_mixed_after_resolve(kp, f, 0, c->stream);
    }
    launch_post_b(kp, f, c->stream);
    c->launches += 6;
  } else {
    if (kp.resolve_period > 0 && h.kstep >= h.next_resolve) {
      // periodic full re-solve: bring the FP32 field up to date, re-solve it
      // (FP32 pairs or FP64) with the same mean strain and offsets, record the
      // difference
      launch_mixed(kp, f, 1, c->stream);
      double zero[4] = {0, 0, 0, 0};
      CK(cudaMemcpyAsync(c->err_dev, zero, sizeof(zero), cudaMemcpyHostToDevice, c->stream));
      solve_dev(c, f.ctl->eps_avg_applied, f.ctl->u, c->err_dev);
      launch_mixed_after_resolve(kp, f, 1, c->stream);
      double e[4];
      CK(cudaMemcpyAsync(e, c->err_dev, sizeof(e), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      // relative L2 norm and max norm of the deviatoric stress difference
      c->err_rms = std::sqrt(e[1] / std::max(e[2], 1e-300));
      c->err_max = std::sqrt(e[0] / std::max(e[3], 1e-300));
      c->err_rms_worst = std::max(c->err_rms_worst, c->err_rms);
      c->err_max_worst = std::max(c->err_max_worst, c->err_max);
      c->n_resolves++;
      h.next_resolve += kp.resolve_period;
      CK(cudaMemcpyAsync(&f.ctl->next_resolve, &h.next_resolve, sizeof(long long), cudaMemcpyHostToDevice, c->stream));
      c->launches += 2;
    }
    if (h.print_done) {
      solve_dev(c, f.ctl->eps_avg, nullptr, f.scratch);
      launch_mixed_after_resolve(kp, f, 0, c->stream);
      launch_post_b(kp, f, c->stream);
      c->launches += 2;
    }
  }
  int st = sync_ctl(c);
  if (st) return st;
  if (h.stopped || h.status || h.halt_reason == kHaltTarget ||
      (h.max_kstep >= 0 && h.kstep >= h.max_kstep) || (h.max_step >= 0 && h.step >= h.max_step)) {
    *done = 1;
    return STZ_OK;
  }
  // resume
  h.halt = 0;
  h.halt_reason = kHaltNone;
  h.step_kind = kNone;
  CK(cudaMemcpyAsync(&f.ctl->halt, &h.halt, sizeof(int) * 2, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(&f.ctl->step_kind, &h.step_kind, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  return STZ_OK;
}

}  // namespace
}  // namespace stz

using namespace stz;

// ============================================================= C ABI
extern "C" const char* stz_last_error(void) { return g_err; }

namespace stz {
int create_ctx(const stz_params* pin, stz_ctx** out, int units_per_block);
}

extern "C" int stz_create(const stz_params* pin, stz_ctx** out) { return stz::create_ctx(pin, out, 0); }

int stz::create_ctx(const stz_params* pin, stz_ctx** out, int units_per_block) {
  if (!pin || !out) return STZ_ERR_INVALID;
  *out = nullptr;
  const stz_params& p = *pin;
  const bool ref2d = p.model == STZ_MODEL_REF2D;
  if (p.model != STZ_MODEL_REF2D && p.model != STZ_MODEL_GLOBAL3D) { set_error("unknown model"); return STZ_ERR_INVALID; }
  if ((ref2d && p.n[0] != 1) || !good_len(p.n[0]) || !good_len(p.n[1]) || !good_len(p.n[2]) || p.n[2] < 2 ||
      p.n[2] % 2) {
    set_error("grid %dx%dx%d not supported (extents 2^a 3^b, fastest even; 2D needs n[0] == 1)", p.n[0], p.n[1], p.n[2]);
    return STZ_ERR_INVALID;
  }
  if (!(p.mu > 0) || !(p.temperature > 0)) { set_error("mu and temperature must be positive"); return STZ_ERR_INVALID; }
  if (!ref2d && p.softening) { set_error("softening is implemented for the reference 2D model only"); return STZ_ERR_UNSUPPORTED; }
  if (!ref2d && (p.xmro_frac > 0 || p.init_mro != 0)) {
    set_error("crystal-like MRO sites belong to the reference 2D model");
    return STZ_ERR_UNSUPPORTED;
  }
  const bool mixed = p.precision == STZ_PREC_MIXED;
  if (mixed && ref2d) { set_error("the mixed form is implemented for the 3D model"); return STZ_ERR_UNSUPPORTED; }
  if (mixed && (p.n[2] % 4 || p.n[2] > 512 || p.n[1] > 512)) {
    // lines are staged by 16-byte bulk copies into shared memory, two per
    // warp; the selection walks a line or a plane's lines with one warp
    set_error("the mixed form needs the fastest extent a multiple of 4 and n1, n2 at most 512 (got %dx%dx%d)",
              p.n[0], p.n[1], p.n[2]);
    return STZ_ERR_UNSUPPORTED;
  }
  int solver = p.solver;
  if (solver == STZ_SOLVER_AUTO) solver = mixed ? STZ_SOLVER_KERNEL : STZ_SOLVER_FFT;
  if (mixed && solver != STZ_SOLVER_KERNEL) { set_error("the mixed form uses the incremental (kernel) solver"); return STZ_ERR_UNSUPPORTED; }
  // FP64 forms: the FFT re-solve after every event (the reference's method) or
  // the incremental update (the solve's response to one voxel, precomputed)

  stz_ctx* c = new stz_ctx();
  c->p = p;
  c->p.solver = solver;
  int st = STZ_OK;
  KParams& kp = c->kp;
  Fields& f = c->f;
  if (cudaSetDevice(p.device) != cudaSuccess) { set_error("cudaSetDevice(%d) failed", p.device); delete c; return STZ_ERR_CUDA; }
  cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  cudaEventCreate(&c->ev0);
  cudaEventCreate(&c->ev1);
  cudaEventCreate(&c->kev0);
  cudaEventCreate(&c->kev1);

  kp.model = p.model;
  kp.nc = ref2d ? 3 : 6;
  kp.incr64 = !mixed && solver == STZ_SOLVER_KERNEL;
  kp.n0 = p.n[0]; kp.n1 = p.n[1]; kp.n2 = p.n[2];
  kp.nh = kp.n2 / 2 + 1;
  kp.N = (long long)kp.n0 * kp.n1 * kp.n2;
  kp.Nk = (long long)kp.n0 * kp.n1 * kp.nh;
  if (mixed) {
    // Units of mirror-grouped lines (one d0, two d1); one wave of resident
    // blocks walks them, or, with units_per_block > 0 (batch members, where
    // the other replicas fill the GPU), that many units per block.
    const int kt0 = kp.n0 / 2 + 1, kt1 = kp.n1 / 2 + 1;
    kp.mx_c1 = (kt1 + 1) / 2;
    kp.mx_units = kt0 * kp.mx_c1;
    // u / mx_c1 as a multiply-high: exact while u * mx_c1 < 2^32 (u < 2^22
    // units for extents up to 512, mx_c1 <= 129)
    kp.c1_magic = (unsigned)((((uint64_t)1 << 32) + (uint64_t)kp.mx_c1 - 1) / (uint64_t)kp.mx_c1);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p.device);
    const long long wave = (long long)std::max(sms, 1) * mixed_blocks_per_sm(kp.n2);
    const long long nb = units_per_block > 0 ? (kp.mx_units + units_per_block - 1) / units_per_block
                                             : std::min<long long>(kp.mx_units, wave);
    kp.nblk = (int)std::max(1LL, nb);
    kp.bsites = 0;
  } else {
    // sites per thread: kSptFp64 while that still gives four blocks per SM,
    // fewer on smaller grids (a 512^2 grid at four per thread is 256 blocks,
    // under two per SM, and the FP64 rate pass needs the warps to cover its
    // latencies)
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p.device);
    int spt = kSptFp64;
    while (spt > 1 && (kp.N + (long long)kRateThreads * spt - 1) / ((long long)kRateThreads * spt) <
                          4LL * std::max(sms, 1))
      spt >>= 1;
    kp.bsites = kRateThreads * spt;
    kp.nblk = (int)((kp.N + kp.bsites - 1) / kp.bsites);
  }
  kp.ngroups = (kp.nblk + kGroup - 1) / kGroup;
  kp.adv_q2 = kRateThreads / kp.n2;
  kp.adv_r2 = kRateThreads % kp.n2;
  kp.loading = p.loading;
  kp.softening = p.softening;
  kp.sf_scheme = p.sf_scheme;
  kp.no_subtract_error = p.no_subtract_error;
  kp.shear_quirk = p.shear_elastic_quirk;
  kp.lambda = p.lambda; kp.mu = p.mu; kp.young = p.young; kp.poisson = p.poisson;
  kp.kT = p.temperature * kBoltz * kJInEv;
  kp.inv_kT = 1.0 / kp.kT;
  kp.vt = p.voxel_volume * p.trial_frequency;
  kp.V0 = p.voxel_volume;
  kp.w_scale = kp.V0 * 1e-18 * kJInEv / (2 * kp.kT);
  kp.dt = p.strain_rate > 0 ? p.strain_increment / p.strain_rate : INFINITY;
  kp.gamma0 = p.gamma0;
  kp.perm_soft = p.perm_soft; kp.temp_soft = p.temp_soft; kp.perm_soft_cap = p.perm_soft_cap; kp.t_temp = p.t_temp;
  kp.perm_soft_mro = p.perm_soft_mro; kp.temp_soft_mro = p.temp_soft_mro;
  kp.no_sf_xtal_mro = p.no_sf_xtal_mro;
  kp.xq0amp = p.xq0amp; kp.random_ratio = p.random_ratio;
  kp.end_strain = p.end_strain;
  kp.strain_rate = p.strain_rate;
  kp.strain_increment = p.strain_increment;
  kp.print_thr = p.print_period * p.strain_increment * 0.99;
  for (int i = 0; i < 6; i++) kp.applied[i] = p.applied_stress[i];
  kp.kt0 = kp.n0 / 2 + 1; kp.kt1 = kp.n1 / 2 + 1; kp.kt2 = kp.n2 / 2 + 1;
  kp.log_cap = p.log_capacity > 0 ? p.log_capacity : (1 << 20);
  kp.fast_inv = mixed ? 1 : 0;
  kp.inv_2mu = 1.0 / (2.0 * p.mu);
  kp.inv_lam_coef = p.lambda / (2.0 * p.mu * ((ref2d ? 2.0 : 3.0) * p.lambda + 2.0 * p.mu));
  kp.invN = 1.0 / (double)((long long)p.n[0] * p.n[1] * p.n[2]);
  kp.resolve_period = mixed ? p.resolve_period : 0;
  kp.sel_slack = selection_slack(kp.n2, p.sel_slack_shift);
  kp.general_pass = p.main_pass_general ? 1 : 0;

  const long long N = kp.N;
  const int nc = kp.nc;
  auto fail = [&](int code) {
    stz_destroy(c);
    return code;
  };
  if ((st = dalloc(&f.ctl, 1))) return fail(st);
  if ((st = dalloc(&f.eps0, (size_t)nc * N))) return fail(st);
  if ((st = dalloc(&f.prev_deps, (size_t)nc * N))) return fail(st);
  if ((st = dalloc(&f.amark, (size_t)N))) return fail(st);
  if (mixed) {
    if ((st = dalloc(&f.lsum, (size_t)STZ_MODES * kp.n0 * kp.n1))) return fail(st);
    if ((st = dalloc(&f.lbnd, (size_t)STZ_MODES * kp.n0 * kp.n1))) return fail(st);
    if ((st = dalloc(&f.psum, (size_t)(STZ_MODES + 1) * kp.n0))) return fail(st);
  } else {
    if ((st = dalloc(&f.part, (size_t)STZ_MODES * kp.nblk))) return fail(st);
    if ((st = dalloc(&f.gsum, (size_t)STZ_MODES * kp.ngroups))) return fail(st);
    if ((st = dalloc(&f.gticket, (size_t)kp.ngroups))) return fail(st);
  }
  if ((st = dalloc(&f.log, (size_t)kp.log_cap))) return fail(st);
  if ((st = dalloc(&c->err_dev, 4))) return fail(st);
  {
    double2* sp = nullptr;
    if ((st = dalloc(&sp, (size_t)nc * kp.Nk))) return fail(st);
    f.spec = sp;
  }
  // scratch for error statistics nobody reads (3 doubles)
  if ((st = dalloc(&f.scratch, 8))) return fail(st);
  if (mixed) {
    if ((st = dalloc(&f.sdev, (size_t)5 * N))) return fail(st);
    if ((st = dalloc(&f.dF32, (size_t)N))) return fail(st);
  } else {
    if ((st = dalloc(&f.sig, (size_t)nc * N))) return fail(st);
  }
  if (ref2d) {
    if ((st = dalloc(&f.Q0, (size_t)STZ_MODES * N))) return fail(st);
    if ((st = dalloc(&f.deps, (size_t)STZ_MODES * 3 * N))) return fail(st);
    if ((st = dalloc(&f.dnorm, (size_t)STZ_MODES * N))) return fail(st);
    if ((st = dalloc(&f.perm_soft, (size_t)N))) return fail(st);
    if ((st = dalloc(&f.temp_soft, (size_t)N))) return fail(st);
    if ((st = dalloc(&f.tlast, (size_t)N))) return fail(st);
  } else {
    if ((st = dalloc(&f.dF, (size_t)N))) return fail(st);
  }
  FFTPlan* plan = new FFTPlan();
  c->fft = plan;
  if ((st = fft_plan_create(plan, kp.n0, kp.n1, kp.n2, nc))) {
    set_error("FFT plan for %dx%dx%d failed", kp.n0, kp.n1, kp.n2);
    return fail(st);
  }
  // tiles and radix order timed for this grid (once per process and shape)
  if ((st = fft_autotune(plan, c->stream, c->fft_tuned, mixed && !c->p.resolve_fp64 ? 1 : 0))) {
    set_error("FFT schedule tuning failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(st);
  }
  kp.c2r_blocks = fft_c2r_blocks(*plan);
  if (!mixed && (st = dalloc(&f.msum, (size_t)nc * kp.c2r_blocks))) return fail(st);
  MT rng;
  mt_seed(&rng, (unsigned long)p.seed);
  st = ref2d ? init_ref2d(c, &rng) : init_global3d(c, &rng);
  if (st) return fail(st);
  if (mixed) mixed_constants(c);

  // control block
  Ctl& h = c->host_ctl;
  std::memset(&h, 0, sizeof(h));
  h.rng = rng;
  h.step_kind = kNone;
  h.max_kstep = -1;
  h.max_step = -1;
  h.next_resolve = kp.resolve_period > 0 ? kp.resolve_period : 0;
  if (p.loading == STZ_LOAD_STRESS) host_iso_inv(kp, p.applied_stress, h.eps_avg);
  for (int i = 0; i < 6; i++) h.eps_avg_applied[i] = h.eps_avg[i];
  {
    // mean stress of the initial solve: C:(eps_avg - 0)
    double e[6];
    for (int i = 0; i < 6; i++) e[i] = h.eps_avg[i];
    const int nd = nc == 3 ? 2 : 3;
    double tr = 0;
    for (int i = 0; i < nd; i++) tr += e[i];
    for (int i = 0; i < nc; i++) h.stress[i] = (i < nd ? kp.lambda * tr : 0.0) + 2.0 * kp.mu * e[i];
  }
  if (cudaMemcpy(f.ctl, &h, sizeof(Ctl), cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("control block upload failed");
    return fail(STZ_ERR_CUDA);
  }
  // initial solve (bmg.c:117-124)
  if (mixed) {
    if ((st = build_response_table(c))) return fail(st);
    solve_dev(c, f.ctl->eps_avg, nullptr, f.scratch);
  } else {
    if (kp.incr64 && (st = build_response_table64(c))) return fail(st);
    solve_plain(c, nullptr, f.ctl->eps_avg);
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
    set_error("initial solve failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(STZ_ERR_CUDA);
  }
  c->launches = 0;
  *out = c;
  return STZ_OK;
}

extern "C" void stz_destroy(stz_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->p.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  Fields& f = c->f;
  void* ptrs[] = {f.eps0, f.sig, f.sdev, f.dF, f.dF32, f.Q0, f.Q1, f.deps, f.dnorm, f.rtab64, f.mro, f.prev_deps, f.perm_soft, f.temp_soft,
                  f.tlast, f.amark, f.part, f.gsum, f.gticket, f.lsum, f.lbnd, f.psum, f.spec, f.ktab, f.log,
                  f.ctl, f.scratch, f.msum, c->err_dev, c->l2buf, c->qbuf, f.lam_site, f.mu_site,
                  f.inh_tau0, f.inh_eeff, f.inh_last, f.inh_part};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->fft) {
    fft_plan_destroy(plan_of(c));
    delete plan_of(c);
  }
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->kev0) cudaEventDestroy(c->kev0);
  if (c->kev1) cudaEventDestroy(c->kev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int stz_run(stz_ctx* c, int64_t max_steps, int64_t max_events) {
  if (!c) return STZ_ERR_INVALID;
  int st;
  cudaSetDevice(c->p.device);
  if ((st = sync_ctl(c))) return st;
  Ctl& h = c->host_ctl;
  if (h.status) return h.status;
  const long long tk = max_events > 0 ? h.kstep + max_events : -1;
  const long long ts = max_steps > 0 ? h.step + max_steps : -1;
  if ((st = set_targets(c, tk, ts))) return st;
  const bool mixed = c->f.sdev != nullptr;
  const int batch = mixed ? 64 : 16;
  if (c->use_graph && (st = capture_plain_graph(c, batch))) return st;
  for (;;) {
    if (c->use_graph) {
      if (cudaGraphLaunch(c->graph, c->stream) != cudaSuccess) {
        set_error("graph launch failed: %s", cudaGetErrorString(cudaGetLastError()));
        return STZ_ERR_CUDA;
      }
      c->launches += c->graph_launches;
    } else {
      for (int i = 0; i < batch; i++) {
        if (mixed) { launch_mixed(c->kp, c->f, 0, c->stream); c->launches += kMixedLaunches; }
        else enqueue_plain_step(c);
      }
    }
    if ((st = sync_ctl(c))) return st;
    if ((st = drain_log(c))) return st;
    if (h.status) { set_error("device reported status %d", h.status); return h.status; }
    if (mixed && h.halt) {
      int done = 0;
      if ((st = mixed_service(c, &done))) return st;
      if ((st = drain_log(c))) return st;
      if (done) break;
      continue;
    }
    if (h.halt) break;
  }
  return h.status;
}

extern "C" int stz_solve(stz_ctx* c) {
  if (!c) return STZ_ERR_INVALID;
  cudaSetDevice(c->p.device);
  if (c->f.sdev) {
    solve_dev(c, c->f.ctl->eps_avg, nullptr, c->f.scratch);
    launch_mixed_after_resolve(c->kp, c->f, 0, c->stream);
  } else {
    solve_plain(c, nullptr, c->f.ctl->eps_avg);
    // Stress = mean of the solved field (AvgStress), u = 0
    const int nc = c->kp.nc, nb = c->kp.c2r_blocks;
    std::vector<double> ms((size_t)nc * nb);
    CK(cudaMemcpyAsync(ms.data(), c->f.msum, sizeof(double) * ms.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double st6[6] = {0, 0, 0, 0, 0, 0}, z[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < nc; k++) {
      double acc = 0;
      for (int b = 0; b < nb; b++) acc += ms[(size_t)k * nb + b];
      st6[k] = acc / (double)c->kp.N;
    }
    CK(cudaMemcpyAsync(c->f.ctl->stress, st6, sizeof(st6), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->f.ctl->u, z, sizeof(z), cudaMemcpyHostToDevice, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return STZ_OK;
}

extern "C" int stz_get_scalars(stz_ctx* c, stz_scalars* o) {
  if (!c || !o) return STZ_ERR_INVALID;
  cudaSetDevice(c->p.device);
  int st = sync_ctl(c);
  if (st) return st;
  const Ctl& h = c->host_ctl;
  std::memset(o, 0, sizeof(*o));
  o->time = h.totime;
  for (int i = 0; i < 6; i++) {
    o->eps_avg[i] = h.eps_avg[i];
    o->stress[i] = h.stress[i];
    o->eps0_avg[i] = h.eps0_sum[i] / (double)c->kp.N;
  }
  o->step = h.step; o->kstep = h.kstep; o->astep = h.astep; o->estep = h.estep;
  o->n_print = h.n_print;
  o->n_events_logged = (int64_t)c->host_log.size();
  o->stopped = h.stopped;
  o->status = h.status;
  o->stress_err_max = c->err_max;
  o->stress_err_rms = c->err_rms;
  o->near_ties = h.near_ties;
  o->log_dropped = h.nlog_dropped;
  o->n_resolves = c->n_resolves;
  o->stress_err_rms_worst = c->err_rms_worst;
  o->stress_err_max_worst = c->err_max_worst;
  o->rejections = h.rejections;
  return STZ_OK;
}

extern "C" int stz_get_events(stz_ctx* c, int64_t first, stz_event* out, int64_t cap, int64_t* n) {
  if (!c || (!out && cap > 0)) return STZ_ERR_INVALID;
  int64_t k = 0;
  for (int64_t i = first; i < (int64_t)c->host_log.size() && k < cap; i++) out[k++] = c->host_log[(size_t)i];
  if (n) *n = k;
  return STZ_OK;
}

static int field_ptr(stz_ctx* c, int which, int comp, double** d64, float** d32) {
  const long long N = c->kp.N;
  const int nc = c->kp.nc;
  Fields& f = c->f;
  *d64 = nullptr;
  *d32 = nullptr;
  switch (which) {
    case STZ_FIELD_SIGMA:
      if (comp < 0 || comp >= nc || !f.sig) return STZ_ERR_INVALID;
      *d64 = f.sig + (size_t)comp * N;
      return STZ_OK;
    case STZ_FIELD_EPS0:
      if (comp < 0 || comp >= nc) return STZ_ERR_INVALID;
      *d64 = f.eps0 + (size_t)comp * N;
      return STZ_OK;
    case STZ_FIELD_DF:
      if (f.Q0) {
        if (comp < 0 || comp >= STZ_MODES) return STZ_ERR_INVALID;
        *d64 = f.Q0 + (size_t)comp * N;
      } else {
        if (comp != 0) return STZ_ERR_INVALID;
        *d64 = f.dF;
      }
      return STZ_OK;
    case STZ_FIELD_DEPS:
      if (!f.deps || comp < 0 || comp >= 3 * STZ_MODES) return STZ_ERR_INVALID;
      *d64 = f.deps + (size_t)comp * N;
      return STZ_OK;
    case STZ_FIELD_TLAST: *d64 = f.tlast; return f.tlast ? STZ_OK : STZ_ERR_INVALID;
    case STZ_FIELD_PERM_SOFT: *d64 = f.perm_soft; return f.perm_soft ? STZ_OK : STZ_ERR_INVALID;
    case STZ_FIELD_TEMP_SOFT: *d64 = f.temp_soft; return f.temp_soft ? STZ_OK : STZ_ERR_INVALID;
    case STZ_FIELD_PREV_DEPS:
      if (comp < 0 || comp >= nc) return STZ_ERR_INVALID;
      *d64 = f.prev_deps + (size_t)comp * N;
      return STZ_OK;
  }
  return STZ_ERR_INVALID;
}

extern "C" int stz_get_field(stz_ctx* c, int32_t which, int32_t comp, double* host, int64_t count) {
  if (!c || !host || count != c->kp.N) return STZ_ERR_INVALID;
  cudaSetDevice(c->p.device);
  const long long N = c->kp.N;
  if (which == STZ_FIELD_MRO) {
    if (c->kp.model != STZ_MODEL_REF2D || comp < 0 || comp > 1 || (long long)c->mro_h.size() != N)
      return STZ_ERR_INVALID;
    for (long long s = 0; s < N; s++) host[s] = comp == 0 ? (double)c->mro_h[(size_t)s] : c->mro_theta_h[(size_t)s];
    return STZ_OK;
  }
  if (which == STZ_FIELD_LAMBDA || which == STZ_FIELD_MU) {
    if (comp != 0) return STZ_ERR_INVALID;
    const std::vector<double>& h = which == STZ_FIELD_LAMBDA ? c->lam_h : c->mu_h;
    const double u = which == STZ_FIELD_LAMBDA ? c->kp.lambda : c->kp.mu;
    for (long long s = 0; s < N; s++) host[s] = h.empty() ? u : h[(size_t)s];
    return STZ_OK;
  }
  if (which == STZ_FIELD_Q) {
    if (comp < 0 || comp >= STZ_MODES) return STZ_ERR_INVALID;
    // a persistent buffer: the reference-style driver reads every mode each step
    if (!c->qbuf && dalloc(&c->qbuf, (size_t)N)) return STZ_ERR_NOMEM;
    launch_q_mode(c->kp, c->f, comp, c->qbuf, c->stream);
    CK(cudaMemcpyAsync(host, c->qbuf, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return STZ_OK;
  }
  if (which == STZ_FIELD_SDEV) {
    if (!c->f.sdev || comp < 0 || comp >= 5) return STZ_ERR_INVALID;
    launch_mixed(c->kp, c->f, 1, c->stream);  // apply the pending update
    std::vector<float> hf((size_t)N);
    CK(cudaMemcpyAsync(hf.data(), c->f.sdev + (size_t)comp * N, sizeof(float) * N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (long long s = 0; s < N; s++) host[s] = hf[(size_t)s];
    return STZ_OK;
  }
  if (which == STZ_FIELD_SIGMA && c->f.sdev) {
    // mixed form: the full field comes from an FP64 solve of the current state
    // (the stored FP32 field holds only the deviatoric coordinates)
    double* tmp = nullptr;
    if (dalloc(&tmp, (size_t)6 * N)) return STZ_ERR_NOMEM;
    SolveArgs a{};
    a.eps = c->f.eps0;
    a.ebar = c->f.ctl->eps_avg_applied;
    a.lambda = c->kp.lambda;
    a.mu = c->kp.mu;
    a.out = kOutSig64;
    a.sig64 = tmp;
    a.spec = c->f.spec;
    fft_solve(*plan_of(c), a, c->stream, nullptr);
    cudaMemcpyAsync(host, tmp + (size_t)comp * N, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream);
    CK(cudaStreamSynchronize(c->stream));
    cudaFree(tmp);
    sync_ctl(c);
    for (long long s = 0; s < N; s++) host[s] += c->host_ctl.u[comp];
    return STZ_OK;
  }
  double* d64;
  float* d32;
  int st = field_ptr(c, which, comp, &d64, &d32);
  if (st) return st;
  CK(cudaMemcpyAsync(host, d64, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (which == STZ_FIELD_SIGMA) {
    sync_ctl(c);
    for (long long s = 0; s < N; s++) host[s] += c->host_ctl.u[comp];
  }
  return STZ_OK;
}

// Displacement field of the current eigenstrain (HomogeneousStressSolver with
// uflag 2, elastic.c:873-900; DispField, io.c:137-240, without the supercell
// position the caller adds): one FP64 solve whose Green's pass writes
// u_hat = -i (F - alpha G g)/(mu |k|), into a temporary buffer (print-time only).
extern "C" int stz_get_displacement(stz_ctx* c, double* host, int64_t count) {
  if (!c || !host) return STZ_ERR_INVALID;
  const long long N = c->kp.N;
  const int dim = c->kp.n0 > 1 ? 3 : 2;
  if (count != (int64_t)dim * N) return STZ_ERR_INVALID;
  cudaSetDevice(c->p.device);
  double* tmp = nullptr;
  if (dalloc(&tmp, (size_t)dim * N)) return STZ_ERR_NOMEM;
  SolveArgs a{};
  a.eps = c->f.eps0;
  a.lambda = c->kp.lambda;
  a.mu = c->kp.mu;
  a.out = kOutSig64;
  a.sig64 = tmp;
  a.spec = c->f.spec;
  a.disp = 1;
  fft_solve(*plan_of(c), a, c->stream, &c->launches);
  cudaMemcpyAsync(host, tmp, sizeof(double) * dim * N, cudaMemcpyDeviceToHost, c->stream);
  const cudaError_t e = cudaStreamSynchronize(c->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) {
    set_error("displacement solve: %s", cudaGetErrorString(e));
    return STZ_ERR_CUDA;
  }
  c->d2h_bytes += (int64_t)sizeof(double) * dim * N;
  return STZ_OK;
}

extern "C" int stz_fft_schedule(stz_ctx* c, int32_t* tiles, int32_t* radices) {
  if (!c || !c->fft) return STZ_ERR_INVALID;
  const FFTPlan& p = *plan_of(c);
  if (tiles)
    for (int k = 0; k < 4; k++) tiles[k] = c->fft_tuned[k];
  if (radices) {
    const Sched* sc[3] = {&p.sh, &p.s1, &p.s0};
    for (int a = 0; a < 3; a++)
      for (int k = 0; k < 12; k++) radices[a * 12 + k] = k < sc[a]->nst ? sc[a]->r[k] : 0;
  }
  return STZ_OK;
}

extern "C" int stz_set_mean_strain(stz_ctx* c, const double* eps_avg) {
  if (!c || !eps_avg) return STZ_ERR_INVALID;
  cudaSetDevice(c->p.device);
  int st = sync_ctl(c);
  if (st) return st;
  for (int k = 0; k < c->kp.nc; k++) c->host_ctl.eps_avg[k] = eps_avg[k];
  CK(cudaMemcpyAsync(c->f.ctl->eps_avg, c->host_ctl.eps_avg, sizeof(double) * 6, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return STZ_OK;
}

// The site moduli of a plain form (and the buffers of its fixed point),
// allocated on first use with the params' uniform values.
static int ensure_moduli(stz_ctx* c) {
  if (!c->lam_h.empty()) return STZ_OK;
  const long long N = c->kp.N;
  const int nc = c->kp.nc;
  int st;
  if ((st = dalloc(&c->f.lam_site, (size_t)N)) || (st = dalloc(&c->f.mu_site, (size_t)N)) ||
      (st = dalloc(&c->f.inh_tau0, (size_t)nc * N)) || (st = dalloc(&c->f.inh_eeff, (size_t)nc * N)) ||
      (st = dalloc(&c->f.inh_last, (size_t)nc * N)) || (st = dalloc(&c->f.inh_part, (size_t)kInhomBlocks)))
    return st;
  c->lam_h.assign((size_t)N, c->kp.lambda);
  c->mu_h.assign((size_t)N, c->kp.mu);
  CK(cudaMemcpyAsync(c->f.lam_site, c->lam_h.data(), sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->f.mu_site, c->mu_h.data(), sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
  return STZ_OK;
}

extern "C" int stz_set_field(stz_ctx* c, int32_t which, int32_t comp, const double* host, int64_t count) {
  if (!c || !host || count != c->kp.N || which == STZ_FIELD_MRO) return STZ_ERR_INVALID;
  cudaSetDevice(c->p.device);
  if (which == STZ_FIELD_LAMBDA || which == STZ_FIELD_MU) {
    // the response tables of the mixed and the FP64 incremental form assume
    // one uniform medium
    if (c->f.sdev || c->kp.incr64) return STZ_ERR_UNSUPPORTED;
    if (comp != 0) return STZ_ERR_INVALID;
    int st = ensure_moduli(c);
    if (st) return st;
    std::vector<double>& h = which == STZ_FIELD_LAMBDA ? c->lam_h : c->mu_h;
    std::copy(host, host + count, h.begin());
    CK(cudaMemcpyAsync(which == STZ_FIELD_LAMBDA ? c->f.lam_site : c->f.mu_site, host, sizeof(double) * count,
                       cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->h2d_bytes += (int64_t)sizeof(double) * count;
    int varies = 0;
    for (long long s = 0; s < count && !varies; s++)
      varies = c->lam_h[(size_t)s] != c->kp.lambda || c->mu_h[(size_t)s] != c->kp.mu;
    c->inhom = varies;
    // the fixed point's iteration count depends on the data: no graph
    if (c->inhom) c->use_graph = 0;
    return STZ_OK;
  }
  double* d64;
  float* d32;
  int st = field_ptr(c, which, comp, &d64, &d32);
  if (st) return st;
  CK(cudaMemcpyAsync(d64, host, sizeof(double) * c->kp.N, cudaMemcpyHostToDevice, c->stream));
  if (which == STZ_FIELD_DF && c->f.dF32) launch_fill_f32(c->f.dF, c->f.dF32, c->kp.N, c->stream);
  if (which == STZ_FIELD_DEPS && c->f.dnorm) launch_mode_norms(c->kp, c->f, c->stream);
  CK(cudaStreamSynchronize(c->stream));
  return STZ_OK;
}

extern "C" int stz_elastic_energy(stz_ctx* c, double* out) {
  if (!c || !out) return STZ_ERR_INVALID;
  const long long N = c->kp.N;
  const int nc = c->kp.nc;
  std::vector<double> sig((size_t)nc * N);
  for (int comp = 0; comp < nc; comp++) {
    int st = stz_get_field(c, STZ_FIELD_SIGMA, comp, sig.data() + (size_t)comp * N, N);
    if (st) return st;
  }
  // ElasticEnergy (elastic.c:533-547)
  double e = 0;
  for (long long s = 0; s < N; s++) {
    double sg[6] = {0, 0, 0, 0, 0, 0}, el[6];
    for (int comp = 0; comp < nc; comp++) sg[comp] = sig[(size_t)comp * N + s];
    host_iso_inv(c->kp, sg, el);
    double acc = 0;
    for (int comp = 0; comp < nc; comp++) acc += ((nc == 3 ? comp == 2 : comp >= 3) ? 2.0 : 1.0) * sg[comp] * el[comp];
    e += 0.5 * acc;
  }
  *out = e;
  return STZ_OK;
}

extern "C" int stz_sync(stz_ctx* c) {
  if (!c) return STZ_ERR_INVALID;
  CK(cudaStreamSynchronize(c->stream));
  return STZ_OK;
}

extern "C" int stz_timer_start(stz_ctx* c) {
  if (!c) return STZ_ERR_INVALID;
  CK(cudaEventRecord(c->ev0, c->stream));
  return STZ_OK;
}

extern "C" int stz_timer_stop(stz_ctx* c, float* ms) {
  if (!c || !ms) return STZ_ERR_INVALID;
  CK(cudaEventRecord(c->ev1, c->stream));
  CK(cudaEventSynchronize(c->ev1));
  CK(cudaEventElapsedTime(ms, c->ev0, c->ev1));
  return STZ_OK;
}

extern "C" int stz_flush_l2(stz_ctx* c) {
  if (!c) return STZ_ERR_INVALID;
  if (!c->l2buf) {
    // a buffer larger than the 126 MB L2, allocated on first use
    c->l2flush_bytes = (size_t)256 << 20;
    if (cudaMalloc(&c->l2buf, c->l2flush_bytes) != cudaSuccess) {
      c->l2buf = nullptr;
      c->l2flush_bytes = 0;
      set_error("L2 flush buffer allocation failed");
      return STZ_ERR_NOMEM;
    }
  }
  launch_l2_flush(c->l2buf, c->l2flush_bytes, c->stream);
  c->launches += 1;
  return STZ_OK;
}

extern "C" int64_t stz_kernel_launches(stz_ctx* c) { return c ? c->launches : 0; }

extern "C" int stz_selftest_wait(int32_t device, int32_t tries, int32_t* status, double* ms, int32_t* kernel_tries) {
  if (!status || tries < 1) return STZ_ERR_INVALID;
  CK(cudaSetDevice(device));
  int* d = nullptr;
  int st;
  if ((st = dalloc(&d, 1))) return st;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int kmax = 0;
  CK(cudaEventRecord(e0, 0));
  if (wait_selftest(tries, d, &kmax, 0)) {
    cudaFree(d);
    set_error("wait self-test launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    return STZ_ERR_CUDA;
  }
  CK(cudaEventRecord(e1, 0));
  CK(cudaEventSynchronize(e1));
  float t = 0;
  CK(cudaEventElapsedTime(&t, e0, e1));
  int h = -1;
  CK(cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost));
  cudaFree(d);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *status = h;
  if (ms) *ms = t;
  if (kernel_tries) *kernel_tries = kmax;
  return STZ_OK;
}

extern "C" int stz_phase_times(stz_ctx* c, double* main_us, double* tail_us, int64_t* n) {
  if (!c) return STZ_ERR_INVALID;
  int st = sync_ctl(c);
  if (st) return st;
  const Ctl& h = c->host_ctl;
  const double k = h.prof_n ? 1e-3 / (double)h.prof_n : 0.0;
  if (main_us) *main_us = (double)h.prof_main_ns * k;
  if (tail_us) *tail_us = (double)h.prof_tail_ns * k;
  if (n) *n = (int64_t)h.prof_n;
  if (std::getenv("STZ_PHASE_DETAIL"))
    std::fprintf(stderr,
                 "stz tail parts (us): sums %.2f decide %.2f search %.2f (planes %.2f lines %.2f sites %.2f) "
                 "commit %.2f\n",
                 h.prof_part_ns[0] * k, h.prof_part_ns[1] * k, h.prof_part_ns[2] * k, h.prof_part_ns[4] * k,
                 h.prof_part_ns[5] * k, h.prof_part_ns[6] * k, h.prof_part_ns[3] * k);
  return STZ_OK;
}

extern "C" int stz_transfer_bytes(stz_ctx* c, int64_t* h2d, int64_t* d2h) {
  if (!c) return STZ_ERR_INVALID;
  if (h2d) *h2d = c->h2d_bytes;
  if (d2h) *d2h = c->d2h_bytes;
  return STZ_OK;
}

// Average device time of the per-step kernel: runs `steps` steps launching
// that kernel directly between CUDA events (no graph), on the context's
// stream. which = 0: the per-step rate/update kernel.
// Lead of the hold kernel queued before each timed mixed-form launch: long
// enough for the host to queue the event and the launches behind it.
constexpr unsigned long long kHoldNs = 40000;

extern "C" int stz_kernel_time(stz_ctx* c, int32_t which, double* ms_avg, int64_t* launches) {
  if (!c || !ms_avg) return STZ_ERR_INVALID;
  cudaSetDevice(c->p.device);
  int st = sync_ctl(c);
  if (st) return st;
  const int steps = launches && *launches > 0 ? (int)*launches : 64;
  const bool mixed = c->f.sdev != nullptr;
  if (!mixed) {
    // FP64 forms: the rate kernel (rates, sums, selection and commit of the
    // step in its last block) of `steps` driver steps, each launched alone
    *ms_avg = 0;
    if (which != 0) return STZ_ERR_UNSUPPORTED;
    Ctl& h = c->host_ctl;
    if ((st = set_targets(c, -1, h.step + steps))) return st;
    double tot = 0;
    int n = 0;
    for (int i = 0; i < steps && !h.halt && !h.stopped; i++) {
      enqueue_plain_step(c, c->kev0, c->kev1);
      CK(cudaStreamSynchronize(c->stream));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, c->kev0, c->kev1));
      tot += ms;
      n++;
      if ((st = sync_ctl(c))) return st;
      if ((st = drain_log(c))) return st;
      if (h.status) return h.status;
    }
    *ms_avg = n ? tot / n : 0;
    if (launches) *launches = n;
    return STZ_OK;
  }
  if (which == 1) {
    // update-only variant: streams the stress field (read + write) and the
    // response table; state is unchanged after its first launch
    double tot = 0;
    for (int i = 0; i < steps; i++) {
      launch_hold(kHoldNs, c->stream);
      CK(cudaEventRecord(c->kev0, c->stream));
      launch_mixed_main(c->kp, c->f, 1, c->stream);
      CK(cudaEventRecord(c->kev1, c->stream));
      launch_mixed_tail(c->kp, c->f, 1, c->stream);
      CK(cudaEventSynchronize(c->kev1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, c->kev0, c->kev1));
      tot += ms;
    }
    CK(cudaStreamSynchronize(c->stream));
    c->launches += 3 * steps;
    *ms_avg = tot / steps;
    if (launches) *launches = steps;
    return STZ_OK;
  }
  // run on a private copy of the targets: the kernel halts on its own rules
  Ctl& h = c->host_ctl;
  if ((st = set_targets(c, h.kstep + steps, -1))) return st;
  double tot = 0;
  int n = 0;
  for (int i = 0; i < steps; i++) {
    // which 0: the grid-wide update/rate kernel alone; 2: the whole event
    // (that kernel plus the selection/commit kernel)
    launch_hold(kHoldNs, c->stream);
    CK(cudaEventRecord(c->kev0, c->stream));
    launch_mixed_main(c->kp, c->f, 0, c->stream);
    if (which == 0) CK(cudaEventRecord(c->kev1, c->stream));
    launch_mixed_tail(c->kp, c->f, 0, c->stream);
    if (which != 0) CK(cudaEventRecord(c->kev1, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->kev0, c->kev1));
    if ((st = sync_ctl(c))) return st;
    if ((st = drain_log(c))) return st;
    if (h.halt) {
      int done = 0;
      if ((st = mixed_service(c, &done))) return st;
      drain_log(c);
      if (done) break;
      continue;  // a serviced step is not a plain launch; do not time it
    }
    tot += ms;
    n++;
  }
  c->launches += (kMixedLaunches + 1) * steps;
  *ms_avg = n ? tot / n : 0;
  if (launches) *launches = n;
  return STZ_OK;
}

// ============================================================= batches
struct stz_batch {
  std::vector<stz_ctx*> reps;
  int device = 0;
  cudaStream_t stream = nullptr;
  stz::BatchDesc* d_desc = nullptr;
  int* d_blk_rep = nullptr;
  int* d_rep_first = nullptr;
  stz::BatchStatus* d_status = nullptr;
  std::vector<stz::BatchStatus> h_status;
  int total_blocks = 0;
  int max_n0 = 1;  // largest plane count (grid x of the plane-sum kernel)
  stz::BatchLaunch bl;  // per line-length class: block range, longest line, stream
  int shared_modes = 0;  // every replica has the same modes (kernel-parameter path)
  stz::ModeSet modes{};
  cudaGraphExec_t graph = nullptr;
  int graph_rounds = 0;
  int64_t launches = 0;
  int64_t min_log_cap = 0;
};

extern "C" void stz_batch_destroy(stz_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (stz_ctx* c : b->reps) stz_destroy(c);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (int c = 0; c < stz::kBatchClasses; c++) {
    if (b->bl.side[c]) cudaStreamDestroy(b->bl.side[c]);
    if (b->bl.join[c]) cudaEventDestroy(b->bl.join[c]);
  }
  if (b->bl.fork) cudaEventDestroy(b->bl.fork);
  cudaFree(b->d_desc);
  cudaFree(b->d_blk_rep);
  cudaFree(b->d_rep_first);
  cudaFree(b->d_status);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

extern "C" int stz_batch_create(const stz_params* params, int32_t count, stz_batch** out) {
  if (!params || count < 1 || !out) return STZ_ERR_INVALID;
  *out = nullptr;
  stz_batch* b = new stz_batch();
  b->device = params[0].device;
  for (int i = 0; i < count; i++) {
    stz_params p = params[i];
    if (p.model != STZ_MODEL_GLOBAL3D || p.precision != STZ_PREC_MIXED || p.device != b->device) {
      set_error("batch replica %d: batches hold mixed-form 3D replicas on one device", i);
      stz_batch_destroy(b);
      return STZ_ERR_UNSUPPORTED;
    }
    if (p.log_capacity <= 0) p.log_capacity = 1 << 15;
    stz_ctx* c = nullptr;
    // batches: sixteen line units per block
    const int st = stz::create_ctx(&p, &c, 16);
    if (st) {
      stz_batch_destroy(b);
      return st;
    }
    c->use_graph = 0;
    b->reps.push_back(c);
  }
  cudaSetDevice(b->device);
  cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  std::vector<stz::BatchDesc> desc(count);
  std::vector<int> blk_rep, first(count);
  // blocks grouped by line-length class, replicas in order within a class
  for (int c = 0; c < stz::kBatchClasses; c++) {
    b->bl.start[c] = (int)blk_rep.size();
    for (int i = 0; i < count; i++) {
      const stz::KParams& kp = b->reps[i]->kp;
      if ((kp.general_pass ? stz::kBatchClasses - 1 : stz::batch_class(kp.n2)) != c) continue;
      first[i] = (int)blk_rep.size();
      for (int k = 0; k < kp.nblk; k++) blk_rep.push_back(i);
      b->bl.max_n2[c] = std::max(b->bl.max_n2[c], kp.n2);
    }
    b->bl.count[c] = (int)blk_rep.size() - b->bl.start[c];
  }
  for (int i = 0; i < count; i++) {
    desc[i].kp = b->reps[i]->kp;
    desc[i].f = b->reps[i]->f;
    b->min_log_cap = i == 0 ? b->reps[i]->kp.log_cap : std::min<int64_t>(b->min_log_cap, b->reps[i]->kp.log_cap);
  }
  b->total_blocks = (int)blk_rep.size();
  cudaEventCreateWithFlags(&b->bl.fork, cudaEventDisableTiming);
  for (int c = 0; c < stz::kBatchClasses; c++) {
    cudaStreamCreateWithFlags(&b->bl.side[c], cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&b->bl.join[c], cudaEventDisableTiming);
  }
  // one mode set for every replica: the batched kernel takes it as parameters
  b->shared_modes = 1;
  for (auto* c : b->reps)
    b->shared_modes &= std::memcmp(c->kp.mdev2, b->reps[0]->kp.mdev2, sizeof(c->kp.mdev2)) == 0 &&
                       std::memcmp(c->kp.mdev_raw, b->reps[0]->kp.mdev_raw, sizeof(c->kp.mdev_raw)) == 0;
  std::memcpy(b->modes.mdev2, b->reps[0]->kp.mdev2, sizeof(b->modes.mdev2));
  std::memcpy(b->modes.mdev_raw, b->reps[0]->kp.mdev_raw, sizeof(b->modes.mdev_raw));
  b->max_n0 = 1;
  for (auto* c : b->reps) b->max_n0 = std::max(b->max_n0, c->kp.n0);
  int st = STZ_OK;
  if ((st = dalloc(&b->d_desc, (size_t)count)) || (st = dalloc(&b->d_blk_rep, blk_rep.size())) ||
      (st = dalloc(&b->d_rep_first, (size_t)count)) || (st = dalloc(&b->d_status, (size_t)count))) {
    stz_batch_destroy(b);
    return st;
  }
  cudaMemcpy(b->d_desc, desc.data(), sizeof(stz::BatchDesc) * count, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_blk_rep, blk_rep.data(), sizeof(int) * blk_rep.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_rep_first, first.data(), sizeof(int) * count, cudaMemcpyHostToDevice);
  b->h_status.resize(count);
  *out = b;
  return STZ_OK;
}

extern "C" int stz_batch_size(stz_batch* b) { return b ? (int)b->reps.size() : 0; }

extern "C" stz_ctx* stz_batch_replica(stz_batch* b, int32_t i) {
  if (!b || i < 0 || i >= (int)b->reps.size()) return nullptr;
  return b->reps[(size_t)i];
}

namespace {
int batch_capture(stz_batch* b, int rounds) {
  if (b->graph && b->graph_rounds == rounds) return STZ_OK;
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  for (int r = 0; r < rounds; r++)
    launch_mixed_batched(b->d_desc, b->d_blk_rep, b->d_rep_first, b->bl, b->d_status, (int)b->reps.size(),
                         b->max_n0, b->shared_modes ? &b->modes : nullptr, b->stream);
  CK(cudaStreamEndCapture(b->stream, &g));
  CK(cudaGraphInstantiate(&b->graph, g, 0));
  cudaGraphDestroy(g);
  b->graph_rounds = rounds;
  return STZ_OK;
}
}  // namespace

extern "C" int stz_batch_run(stz_batch* b, int64_t events) {
  if (!b || events < 1) return STZ_ERR_INVALID;
  cudaSetDevice(b->device);
  int st;
  const int n = (int)b->reps.size();
  for (stz_ctx* c : b->reps) {
    if ((st = sync_ctl(c))) return st;
    if (c->host_ctl.status) return c->host_ctl.status;
    if ((st = set_targets(c, c->host_ctl.kstep + events, -1))) return st;
    CK(cudaStreamSynchronize(c->stream));
  }
  const int rounds = 16;
  if ((st = batch_capture(b, rounds))) return st;
  int64_t since_drain = 0;
  for (;;) {
    if (cudaGraphLaunch(b->graph, b->stream) != cudaSuccess) {
      set_error("batch graph launch failed: %s", cudaGetErrorString(cudaGetLastError()));
      return STZ_ERR_CUDA;
    }
    b->launches += kMixedLaunches * rounds;
    for (stz_ctx* c : b->reps) c->launches += kMixedLaunches * rounds;
    since_drain += rounds;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(b->h_status.data(), b->d_status, sizeof(stz::BatchStatus) * n, cudaMemcpyDeviceToHost,
                       b->stream));
    CK(cudaStreamSynchronize(b->stream));
    bool active = false;
    const bool drain_all = since_drain * 2 >= b->min_log_cap;
    for (int i = 0; i < n; i++) {
      stz_ctx* c = b->reps[(size_t)i];
      const stz::BatchStatus& s = b->h_status[(size_t)i];
      if (s.status) {
        set_error("batch replica %d: device status %d", i, s.status);
        return s.status;
      }
      if (!s.halt) {
        active = true;
        if (drain_all) {
          if ((st = sync_ctl(c)) || (st = drain_log(c))) return st;
        }
        continue;
      }
      if ((st = sync_ctl(c))) return st;
      if ((st = drain_log(c))) return st;
      if (s.stopped || s.halt_reason == stz::kHaltTarget || s.halt_reason == stz::kHaltStop) continue;
      int done = 0;
      if ((st = mixed_service(c, &done))) return st;
      if ((st = drain_log(c))) return st;
      if (!done) active = true;
    }
    if (drain_all) since_drain = 0;
    if (!active) break;
  }
  for (stz_ctx* c : b->reps) {
    if ((st = sync_ctl(c)) || (st = drain_log(c))) return st;
  }
  return STZ_OK;
}
