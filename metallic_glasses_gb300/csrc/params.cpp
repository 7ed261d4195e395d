// params.cpp -- defaults and the reference 'input' file.
//
// stz_params_from_input_file accepts the labelled file read by ReadInput
// (io.c:4-101): the same labels, in the same order, each followed by its
// value(s) and a blank line. A label that does not match is reported and the
// field keeps its previous value, as the reference does (io.c:10-12). The
// derived constants follow Init() with LOW_T (init.c:18-27, 44-68).
#include <cmath>
#include <cstdio>
#include <cstring>

#include "stz_internal.h"

namespace {

constexpr double kEvInJ = 1.60217733e-19;   // bmg.h:71
constexpr double kBoltzmann = 1.380658e-23; // bmg.h:75

double kt_ev(double T) { return T * kBoltzmann * (1 / kEvInJ); }

}  // namespace

extern "C" int stz_params_default(stz_params* p, int32_t model) {
  if (!p) return STZ_ERR_INVALID;
  std::memset(p, 0, sizeof(*p));
  p->model = model;
  p->trial_frequency = 1e13;
  p->resolve_period = 1000;
  p->solver = STZ_SOLVER_FFT;
  p->precision = STZ_PREC_FP64;
  p->perm_soft = 13;
  p->temp_soft = 39;
  p->perm_soft_cap = -std::log(0.6);
  p->perm_soft_mro = 20;  // PermSoftmro, TempSoftmro (init.c:61-63)
  p->temp_soft_mro = 60;
  p->no_sf_xtal_mro = 1;  // bmgFlags.h as shipped
  p->sf_scheme = STZ_SF_SQUARE_FWD;
  if (model == STZ_MODEL_REF2D) {
    // the reference's compile-time constants (bmg.h:23-94) and shipped input
    p->n[0] = 1; p->n[1] = 512; p->n[2] = 512;
    p->temperature = 300.;
    p->voxel_volume = 0.7 * 0.7 * 1.0;
    p->gamma0 = 0.14;
    p->q0_sd = 0.25;
    p->q0_mean = 2.0;
    p->loading = STZ_LOAD_TENSION;
    p->shear_elastic_quirk = 1;
    double E = 69.46, nu = 0.365 * 2;
    p->young = E; p->poisson = nu;
    p->mu = E / (2 + 2 * nu);
    p->lambda = E * nu / (1 - nu * nu);
    p->strain_rate = 1e-4;
    p->strain_increment = 1e-4;
    p->end_strain = 0.06;
    p->print_period = 5;
    p->softening = 1;
    p->seed = 123;
    p->random_ratio = 0.2;
    p->xq0amp = 2.0;
    p->t_temp = 1 / (p->trial_frequency * std::exp(-0.37 / kt_ev(p->temperature)));
    return STZ_OK;
  }
  if (model == STZ_MODEL_GLOBAL3D) {
    p->n[0] = 64; p->n[1] = 64; p->n[2] = 64;
    double mu = 35.0, nu = 0.35;
    p->mu = mu;
    p->poisson = nu;
    p->lambda = 2 * mu * nu / (1 - 2 * nu);
    p->young = 2 * mu * (1 + nu);
    p->temperature = 455.;
    p->voxel_volume = 1.0;
    p->gamma0 = 0.1;
    p->df_kind = STZ_DF_TRUNC_NORMAL;
    p->q0_mean = 1.2; p->q0_sd = 0.1; p->q0_trunc = 3.0; p->q0_corr_len = 4.0;
    p->loading = STZ_LOAD_SHEAR;
    p->strain_rate = 0.5e-4;
    p->strain_increment = 1e-4;
    p->end_strain = 0.025;
    p->print_period = 5;
    p->softening = 0;
    p->seed = 0;
    p->t_temp = 1 / (p->trial_frequency * std::exp(-0.37 / kt_ev(p->temperature)));
    return STZ_OK;
  }
  return STZ_ERR_INVALID;
}

extern "C" int stz_params_from_input_file(stz_params* p, const char* path) {
  if (!p || !path) return STZ_ERR_INVALID;
  FILE* f = std::fopen(path, "r");
  if (!f) {
    stz::set_error("cannot open input file '%s'", path);
    return STZ_ERR_IO;
  }
  double E = 0, nu = 0, q0amp = 0, rate = 0, inc = 0, rr = 0, end = 0, relx = 0, xs = 0, xq = 0,
         resi = 0, xfrac = 0, xq0 = 0;
  int seed = 0, pp = 0, soft = 0, initmro = 0;
  char resfile[256] = {0};
  struct Field {
    const char* fmt;
    int want;
    void* a;
    void* b;
  };
  const Field fields[] = {
      {"Moduli(E, nu):\n%lf %lf\n\n", 2, &E, &nu},
      {"Stress-free energy barrier:\n%lf\n\n", 1, &q0amp, nullptr},
      {"Applied strain rate:\n%lf\n\n", 1, &rate, nullptr},
      {"Strain increment:\n%lf\n\n", 1, &inc, nullptr},
      {"Random seed:\n%d\n\n", 1, &seed, nullptr},
      {"Random ratio of fluctuation in energy barrier:\n%lf\n\n", 1, &rr, nullptr},
      {"Print period:\n%d\n\n", 1, &pp, nullptr},
      {"End Strain:\n%lf\n\n", 1, &end, nullptr},
      {"Softening Flag:\n%d\n\n", 1, &soft, nullptr},
      {"Relaxation Time:\n%lf\n\n", 1, &relx, nullptr},
      {"Characteristic Xtal shear:\n%lf\n\n", 1, &xs, nullptr},
      {"Barrier for Xtal shear:\n%lf\n\n", 1, &xq, nullptr},
      {"Ratio for generating residual stress:\n%lf\n\n", 1, &resi, nullptr},
      {"Residual stress data file:\n%255s\n\n", 1, resfile, nullptr},
      {"Volume fraction of crystal-like MRO:\n%lf\n\n", 1, &xfrac, nullptr},
      {"Initialization condition for MRO:\n%d\n\n", 1, &initmro, nullptr},
      {"Stress-free energy barrier for crystal-like MRO:\n%lf\n\n", 1, &xq0, nullptr},
  };
  int mismatches = 0;
  for (const Field& fd : fields) {
    int got = fd.b ? std::fscanf(f, fd.fmt, fd.a, fd.b) : std::fscanf(f, fd.fmt, fd.a);
    if (got != fd.want) {
      std::fprintf(stderr, "stz: input file: could not match '%.40s'\n", fd.fmt);
      mismatches++;
    }
  }
  std::fclose(f);
  if (mismatches == (int)(sizeof(fields) / sizeof(fields[0]))) {
    stz::set_error("input file '%s' has none of the expected labels", path);
    return STZ_ERR_IO;
  }
  // Init() under LOW_T (init.c:26-27, 44): 2D moduli from (E, nu)
  nu *= 2;
  double mu = E / (2 + 2 * nu);
  p->young = E;
  p->poisson = nu;
  p->mu = mu;
  p->lambda = E * nu / (1 - nu * nu);
  p->q0_mean = q0amp;
  p->strain_rate = rate;
  p->strain_increment = inc;
  p->seed = (uint64_t)(uint32_t)seed;
  p->random_ratio = rr;
  p->print_period = pp;
  p->end_strain = end;
  p->softening = soft;
  p->xmro_frac = xfrac;
  p->init_mro = initmro;
  p->xq0amp = xq0;
  p->t_temp = 1 / (p->trial_frequency * std::exp(-0.37 / kt_ev(p->temperature)));
  (void)relx; (void)xs; (void)xq; (void)resi;
  return STZ_OK;
}

extern "C" int64_t stz_sizeof(int32_t which) {
  switch (which) {
    case 0: return (int64_t)sizeof(stz_params);
    case 1: return (int64_t)sizeof(stz_event);
    case 2: return (int64_t)sizeof(stz_scalars);
  }
  return -1;
}
