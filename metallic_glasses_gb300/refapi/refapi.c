/* refapi.c -- the reference's own entry points on the GB300 engine.
 *
 * A drop-in for the reference's init.c, elastic.c, evolution.c and io.c in
 * the 2D model: compiled against the user's bmg.h / my_fft.h / bmgFlags.h
 * (the grid size NX x NY, the flags and the global state come from there),
 * it defines the functions the reference's main (bmg.c) calls, with the same
 * names and signatures (bmg.h:149-152, 216-232, 295-311, 329, 352, 375), and
 * runs them on one GB300 through the engine's C ABI (stz_api.h). The
 * reference's main links against it unchanged.
 *
 * State. The device holds the simulation; the globals of bmg.h are host
 * mirrors, filled where the reference's main reads them:
 *   ActEnergy          Q[m] for every mode (main scans it for Q < 0)
 *   KMC, athermal      totime, EpsAvg, Stress, kstep/astep/estep after the step
 *   solvers            Sigma, Stress, EpsAvg (and TotEps = C^-1:Sigma + Eps0)
 *   RecordPrep         Eps0, Sigma, then EqStrain / EqStress (io.c:260-273)
 *   Energy_Init/DStrain Q0, Q1 (initial copy), DEps0
 * A host write to EpsAvg before a solve is passed to the device; other host
 * writes to mirrors are not (the device state stays authoritative).
 *
 * The KMC step of the engine takes the same branch as the reference's main
 * (athermal when some Q < 0, else thermal or elastic), so KMC() and
 * athermal_plasticity() both advance one driver step. The print-time re-solve
 * (bmg.c:292-295) is the main's own solver call with uflag 2, after the step,
 * as in the reference: the engine's internal print test is switched off, so
 * the globals after KMC() hold the state before that re-solve.
 *
 * The uflag-1/2 solves and DispField fill the positions XR: the engine's
 * displacement field of the eigenstrain plus the supercell position, as
 * elastic.c:866-900 and io.c:137-240 write them.
 *
 * Spatially varying Lambda/Mu passed to InhomogeneousStressSolver go to the
 * engine, whose solves (those of the steps too) then run the reference's
 * polarisation fixed point.
 *
 * Crystal-like MRO sites (init.c:350-437): the engine draws the map (InitMRO
 * 0) or takes the one Alloc reads from MROstructure.ms (InitMRO 1); Alloc
 * fills MRO/MROthe0 from it and writes Initial_MROstructure, and actQ.out
 * records the chosen site's MRO type, as the reference does.
 *
 * Not provided: SOC counters (UpdateSOC leaves main's arrays as they are),
 * residual-stress generation.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "bmg.h"
#include "my_fft.h"
#include "stz_api.h"

/* bmgFlags.h switches whose physics the engine does not implement. Each one
 * stops the build here, so that a drop-in build never runs the default
 * physics in place of the switched-on one. Switches that only change what
 * ParameterPrint/PrintFlags print (PRE_RELAXATION, RESIDUAL_STRESS,
 * UNIFORM_DEFECTS) or that no reference source reads (STZ_DILATATION,
 * FCC_SYMMETRY, TWO_FOLD_SYMMETRY) are accepted. */
#if defined(STRAIN_RATE_SENSITIVITY) || defined(LOCAL_RATE_V2)
#error "refapi: STRAIN_RATE_SENSITIVITY / LOCAL_RATE_V2 (rate-sensitive barriers, init.c:670-682) are not implemented by the engine"
#endif
/* The two relaxation laws divide by tPerm, which the reference never assigns
 * (0.0 from bmg.h:177; init.c:50,53 are commented out). */
#if defined(RELX_BIMOLE_FLAG) || defined(RELX_FVT_FLAG)
#error "refapi: RELX_BIMOLE_FLAG / RELX_FVT_FLAG (softening relaxation laws, init.c:717-724) are not implemented by the engine; in the reference they divide by tPerm, which is never assigned (0.0)"
#endif
#if defined(AVG_PERMSOFTENING)
#error "refapi: AVG_PERMSOFTENING (the grid-mean permanent softening, init.c:692-709, 725-729) is not implemented by the engine"
#endif
#if defined(HEAT_CONDUCT)
#error "refapi: HEAT_CONDUCT (local heating and conduction, elastic.c:549-582, evolution.c:247-249) is not implemented by the engine"
#endif
#if defined(RESIDUAL_STRESS_CONST) || defined(RESIDUAL_STRESS_RELX)
#error "refapi: RESIDUAL_STRESS_CONST / RESIDUAL_STRESS_RELX (residual-stress work terms, init.c:576-583, bmg.c:86-102) are not implemented by the engine"
#endif
#if defined(XTAL_VARIANTS)
#error "refapi: XTAL_VARIANTS (crystal variants, init.c:9-17, elastic.c:9, 398) is not implemented by the engine"
#endif
#if defined(STRESS_FREE_BOUNDARY)
#error "refapi: STRESS_FREE_BOUNDARY (elastic.c:220-262) is not implemented by the engine"
#endif
/* Without MICRO_MEMORY the reference declares no PreDEps0 (bmg.h:236-240), so
 * its ActEnergy compiles only when the scheme it takes is SF_EVEN, the one
 * scheme that reads no memory. That build is the engine's SF_EVEN (its memory
 * then unused); the others are refused, as the reference does not build. */
#if !defined(MICRO_MEMORY) && (defined(SF_LINEAR_FWD) || defined(SF_LINEAR_BWD) || !defined(SF_EVEN))
#error "refapi: builds without MICRO_MEMORY need SF_EVEN as the softening-direction scheme (the other schemes read PreDEps0, which the reference declares only under MICRO_MEMORY, bmg.h:236-240)"
#endif
/* ActEnergy sets its direction modifier under one of six names only
 * (init.c:590-642); with none of them defined it reads the variable
 * uninitialised (init.c:563). bmgFlags.h:35 spells the cubic scheme
 * SF_Cubic_FWD, a name init.c does not test. */
#if !defined(SF_LINEAR_FWD) && !defined(SF_LINEAR_BWD) && !defined(SF_EVEN) && !defined(SF_SQUARE_FWD) && \
    !defined(SF_CUBIC_FWD) && !defined(SF_GAUSS_FWD)
#if defined(SF_Cubic_FWD)
#error "refapi: SF_Cubic_FWD selects no scheme in ActEnergy (init.c:622 tests SF_CUBIC_FWD); define SF_CUBIC_FWD"
#else
#error "refapi: no softening-direction scheme (SF_LINEAR_FWD, SF_LINEAR_BWD, SF_EVEN, SF_SQUARE_FWD, SF_CUBIC_FWD, SF_GAUSS_FWD) is defined; ActEnergy would read its direction modifier uninitialised (init.c:563)"
#endif
#endif

static stz_ctx* g_ctx = NULL;
static stz_params g_p;
static int64_t g_events_seen = 0;  /* events already written to fq */
static int g_any_mro = 0;          /* the map holds crystal-like sites */
static real* g_q0_seen[MODES];     /* Q0 as RecordPrep read it from the device */
static int g_q0_check = 0;         /* compare the Q0 mirror before the next step */
static double g_epsavg_dev[3];     /* EpsAvg as last read from the device */

static void fail(const char* what, int code) {
  fprintf(stderr, "refapi: %s failed (%d): %s\n", what, code, stz_last_error());
  MPI_Abort(MPI_COMM_WORLD, -1);
}

static real* alloc_field(void) {
  real* p = (real*)calloc((size_t)NXY, sizeof(real));
  if (!p) fail("allocation", STZ_ERR_NOMEM);
  return p;
}

/* the engine's scalars into the reference's globals */
static void pull_scalars(void) {
  stz_scalars s;
  int st = stz_get_scalars(g_ctx, &s);
  if (st) fail("stz_get_scalars", st);
  totime = s.time;
  for (int c = 0; c < 3; c++) {
    EpsAvg[c] = s.eps_avg[c];
    g_epsavg_dev[c] = s.eps_avg[c];
    Stress[c] = s.stress[c];
  }
  kstep = (int)s.kstep;
  astep = (int)s.astep;
  estep = (int)s.estep;
}

static void pull_field(int which, int comp, real* host) {
  int st = stz_get_field(g_ctx, which, comp, host, (int64_t)NXY);
  if (st) fail("stz_get_field", st);
}

/* ------------------------------------------------------------- set-up */

/* io.c:4-101: the labelled input file, into the reference's globals */
void ReadInput(FILE* in) {
  char res[80] = {0};
  struct {
    const char* fmt;
    int want;
    void* a;
    void* b;
  } f[] = {
      {"Moduli(E, nu):\n%lf %lf\n\n", 2, &E, &nu},
      {"Stress-free energy barrier:\n%lf\n\n", 1, &Q0amp, NULL},
      {"Applied strain rate:\n%lf\n\n", 1, &strainrate, NULL},
      {"Strain increment:\n%lf\n\n", 1, &strainincrement, NULL},
      {"Random seed:\n%d\n\n", 1, &seed, NULL},
      {"Random ratio of fluctuation in energy barrier:\n%lf\n\n", 1, &RandomRatio, NULL},
      {"Print period:\n%d\n\n", 1, &printperiod, NULL},
      {"End Strain:\n%lf\n\n", 1, &EndStrain, NULL},
      {"Softening Flag:\n%d\n\n", 1, &softening_FLAG, NULL},
      {"Relaxation Time:\n%lf\n\n", 1, &RelxTime, NULL},
      {"Characteristic Xtal shear:\n%lf\n\n", 1, &XtalShear, NULL},
      {"Barrier for Xtal shear:\n%lf\n\n", 1, &XtalQ0amp, NULL},
      {"Ratio for generating residual stress:\n%lf\n\n", 1, &ResiRatio, NULL},
      {"Residual stress data file:\n%79s\n\n", 1, res, NULL},
      {"Volume fraction of crystal-like MRO:\n%lf\n\n", 1, &xMROFrac, NULL},
      {"Initialization condition for MRO:\n%d\n\n", 1, &InitMRO, NULL},
      {"Stress-free energy barrier for crystal-like MRO:\n%lf\n\n", 1, &xQ0amp, NULL},
  };
  for (size_t i = 0; i < sizeof(f) / sizeof(f[0]); i++) {
    int got = f[i].b ? fscanf(in, f[i].fmt, f[i].a, f[i].b) : fscanf(in, f[i].fmt, f[i].a);
    if (got != f[i].want) fprintf(stderr, "ReadInput: could not match '%.40s'\n", f[i].fmt);
  }
  memcpy(ResStressDataFile, res, sizeof(res));
}

/* init.c:6-75: derived constants. The 2D material branch in Init()'s order
 * (XTAL_VARIANTS is refused above): LOW_T from the input's moduli, or a
 * high-temperature alloy whose moduli and barrier amplitude replace the
 * input's, from the constants of the caller's bmg.h (bmg.h:36-48); then the
 * common part. */
void Init(void) {
#if defined(LOW_T)
  nu *= 2;
  mu = E / (2 + 2 * nu);
#elif defined(HIGH_T_Vit1)
  {
    const double glass = tanh((T__K - Tg__K) / DeltaE);
    E = (E_gl + E_sc) / 2. - (E_gl - E_sc) * glass / 2. - k_E * (T__K - Tg__K);
    nu = (nu_gl + nu_sc) / 2. - (nu_gl - nu_sc) * glass / 2.;
  }
  mu = E / (2 + 2 * nu);
  Q0amp = 2.2;
#elif defined(HIGH_T_PdNiP)
  E = 96;
  nu = 0.36;
  mu = E / (2 + 2 * nu);
  Q0amp = 3.0;
#else
#error "refapi: no material branch of Init() (LOW_T, HIGH_T_Vit1 or HIGH_T_PdNiP) is defined"
#endif
  lambda = E * nu / (1 - nu * nu);
  alpha = (1 + nu) / 2;
  beta = nu;
  dt = strainincrement / strainrate;
  tTemp = 1 / (TRIAL_FREQUENCY * exp(-0.37 / kT));
  tResi = 1 / (TRIAL_FREQUENCY * exp(-1.80 / kT));
  PermSoft = 13;
  PermSoftmro = 20;
  TempSoft = 39;
  TempSoftmro = 60;
  PermSofteningCap = -log(0.6);
}

/* single device: the whole grid is this rank's slab */
void FFT_MPI_Init(void) {
  lnx = NX;
  lxs = 0;
  lnyt = NY;
  lyst = 0;
  lsize = NXY;
}

void Rand_Init(void) {}  /* the engine seeds its generator from the input seed */
void Grad(void) {}       /* wave vectors are formed on the fly by the solve */

/* init.c:225-349: the fields, then the engine context (its initial draws
 * follow the reference's order: MRO map, Q0, mode eigenstrains) */
void Alloc(void) {
  for (int m = 0; m < MODES; m++) {
    Q[m] = alloc_field();
    Q0[m] = alloc_field();
    Q1[m] = alloc_field();
    Work[m] = alloc_field();
    for (int c = 0; c < DE; c++) DEps0[m][c] = alloc_field();
  }
  for (int c = 0; c < DE; c++) {
    Eps0[c] = alloc_field();
    Sigma[c] = alloc_field();
    TotEps[c] = alloc_field();
  }
  XR[0] = alloc_field();
  XR[1] = alloc_field();
  tlast = alloc_field();
  PermSoftening = alloc_field();
  TempSoftening = alloc_field();
  Softening = alloc_field();
#ifdef INHOM_ELAST
  Lambda = alloc_field();
  Mu = alloc_field();
  for (int s = 0; s < NXY; s++) {
    Lambda[s] = lambda;
    Mu[s] = mu;
  }
#endif

  stz_params_default(&g_p, STZ_MODEL_REF2D);
  g_p.n[0] = 1;
  g_p.n[1] = NX;
  g_p.n[2] = NY;
  g_p.young = E;
  g_p.poisson = nu;
  g_p.mu = mu;
  g_p.lambda = lambda;
  g_p.temperature = T__K;
  g_p.voxel_volume = VOXEL0;
  g_p.gamma0 = GAMMA0;
  g_p.q0_mean = Q0amp;
  g_p.random_ratio = RandomRatio;
  g_p.strain_rate = strainrate;
  g_p.strain_increment = strainincrement;
  g_p.end_strain = EndStrain;
  /* the reference's main runs the print-time re-solve itself, after the step
   * (bmg.c:181-295, the uflag-2 solve): the engine's own print test is off */
  g_p.print_period = 1 << 30;
  g_p.softening = softening_FLAG;
  g_p.seed = (uint64_t)(uint32_t)seed;
  g_p.perm_soft = PermSoft;
  g_p.temp_soft = TempSoft;
  g_p.perm_soft_cap = PermSofteningCap;
  g_p.t_temp = tTemp;
  g_p.xmro_frac = xMROFrac;
  g_p.init_mro = InitMRO;
  g_p.xq0amp = xQ0amp;
  g_p.perm_soft_mro = PermSoftmro;
  g_p.temp_soft_mro = TempSoftmro;
#if defined(NO_SF_XTAL_MRO)
  g_p.no_sf_xtal_mro = 1;
#else
  g_p.no_sf_xtal_mro = 0;
#endif
  MRO = (int*)calloc((size_t)NXY, sizeof(int));
  MROthe0 = alloc_field();
  int32_t* mro_in = NULL;
  if (!MRO) fail("allocation", STZ_ERR_NOMEM);
  if (InitMRO == 1) {
    /* init.c:398-420: one "i j type angle" line per site of this rank's slab */
    FILE* fp = fopen("MROstructure.ms", "r");
    if (!fp) {
      perror("MROstructure.ms");
      MPI_Abort(MPI_COMM_WORLD, -1);
    }
    mro_in = (int32_t*)calloc((size_t)NXY, sizeof(int32_t));
    if (!mro_in) fail("allocation", STZ_ERR_NOMEM);
    char buffer[80] = {0};
    for (int i = 0; i < lnx; i++)
      for (int j = 0; j < NY; j++) {
        const int m = i * NY + j;
        int ii = 0, jj = 0, t = 0;
        double th = 0;
        if (!fgets(buffer, 80, fp) || sscanf(buffer, "%d %d %d %lf", &ii, &jj, &t, &th) != 4 ||
            (ii - 1 - lxs) * NY + jj - 1 != m) {
          perror("Error in reading MROstructure.ms file (inconsistent index system)!!\n");
          MPI_Abort(MPI_COMM_WORLD, -1);
        }
        mro_in[m] = t;
        MROthe0[m] = th;
      }
    fclose(fp);
    g_p.mro_type = mro_in;
    g_p.mro_theta = MROthe0;
  }
#if defined(TENSION)
  g_p.loading = STZ_LOAD_TENSION;
#elif defined(SHEAR)
  g_p.loading = STZ_LOAD_SHEAR;
#elif defined(COMPRESSION)
  g_p.loading = STZ_LOAD_COMPRESSION;
#endif
  /* the first scheme defined in ActEnergy's order wins (init.c:590-642) */
#if defined(SF_LINEAR_FWD)
  g_p.sf_scheme = STZ_SF_LINEAR_FWD;
#elif defined(SF_LINEAR_BWD)
  g_p.sf_scheme = STZ_SF_LINEAR_BWD;
#elif defined(SF_EVEN)
  g_p.sf_scheme = STZ_SF_EVEN;
#elif defined(SF_SQUARE_FWD)
  g_p.sf_scheme = STZ_SF_SQUARE_FWD;
#elif defined(SF_CUBIC_FWD)
  g_p.sf_scheme = STZ_SF_CUBIC_FWD;
#elif defined(SF_GAUSS_FWD)
  g_p.sf_scheme = STZ_SF_GAUSS_FWD;
#endif
#ifdef NO_SUBTRACT_ERROR
  g_p.no_subtract_error = 1;
#endif
  g_p.log_capacity = 1 << 16;
  int st = stz_create(&g_p, &g_ctx);
  if (st) fail("stz_create", st);
  free(mro_in);
  g_p.mro_type = NULL;
  g_p.mro_theta = NULL;
  g_events_seen = 0;
  /* the map the engine holds (ten-fold sites of a structure file may have
   * become two-fold), as init.c:437 writes it */
  real* tmp = alloc_field();
  pull_field(STZ_FIELD_MRO, 0, tmp);
  for (int s = 0; s < NXY; s++) {
    MRO[s] = (int)tmp[s];
    g_any_mro |= MRO[s] != 0;
  }
  free(tmp);
  if (g_any_mro)
    for (int m = 0; m < MODES; m++) g_q0_seen[m] = alloc_field();
  pull_field(STZ_FIELD_MRO, 1, MROthe0);
  WriteMROMPI_INT(MRO, "Initial_MROstructure", 0);
}

/* init.c:181-198: the barriers the engine drew, and their initial copy Q1 */
void Energy_Init(void) {
  for (int m = 0; m < MODES; m++) {
    pull_field(STZ_FIELD_DF, m, Q0[m]);
    memcpy(Q1[m], Q0[m], sizeof(real) * NXY);
  }
  pull_field(STZ_FIELD_TLAST, 0, tlast);
}

/* elastic.c:115-140: the mode eigenstrains the engine drew */
void DStrain(void) {
  for (int m = 0; m < MODES; m++)
    for (int c = 0; c < DE; c++) pull_field(STZ_FIELD_DEPS, m * 3 + c, DEps0[m][c]);
}

/* ------------------------------------------------------------- solves */

static void solve_into(real** epso, real** sigmao, real* stress, real* epsavg) {
  int moved = 0;
  for (int c = 0; c < 3; c++) moved |= epsavg[c] != g_epsavg_dev[c];
  if (moved) {
    double e6[6] = {epsavg[0], epsavg[1], epsavg[2], 0, 0, 0};
    int st = stz_set_mean_strain(g_ctx, e6);
    if (st) fail("stz_set_mean_strain", st);
  }
  int st = stz_solve(g_ctx);
  if (st) fail("stz_solve", st);
  for (int c = 0; c < DE; c++) pull_field(STZ_FIELD_SIGMA, c, sigmao[c]);
  pull_scalars();
  for (int c = 0; c < 3; c++) {
    stress[c] = Stress[c];
    epsavg[c] = EpsAvg[c];
  }
  if (epso) {
    /* total strain = elastic strain (isotropic compliance) + eigenstrain */
    real* e0[DE];
    for (int c = 0; c < DE; c++) {
      e0[c] = alloc_field();
      pull_field(STZ_FIELD_EPS0, c, e0[c]);
    }
    for (int s = 0; s < NXY; s++) {
      const real s0 = sigmao[0][s], s1 = sigmao[1][s], s2 = sigmao[2][s];
      const real tr = s0 + s1;
      epso[0][s] = (s0 - lambda / (2 * lambda + 2 * mu) * tr) / (2 * mu) + e0[0][s];
      epso[1][s] = (s1 - lambda / (2 * lambda + 2 * mu) * tr) / (2 * mu) + e0[1][s];
      epso[2][s] = s2 / (2 * mu) + e0[2][s];
    }
    for (int c = 0; c < DE; c++) free(e0[c]);
  }
}

/* Positions of the print step (elastic.c:866-870, io.c:151-155 and 204):
 * the supercell position with the mean strain epsavg plus the displacement
 * field of the current eigenstrain from the engine. */
static void positions(real** xr, const real* epsavg) {
  real* u = (real*)malloc(sizeof(real) * 2 * NXY);
  if (!u) fail("malloc", STZ_ERR_NOMEM);
  int st = stz_get_displacement(g_ctx, u, (int64_t)2 * NXY);
  if (st) fail("stz_get_displacement", st);
  for (int i = 0; i < lnx; i++)
    for (int j = 0; j < NY; j++) {
      const int idx = i * NY + j;
      xr[0][idx] = (i + lxs) * (1 + epsavg[0]) * LX + j * epsavg[2] * LY + u[idx];
      xr[1][idx] = (i + lxs) * epsavg[2] * LX + j * (1 + epsavg[1]) * LY + u[NXY + idx];
    }
  free(u);
}

#ifdef INHOM_ELAST
/* elastic.c:977-1066: the engine's solve with the site moduli Lambdao, Muo
 * (a uniform medium is one homogeneous solve; a varying one is the
 * polarisation fixed point around lambda_, mu_). The moduli go to the device
 * when they differ from what it holds. */
void InhomogeneousStressSolver(real* Lambdao, real* Muo, real** eps0o, real* epsavg, real lambda_, real mu_,
                               real** uo, real** epso, real** sigmao, real* stress, int uflag) {
  static real* held[2] = {NULL, NULL};  /* the moduli last passed to the engine */
  real* mod[2] = {Lambdao, Muo};
  const real uni[2] = {lambda_, mu_};
  (void)eps0o;
  for (int k = 0; k < 2; k++) {
    int push = 0;
    for (int s = 0; s < NXY && !push; s++) push = held[k] ? mod[k][s] != held[k][s] : mod[k][s] != uni[k];
    if (!push) continue;
    if (!held[k]) held[k] = alloc_field();
    for (int s = 0; s < NXY; s++) held[k][s] = mod[k][s];
    int st = stz_set_field(g_ctx, k ? STZ_FIELD_MU : STZ_FIELD_LAMBDA, 0, mod[k], NXY);
    if (st) fail("stz_set_field (moduli)", st);
  }
  solve_into(epso, sigmao, stress, epsavg);
  if (uflag != 0 && uo) positions(uo, epsavg);
}

/* elastic.c:779-900 */
void HomogeneousStressSolver(real lambda_, real mu_, real** eps0o, real* epsavg, real** uo, real** epso,
                             real** sigmao, real* stress, int uflag) {
  (void)lambda_;
  (void)mu_;
  (void)eps0o;
  solve_into(epso, sigmao, stress, epsavg);
  if (uflag != 0 && uo) positions(uo, epsavg);
}
#endif

/* elastic.c: the solve on the global fields */
void HomStressSolver(void) { solve_into(TotEps, Sigma, Stress, EpsAvg); }

/* io.c:137-240: positions of the print step from Eps0 and EpsAvg */
void DispField(real* xr[2]) { positions(xr, EpsAvg); }

/* ------------------------------------------------------------- the step */

void SofteningFactor(void) {}  /* computed per site inside the rate pass */

/* init.c:561-690: Q for every mode at the current stress */
void ActEnergy(int step_) {
  (void)step_;
  for (int m = 0; m < MODES; m++) pull_field(STZ_FIELD_Q, m, Q[m]);
}

/* Q0 modes that main changed since RecordPrep go to the device */
static void sync_q0(void) {
  if (!g_q0_check) return;
  g_q0_check = 0;
  for (int m = 0; m < MODES; m++)
    if (memcmp(g_q0_seen[m], Q0[m], sizeof(real) * NXY) != 0) {
      int st = stz_set_field(g_ctx, STZ_FIELD_DF, m, Q0[m], (int64_t)NXY);
      if (st) fail("stz_set_field", st);
    }
}

/* one driver step on the device, then the globals and the actQ.out records
 * of evolution.c:243 */
static void one_step(void) {
  sync_q0();
  int st = stz_run(g_ctx, 1, 0);
  if (st) fail("stz_run", st);
  pull_scalars();
  stz_event ev[256];
  for (;;) {
    int64_t n = 0;
    st = stz_get_events(g_ctx, g_events_seen, ev, 256, &n);
    if (st) fail("stz_get_events", st);
    if (n <= 0) break;
    for (int64_t i = 0; i < n; i++)
      if (ev[i].kind == STZ_EV_THERMAL && rank == 0 && fq) {
        /* evolution.c:206,243: the chosen site's MRO type and its Q */
        fprintf(fq, "%d\t%.6e\n", MRO[ev[i].site], ev[i].q);
        fflush(fq);
      }
    g_events_seen += n;
    if (n < 256) break;
  }
}

void KMC(void) { one_step(); }
void athermal_plasticity(void) { one_step(); }

void UpdateSOC(void) {}

/* elastic.c:533-547 */
void ElasticEnergy(void) {
  double e = 0;
  int st = stz_elastic_energy(g_ctx, &e);
  if (st) fail("stz_elastic_energy", st);
  elEnergy = e;
}

/* ------------------------------------------------------------- records */

/* io.c:260-273 */
void RecordPrep(void) {
  for (int c = 0; c < DE; c++) {
    pull_field(STZ_FIELD_EPS0, c, Eps0[c]);
    pull_field(STZ_FIELD_SIGMA, c, Sigma[c]);
  }
  /* the reference's main resets Q0 to Q1 right after RecordPrep in its print
   * block (bmg.c:214-221). Crystal-like sites change Q0 when they transform,
   * so the mirror is brought up to date here and what main writes to it is
   * passed to the device before the next step (sync_q0). */
  if (g_any_mro) {
    for (int m = 0; m < MODES; m++) {
      pull_field(STZ_FIELD_DF, m, Q0[m]);
      memcpy(g_q0_seen[m], Q0[m], sizeof(real) * NXY);
    }
    g_q0_check = 1;
  }
  EqStrain = (real*)malloc((size_t)lsize * sizeof(real));
  EqStress = (real*)malloc((size_t)lsize * sizeof(real));
  for (int s = 0; s < NXY; s++) {
    EqStrain[s] = sqrt(Eps0[0][s] * Eps0[0][s] + Eps0[2][s] * Eps0[2][s]);
    EqStress[s] = sqrt(Sigma[0][s] * Sigma[0][s] + Sigma[2][s] * Sigma[2][s]);
  }
}

void RecordFree(void) {
  free(EqStrain);
  free(EqStress);
  EqStrain = EqStress = NULL;
}

/* io.c:289-347: a field as the reference's binary record "<s>_S<step>.iout",
 * the raw native values of the ranks' slabs in rank order (what MPI-IO
 * writes with the view rank * lsize). Here one rank holds the whole grid, so
 * rank 0 writes the file alone; the bytes are those of a single-rank run of
 * the reference. A file that cannot be written ends the run, as the
 * reference's other record files do. */
static void write_record(const void* field, size_t elem, const char* s, int step) {
  if (rank != 0) return;
  char fname[256];
  snprintf(fname, sizeof fname, "%s_S%03d.iout", s, step);
  FILE* f = fopen(fname, "wb");
  if (!f || fwrite(field, elem, (size_t)lsize, f) != (size_t)lsize) {
    perror(fname);
    if (f) fclose(f);
    MPI_Abort(MPI_COMM_WORLD, -1);
    return;
  }
  fclose(f);
}

void WriteScalarMPI(real* field, char* s, int step) { write_record(field, sizeof(real), s, step); }
void WriteScalarMPI_INT(int* field, char* s, int step) { write_record(field, sizeof(int), s, step); }
/* the reference copies the map before writing it; the bytes are the same */
void WriteMROMPI_INT(int* field, char* s, int step) { write_record(field, sizeof(int), s, step); }

void ParameterPrint(void) {
  /* the reference's text, byte for byte (io.c:103-135), so that logs of a
   * drop-in build compare with the reference's */
  printf("\nSimulation Geometry:\n");
  printf("System size:\t[%d x %d]\n", NX, NY);
  printf("Voxel size:\t[%.3fnm x %.3fnm]\n", (double)LX, (double)LY);
  printf("\nMaterial Properties at T=%f\n", (double)T__K);
  printf("Activation energy barrier amplituide: \t%.3f\n", Q0amp);
  printf("Young's modulus:\t%.3f\n", E);
  printf("Shear modulus:\t%.3f\n", mu);
  printf("Poisson's ratio:\t%.3f\n", nu);
  printf("\nPEL Parameters:\n");
  printf("# of STZ modes:\t%d\n", MODES);
  printf("Stress-free energy barrier prefactor:\t%.3f\n", Q0amp);
  printf("\nSoftening Parameters:\n");
  printf("Permanent softening prefactor:\t%.3f\n", PermSoft);
  printf("Temporary softening prefactor:\t%.3f\n", TempSoft);
  printf("PermSoftening cap:\t%.3f\n", PermSofteningCap);
  printf("\nSimulation Environment:\n");
  printf("Applied strain rate:\t%.3e\n", strainrate);
  printf("Strain increment in recording data:\t%.3e\n", strainincrement);
  printf("End Strain:\t%.3f\n", EndStrain);
  printf("Softening model: %s\n", softening_FLAG == 0 ? "OFF" : "ON");
  printf("Relaxation time:\t%.3e\n", RelxTime);
  printf("Ratio for generating residual stress:\t%.3f\n", ResiRatio);
}

void PrintFlags(void) {
  /* the reference's list and order (io.c:374-434); the switches it also
   * lists that this layer refuses cannot be defined here */
  printf("Active flags in bmgFlags.h:\n");
#ifdef COMPRESSION
  printf("#define COMPRESSION\n");
#endif
#ifdef TENSION
  printf("#define TENSION\n");
#endif
#ifdef SHEAR
  printf("#define SHEAR\n");
#endif
#ifdef PRE_RELAXATION
  printf("#define PRE_RELAXATION\n");
#endif
#ifdef RESIDUAL_STRESS
  printf("#define RESIDUAL_STRESS\n");
#endif
#ifdef UNIFORM_DEFECTS
  printf("#define UNIFORM_DEFECTS\n");
#endif
#ifdef LOW_T
  printf("#define LOW_T\n");
#endif
#ifdef HIGH_T_Vit1
  printf("#define HIGH_T_Vit1\n");
#endif
}

/* init.c:499-559 */
void Free(void) {
  stz_destroy(g_ctx);
  g_ctx = NULL;
  for (int m = 0; m < MODES; m++) {
    free(Q[m]);
    free(Q0[m]);
    free(Q1[m]);
    free(Work[m]);
    for (int c = 0; c < DE; c++) free(DEps0[m][c]);
  }
  for (int c = 0; c < DE; c++) {
    free(Eps0[c]);
    free(Sigma[c]);
    free(TotEps[c]);
  }
  free(XR[0]);
  free(XR[1]);
  free(tlast);
  free(PermSoftening);
  free(TempSoftening);
  free(Softening);
  free(MRO);
  free(MROthe0);
  MRO = NULL;
  MROthe0 = NULL;
  for (int m = 0; m < MODES; m++) {
    free(g_q0_seen[m]);
    g_q0_seen[m] = NULL;
  }
  g_any_mro = 0;
  g_q0_check = 0;
#ifdef INHOM_ELAST
  free(Lambda);
  free(Mu);
#endif
}

/* the engine context behind the reference API (for callers that want the
 * event log or the handle API alongside it) */
stz_ctx* stz_refapi_context(void) { return g_ctx; }
