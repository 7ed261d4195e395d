/* Test driver of the reference API on the GB300 engine: the call sequence
 * of the reference's main loop (bmg.c:30-410, 2D, INHOM_ELAST), without its
 * text output files, stopped after REFAPI_MAX_EVENTS thermal events. It writes
 *   steps.txt   per driver step: step kind time EpsAvg[3] Stress[3]
 *               (kind 0 thermal, 1 athermal, 2 elastic)
 *   events.txt  per transformation: step kind site mode (from the engine log)
 *   X1R%03d_P00.out, X2R%03d_P00.out  the positions XR of the prints listed in
 *               REFAPI_XR_PRINTS (comma-separated print numbers; all prints when
 *               unset), named and formatted as the reference's main writes them
 *               (bmg.c:300-330)
 *   Strain_0c_S%03d.iout, Stress_0c_S%03d.iout  Eps0 and Sigma of the same
 *               prints through WriteScalarMPI, where the reference's main writes
 *               them under FULL_TENSOR_RECORD (bmg.c:269-277)
 * in the working directory, which holds the reference's "input" file. */
#define BMG_GLOBALS_ONCE
#include "bmg.h"
#include "my_fft.h"
#undef BMG_GLOBALS_ONCE
#include "stz_api.h"

stz_ctx* stz_refapi_context(void);

int main(int argc, char** argv) {
  int i, j, m, idx;
  const char* cap = getenv("REFAPI_MAX_EVENTS");
  const int max_events = cap ? atoi(cap) : 1000;
  FILE* f1 = fopen("input", "r");
  if (!f1) { perror("input"); return 2; }
  ReadInput(f1);
  fclose(f1);
  MPI_Init(&argc, &argv);
  MPI_Comm_size(MPI_COMM_WORLD, &totnodes);
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  Init();
  fq = fopen("actQ.out", "w");
  FFT_MPI_Init();
  Rand_Init();
  Alloc();
  Grad();
  Energy_Init();
  DStrain();
  EpsAvg[0] = 0.; EpsAvg[1] = 0.; EpsAvg[2] = 0.;
  InhomogeneousStressSolver(Lambda, Mu, Eps0, EpsAvg, lambda, mu, XR, TotEps, Sigma, Stress, 0);
  FILE* fs = fopen("steps.txt", "w");
  real last_print = 0.0;
  int n_print = 1;
  const char* xr_list = getenv("REFAPI_XR_PRINTS");
#ifdef TENSION
  const int lc = 0;
#else
  const int lc = 2;
#endif
  while (1) {
    step++;
    if (softening_FLAG == 1) SofteningFactor();
    ActEnergy(step);
    int flag = 0;
    for (m = 0; m < MODES; m++)
      space_loop {
        idx = i * NY + j;
        if (Q[m][idx] < 0) flag++;
      }
    const int k0 = kstep, a0 = astep;
    if (flag > 0) {
      athermal_plasticity();
    } else {
      UpdateSOC();
      KMC();
    }
    ElasticEnergy();
    const int kind = kstep > k0 ? 0 : (astep > a0 ? 1 : 2);
    fprintf(fs, "%d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", step, kind, totime, EpsAvg[0], EpsAvg[1],
            EpsAvg[2], Stress[0], Stress[1], Stress[2]);
    if (fabs(EpsAvg[lc] - last_print) >= (printperiod * strainincrement * 0.99)) {
      last_print = EpsAvg[lc];
      int want = !xr_list;
      if (xr_list) {
        const char* q = xr_list;
        while (*q && !want) {
          if (atoi(q) == n_print) want = 1;
          while (*q && *q != ',') q++;
          if (*q == ',') q++;
        }
      }
      RecordPrep();
      for (m = 0; m < MODES; m++)
        for (i = 0; i < lnx; i++)
          for (j = 0; j < NY; j++) Q0[m][i * NY + j] = Q1[m][i * NY + j];
      for (int c = 0; c < 3 && want; c++) {
        char fname[32];
        sprintf(fname, "Strain_%02d", c + 1);
        WriteScalarMPI(Eps0[c], fname, n_print);
        sprintf(fname, "Stress_%02d", c + 1);
        WriteScalarMPI(Sigma[c], fname, n_print);
      }
      RecordFree();
      InhomogeneousStressSolver(Lambda, Mu, Eps0, EpsAvg, lambda, mu, XR, TotEps, Sigma, Stress, 2);
      n_print++;
      for (int a = 0; a < 2 && want; a++) {
        char fname[64];
        sprintf(fname, "X%dR%03d_P%02d.out", a + 1, n_print - 1, rank);
        FILE* fx = fopen(fname, "w");
        if (!fx) { perror(fname); return 2; }
        for (i = 0; i < lnx; i++) {
          for (j = 0; j < NY; j++) fprintf(fx, "%lf ", XR[a][i * NY + j]);
          fprintf(fx, "\n");
        }
        fclose(fx);
      }
    }
    if (kstep >= max_events) break;
#ifdef TENSION
    if (fabs(EpsAvg[0]) > EndStrain) break;
    if (Stress[0] < -0.5) break;
#else
    if (fabs(EpsAvg[2]) > EndStrain) break;
    if (fabs(Stress[2]) < EPSILON) break;
#endif
  }
  fclose(fs);
  FILE* fe = fopen("events.txt", "w");
  stz_ctx* ctx = stz_refapi_context();
  int64_t first = 0;
  stz_event ev[512];
  for (;;) {
    int64_t n = 0;
    if (stz_get_events(ctx, first, ev, 512, &n) || n <= 0) break;
    for (int64_t k = 0; k < n; k++)
      if (ev[k].kind != STZ_EV_ELASTIC)
        fprintf(fe, "%lld %d %lld %d\n", (long long)ev[k].step, ev[k].kind, (long long)ev[k].site, ev[k].mode);
    first += n;
  }
  fclose(fe);
  if (fq) fclose(fq);
  Free();
  MPI_Finalize();
  return 0;
}
