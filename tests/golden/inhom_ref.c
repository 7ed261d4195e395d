/* Fixture generator (test infrastructure; compiled only where the reference
 * tree is present, by make_golden.py): the reference's own
 * InhomogeneousStressSolver (elastic.c:977-1066) on a spatially varying
 * medium. The reference sources io.c, init.c, elastic.c and evolution.c are
 * compiled unmodified against the single-rank stand-ins of oracle/shim; this
 * file is their main. It reads the "input" file of the working directory,
 * sets up the reference's state (Init ... DStrain), then overwrites
 *   Eps0     with a deterministic pattern of transformed sites,
 *   Lambda, Mu with a deterministic field between 0.7 and 1.3 of lambda, mu,
 *   EpsAvg   with a mean strain above the solver's 1e-4 convergence floor,
 * calls InhomogeneousStressSolver(..., uflag 0) and writes inhom.bin:
 *   int64 NX, NY; float64 lambda, mu, EpsAvg[3], Stress[3];
 *   float64 Eps0[3][N], Lambda[N], Mu[N], Sigma[3][N]. */
#define BMG_GLOBALS_ONCE
#include "bmg.h"
#include "my_fft.h"
#undef BMG_GLOBALS_ONCE

static double frac(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

int main(int argc, char** argv) {
  int i, j, c, idx;
  FILE* f1 = fopen("input", "r");
  if (!f1) { perror("input"); return 2; }
  ReadInput(f1);
  fclose(f1);
  MPI_Init(&argc, &argv);
  MPI_Comm_size(MPI_COMM_WORLD, &totnodes);
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  Init();
  FFT_MPI_Init();
  Rand_Init();
  Alloc();
  Grad();
  Energy_Init();
  DStrain();
  space_loop {
    idx = i * NY + j;
    for (c = 0; c < DE; c++) Eps0[c][idx] = 0.0;
    /* one site in eight carries a mode strain of its own */
    if (frac(3 * (unsigned long long)idx + 1) < 0.125) {
      const int m = (int)(frac(5 * (unsigned long long)idx + 2) * MODES) % MODES;
      for (c = 0; c < DE; c++) Eps0[c][idx] = DEps0[m][c][idx];
    }
    const double a = 0.7 + 0.6 * frac(7 * (unsigned long long)idx + 3);
    const double b = 0.7 + 0.6 * frac(11 * (unsigned long long)idx + 4);
    Lambda[idx] = a * lambda;
    Mu[idx] = b * mu;
  }
  EpsAvg[0] = 2.0e-3;
  EpsAvg[1] = -7.0e-4;
  EpsAvg[2] = 1.1e-3;
  InhomogeneousStressSolver(Lambda, Mu, Eps0, EpsAvg, lambda, mu, XR, TotEps, Sigma, Stress, 0);
  FILE* fo = fopen("inhom.bin", "wb");
  if (!fo) { perror("inhom.bin"); return 2; }
  const long long hdr[2] = {NX, NY};
  fwrite(hdr, sizeof(long long), 2, fo);
  const double sc[8] = {lambda, mu, EpsAvg[0], EpsAvg[1], EpsAvg[2], Stress[0], Stress[1], Stress[2]};
  fwrite(sc, sizeof(double), 8, fo);
  for (c = 0; c < DE; c++) fwrite(Eps0[c], sizeof(double), NXY, fo);
  fwrite(Lambda, sizeof(double), NXY, fo);
  fwrite(Mu, sizeof(double), NXY, fo);
  for (c = 0; c < DE; c++) fwrite(Sigma[c], sizeof(double), NXY, fo);
  fclose(fo);
  MPI_Finalize();
  return 0;
}
