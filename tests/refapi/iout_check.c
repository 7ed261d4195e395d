/* Test program for the .iout record writers of the drop-in layer (io.c:289-347
 * in the reference): writes a known FP64 field and a known int field through
 * WriteScalarMPI / WriteScalarMPI_INT as the reference's main calls them, in
 * the working directory. No device work is done. */
#define BMG_GLOBALS_ONCE
#include "bmg.h"
#include "my_fft.h"
#undef BMG_GLOBALS_ONCE

int main(int argc, char** argv) {
  MPI_Init(&argc, &argv);
  MPI_Comm_size(MPI_COMM_WORLD, &totnodes);
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  FFT_MPI_Init();
  real* f = (real*)malloc(sizeof(real) * NXY);
  int* g = (int*)malloc(sizeof(int) * NXY);
  for (int s = 0; s < NXY; s++) {
    f[s] = 0.25 * s - 3.0;
    g[s] = 7 * s - 11;
  }
  char name[32];
  sprintf(name, "Stress_%02d", 2);
  WriteScalarMPI(f, name, 12);
  WriteScalarMPI_INT(g, "Map", 3);
  free(f);
  free(g);
  MPI_Finalize();
  return 0;
}
