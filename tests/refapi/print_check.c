/* Test program for the drop-in layer's start-up printout: reads ./input,
 * derives the constants and prints the flag and parameter blocks, in the
 * order the reference's main does (bmg.c:42, 60-81). No device work is
 * done. */
#define BMG_GLOBALS_ONCE
#include "bmg.h"
#include "my_fft.h"
#undef BMG_GLOBALS_ONCE

int main(int argc, char** argv) {
  MPI_Init(&argc, &argv);
  MPI_Comm_size(MPI_COMM_WORLD, &totnodes);
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  PrintFlags();
  FILE* in = fopen("input", "r");
  if (!in) return 2;
  ReadInput(in);
  fclose(in);
  Init();
  ParameterPrint();
  MPI_Finalize();
  return 0;
}
