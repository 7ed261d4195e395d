/* Test program for the material branches of the drop-in layer's Init()
 * (init.c:6-75 in the reference): sets the input file's moduli and barrier
 * amplitude, calls Init() as the reference's main does after ReadInput, and
 * prints the derived E, nu, mu, lambda and Q0amp. No device work is done. */
#define BMG_GLOBALS_ONCE
#include "bmg.h"
#include "my_fft.h"
#undef BMG_GLOBALS_ONCE

int main(void) {
  E = 69.46;
  nu = 0.365;
  Q0amp = 2.0;
  strainincrement = 1e-4;
  strainrate = 1e-4;
  Init();
  printf("%.17g %.17g %.17g %.17g %.17g\n", E, nu, mu, lambda, Q0amp);
  return 0;
}
