/* Test-only stand-in for the reference's my_fft.h: the slab globals. */
#ifndef H_MY_FFT
#define H_MY_FFT
#include "bmg.h"
#ifdef BMG_GLOBALS_ONCE
int rank = 0, totnodes = 0;
int lnx = 0, lxs = 0, lnyt = 0, lyst = 0, lsize = 0;
#else
extern int rank, totnodes;
extern int lnx, lxs, lnyt, lyst, lsize;
#endif
#endif
