/* TEST INFRASTRUCTURE ONLY. Stand-in for gsl_ran_gaussian (polar method). */
#ifndef STZ_SHIM_GSL_RANDIST_H
#define STZ_SHIM_GSL_RANDIST_H
#include "gsl_rng.h"
double gsl_ran_gaussian(const gsl_rng* r, double sigma);
#endif
