/*
 * TEST INFRASTRUCTURE ONLY. Stand-in for the part of GSL's random number
 * interface used by the reference: gsl_rng_default is mt19937 (GSL's
 * default generator), seeded from gsl_rng_default_seed at allocation.
 */
#ifndef STZ_SHIM_GSL_RNG_H
#define STZ_SHIM_GSL_RNG_H
typedef struct { const char* name; } gsl_rng_type;
typedef struct gsl_rng gsl_rng;
extern const gsl_rng_type* gsl_rng_default;
extern unsigned long int gsl_rng_default_seed;
gsl_rng* gsl_rng_alloc(const gsl_rng_type* T);
void gsl_rng_free(gsl_rng* r);
double gsl_rng_uniform(const gsl_rng* r);
double gsl_rng_uniform_pos(const gsl_rng* r);
#endif
