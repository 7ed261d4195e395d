/*
 * stz_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (FP64, plain C) of the reference's STZ kinetic Monte Carlo
 * step, used as the correctness oracle by tests/, by __graft_entry__.smoke()
 * and as the CPU baseline leg of bench.py. Nothing in the product links it.
 *
 * Parity pinning: the 2D model is checked against the reference's own sources
 * compiled unmodified against single-rank stand-ins for MPI, FFTW 2 and GSL
 * (oracle/Makefile, target _ref/ref2d) and against fixtures produced by that
 * build (tests/golden/). The 3D model generalises the same formulas; there is
 * no reference code for 3D, so its parity rests on the 2D pinning plus the
 * invariants tested in tests/ (equilibrium, compatibility, mean stress).
 *
 * Third-party algorithms restated here (absent from the reference tree):
 *   GSL mt19937 generator (gsl_rng_default; rng/mt.c of GSL 1.x/2.x, version
 *     not pinned by the reference Makefile), gsl_rng_uniform = u32 / 2^32,
 *     gsl_rng_uniform_pos rejects 0, gsl_ran_gaussian = polar Box-Muller as
 *     restated by the reference itself at init.c:207-223.
 *   FFTW 2.x fftwnd_mpi: unnormalised complex DFT, sign -1 forward, +1 backward.
 */
#ifndef STZ_ORACLE_H
#define STZ_ORACLE_H

#include <stdint.h>
#include "../include/stz_api.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- GSL-convention MT19937 ------------------------------------------------ */
typedef struct or_rng { uint32_t mt[624]; int mti; } or_rng;
void     or_rng_seed(or_rng* r, unsigned long s);
uint32_t or_rng_get(or_rng* r);
double   or_rng_uniform(or_rng* r);
double   or_rng_uniform_pos(or_rng* r);
double   or_ran_gaussian(or_rng* r, double sigma);

/* ---- complex FFT on interleaved (re,im) doubles ---------------------------- */
/* In-place unnormalised DFT of an n0 x n1 x n2 array (n2 fastest) along every
 * axis of extent > 1. sign = -1 forward, +1 backward. Extents: 2^a 3^b. */
int  or_fft3(int n0, int n1, int n2, double* data, int sign);

/* ---- model ------------------------------------------------------------------ */
typedef struct or_model or_model;

or_model* or_create(const stz_params* p, int* status);
void      or_destroy(or_model* m);
/* The driver loop (bmg.c:138-411) until max_steps iterations or max_events
 * thermal events, or a stop condition. Returns a stz status code. */
int  or_run(or_model* m, int64_t max_steps, int64_t max_events);
int  or_solve(or_model* m);        /* InhomogeneousStressSolver(...,0) */
int  or_get_scalars(or_model* m, stz_scalars* out);
int64_t or_num_events(or_model* m);
int  or_get_events(or_model* m, int64_t first, stz_event* out, int64_t cap, int64_t* n);
int  or_get_field(or_model* m, int which, int comp, double* out, int64_t count);
int  or_set_field(or_model* m, int which, int comp, const double* in, int64_t count);
int  or_elastic_energy(or_model* m, double* out);
int  or_set_mean_strain(or_model* m, const double* eps_avg);
/* Forced path: the next n thermal events take (sites[k], modes[k]) after
 * discarding draws[k] - 1 generator words; or_get_checks returns per event
 * the oracle's own choice with the same words, the dice, the forced element's
 * cumulative interval (fractions of the total rate), the total rate and the
 * words the own choice took. */
int  or_force_path(or_model* m, const int64_t* sites, const int32_t* modes, const int32_t* draws, int64_t n);
int64_t or_get_checks(or_model* m, double* out, int64_t cap);
/* Own choices by line bounds of slack 2^-slack with rejection (slack > 0), the
 * rule of the engine's mixed form, instead of the reference's (slack 0). For
 * tests of the engine's rejection path only. */
int  or_set_bounded_selection(or_model* m, int slack);
/* Parameters without the engine library: defaults per model (the reference's
 * constants for REF2D, the 3D study's for GLOBAL3D) and the reference's
 * labelled input file through Init() under LOW_T (io.c:4-101, init.c:6-75). */
int  or_params_default(stz_params* p, int model);
int  or_params_from_input_file(stz_params* p, const char* path);
/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int  or_threads(void);
void or_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
