/*
 * TEST INFRASTRUCTURE ONLY. Single-rank stand-in for the FFTW 2.x MPI
 * interface used by the reference STZ code: an unnormalised complex 2D DFT
 * (sign -1 forward, +1 backward) in normal order, computed by the oracle's
 * FFT. The whole grid is the local slab (lnx = NX, lxs = 0).
 */
#ifndef STZ_SHIM_FFTW_MPI_H
#define STZ_SHIM_FFTW_MPI_H
#include <stddef.h>
#include "mpi.h"

typedef double fftw_real;
typedef struct { fftw_real re, im; } fftw_complex;
typedef enum { FFTW_FORWARD = -1, FFTW_BACKWARD = 1 } fftw_direction;
typedef enum { FFTW_NORMAL_ORDER = 0, FFTW_TRANSPOSED_ORDER = 1 } fftwnd_mpi_output_order;
#define FFTW_ESTIMATE 0
typedef struct stz_shim_plan* fftwnd_mpi_plan;

fftwnd_mpi_plan fftw2d_mpi_create_plan(MPI_Comm comm, int nx, int ny, fftw_direction dir, int flags);
void fftwnd_mpi_local_sizes(fftwnd_mpi_plan p, int* local_nx, int* local_x_start,
                            int* local_ny_after_transpose, int* local_y_start_after_transpose,
                            int* total_local_size);
void fftwnd_mpi(fftwnd_mpi_plan p, int n_fields, fftw_complex* local_data, fftw_complex* work,
                fftwnd_mpi_output_order order);
void fftwnd_mpi_destroy_plan(fftwnd_mpi_plan p);
void* fftw_malloc(size_t n);
void fftw_free(void* p);
#endif

/*
 * Outside the include guard on purpose. The reference fixes the grid with
 * '#define NX 512' / '#define NY 512' in bmg.h, and every translation unit
 * includes this header a second time (through my_fft.h) after bmg.h. When the
 * build passes -DSTZ_SHIM_NX=.. -DSTZ_SHIM_NY=.., the second inclusion
 * replaces the grid size for the rest of the translation unit, so the
 * unmodified sources run at a test-sized grid. bmgFlags.h switches change
 * the same way:
 *   STZ_SHIM_LOAD_SHEAR   SHEAR in place of TENSION;
 *   STZ_SHIM_XTAL_SF_OFF  NO_SF_XTAL_MRO taken out;
 *   STZ_SHIM_NO_LOW_T     LOW_T taken out, for a HIGH_T_* material branch
 *                         defined on the command line (bmg.h's Tg__K needs it
 *                         before this point);
 *   STZ_SHIM_SF=k         the softening-direction scheme, k as STZ_SF_*
 *                         (0 LINEAR_FWD, 1 LINEAR_BWD, 2 EVEN, 3 SQUARE_FWD,
 *                         4 CUBIC_FWD, 5 GAUSS_FWD: the names ActEnergy tests).
 * Every unit includes my_fft.h after bmg.h, so its code sees the changed
 * switches; only bmg.h's own declarations were made before this point, which
 * is why a switch that bmg.h reads (MICRO_MEMORY) cannot change here.
 */
#if defined(NX) && defined(STZ_SHIM_NX)
#undef NX
#define NX STZ_SHIM_NX
#endif
#if defined(NY) && defined(STZ_SHIM_NY)
#undef NY
#define NY STZ_SHIM_NY
#endif
#if defined(H_BMGFLAGS) && defined(STZ_SHIM_LOAD_SHEAR)
#undef TENSION
#undef COMPRESSION
#ifndef SHEAR
#define SHEAR
#endif
#endif
#if defined(H_BMGFLAGS) && defined(STZ_SHIM_NO_LOW_T)
#undef LOW_T
#endif
#if defined(H_BMGFLAGS) && defined(STZ_SHIM_XTAL_SF_OFF)
#undef NO_SF_XTAL_MRO
#endif
#if defined(H_BMGFLAGS) && defined(STZ_SHIM_SF)
#undef SF_LINEAR_FWD
#undef SF_LINEAR_BWD
#undef SF_EVEN
#undef SF_SQUARE_FWD
#undef SF_CUBIC_FWD
#undef SF_GAUSS_FWD
#if STZ_SHIM_SF == 0
#define SF_LINEAR_FWD
#elif STZ_SHIM_SF == 1
#define SF_LINEAR_BWD
#elif STZ_SHIM_SF == 2
#define SF_EVEN
#elif STZ_SHIM_SF == 3
#define SF_SQUARE_FWD
#elif STZ_SHIM_SF == 4
#define SF_CUBIC_FWD
#elif STZ_SHIM_SF == 5
#define SF_GAUSS_FWD
#else
#error "STZ_SHIM_SF must be 0..5"
#endif
#endif
