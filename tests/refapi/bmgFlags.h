/* Test build flags for the reference-API driver: the configuration of the
 * 2D fixtures (tension loading, square-forward softening directions, the
 * low-temperature material branch, micro memory, the inhomogeneous-solver
 * entry point, the reduced softening of crystal-like sites). Written for the
 * tests; the names are the reference's. REFAPI_TEST_NO_SF leaves the
 * softening-direction scheme to the command line, REFAPI_TEST_HIGH_T the
 * material branch (HIGH_T_Vit1 or HIGH_T_PdNiP in place of LOW_T). */
#ifndef H_BMGFLAGS
#define H_BMGFLAGS
#ifdef REFAPI_TEST_SHEAR
#define SHEAR
#else
#define TENSION
#endif
#ifndef REFAPI_TEST_NO_SF
#define SF_SQUARE_FWD
#endif
#ifndef REFAPI_TEST_HIGH_T
#define LOW_T
#endif
#ifndef REFAPI_TEST_NO_MICRO_MEMORY
#define MICRO_MEMORY
#endif
#define INHOM_ELAST
#define NO_SF_XTAL_MRO
#endif
