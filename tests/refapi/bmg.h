/* Test-only stand-in for the reference's bmg.h: the names, types and
 * constants the reference API (and its main) use, declared for the driver
 * test of the GB300 drop-in (metallic_glasses_gb300/refapi/refapi.c). The
 * grid size comes from REFAPI_NX / REFAPI_NY; the physical constants are the
 * reference's shipped values (2D model). The globals are defined in the unit
 * that defines BMG_GLOBALS_ONCE, as in the reference. */
#ifndef H_BMG_MPI
#define H_BMG_MPI
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>
#include "bmgFlags.h"

typedef double real;
#define MPI_real MPI_DOUBLE
#ifndef REFAPI_NX
#define REFAPI_NX 32
#endif
#ifndef REFAPI_NY
#define REFAPI_NY 32
#endif
#define NX REFAPI_NX
#define NY REFAPI_NY
#define NXY (NX * NY)
#define DIM 2
#define DE 3
#define MODES 20
#define T__K 300.
#if defined(HIGH_T_Vit1)
#define Tg__K 623.
#elif defined(HIGH_T_PdNiP)
#define Tg__K 587.5
#endif
#define TRIAL_FREQUENCY 1e13
#define E_gl 80.7
#define E_sc 30.0
#define k_E 39.0E-3
#define DeltaE 24.0
#define nu_gl 0.360
#define nu_sc 0.447
#define EV_IN_J 1.60217733e-19
#define J_IN_EV (1 / EV_IN_J)
#define EPSILON 1e-17
#define BOLZ 1.380658e-23
#define kT (T__K * BOLZ * J_IN_EV)
#define LX 0.7
#define LY 0.7
#define LZ 1.0
#define VOXEL0 (LX * LY * LZ)
#define GAMMA0 0.14
#define space_loop for (i = 0; i < lnx; i++) for (j = 0; j < NY; j++)

#ifdef BMG_GLOBALS_ONCE
#define G(decl, init) decl = init
#else
#define G(decl, init) extern decl
#endif
G(real E, 0); G(real nu, 0); G(real mu, 0); G(real lambda, 0); G(real alpha, 0); G(real beta, 0);
G(real Q0amp, 0); G(real XtalQ0amp, 0); G(real XtalShear, 0);
G(real* Work[MODES], {0}); G(real* Q0[MODES], {0}); G(real* Q1[MODES], {0}); G(real* Q[MODES], {0});
G(real* tlast, 0); G(int softening_FLAG, 0);
G(real PermSoft, 0); G(real PermSoftmro, 0); G(real TempSoft, 0); G(real TempSoftmro, 0);
G(real PermSofteningCap, 0);
G(real* PermSoftening, 0); G(real* TempSoftening, 0); G(real* Softening, 0);
G(real xQ0amp, 0); G(real xMROFrac, 0); G(int InitMRO, 0); G(real tTemp, 0); G(real tResi, 0);
G(int* MRO, 0); G(real* MROthe0, 0);
G(real strainrate, 0); G(real strainincrement, 0); G(real totime, 0); G(real dt, 0);
G(real RandomRatio, 0); G(int printperiod, 0); G(real EndStrain, 0); G(real elEnergy, 0);
G(real RelxTime, 0);
G(real* DEps0[MODES][DE], {{0}}); G(real* Eps0[DE], {0}); G(real* Sigma[DE], {0});
G(real* TotEps[DE], {0}); G(char ResStressDataFile[80], {0}); G(real ResiRatio, 0);
G(real Stress[3], {0}); G(real EpsAvg[3], {0}); G(real* EqStrain, 0); G(real* EqStress, 0);
G(real* XR[2], {0}); G(real* Lambda, 0); G(real* Mu, 0); G(int seed, 0);
G(int step, 0); G(int astep, 0); G(int kstep, 0); G(int estep, 0);
G(FILE* fq, 0);
#undef G

void ReadInput(FILE* in);
void Init(void);
void FFT_MPI_Init(void);
void Grad(void);
void Rand_Init(void);
void Energy_Init(void);
void Alloc(void);
void Free(void);
void DStrain(void);
void ParameterPrint(void);
void PrintFlags(void);
void RecordPrep(void);
void RecordFree(void);
void WriteScalarMPI(real* field, char* s, int step);
void WriteScalarMPI_INT(int* field, char* s, int step);
void WriteMROMPI_INT(int* field, char* s, int step);
void DispField(real* XR[2]);
void ActEnergy(int step);
void SofteningFactor(void);
void ElasticEnergy(void);
void UpdateSOC(void);
void KMC(void);
void athermal_plasticity(void);
void HomStressSolver(void);
void HomogeneousStressSolver(real lambda, real mu, real** eps0o, real* epsavg, real** uo, real** epso,
                             real** sigmao, real* stress, int uflag);
void InhomogeneousStressSolver(real* Lambdao, real* Muo, real** eps0o, real* epsavg, real lambda, real mu,
                               real** uo, real** epso, real** sigmao, real* stress, int uflag);
#endif
