// fft.cuh -- hand-written 2D/3D real-to-complex FFT for the Green's-function
// elastic solve (replaces the FFTW 2 MPI plans of init.c:77-110 and the solve
// of elastic.c:779-828).
#pragma once
#include <cuda_runtime.h>

#include "stz_internal.h"

namespace stz {

// Radix schedule of one transform length (radices 8, 4, 3, 2).
struct Sched {
  int n = 1;
  int nst = 0;
  int r[12] = {0};
};

// What the inverse half of a solve writes.
enum SolveOut {
  kOutSig64 = 0,   // sigma[c][s] (FP64), the plain forms
  kOutSig32 = 1,   // sigma[c][s] (FP32 buffer), mixed form with per-event FFT
  kOutDev32 = 2    // deviatoric coordinates (FP32) + error statistics against the
                   // field they replace, mixed form re-solve
};

struct FFTPlan {
  int n0, n1, n2, h, nh, nc;
  long long N, Nk;
  Sched sh, s1, s0;
  // twiddles exp(-2 pi i k / n): half length h, axis-1 length, axis-0 length,
  // and the real-FFT post twiddle of length n2 (k = 0..h)
  double2 *tw_h = nullptr, *tw_1 = nullptr, *tw_0 = nullptr, *tw_p = nullptr;
  float2 *tw_hf = nullptr, *tw_1f = nullptr, *tw_0f = nullptr, *tw_pf = nullptr;
  float4 *tw_hd = nullptr, *tw_1d = nullptr, *tw_0d = nullptr, *tw_pd = nullptr;  // FP32 pairs (hi, lo) x 2
  // tiles (lines per block) of each pass
  int L_x = 0, L_y = 0, L_g = 0;
  size_t smem_x = 0, smem_y = 0, smem_g = 0, smem_c2r = 0;
};

int fft_plan_create(FFTPlan* p, int n0, int n1, int n2, int nc);
// Chooses the tiles (lines per block of each pass) and the radix order of the
// plan by timing solves of a fixed eigenstrain in FP64 (pair = 0) or in FP32
// pairs (pair = 1), once per device, grid shape and precision per process
// (cached); a candidate is admitted only if its result equals the default
// schedule's within 1e-10. chosen (optional, 4 ints): the tiles L_x, L_y, L_g
// and the number of candidates rejected.
int fft_autotune(FFTPlan* p, cudaStream_t st, int* chosen, int pair);
// A plan whose twiddle tables are written into caller-provided device storage
// of at least fft_twiddle_count() elements (FP64 transforms only).
size_t fft_twiddle_count(int n0, int n1, int n2);
int fft_plan_init_in(FFTPlan* p, int n0, int n1, int n2, int nc, double2* storage, size_t cap, cudaStream_t st);
// number of blocks of the C2R pass (the length of one component's msum row)
int fft_c2r_blocks(const FFTPlan& p);
void fft_plan_destroy(FFTPlan* p);

struct SolveArgs {
  const double* eps;     // [nc][N] eigenstrain (FP64)
  const double* ebar;    // device: mean strain for the k = 0 term (nc doubles), or null = 0
  const double* uadd;    // device: uniform stress added after the solve (nc), or null
  double lambda, mu;
  const int* gate;       // device: skip everything when *gate == 0 (null = always run)
  int out;               // SolveOut
  double* sig64;         // kOutSig64
  float* sig32;          // kOutSig32
  float* sdev;           // kOutDev32 (read for the error, then overwritten)
  double* err;           // kOutDev32: err[0] = max |d s|^2, err[1] = sum |d s|^2,
                         // err[2] = sum |s|^2, err[3] = max |s|^2 (s: the FP64 result)
  double* msum;          // kOutSig64, optional: per-(component, block) sums of the
                         // solved field, [nc][fft_c2r_blocks] (for the mean stress)
  int fp32;              // run the transform in FP32 (eps converted on load)
  int pair;              // run the transform in FP32 pairs (about 48 bits; eps split on load)
  int disp;              // kOutSig64 only: write the displacement field ([dim][N], dim = 2 in 2D,
                         // 3 in 3D; zero mean) instead of the stress
  void* spec;            // [nc][Nk] complex scratch (double2, or float2 when fp32)
  int ortho_mean;        // 1: the k = 0 term is C:(N ebar - eps_hat(0)) (always 1 here)
};

// Full Green's-function solve: sigma = C:(eps - eps*) with <eps> = ebar.
int fft_solve(const FFTPlan& p, const SolveArgs& a, cudaStream_t st, int64_t* launches);

// Forward R2C of one real field (for the barrier-field generator), the
// spectrum filter exp(-k^2 l^2 / 4) with the mean removed, and the inverse.
int fft_filter_gaussian(const FFTPlan& p, double* field, double corr_len, void* spec, cudaStream_t st);

}  // namespace stz
