// noalloc.cu -- the Green's-function stress solve without any device
// allocation, for callers that cannot call cudaMalloc.
//
// Some callers run where allocating device memory is not allowed or not
// possible: code that executes inside another framework's memory budget or
// pool, or in a process whose allocator is owned by someone else. They still
// own their input and output buffers. This entry point performs
// the same solve as stz_solve (the reference's HomogeneousStressSolver with
// uflag 0) on buffers the caller passes, and keeps its scratch -- the half
// spectrum, the twiddle tables and the mean strain -- in one file-scope
// device array of fixed size. Every GPU that loads this library holds that
// array (about 13 MB) until the process exits. Each call uploads its twiddle
// tables and the mean strain from host memory and synchronises the stream
// before it returns.
#include <cstdio>
#include <cstring>

#include "fft.cuh"
#include "stz_internal.h"

namespace {

// Largest half spectrum the array holds: six components of a 64^3 grid
// (nc * n0 * n1 * (n2/2 + 1) complex values); 2D grids up to 512^2 fit too.
constexpr size_t kNoAllocSpec = (size_t)6 * 64 * 64 * 33;
// Twiddle tables and the mean strain behind the spectrum.
constexpr size_t kNoAllocExtra = 8192;

static __device__ __align__(256) double2 g_noalloc_scratch[kNoAllocSpec + kNoAllocExtra];

// Device address of the array, looked up once per device (host code may not
// use the symbol itself as a device address).
constexpr int kMaxDevices = 64;
double2* g_scratch_addr[kMaxDevices] = {nullptr};

int scratch_for_current_device(double2** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    stz::set_error("stz_solve_noalloc: no usable current device");
    return STZ_ERR_CUDA;
  }
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      stz::set_error("stz_solve_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return STZ_ERR_CUDA;
    }
    g_scratch_addr[dev] = reinterpret_cast<double2*>(p);
  }
  *out = g_scratch_addr[dev];
  return STZ_OK;
}

}  // namespace

extern "C" int stz_solve_noalloc(int32_t dim, int32_t n0, int32_t n1, int32_t n2, double lambda, double mu,
                                 const double* eps0_dev, const double* eps_avg, double* sigma_dev, void* stream) {
  if ((dim != 2 && dim != 3) || !eps0_dev || !sigma_dev || !eps_avg || !(mu > 0)) {
    stz::set_error("stz_solve_noalloc: invalid arguments");
    return STZ_ERR_INVALID;
  }
  if (dim == 2 && n0 != 1) {
    stz::set_error("stz_solve_noalloc: a 2D grid has n0 == 1");
    return STZ_ERR_INVALID;
  }
  const int nc = dim == 2 ? 3 : 6;
  if (n0 < 1 || n1 < 1 || n2 < 2 || n2 % 2) {
    stz::set_error("stz_solve_noalloc: grid %dx%dx%d not supported", n0, n1, n2);
    return STZ_ERR_INVALID;
  }
  const size_t spec = (size_t)nc * n0 * n1 * (n2 / 2 + 1);
  const size_t tw = stz::fft_twiddle_count(n0, n1, n2);
  if (spec > kNoAllocSpec || tw + 8 > kNoAllocExtra) {
    stz::set_error("stz_solve_noalloc: grid %dx%dx%d needs %zu spectrum values, the fixed scratch holds %zu "
                   "(6 components of 64^3)", n0, n1, n2, spec, kNoAllocSpec);
    return STZ_ERR_INVALID;
  }
  double2* base = nullptr;
  int st = scratch_for_current_device(&base);
  if (st) return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  double2* extra = base + kNoAllocSpec;
  stz::FFTPlan plan;
  if ((st = stz::fft_plan_init_in(&plan, n0, n1, n2, nc, extra, kNoAllocExtra - 8, s))) {
    if (st == STZ_ERR_INVALID)
      stz::set_error("stz_solve_noalloc: grid %dx%dx%d not supported by the FFT", n0, n1, n2);
    else
      stz::set_error("stz_solve_noalloc: twiddle upload failed: %s", cudaGetErrorString(cudaGetLastError()));
    return st;
  }
  // the mean strain goes behind the twiddles (8 values of 16 bytes reserved)
  double* ebar = reinterpret_cast<double*>(extra + (kNoAllocExtra - 8));
  double eb[6] = {0, 0, 0, 0, 0, 0};
  for (int c = 0; c < nc; c++) eb[c] = eps_avg[c];
  if (cudaMemcpyAsync(ebar, eb, sizeof(eb), cudaMemcpyHostToDevice, s) != cudaSuccess) {
    stz::set_error("stz_solve_noalloc: copy of the mean strain failed");
    return STZ_ERR_CUDA;
  }
  stz::SolveArgs a{};
  a.eps = eps0_dev;
  a.ebar = ebar;
  a.lambda = lambda;
  a.mu = mu;
  a.out = stz::kOutSig64;
  a.sig64 = sigma_dev;
  a.spec = base;
  st = stz::fft_solve(plan, a, s, nullptr);
  if (st) return st;
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    stz::set_error("stz_solve_noalloc: %s", cudaGetErrorString(e));
    return STZ_ERR_CUDA;
  }
  return STZ_OK;
}
