// mt19937.cuh -- MT19937 with GSL's conventions, usable on host and device.
//
// Matsumoto & Nishimura (1998). Seeding is GSL's mt_set: the 1812433253
// recurrence with seed 0 replaced by 4357; gsl_rng_uniform = u32 / 2^32;
// gsl_rng_uniform_pos rejects 0; gsl_ran_gaussian is the polar Box-Muller
// method, in the form the reference restates it (init.c:207-223). The
// products in the polar test are rounded separately (no fused multiply-add),
// so the accept/reject decisions and the draws match a host build without
// contraction bit for bit.
#pragma once
#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define STZ_HD __host__ __device__ __forceinline__
#else
#define STZ_HD inline
#endif

namespace stz {

struct MT {
  uint32_t mt[624];
  int32_t mti;
};

STZ_HD void mt_seed(MT* r, unsigned long s) {
  if (s == 0) s = 4357;
  r->mt[0] = (uint32_t)(s & 0xffffffffUL);
  for (int i = 1; i < 624; i++)
    r->mt[i] = (uint32_t)(1812433253UL * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (unsigned long)i);
  r->mti = 624;
}

STZ_HD void mt_twist(MT* r) {
  const uint32_t UP = 0x80000000u, LO = 0x7fffffffu, A = 0x9908b0dfu;
  int k;
  for (k = 0; k < 624 - 397; k++) {
    uint32_t y = (r->mt[k] & UP) | (r->mt[k + 1] & LO);
    r->mt[k] = r->mt[k + 397] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
  }
  for (; k < 623; k++) {
    uint32_t y = (r->mt[k] & UP) | (r->mt[k + 1] & LO);
    r->mt[k] = r->mt[k + 397 - 624] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
  }
  uint32_t y = (r->mt[623] & UP) | (r->mt[0] & LO);
  r->mt[623] = r->mt[396] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
  r->mti = 0;
}

// The output tempering of one state word.
STZ_HD uint32_t mt_temper(uint32_t k) {
  k ^= (k >> 11);
  k ^= (k << 7) & 0x9d2c5680u;
  k ^= (k << 15) & 0xefc60000u;
  k ^= (k >> 18);
  return k;
}

STZ_HD uint32_t mt_next(MT* r) {
  if (r->mti >= 624) mt_twist(r);
  return mt_temper(r->mt[r->mti++]);
}

STZ_HD double mt_uniform(MT* r) { return mt_next(r) / 4294967296.0; }

STZ_HD double mt_uniform_pos(MT* r) {
  double x;
  do { x = mt_uniform(r); } while (x == 0);
  return x;
}

STZ_HD double dmul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
STZ_HD double dadd_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}

STZ_HD double mt_gaussian(MT* r, double sigma) {
  double x, y, r2;
  do {
    x = -1 + 2 * mt_uniform_pos(r);
    y = -1 + 2 * mt_uniform_pos(r);
    r2 = dadd_rn(dmul_rn(x, x), dmul_rn(y, y));
  } while (r2 > 1.0 || r2 == 0);
  return dmul_rn(dmul_rn(sigma, y), sqrt(-2.0 * log(r2) / r2));
}

}  // namespace stz
