// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), usable on host and
// device, and the Box-Muller normal pair built from it. Dynamics noise and the
// synthetic-mesh generators both draw from it, so a draw is a pure function of
// (seed, counter) and identical on CPU and GPU up to libm rounding.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define UMCP_HD __host__ __device__ __forceinline__
#else
#define UMCP_HD inline
#endif

namespace umcp {

struct philox_out { uint32_t v[4]; };

UMCP_HD void philox_mulhilo(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

UMCP_HD philox_out philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
  for (int round = 0; round < 10; ++round) {
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(0xD2511F53u, c0, &hi0, &lo0);
    philox_mulhilo(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  philox_out o;
  o.v[0] = c0; o.v[1] = c1; o.v[2] = c2; o.v[3] = c3;
  return o;
}

// Uniform in the open interval (0,1) with 53 random bits from two words.
UMCP_HD double philox_u53(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return ((double)m + 0.5) * (1.0 / 9007199254740992.0);
}

}  // namespace umcp
