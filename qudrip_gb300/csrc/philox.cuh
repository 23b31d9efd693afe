// philox.cuh -- Philox4x32-10 counter-based generator (J. K. Salmon, M. A.
// Moraes, R. O. Dror and D. E. Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC11), identical on host and device so a CPU restatement can
// replay every trajectory's random decisions.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#endif
#endif

namespace qd {

__host__ __device__ inline void philox_mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

// 10 rounds on counter c with key k; returns 4 words in c.
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(M0, c[0], hi0, lo0);
    philox_mulhilo(M1, c[2], hi1, lo1);
    const uint32_t n0 = hi1 ^ c[1] ^ k0;
    const uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += W0;
    k1 += W1;
  }
}

// Two uniform doubles in [0, 1) (53 random bits each) for (seed, stream, step).
__host__ __device__ inline void philox_uniform2(uint64_t seed, uint32_t stream, uint32_t step, double& u1,
                                                double& u2) {
  uint32_t c[4] = {step, stream, 0u, 0u};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  u1 = ((double)(c[0] >> 5) * 67108864.0 + (double)(c[1] >> 6)) * (1.0 / 9007199254740992.0);
  u2 = ((double)(c[2] >> 5) * 67108864.0 + (double)(c[3] >> 6)) * (1.0 / 9007199254740992.0);
}

}  // namespace qd
