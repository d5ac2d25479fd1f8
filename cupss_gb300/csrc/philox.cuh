// Counter-based Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
// as easy as 1, 2, 3", SC'11) and a Box-Muller normal pair.
//
// Replaces the reference's host-API cuRAND Philox generator + real-space noise FFT
// (src/field_init.cpp:130-137, src/field.cpp:300-316): the noise is drawn directly in
// Fourier space inside the update, so it costs no memory traffic.
#pragma once
#if !defined(__CUDACC_RTC__)
#include <cstdint>
#include <cuda_runtime.h>
#endif

namespace cupssgb {

#if defined(__CUDACC__)
__device__ __forceinline__ void philox4x32_10(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                                              uint32_t k0, uint32_t k1) {
  constexpr uint32_t kM0 = 0xD2511F53u, kM1 = 0xCD9E8D57u;
  constexpr uint32_t kW0 = 0x9E3779B9u, kW1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    // one widening 32x32 -> 64 multiply gives both halves of each product
    const unsigned long long p0 = (unsigned long long)kM0 * c0;
    const unsigned long long p1 = (unsigned long long)kM1 * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += kW0;
    k1 += kW1;
  }
}

// NB independent Philox4x32-10 blocks c[b] under one key, advanced round by round: the
// rounds form a loop (not unrolled) whose body updates all NB blocks, so the blocks'
// independent multiply chains overlap while the code stays NB rounds long.  Same values
// as philox4x32_10 on each block.
template <int NB>
__device__ __forceinline__ void philox4x32_10_batch(uint32_t (&c)[NB][4], uint32_t k0, uint32_t k1) {
  constexpr uint32_t kM0 = 0xD2511F53u, kM1 = 0xCD9E8D57u;
  constexpr uint32_t kW0 = 0x9E3779B9u, kW1 = 0xBB67AE85u;
#pragma unroll 1
  for (int r = 0; r < 10; ++r) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const unsigned long long p0 = (unsigned long long)kM0 * c[b][0];
      const unsigned long long p1 = (unsigned long long)kM1 * c[b][2];
      const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
      const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
      const uint32_t n0 = hi1 ^ c[b][1] ^ k0, n2 = hi0 ^ c[b][3] ^ k1;
      c[b][0] = n0;
      c[b][1] = lo1;
      c[b][2] = n2;
      c[b][3] = lo0;
    }
    k0 += kW0;
    k1 += kW1;
  }
}

// Box-Muller: two standard normals from two 32-bit words.
//   u1 = ((a >> 8) + 1) 2^-24 in (0, 1],  u2 = (b >> 8) 2^-24 in [0, 1)
//   r = sqrt(-2 ln u1),  theta = 2 pi (u2 - 1/2) in [-pi, pi)
// ln and sin/cos use the hardware approximations (absolute error near 2^-21 on the
// arguments here); the clamp keeps -2 ln u1 >= 0 where u1 rounds to 1.
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& g1, float& g2) {
  const float u1 = (float)((a >> 8) + 1u) * 5.9604644775390625e-08f;
  const float u2 = (float)(b >> 8) * 5.9604644775390625e-08f;
  const float r = sqrtf(fmaxf(-2.0f * __logf(u1), 0.0f));
  float sn, cs;
  __sincosf(6.2831853071795864769f * (u2 - 0.5f), &sn, &cs);
  g1 = r * cs;
  g2 = r * sn;
}

// Four standard normals from counter (ctr, step, fid, 0) under key (k0, k1):
// (g1, g2) from words 0, 1 and (g3, g4) from words 2, 3.
__device__ __forceinline__ void philox_normal4(uint32_t ctr, uint32_t step, uint32_t fid, uint32_t k0,
                                               uint32_t k1, float& g1, float& g2, float& g3, float& g4) {
  uint32_t c0 = ctr, c1 = step, c2 = fid, c3 = 0u;
  philox4x32_10(c0, c1, c2, c3, k0, k1);
  box_muller(c0, c1, g1, g2);
  box_muller(c2, c3, g3, g4);
}

// Two standard normals from words 0, 1 of counter (ctr, step, fid, 0).
__device__ __forceinline__ void philox_normal2(uint32_t ctr, uint32_t step, uint32_t fid, uint32_t k0,
                                               uint32_t k1, float& g1, float& g2) {
  uint32_t c0 = ctr, c1 = step, c2 = fid, c3 = 0u;
  philox4x32_10(c0, c1, c2, c3, k0, k1);
  box_muller(c0, c1, g1, g2);
}
#endif

}  // namespace cupssgb
