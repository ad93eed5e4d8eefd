// Counter-based Gaussian thermal noise, generated inside the LLG kernels.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11) keyed by the 64-bit seed, counter (spin, replica,
// step low, step high), followed by Box-Muller.  The logarithm and sin/cos are
// short series evaluated with correctly rounded single-precision operations
// (__fmaf_rn etc.), so the normals are the same floats on every device and
// in the CPU restatement used to check the kernels:
//   ln u    = e ln2 + 2 atanh((m-1)/(m+1)), u = m 2^e, m in (sqrt(1/2), sqrt 2],
//             atanh series to the f^9 term (error < 4e-10 relative)
//   sin, cos of 2 pi k / 2^24: quadrant from the top two bits, remainder
//             r in [-1/2, 1/2) and Taylor series of sin(pi r / 2) to r^9,
//             cos(pi r / 2) to r^8 (truncation < 3e-8)
// The reference draws its noise from cuRAND XORWOW
// (src/jams/thermostats/cuda_thermostat_classical.cc:54); the variates differ,
// the distribution is the same N(0, 1).
#pragma once

#include <cstdint>

namespace jams_llg {

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    // one 32 x 32 -> 64-bit multiply per word gives both halves
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
    const uint32_t n0 = hi1 ^ c[1] ^ k0;
    const uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
}

// the same generator with the 10 round keys precomputed (keys[2r], keys[2r+1]
// = round r key words); gives the same words as philox4x32_10
__device__ __forceinline__ void philox4x32_10_keyed(uint32_t c[4], const uint32_t* keys) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ keys[2 * r];
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ keys[2 * r + 1];
    c[1] = (uint32_t)p1;
    c[3] = (uint32_t)p0;
    c[0] = n0;
    c[2] = n2;
  }
}

__device__ __forceinline__ float noise_log(float u) {
  const uint32_t b = __float_as_uint(u);
  int32_t e = (int32_t)(b >> 23) - 127;
  uint32_t mb = (b & 0x007FFFFFu) | 0x3F800000u;
  if (mb > 0x3FB504F3u) {
    mb -= 0x00800000u;
    e += 1;
  }
  const float m = __uint_as_float(mb);
  const float f = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float f2 = __fmul_rn(f, f);
  float p = 0x1.c71c72p-4f;
  p = __fmaf_rn(p, f2, 0x1.24924ap-3f);
  p = __fmaf_rn(p, f2, 0x1.99999ap-3f);
  p = __fmaf_rn(p, f2, 0x1.555556p-2f);
  p = __fmaf_rn(p, f2, 1.0f);
  const float lnm = __fmul_rn(2.0f, __fmul_rn(f, p));
  return __fmaf_rn((float)e, 0x1.62e430p-1f, lnm);
}

__device__ __forceinline__ void noise_sincos(uint32_t k, float* s_out, float* c_out) {
  uint32_t q = k >> 22;
  int32_t j = (int32_t)(k & 0x3FFFFFu);
  if (j >= (1 << 21)) {
    q += 1;
    j -= (1 << 22);
  }
  const float r = __fmul_rn((float)j, 0x1.0p-22f);
  const float r2 = __fmul_rn(r, r);
  float sp = 0x1.507834p-13f;
  sp = __fmaf_rn(sp, r2, -0x1.32d2ccp-8f);
  sp = __fmaf_rn(sp, r2, 0x1.466bc6p-4f);
  sp = __fmaf_rn(sp, r2, -0x1.4abbcep-1f);
  sp = __fmaf_rn(sp, r2, 0x1.921fb6p+0f);
  const float sn = __fmul_rn(sp, r);
  float cp = 0x1.e1f506p-11f;
  cp = __fmaf_rn(cp, r2, -0x1.55d3c8p-6f);
  cp = __fmaf_rn(cp, r2, 0x1.03c1f0p-2f);
  cp = __fmaf_rn(cp, r2, -0x1.3bd3ccp+0f);
  const float cs = __fmaf_rn(cp, r2, 1.0f);
  switch (q & 3u) {
    case 0: *s_out = sn; *c_out = cs; break;
    case 1: *s_out = cs; *c_out = -sn; break;
    case 2: *s_out = -sn; *c_out = -cs; break;
    default: *s_out = -cs; *c_out = sn; break;
  }
}

// three N(0,1) floats for (seed, replica, step, spin)
__device__ __forceinline__ void noise_normals(uint64_t seed, uint32_t replica, uint64_t step,
                                              uint32_t spin, float out[3]) {
  uint32_t c[4] = {spin, replica, (uint32_t)step, (uint32_t)(step >> 32)};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const float u1 = __fmul_rn((float)((c[0] >> 8) + 1u), 0x1.0p-24f);
  const float u2 = __fmul_rn((float)((c[2] >> 8) + 1u), 0x1.0p-24f);
  const float r1 = __fsqrt_rn(__fmul_rn(-2.0f, noise_log(u1)));
  const float r2 = __fsqrt_rn(__fmul_rn(-2.0f, noise_log(u2)));
  float s1, c1, s2, c2;
  noise_sincos(c[1] >> 8, &s1, &c1);
  noise_sincos(c[3] >> 8, &s2, &c2);
  out[0] = __fmul_rn(r1, c1);
  out[1] = __fmul_rn(r1, s1);
  out[2] = __fmul_rn(r2, c2);
}

}  // namespace jams_llg
