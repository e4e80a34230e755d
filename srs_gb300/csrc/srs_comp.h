// srs_comp.h — compact storage of the Euler compensation terms.
//
// The FP32 engines keep, per element and species, the rounding error c of
// the last compensated Euler update t = u + y (Kahan: c = (t - u) - y), and
// subtract it from the next increment.  |c| <= ulp(t) / 2.  The large-mesh
// form of the plain FP32 engine stores c as an IEEE half of c * 2^24
// (round to nearest even, clamped to the half range), 10 bytes per element
// for the five species instead of 20:
//   q = half(clamp(c * 2^24, +-65504)),   c' = float(q) * 2^-24.
// Concentrations stay below 2^15 uM, so |c * 2^24| <= 2^15 and the clamp only
// matters for a diverged state; c' keeps 11 significant bits of c (the
// accumulator keeps about 35), down to |c| = 2^-38 (c * 2^24 >= 2^-14, the
// half's normal range), i.e. for states above about 6e-5 uM.  Both scalings
// are exact powers of two, and the conversion is IEEE round-to-nearest-even
// (the device's conversion; the CPU oracle restates it with the compiler's
// _Float16), and reading back is exact on host and device alike.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#include <cuda_fp16.h>
#define SRS_COMP_FN __host__ __device__ __forceinline__
#else
#define SRS_COMP_FN inline
#endif

namespace srs {

constexpr float kCompScale = 16777216.0f;          // 2^24
constexpr float kCompInvScale = 1.0f / 16777216.0f;  // 2^-24

// IEEE binary16 to binary32 (exact).
inline float comp_half_to_float_host(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  const int e = (h >> 10) & 0x1F;
  const uint32_t m = h & 0x3FFu;
  float v;
  if (e == 0) {
    v = (float)m * (1.0f / 16777216.0f);  // subnormal: m * 2^-24, exact
  } else {
    uint32_t b = ((uint32_t)(e - 15 + 127) << 23) | (m << 13);
    memcpy(&v, &b, 4);
  }
  uint32_t vb;
  memcpy(&vb, &v, 4);
  vb |= sign;
  memcpy(&v, &vb, 4);
  return v;
}

SRS_COMP_FN float comp_clamp(float v) {
  return fminf(fmaxf(v, -65504.0f), 65504.0f);  // a NaN becomes -65504 on both sides
}

// Host side: the compensation term held in the stored 16 bits.
inline float comp_decode_host(uint16_t q) { return comp_half_to_float_host(q) * kCompInvScale; }

#ifdef __CUDACC__
// Device side, the same values: two species per instruction.
__device__ __forceinline__ __half2 comp_encode2(float a, float b) {
  return __floats2half2_rn(comp_clamp(a * kCompScale), comp_clamp(b * kCompScale));
}
__device__ __forceinline__ float2 comp_decode2(__half2 q) {
  const float2 f = __half22float2(q);
  return make_float2(f.x * kCompInvScale, f.y * kCompInvScale);
}
__device__ __forceinline__ __half comp_encode1(float a) {
  return __float2half_rn(comp_clamp(a * kCompScale));
}
__device__ __forceinline__ float comp_decode1(__half q) { return __half2float(q) * kCompInvScale; }

// the stored layout: ushort4 (x, y, z, w) of the four mobile species, ushort
// of the immobile buffer
__device__ __forceinline__ float4 comp_load4(ushort4 q) {
  const float2 a = comp_decode2(__halves2half2(__ushort_as_half(q.x), __ushort_as_half(q.y)));
  const float2 b = comp_decode2(__halves2half2(__ushort_as_half(q.z), __ushort_as_half(q.w)));
  return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ ushort4 comp_store4(float4 c) {
  const __half2 a = comp_encode2(c.x, c.y), b = comp_encode2(c.z, c.w);
  return make_ushort4(__half_as_ushort(__low2half(a)), __half_as_ushort(__high2half(a)),
                      __half_as_ushort(__low2half(b)), __half_as_ushort(__high2half(b)));
}
__device__ __forceinline__ float comp_load1(unsigned short q) { return comp_decode1(__ushort_as_half(q)); }
__device__ __forceinline__ unsigned short comp_store1(float c) { return __half_as_ushort(comp_encode1(c)); }
#endif

}  // namespace srs
