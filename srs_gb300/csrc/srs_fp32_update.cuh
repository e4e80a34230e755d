// srs_fp32_update.cuh — the FP32 element update shared by the plain and the
// resident engines (deviation form, compensated Euler; see k_fp32.cu).
#pragma once
#include "srs_engine.h"

namespace srs {

// One element, one step.  o/im: state, cm/ci: compensation (updated in place),
// s1..s4: neighbour states, a: off-diagonal coefficients.
// flags: bit0 JSR, bit1 TropC, bit2 carries channel entries.
__device__ __forceinline__ void tet_update(const Consts32& k, float4 o, float im, float4 s1,
                                           float4 s2, float4 s3, float4 s4, float4 a,
                                           uint32_t fl, float bsl, float kb, float flux,
                                           float4& cm, float& ci, float4* out, float* im_out,
                                           float* g_out = nullptr) {
  float dx = a.x * (s1.x - o.x);
  dx = fmaf(a.y, s2.x - o.x, dx);
  dx = fmaf(a.z, s3.x - o.x, dx);
  dx = fmaf(a.w, s4.x - o.x, dx);
  float dy = a.x * (s1.y - o.y);
  dy = fmaf(a.y, s2.y - o.y, dy);
  dy = fmaf(a.z, s3.y - o.y, dy);
  dy = fmaf(a.w, s4.y - o.y, dy);
  float dz = a.x * (s1.z - o.z);
  dz = fmaf(a.y, s2.z - o.z, dz);
  dz = fmaf(a.z, s3.z - o.z, dz);
  dz = fmaf(a.w, s4.z - o.z, dz);
  float dw = a.x * (s1.w - o.w);
  dw = fmaf(a.y, s2.w - o.w, dw);
  dw = fmaf(a.z, s3.w - o.w, dw);
  dw = fmaf(a.w, s4.w - o.w, dw);
  if (kb != 0.0f) {  // Dirichlet faces hold the resting values
    dx = fmaf(-kb, o.x, dx);
    dy = fmaf(-kb, o.y, dy);
    dz = fmaf(-kb, o.z, dz);
    dw = fmaf(-kb, o.w, dw);
  }
  float rca = k.D[0] * dx, ratp = k.D[1] * dy, rcmdn = k.D[2] * dz, rdye = k.D[3] * dw;
  float rim = 0.0f;
  const float u = o.x;
  float c;
  if (!(fl & 1u)) {
    c = k.c0 + u;
    float rb;
    if (fl & 2u) {
      rb = fmaf(k.kon[3], fmaf(k.bfree[3], u, -im * c), -k.koff[3] * im);
      rca -= rb;
      rim = rb;
      float Ki = c * k.inv_kdi;
      Ki = Ki * Ki;  // K_i = (c / K_D_i)^2 (cpu/RunSimulation.cpp:83-84)
      float Ki2 = Ki * Ki;
      float den = fmaf(Ki2, k.sd2, fmaf(Ki, k.sd1, k.sd0));
      float num = fmaf(Ki2, 3.24873e12f, fmaf(Ki, k.sn1, -k.sn0));
      rca = fmaf(-k.serca_scale, num / den, rca);
    }
    rb = fmaf(k.kon[0], fmaf(k.bfree[0], u, -o.w * c), -k.koff[0] * o.w);
    rca -= rb;
    rdye += rb;
    rb = fmaf(k.kon[1], fmaf(k.bfree[1], u, -o.y * c), -k.koff[1] * o.y);
    rca -= rb;
    ratp += rb;
    rb = fmaf(k.kon[2], fmaf(k.bfree[2], u, -o.z * c), -k.koff[2] * o.z);
    rca -= rb;
    rcmdn += rb;
  } else {
    c = k.c0j + u;
    float rb = fmaf(k.kon[4], fmaf(k.bfree[4], u, -im * c), -k.koff[4] * im);
    rca -= rb;
    rim = rb;
    rca += fmaf(-u, k.refill_v, k.refill0);
  }
  rca += flux;
  if (g_out) *g_out = rca;  // Ca rate before the rapid-buffer factor
  if (bsl != 0.0f) {  // rapid SL buffer (cpu/RunSimulation.cpp:15-22): r / (1 + bsl / kc^2)
    const float kc = k.khi + c;
    const float kc2 = kc * kc;
    rca = (rca * kc2) / (kc2 + bsl);
  }
  // compensated Euler: y = dt*r - comp; t = u + y; comp = (t - u) - y
  float y, t;
  y = fmaf(k.dt, rca, -cm.x);
  t = o.x + y;
  cm.x = (t - o.x) - y;
  out->x = t;
  y = fmaf(k.dt, ratp, -cm.y);
  t = o.y + y;
  cm.y = (t - o.y) - y;
  out->y = t;
  y = fmaf(k.dt, rcmdn, -cm.z);
  t = o.z + y;
  cm.z = (t - o.z) - y;
  out->z = t;
  y = fmaf(k.dt, rdye, -cm.w);
  t = o.w + y;
  cm.w = (t - o.w) - y;
  out->w = t;
  y = fmaf(k.dt, rim, -ci);
  t = im + y;
  ci = (t - im) - y;
  *im_out = t;
}


// Packed pairs of FP32 lanes (the f32x2 instructions of sm_100-family GPUs).
// Every lane rounds exactly as the scalar instruction does, so the packed
// update is bit-identical to the scalar one, with half the instructions.
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
      "sub.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 p_bc(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

// tet_update with the four mobile species as two packed pairs, (Ca, ATP)
// and (CMDN, dye): every lane performs the scalar operations of tet_update
// in the same order, so the two give bit-identical results.  The resident
// engine uses it (fewer issued instructions: 251.4 -> 249.3 ms per bench
// launch); the plain engine keeps the scalar form, which measured faster at
// its 40-register budget (0.442 against 0.492 ms per large-mesh step).
__device__ __forceinline__ void tet_update_x2(const Consts32& k, float4 o, float im, float4 s1,
                                           float4 s2, float4 s3, float4 s4, float4 a,
                                           uint32_t fl, float bsl, float kb, float flux,
                                           float4& cm, float& ci, float4* out, float* im_out,
                                           float* g_out = nullptr) {
  const float2 oxy = lo2(o), ozw = hi2(o);
  // d = a.x (s1 - o) + a.y (s2 - o) + a.z (s3 - o) + a.w (s4 - o), left to right
  float2 dxy = p_mul(p_bc(a.x), p_sub(lo2(s1), oxy));
  float2 dzw = p_mul(p_bc(a.x), p_sub(hi2(s1), ozw));
  dxy = p_fma(p_bc(a.y), p_sub(lo2(s2), oxy), dxy);
  dzw = p_fma(p_bc(a.y), p_sub(hi2(s2), ozw), dzw);
  dxy = p_fma(p_bc(a.z), p_sub(lo2(s3), oxy), dxy);
  dzw = p_fma(p_bc(a.z), p_sub(hi2(s3), ozw), dzw);
  dxy = p_fma(p_bc(a.w), p_sub(lo2(s4), oxy), dxy);
  dzw = p_fma(p_bc(a.w), p_sub(hi2(s4), ozw), dzw);
  if (kb != 0.0f) {  // Dirichlet faces hold the resting values
    const float2 nkb = p_bc(-kb);
    dxy = p_fma(nkb, oxy, dxy);
    dzw = p_fma(nkb, ozw, dzw);
  }
  // rxy = (Ca, ATP) rates, rzw = (CMDN, dye) rates
  float2 rxy = p_mul(make_float2(k.D[0], k.D[1]), dxy);
  float2 rzw = p_mul(make_float2(k.D[2], k.D[3]), dzw);
  float rim = 0.0f;
  const float u = o.x;
  float c;
  if (!(fl & 1u)) {
    c = k.c0 + u;
    float rb;
    if (fl & 2u) {
      rb = fmaf(k.kon[3], fmaf(k.bfree[3], u, -im * c), -k.koff[3] * im);
      rxy.x -= rb;
      rim = rb;
      float Ki = c * k.inv_kdi;
      Ki = Ki * Ki;  // K_i = (c / K_D_i)^2 (cpu/RunSimulation.cpp:83-84)
      float Ki2 = Ki * Ki;
      float den = fmaf(Ki2, k.sd2, fmaf(Ki, k.sd1, k.sd0));
      float num = fmaf(Ki2, 3.24873e12f, fmaf(Ki, k.sn1, -k.sn0));
      rxy.x = fmaf(-k.serca_scale, num / den, rxy.x);
    }
    // bound-buffer rates kon (bfree u - B c) - koff B: CMDN and dye packed
    const float2 rb2 = p_fma(make_float2(k.kon[2], k.kon[0]),
                             p_fma(make_float2(k.bfree[2], k.bfree[0]), p_bc(u), p_mul(ozw, p_bc(-c))),
                             p_mul(make_float2(-k.koff[2], -k.koff[0]), ozw));
    rb = fmaf(k.kon[1], fmaf(k.bfree[1], u, -o.y * c), -k.koff[1] * o.y);
    rxy.x -= rb2.y;  // dye
    rxy.x -= rb;     // ATP
    rxy.y += rb;
    rxy.x -= rb2.x;  // CMDN
    rzw = p_add(rzw, rb2);
  } else {
    c = k.c0j + u;
    float rb = fmaf(k.kon[4], fmaf(k.bfree[4], u, -im * c), -k.koff[4] * im);
    rxy.x -= rb;
    rim = rb;
    rxy.x += fmaf(-u, k.refill_v, k.refill0);
  }
  rxy.x += flux;
  if (g_out) *g_out = rxy.x;  // Ca rate before the rapid-buffer factor
  if (bsl != 0.0f) {  // rapid SL buffer (cpu/RunSimulation.cpp:15-22): r / (1 + bsl / kc^2)
    const float kc = k.khi + c;
    const float kc2 = kc * kc;
    rxy.x = (rxy.x * kc2) / (kc2 + bsl);
  }
  // compensated Euler y = dt r - comp; t = u + y; comp = (t - u) - y, taken
  // in negated form: ny = fma(-dt, r, comp) = -y exactly (round-to-nearest is
  // symmetric), t = u - ny, comp = (t - u) + ny.  Zeros keep their scalar
  // signs because no state value is ever -0.
  const float2 ndt = p_bc(-k.dt);
  float2 ny = p_fma(ndt, rxy, lo2(cm));
  const float2 txy = p_sub(oxy, ny);
  const float2 cxy = p_add(p_sub(txy, oxy), ny);
  ny = p_fma(ndt, rzw, hi2(cm));
  const float2 tzw = p_sub(ozw, ny);
  const float2 czw = p_add(p_sub(tzw, ozw), ny);
  cm = make_float4(cxy.x, cxy.y, czw.x, czw.y);
  *out = make_float4(txy.x, txy.y, tzw.x, tzw.y);
  float y = fmaf(k.dt, rim, -ci);
  float t = im + y;
  ci = (t - im) - y;
  *im_out = t;
}

}  // namespace srs
