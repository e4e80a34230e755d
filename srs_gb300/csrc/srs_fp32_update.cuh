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

}  // namespace srs
