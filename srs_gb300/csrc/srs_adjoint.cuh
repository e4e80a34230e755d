// srs_adjoint.cuh — per-element pieces of the reverse sweep shared by the
// adjoints of the resident and the plain FP32 engines.
#pragma once
#include "srs_engine.h"

namespace srs {

__device__ __forceinline__ void kadd(float& s, float& c, float v) {
  float y = v - c;
  float t = s + y;
  c = (t - s) - y;
  s = t;
}

// One buffer reaction r = kon (B - b) c - koff b of an element: adds its
// Jacobian-transpose terms and its kon/koff gradient terms.
__device__ __forceinline__ void adj_buffer(const Consts32& k, const AdjConsts& ak, int q, float c,
                                           float ub, float lb, float w, float& ob, float& oc,
                                           float& dG, float* g, int gi) {
  const float free = k.bfree[q] - ub;
  const float alpha = k.kon[q] * free;
  const float beta = fmaf(k.kon[q], c, k.koff[q]);
  dG -= alpha;            // dF_Ca/dCa (times B)
  ob = fmaf(beta, w - lb, ob);  // dF_Ca/db * lambda_Ca + dF_b/db * lambda_b
  oc = fmaf(alpha, lb, oc);      // dF_b/dCa * lambda_b
  const float d = lb - w;
  g[gi] = fmaf(d * free, c, g[gi]);                  // dr/dkon = (B - b) c
  g[gi + 1] = fmaf(-d, ak.brest[q] + ub, g[gi + 1]);  // dr/dkoff = -b
}

// 1 / B(c), B the rapid-buffer factor of UpdateFastBuffer
// (cpu/RunSimulation.cpp:15-22).
__device__ __forceinline__ float sl_inv_factor(const Consts32& k, float bsl, float c) {
  if (bsl == 0.0f) return 1.0f;
  const float kc = k.khi + c;
  const float kc2 = kc * kc;
  return __fdividef(kc2, kc2 + bsl);
}

// The reverse-step terms of one element that need no neighbour: the
// diffusion-coefficient gradients (from the transposed-diffusion sums S*),
// the buffer reactions and SERCA (cpu/RunSimulation.cpp:70-118), and the
// JSR refill.  x/xim: state x_{n-1}; me: the element's published slot
// (lambda_Ca / B, lambda_ATP, lambda_CMDN, lambda_dye); li: lambda of the
// immobile buffer.  Returns the adjoint rates o* (before the rapid-buffer
// factor for Ca) and dG, d(Ca rate)/dCa times B.
struct AdjTerms {
  float oc, oa, om, oy, oi, dG, c;
};
__device__ __forceinline__ AdjTerms adj_local(const Consts32& k, const AdjConsts& ak, const float4& x,
                                              float xim, const float4& me, float li, bool jsr,
                                              bool trpn, float Sc, float Sa, float Sm, float Sy,
                                              float* g) {
  // D gradients: sum_j lambda_j (L u)_j = sum_j u_j (L^T lambda)_j
  g[SRS_ADJ_D_CA] = fmaf(x.x, Sc, g[SRS_ADJ_D_CA]);
  g[SRS_ADJ_D_ATP] = fmaf(x.y, Sa, g[SRS_ADJ_D_ATP]);
  g[SRS_ADJ_D_CMDN] = fmaf(x.z, Sm, g[SRS_ADJ_D_CMDN]);
  g[SRS_ADJ_D_DYE] = fmaf(x.w, Sy, g[SRS_ADJ_D_DYE]);
  AdjTerms o;
  o.oc = k.D[0] * Sc;
  o.oa = k.D[1] * Sa;
  o.om = k.D[2] * Sm;
  o.oy = k.D[3] * Sy;
  o.oi = 0.0f;
  const float w = me.x;
  o.dG = 0.0f;
  const float c = (jsr ? k.c0j : k.c0) + x.x;
  o.c = c;
  if (!jsr) {
    adj_buffer(k, ak, 0, c, x.w, me.w, w, o.oy, o.oc, o.dG, g, SRS_ADJ_K_ON_DYE);
    adj_buffer(k, ak, 1, c, x.y, me.y, w, o.oa, o.oc, o.dG, g, SRS_ADJ_K_ON_ATP);
    adj_buffer(k, ak, 2, c, x.z, me.z, w, o.om, o.oc, o.dG, g, SRS_ADJ_K_ON_CMDN);
    if (trpn) {
      adj_buffer(k, ak, 3, c, xim, li, w, o.oi, o.oc, o.dG, g, SRS_ADJ_K_ON_TRPN);
      // SERCA v(Ki), Ki = (c / K_D_i)^2 (cpu/RunSimulation.cpp:83-91)
      float Ki = c * k.inv_kdi;
      Ki = Ki * Ki;
      const float den = fmaf(Ki * Ki, k.sd2, fmaf(Ki, k.sd1, k.sd0));
      const float num = fmaf(Ki * Ki, 3.24873e12f, fmaf(Ki, k.sn1, -k.sn0));
      const float iden = __fdividef(1.0f, den);
      const float v = num * iden;
      const float dnum = fmaf(2.0f * Ki, 3.24873e12f, k.sn1);
      const float dden = fmaf(2.0f * Ki, k.sd2, k.sd1);
      const float dv = (dnum - v * dden) * iden * (2.0f * c * k.inv_kdi * k.inv_kdi);
      o.dG = fmaf(-k.serca_scale, dv, o.dG);
      g[SRS_ADJ_A_P] = fmaf(-w * ak.serca_per_ap, v, g[SRS_ADJ_A_P]);
    }
  } else {
    adj_buffer(k, ak, 4, c, xim, li, w, o.oi, o.oc, o.dG, g, SRS_ADJ_K_ON_CSQN);
    o.dG -= k.refill_v;
  }
  return o;
}

// dG into lambda_Ca's rate, then the rapid SL buffer (cpu/RunSimulation.cpp:
// 15-22): F_Ca = G / B(c), so -G B'(c) / B^2 lambda_Ca = 2 bsl G w / (B kc^3),
// with its B_TOT_SL and K_D_SL gradient terms.  w: lambda_Ca / B.
__device__ __forceinline__ void adj_rapid(const Consts32& k, const AdjConsts& ak, float bsl, float c,
                                          float G, float w, float dG, float& oc, float* g) {
  oc = fmaf(dG, w, oc);
  if (bsl != 0.0f) {
    const float kc = k.khi + c;
    const float ikc = __fdividef(1.0f, kc);
    const float bk2 = bsl * ikc * ikc;           // B - 1
    const float GB = __fdividef(G, 1.0f + bk2);  // G / B
    const float t3 = GB * bk2 * ikc;             // G bsl / (B kc^3)
    oc = fmaf(2.0f * t3, w, oc);
    g[SRS_ADJ_B_TOT_SL] = fmaf(-w * GB, bk2 * ak.inv_btot_sl, g[SRS_ADJ_B_TOT_SL]);
    g[SRS_ADJ_K_D_SL] = fmaf(-w * t3, (c - k.khi) * ak.inv_khi, g[SRS_ADJ_K_D_SL]);
  }
}

}  // namespace srs
