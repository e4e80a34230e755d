// srs_math.h — arithmetic shared by the sm_103a kernels and the C++ host:
// counter-based Philox4x32-10 random numbers, project-written log/exp, and
// the stochastic RyR / LCC gating update.
//
// Everything here is written so that the device (nvcc, sm_103a) and a C/C++
// host compiler produce bit-identical results for identical inputs:
//   * every floating-point operation that could be contracted is spelled out
//     with an explicit rounding intrinsic (SRS_FMAF, SRS_FMULF, ...);
//   * no CUDA math-library function is called on this path; log and exp are
//     implemented here from textbook methods (see srs_logf / srs_exp2f).
// This is what makes gating decisions reproducible on the CPU given the same
// local Ca2+ (the reference draws from glibc rand(): cpu/RunSimulation.cpp:208,
// 382-386; its GPU build from per-channel curand XORWOW: gpu/InitFuncs.cu:1722).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define SRS_HD __host__ __device__ __forceinline__
#else
#define SRS_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define SRS_FMAF(a, b, c) __fmaf_rn((a), (b), (c))
#define SRS_FMULF(a, b) __fmul_rn((a), (b))
#define SRS_FADDF(a, b) __fadd_rn((a), (b))
#define SRS_FSUBF(a, b) __fsub_rn((a), (b))
#define SRS_FDIVF(a, b) __fdiv_rn((a), (b))
#define SRS_FMA(a, b, c) __fma_rn((a), (b), (c))
#define SRS_DMUL(a, b) __dmul_rn((a), (b))
#define SRS_DADD(a, b) __dadd_rn((a), (b))
#define SRS_DSUB(a, b) __dsub_rn((a), (b))
#define SRS_DDIV(a, b) __ddiv_rn((a), (b))
#define SRS_F2I_RN(x) __float2int_rn(x)
#define SRS_MULHI(a, b) __umulhi((a), (b))
#else
#include <math.h>
#define SRS_FMAF(a, b, c) fmaf((a), (b), (c))
#define SRS_FMULF(a, b) ((float)((a) * (b)))
#define SRS_FADDF(a, b) ((float)((a) + (b)))
#define SRS_FSUBF(a, b) ((float)((a) - (b)))
#define SRS_FDIVF(a, b) ((float)((a) / (b)))
#define SRS_FMA(a, b, c) fma((a), (b), (c))
#define SRS_DMUL(a, b) ((double)((a) * (b)))
#define SRS_DADD(a, b) ((double)((a) + (b)))
#define SRS_DSUB(a, b) ((double)((a) - (b)))
#define SRS_DDIV(a, b) ((double)((a) / (b)))
#define SRS_F2I_RN(x) ((int)rintf(x))
#define SRS_MULHI(a, b) ((uint32_t)(((uint64_t)(a) * (uint64_t)(b)) >> 32))
#endif

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Counter = (step_lo, step_hi, channel, stream),
// key = (seed_lo, seed_hi).  Stateless: the realization, channel and step
// index select the draw, so no per-channel RNG state is stored or initialised.
// ---------------------------------------------------------------------------
struct srs_u32x4 {
  uint32_t x, y, z, w;
};

SRS_HD srs_u32x4 srs_philox4x32_10(srs_u32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = SRS_MULHI(M0, c.x), lo0 = M0 * c.x;
    uint32_t hi1 = SRS_MULHI(M1, c.z), lo1 = M1 * c.z;
    srs_u32x4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// 52-bit uniform in the open interval (0, 1) from two 32-bit words.
SRS_HD double srs_u01_open(uint32_t hi, uint32_t lo) {
  uint64_t k = ((uint64_t)hi << 20) | (uint64_t)(lo >> 12);
  // k < 2^52, so k + 0.5 and the scaling by 2^-52 are exact in double.
  return ((double)k + 0.5) * 2.220446049250313080847263336181640625e-16;
}

// Two uniforms for (seed, channel, step, stream): stream 0 = residual redraw,
// stream 1 = (unused) reserve, stream 2 = initial residuals / protocol draws.
struct srs_u01x2 {
  double u0, u1;
};
SRS_HD srs_u01x2 srs_uniform2(uint64_t seed, uint32_t channel, uint64_t step,
                              uint32_t stream) {
  srs_u32x4 c;
  c.x = (uint32_t)step;
  c.y = (uint32_t)(step >> 32);
  c.z = channel;
  c.w = stream;
  srs_u32x4 o = srs_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  srs_u01x2 u;
  u.u0 = srs_u01_open(o.x, o.y);
  u.u1 = srs_u01_open(o.z, o.w);
  return u;
}

// ---------------------------------------------------------------------------
// Bit-reproducible logarithms / exponentials.
//   log: x = m * 2^e with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s),
//        s = (m-1)/(m+1), odd power series of atanh (|s| <= 0.1716).
//   exp2: y = k + f, k = rint(y), |f| <= 1/2; 2^f = e^(f ln2) by its Taylor
//        polynomial (Horner form), then scaled by 2^k through the exponent.
// Only +, *, fma and correctly rounded division are used, each with an
// explicit rounding mode, so host and device agree to the bit.
// ---------------------------------------------------------------------------
SRS_HD float srs_bits2f(uint32_t b) {
  union {
    uint32_t u;
    float f;
  } v;
  v.u = b;
  return v.f;
}
SRS_HD uint32_t srs_f2bits(float f) {
  union {
    uint32_t u;
    float f;
  } v;
  v.f = f;
  return v.u;
}
SRS_HD double srs_bits2d(uint64_t b) {
  union {
    uint64_t u;
    double f;
  } v;
  v.u = b;
  return v.f;
}
SRS_HD uint64_t srs_d2bits(double f) {
  union {
    uint64_t u;
    double f;
  } v;
  v.f = f;
  return v.u;
}

// Natural log for positive normal floats (rate arguments are concentrations
// in [1e-6, 1e5] uM; non-positive input returns -1e30f, never NaN).
SRS_HD float srs_logf(float x) {
  if (!(x > 1.17549435e-38f)) return -1e30f;
  uint32_t b = srs_f2bits(x);
  int e = (int)((b >> 23) & 0xff) - 127;
  float m = srs_bits2f((b & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > 1.41421356f) {
    m = SRS_FMULF(m, 0.5f);
    e += 1;
  }
  float s = SRS_FDIVF(SRS_FSUBF(m, 1.0f), SRS_FADDF(m, 1.0f));
  float s2 = SRS_FMULF(s, s);
  // 2*atanh(s) = 2 s (1 + s^2/3 + s^4/5 + s^6/7 + s^8/9 + s^10/11)
  float p = 0.0909090909f;
  p = SRS_FMAF(p, s2, 0.111111111f);
  p = SRS_FMAF(p, s2, 0.142857143f);
  p = SRS_FMAF(p, s2, 0.2f);
  p = SRS_FMAF(p, s2, 0.333333333f);
  p = SRS_FMAF(p, s2, 1.0f);
  float lnm = SRS_FMULF(SRS_FMULF(2.0f, s), p);
  // e * ln2 split in two parts (Cody & Waite) so the sum stays accurate.
  float fe = (float)e;
  return SRS_FMAF(fe, 0.693145752f, SRS_FMAF(fe, 1.42860677e-06f, lnm));
}

// 2^y for y in [-126, 127]; saturates outside.
SRS_HD float srs_exp2f(float y) {
  if (y > 127.0f) y = 127.0f;
  if (y < -126.0f) y = -126.0f;
  int k = SRS_F2I_RN(y);
  float f = SRS_FSUBF(y, (float)k);  // exact: |f| <= 1/2
  float t = SRS_FMULF(f, 0.693147181f);
  // e^t, |t| <= 0.3466: Taylor terms through t^8 (truncation < 1e-9).
  float p = 2.48015873e-05f;          // 1/8!
  p = SRS_FMAF(p, t, 1.98412698e-04f);  // 1/7!
  p = SRS_FMAF(p, t, 1.38888889e-03f);  // 1/6!
  p = SRS_FMAF(p, t, 8.33333333e-03f);  // 1/5!
  p = SRS_FMAF(p, t, 4.16666667e-02f);  // 1/4!
  p = SRS_FMAF(p, t, 1.66666667e-01f);  // 1/3!
  p = SRS_FMAF(p, t, 0.5f);
  p = SRS_FMAF(p, t, 1.0f);
  p = SRS_FMAF(p, t, 1.0f);
  return SRS_FMULF(p, srs_bits2f((uint32_t)(k + 127) << 23));
}

// x^a for x > 0 (a any real): 2^(a * log2 x).
SRS_HD float srs_powf(float x, float a) {
  float l2 = SRS_FMULF(srs_logf(x), 1.44269504f);
  return srs_exp2f(SRS_FMULF(a, l2));
}

// Natural log in double precision for u in (0, 1]: used once per channel
// firing to redraw the residual R = log(U) (cpu/RunSimulation.cpp:208-209).
SRS_HD double srs_log(double x) {
  if (!(x > 2.2250738585072014e-308)) return -1e300;
  uint64_t b = srs_d2bits(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  double m = srs_bits2d((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  if (m > 1.4142135623730951) {
    m = SRS_DMUL(m, 0.5);
    e += 1;
  }
  double s = SRS_DDIV(SRS_DSUB(m, 1.0), SRS_DADD(m, 1.0));
  double s2 = SRS_DMUL(s, s);
  // odd atanh series through s^23 (|s| <= 0.1716: truncation < 1e-19).
  double p = 1.0 / 23.0;
  p = SRS_FMA(p, s2, 1.0 / 21.0);
  p = SRS_FMA(p, s2, 1.0 / 19.0);
  p = SRS_FMA(p, s2, 1.0 / 17.0);
  p = SRS_FMA(p, s2, 1.0 / 15.0);
  p = SRS_FMA(p, s2, 1.0 / 13.0);
  p = SRS_FMA(p, s2, 1.0 / 11.0);
  p = SRS_FMA(p, s2, 1.0 / 9.0);
  p = SRS_FMA(p, s2, 1.0 / 7.0);
  p = SRS_FMA(p, s2, 1.0 / 5.0);
  p = SRS_FMA(p, s2, 1.0 / 3.0);
  p = SRS_FMA(p, s2, 1.0);
  double lnm = SRS_DMUL(SRS_DMUL(2.0, s), p);
  double de = (double)e;
  // ln2 = 0.6931471803691238 + 1.9082149292705877e-10 (Cody-Waite split)
  return SRS_FMA(de, 0.6931471803691238, SRS_FMA(de, 1.9082149292705877e-10, lnm));
}

// ---------------------------------------------------------------------------
// Channel gating.  Constants that depend only on parameters or on the
// membrane potential are prepared once on the host in double precision and
// passed in as floats; everything evaluated per step is below.
// ---------------------------------------------------------------------------
struct srs_gate_consts {
  // RyR (cpu/RunSimulation.cpp:166-227)
  float ryr_kplus;    // RYR_K_PLUS
  float ryr_kminus;   // RYR_K_MINUS (times X, X == 1 when RYR_A_STAR == 0)
  float ryr_eta;      // RYR_ETA
  float ryr_phi0;     // 1 - (1000/RYR_PHI_KD)^RYR_PHI_N
  float ryr_inv_kphi; // 1 / RYR_PHI_KD
  float ryr_phin;     // RYR_PHI_N
  float ryr_astar_half;  // 0.5 * RYR_A_STAR
  float ryr_eps_cc, ryr_eps_oo;
  // LCC (cpu/RunSimulation.cpp:229-400), for the potential in force
  float alpha, beta, gamma_cf;  // alpha(V), beta(V), gammacf
  float lccv_rate_inact_to_act; // yCa_inf / tau_yCa      (state 1 -> 2)
  float lccv_rate_act_to_inact; // (1 - yCa_inf) / tau_yCa (state 2 -> 1)
  double dt;
};

// RyR update given the cleft Ca (ca_ss), JSR Ca and lattice neighbour counts.
// Returns the new open flag; updates the residual *R in place.
// Draw: stream 0 of (seed, channel, step).
SRS_HD int srs_gate_ryr(const srs_gate_consts* g, int open, float ca_ss,
                        float ca_jsr, int n_open_nb, int n_closed_nb, double* R,
                        uint64_t seed, uint32_t channel, uint64_t step) {
  float rate;
  if (open) {
    float X = 1.0f;
    if (g->ryr_astar_half != 0.0f) {
      float arg = SRS_FMULF(g->ryr_astar_half,
                            SRS_FSUBF(SRS_FMULF((float)n_open_nb, g->ryr_eps_oo),
                                      SRS_FMULF((float)n_closed_nb, g->ryr_eps_cc)));
      X = srs_exp2f(SRS_FMULF(arg, 1.44269504f));
    }
    rate = SRS_FMULF(X, g->ryr_kminus);
  } else {
    float phi = SRS_FADDF(g->ryr_phi0,
                          srs_powf(SRS_FMULF(ca_jsr, g->ryr_inv_kphi), g->ryr_phin));
    float X = 1.0f;
    if (g->ryr_astar_half != 0.0f) {
      float arg = SRS_FMULF(g->ryr_astar_half,
                            SRS_FSUBF(SRS_FMULF((float)n_closed_nb, g->ryr_eps_cc),
                                      SRS_FMULF((float)n_open_nb, g->ryr_eps_oo)));
      X = srs_exp2f(SRS_FMULF(arg, 1.44269504f));
    }
    float cpow = srs_powf(ca_ss, g->ryr_eta);
    rate = SRS_FMULF(SRS_FMULF(SRS_FMULF(X, phi), g->ryr_kplus), cpow);
  }
  double r = SRS_DADD(*R, SRS_DMUL((double)rate, g->dt));
  if (r > 0.0) {
    srs_u01x2 u = srs_uniform2(seed, channel, step, 0u);
    r = srs_log(u.u0);
    open = !open;
  }
  *R = r;
  return open;
}

// LCC transition table (cpu/RunSimulation.cpp:279-364): for each of the 12
// Markov states, up to three (target, rate-kind) pairs.  Rate kinds:
//  0 none, 1 k*alpha, 2 k*beta, 3 aL^k * gamma, 4 fL, 5 gL, 6 omega/bL^k,
//  7 k*alpha', 8 k*beta', 9 fL', 10 gL'.  The multiplier k is stored beside.
SRS_HD void srs_lcc_rates(const srs_gate_consts* g, int state, float ca_ss,
                          float rates[3], int targets[3]) {
  const float fL = 0.85f, gL = 2.0f, fLp = 0.005f, gLp = 7.0f;
  const float bL = 1.9356f, aL = 2.0f;
  const float omega = 0.83f * 2.0f * 1.3f * 0.01f;
  float alpha = g->alpha, beta = g->beta;
  float alpha_p = SRS_FMULF(aL, alpha);
  float beta_p = SRS_FDIVF(beta, bL);
  float gam = SRS_FMULF(g->gamma_cf, ca_ss);
  float bL2 = bL * bL, bL3 = bL2 * bL, bL4 = bL3 * bL;
  float aL2 = aL * aL, aL3 = aL2 * aL, aL4 = aL3 * aL;
  rates[0] = rates[1] = rates[2] = 0.0f;
  targets[0] = targets[1] = targets[2] = 0;
  switch (state) {
    case 1: rates[0] = SRS_FMULF(4.0f, alpha); rates[1] = gam; targets[0] = 2; targets[1] = 7; break;
    case 2: rates[0] = beta; rates[1] = SRS_FMULF(3.0f, alpha); rates[2] = SRS_FMULF(aL, gam);
            targets[0] = 1; targets[1] = 3; targets[2] = 8; break;
    case 3: rates[0] = SRS_FMULF(2.0f, beta); rates[1] = SRS_FMULF(2.0f, alpha); rates[2] = SRS_FMULF(aL2, gam);
            targets[0] = 2; targets[1] = 4; targets[2] = 9; break;
    case 4: rates[0] = SRS_FMULF(3.0f, beta); rates[1] = alpha; rates[2] = SRS_FMULF(aL3, gam);
            targets[0] = 3; targets[1] = 5; targets[2] = 10; break;
    case 5: rates[0] = SRS_FMULF(4.0f, beta); rates[1] = fL; rates[2] = SRS_FMULF(aL4, gam);
            targets[0] = 4; targets[1] = 6; targets[2] = 11; break;
    case 6: rates[0] = gL; targets[0] = 5; break;
    case 7: rates[0] = omega; rates[1] = SRS_FMULF(4.0f, alpha_p); targets[0] = 1; targets[1] = 8; break;
    case 8: rates[0] = beta_p; rates[1] = SRS_FDIVF(omega, bL); rates[2] = SRS_FMULF(3.0f, alpha_p);
            targets[0] = 7; targets[1] = 2; targets[2] = 9; break;
    case 9: rates[0] = SRS_FMULF(2.0f, beta_p); rates[1] = SRS_FDIVF(omega, bL2); rates[2] = SRS_FMULF(2.0f, alpha_p);
            targets[0] = 8; targets[1] = 3; targets[2] = 10; break;
    case 10: rates[0] = SRS_FMULF(3.0f, beta_p); rates[1] = SRS_FDIVF(omega, bL3); rates[2] = alpha_p;
             targets[0] = 9; targets[1] = 4; targets[2] = 11; break;
    case 11: rates[0] = SRS_FMULF(4.0f, beta_p); rates[1] = SRS_FDIVF(omega, bL4); rates[2] = fLp;
             targets[0] = 10; targets[1] = 5; targets[2] = 12; break;
    case 12: rates[0] = gLp; targets[0] = 11; break;
    default: break;
  }
}

// LCC update: 12-state Markov chain plus 2-state voltage gate sharing one
// residual (cpu/RunSimulation.cpp:366-398).  *state and *vstate updated in
// place.  Draw: stream 0 of (seed, channel, step); u0 -> new residual,
// u1 -> which transition.
SRS_HD void srs_gate_lcc(const srs_gate_consts* g, int* state, int* vstate,
                         float ca_ss, double* R, uint64_t seed, uint32_t channel,
                         uint64_t step) {
  float tr[3];
  int tg[3];
  srs_lcc_rates(g, *state, ca_ss, tr, tg);
  float vr = (*vstate == 1) ? g->lccv_rate_inact_to_act : g->lccv_rate_act_to_inact;
  float tot = SRS_FADDF(SRS_FADDF(SRS_FADDF(tr[0], tr[1]), tr[2]), vr);
  double r = SRS_DADD(*R, SRS_DMUL((double)tot, g->dt));
  if (r > 0.0) {
    srs_u01x2 u = srs_uniform2(seed, channel, step, 0u);
    r = srs_log(u.u0);
    float pick = SRS_FMULF((float)u.u1, tot);
    float c0 = tr[0], c1 = SRS_FADDF(tr[0], tr[1]), c2 = SRS_FADDF(c1, tr[2]);
    if (pick < c0) {
      *state = tg[0];
    } else if (pick < c1) {
      *state = tg[1];
    } else if (pick < c2) {
      *state = tg[2];
    } else {
      *vstate = (*vstate == 1) ? 2 : 1;
    }
  }
  *R = r;
}

// Initial residual of channel `channel` for realization `seed`
// (cpu/RunSimulation.cpp:452-456 draws these from rand()).
SRS_HD double srs_initial_residual(uint64_t seed, uint32_t channel) {
  srs_u01x2 u = srs_uniform2(seed, channel, 0xFFFFFFFFFFFFFFFFull, 2u);
  return srs_log(u.u0);
}

// Extra draws per realization (LCC open duration, initial random RyR):
// channel index 0xFFFFFF00 + k, stream 2.
SRS_HD double srs_protocol_uniform(uint64_t seed, uint32_t k) {
  srs_u01x2 u = srs_uniform2(seed, 0xFFFFFF00u + k, 0xFFFFFFFFFFFFFFFFull, 2u);
  return u.u0;
}
