// k_adjoint_plain.cu — pathwise adjoint of the FP32 plain engine, for meshes
// too large for the resident engine (a cluster's shared memory holds about
// 64k elements; a release site of 1M tets does not fit).
//
// Same recursion as the resident adjoint (k_adjoint.cu): with the gating
// path of the forward run held fixed,
//   lambda_{n-1} = lambda_n + dt J(x_{n-1})^T lambda_n,
//   dL/dtheta   += dt (dF/dtheta)(x_{n-1})^T lambda_n,
// and lambda_n += dL/dx_n at the line-scan ticks.  Here every array lives in
// HBM in the plain engine's layout ([realization][element], engine
// numbering) and one launch runs one reverse step over all realizations:
//   * pub / nxt: the published slots of the step (lambda_Ca / B(x_{n-1}),
//     lambda_ATP, lambda_CMDN, lambda_dye + tick injection), double
//     buffered; lambda_ATP/CMDN/dye have no other owner storage inside a
//     segment;
//   * lam_c, lam_im, lam_c4q, lam_cimq: the owner state (lambda_Ca, the
//     immobile buffer's lambda, their Kahan compensation as halves,
//     srs_comp.h);
//   * lam: the full lambda at the segment boundaries.
// The transposed diffusion operator gathers the four neighbours' slots with
// the transposed coefficients aT; Dirichlet faces (kb) join the diagonal, and
// their sources of the mobile buffers add kon/koff gradient terms.
//
// Parameter gradients: each thread sums its elements' terms of the step in
// FP32, the block reduces them (one realization per block), and the block's
// FP64 accumulator in `part` (one row per block, no atomics) takes the sum;
// the host adds the rows in a fixed order at the end.
#include "srs_adjoint.cuh"
#include "srs_engine.h"

namespace srs {

namespace {

constexpr int NA = SRS_N_ADJ;
constexpr int ADJP_THREADS = 256;

__device__ __forceinline__ float plain_injection(const AdjPlainArgs& a, const double* coef, int e) {
  double inj = 0.0;
  for (int q = a.wt_ptr[e]; q < a.wt_ptr[e + 1]; ++q) inj += coef[a.wt_idx[q]] * a.wt_w[q];
  return (float)inj;
}

}  // namespace

// Start of a segment: publish lambda_{s1} (with the tick injection of step
// s1) from the boundary arrays.  ib: 1 / B(x_{s1-1}) from the trajectory.
__global__ void __launch_bounds__(ADJP_THREADS) k_adjp_publish(AdjPlainArgs a) {
  const int r = blockIdx.x;
  const double* coef = a.coef_cur ? a.coef_cur + (size_t)r * a.n_samples : nullptr;
  for (int j = blockIdx.y * blockDim.x + threadIdx.x; j < a.N; j += gridDim.y * blockDim.x) {
    const size_t o = (size_t)r * a.N + j;
    const float4 L = a.lam[o];
    const float inj = coef ? plain_injection(a, coef, j) : 0.0f;
    a.nxt[o] = make_float4(L.x * a.ib[o], L.y, L.z, L.w + inj);
    a.lam_c[o] = L.x;
  }
}

// One reverse step t of the segment (x_{n-1} -> x_n, n = s0 + t): reads the
// slots of step n (pub), writes those of step n - 1 (nxt), or the boundary
// lambda when t == 1 (a.last).  Four blocks per SM (64 registers, a few
// spilled): the step waits on memory, and 32 warps per SM hide more of it
// than 24 (1.11 against 0.84 ms per step on the config-4 mesh).
__global__ void __launch_bounds__(ADJP_THREADS, 4) k_adjp_step(AdjPlainArgs a) {
  const int r = blockIdx.x;
  const Consts32& k = a.k;
  const AdjConsts& ak = a.ak;
  const size_t ro = (size_t)r * a.N;
  const float4* pub = a.pub + ro;
  const float4* tu = a.tu + ro;
  const int NR = a.NR, NL = a.NL, W = NR + 2 * NL + 1;
  const int32_t* rec = a.rec + (size_t)r * W;
  const double* coef = a.coef_next ? a.coef_next + (size_t)r * a.n_samples : nullptr;
  float g[NA];
#pragma unroll
  for (int p = 0; p < NA; ++p) g[p] = 0.0f;
  for (int j = blockIdx.y * blockDim.x + threadIdx.x; j < a.N; j += gridDim.y * blockDim.x) {
    const size_t o = ro + j;
    const float4 at = a.aT[j];
    const int4 nb = a.nb[j];
    const float2 bs = a.bs[j];
    const float bsl = fabsf(bs.x);
    const bool trpn = (__float_as_uint(bs.x) >> 31) != 0;
    const float sa = fabsf(bs.y);
    const bool jsr = (__float_as_uint(bs.y) >> 31) != 0;
    const float4 x = tu[j];
    const float2 ig = a.tig[o];
    const float4 me = pub[j];
    const float4 n0 = pub[nb.x], n1 = pub[nb.y], n2 = pub[nb.z], n3 = pub[nb.w];
    float lx = a.lam_c[o], li = a.lam_im[o];
    float4 cm = comp_load4_x2(a.lam_c4q + o);
    float ci = comp_load1(a.lam_cimq[o]);
    // transposed diffusion: S = sum_k aT_k lambda(nb_k) - (sum_k a_k + kb) lambda(self)
    float Sc = at.x * n0.x;
    Sc = fmaf(at.y, n1.x, Sc);
    Sc = fmaf(at.z, n2.x, Sc);
    Sc = fmaf(at.w, n3.x, Sc);
    Sc = fmaf(-sa, me.x, Sc);
    float Sa = at.x * n0.y;
    Sa = fmaf(at.y, n1.y, Sa);
    Sa = fmaf(at.z, n2.y, Sa);
    Sa = fmaf(at.w, n3.y, Sa);
    Sa = fmaf(-sa, me.y, Sa);
    float Sm = at.x * n0.z;
    Sm = fmaf(at.y, n1.z, Sm);
    Sm = fmaf(at.z, n2.z, Sm);
    Sm = fmaf(at.w, n3.z, Sm);
    Sm = fmaf(-sa, me.z, Sm);
    float Sy = at.x * n0.w;
    Sy = fmaf(at.y, n1.w, Sy);
    Sy = fmaf(at.z, n2.w, Sy);
    Sy = fmaf(at.w, n3.w, Sy);
    Sy = fmaf(-sa, me.w, Sy);
    const float w = me.x;
    const AdjTerms lt = adj_local(k, ak, x, ig.x, me, li, jsr, trpn, Sc, Sa, Sm, Sy, g);
    float oc = lt.oc, dG = lt.dG;
    const float c = lt.c;
    if (a.kb) {
      // the Dirichlet source of the mobile buffers (their resting bound level)
      const float kbj = a.kb[j];
      if (kbj != 0.0f) {
        g[SRS_ADJ_K_ON_DYE] = fmaf(me.w * kbj, ak.kb_on[0], g[SRS_ADJ_K_ON_DYE]);
        g[SRS_ADJ_K_OFF_DYE] = fmaf(me.w * kbj, ak.kb_off[0], g[SRS_ADJ_K_OFF_DYE]);
        g[SRS_ADJ_K_ON_ATP] = fmaf(me.y * kbj, ak.kb_on[1], g[SRS_ADJ_K_ON_ATP]);
        g[SRS_ADJ_K_OFF_ATP] = fmaf(me.y * kbj, ak.kb_off[1], g[SRS_ADJ_K_OFF_ATP]);
        g[SRS_ADJ_K_ON_CMDN] = fmaf(me.z * kbj, ak.kb_on[2], g[SRS_ADJ_K_ON_CMDN]);
        g[SRS_ADJ_K_OFF_CMDN] = fmaf(me.z * kbj, ak.kb_off[2], g[SRS_ADJ_K_OFF_CMDN]);
      }
    }
    if (a.flags[j] & 4u) {
      // release flux of this element's channels, with the gating of step n
      for (int q = a.ch_ptr[j]; q < a.ch_ptr[j + 1]; ++q) {
        const ChanEntry32 e = a.ch_list[q];
        if (e.kind < 2) {
          if (rec[e.ch]) {
            const int pe = e.kind == 0 ? a.ryr_jsr[e.ch] : a.ryr_cleft[e.ch];
            const float wo = pub[pe].x;
            const float so = e.kind == 0 ? a.ryr_s_js[e.ch] : a.ryr_s_cl[e.ch];
            const float qv = fmaf(w, e.s, wo * so);
            if (e.kind == 0) {
              oc = fmaf(-k.jr_scale, qv, oc);
              const float cj = k.c0j + tu[pe].x;
              g[SRS_ADJ_V_RYR] = fmaf(qv * ak.v_cell, cj - c, g[SRS_ADJ_V_RYR]);
            } else {
              oc = fmaf(k.jr_scale, qv, oc);
            }
          }
        } else if ((rec[NR + e.ch] == 6 || rec[NR + e.ch] == 12) && rec[NR + NL + e.ch] == 2) {
          const int vs = rec[W - 1];
          dG = fmaf(k.lccA[vs] * k.lccE[vs], e.s, dG);
        }
      }
    }
    adj_rapid(k, ak, bsl, c, ig.y, w, dG, oc, g);
    // compensated update of lambda
    float4 L = make_float4(lx, me.y, me.z, me.w);
    kadd(L.x, cm.x, k.dt * oc);
    kadd(L.y, cm.y, k.dt * lt.oa);
    kadd(L.z, cm.z, k.dt * lt.om);
    kadd(L.w, cm.w, k.dt * lt.oy);
    kadd(li, ci, k.dt * lt.oi);
    a.lam_im[o] = li;
    comp_store4_x2(a.lam_c4q + o, cm);
    a.lam_cimq[o] = comp_store1(ci);
    if (!a.last) {
      const float inj = coef ? plain_injection(a, coef, j) : 0.0f;
      a.nxt[o] = make_float4(L.x * a.ib[o], L.y, L.z, L.w + inj);
      a.lam_c[o] = L.x;
    } else {
      a.lam[o] = L;
    }
  }
  // gradient of the step: warp sums, then the block's FP64 row
  __shared__ float red[ADJP_THREADS / 32][NA];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int p = 0; p < NA; ++p) {
    float v = g[p];
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    if (lane == 0) red[warp][p] = v;
  }
  __syncthreads();
  if (threadIdx.x < NA) {
    double v = 0.0;
    for (int q = 0; q < ADJP_THREADS / 32; ++q) v += (double)red[q][threadIdx.x];
    a.part[((size_t)r * gridDim.y + blockIdx.y) * NA + threadIdx.x] += v;
  }
}

// Blocks per realization of the reverse-step launches: enough blocks for
// several waves over the SMs, at most one element per thread.
int adjp_blocks_per_realization(int N, int R, int n_sm) {
  const int by_elem = (N + ADJP_THREADS - 1) / ADJP_THREADS;
  const int want = (8 * n_sm + R - 1) / R;
  return std::max(1, std::min(by_elem, std::min(want, 65535)));
}

int launch_adjp_publish(const AdjPlainArgs& a, int blocks, cudaStream_t st) {
  k_adjp_publish<<<dim3(a.R, blocks), ADJP_THREADS, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_adjp_step(const AdjPlainArgs& a, int blocks, cudaStream_t st) {
  k_adjp_step<<<dim3(a.R, blocks), ADJP_THREADS, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace srs
