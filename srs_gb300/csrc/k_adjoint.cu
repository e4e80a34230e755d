// k_adjoint.cu — pathwise adjoint of the FP32 resident engine.
//
// The forward map is the explicit Euler step of ExplicitStep
// (cpu/RunSimulation.cpp:591-647), x_n = x_{n-1} + dt F(x_{n-1}; theta, g_{n-1}),
// with the channel states g_{n-1} of every step held fixed: gating is not
// differentiable, so the gradient is the one of the recorded path.  The
// adjoint recursion is
//   lambda_{n-1} = lambda_n + dt J(x_{n-1})^T lambda_n,
//   dL/dtheta   += dt (dF/dtheta)(x_{n-1})^T lambda_n,
// with lambda_n += dL/dx_n injected at the line-scan ticks.
//
// One thread-block cluster holds one realization, partitioned exactly like
// the forward resident engine.  Every step each element publishes
// (lambda_Ca / B_SL, lambda_ATP, lambda_CMDN, lambda_dye) into a
// double-buffered shared-memory slot; after one cluster barrier every element
// gathers its four neighbours' slots (through distributed shared memory when
// they sit in another CTA), so the transposed diffusion operator needs the
// transposed coefficients aT only.  The state x_{n-1}, its Ca rate before the
// rapid-buffer factor (G) and the channel states come from the trajectory
// the forward engine recorded for the segment.  Lambda lives in HBM/L2 in
// owner-only arrays with Kahan compensation, like the forward state.
//
// Parameter gradients: every thread sums its elements' terms in FP32 over up
// to 16 steps; then each warp reduces those sums (warp shuffles) and adds
// them to a per-warp FP64 accumulator in shared memory; at the end of a
// realization the warps' sums
// are added in FP64 to the per-realization gradient, which therefore
// accumulates over all steps and segments (the long reverse sweep) in double
// precision.
#include <type_traits>

#include "srs_adjoint.cuh"
#include "srs_cluster.cuh"
#include "srs_engine.h"

namespace srs {

namespace {

constexpr int NA = SRS_N_ADJ;

}  // namespace

// Shared memory: float4 pub[2][P]; double red[32][NA]; int32 cptr[n_ch+1];
// ChanEntry32 clist[] (16-byte aligned); uint32 base[2][16]; uint16
// sched[P] (16-byte aligned end); then, when
// `own_in_smem`, the owner state float4 c4[P], o[P] (lambda_Ca, lambda_imm,
// its compensation, unused);
// then, when `stage`, three trajectory buffers float4 u[3][P], float2
// ig[3][P] and their mbarriers uint64 bar[3].
size_t adjoint_smem_bytes(int P, int n_chtet, int n_entries, bool own_in_smem, bool stage) {
  // P: element slots of one CTA
  size_t b = (size_t)2 * P * sizeof(float4);
  b += (size_t)32 * NA * sizeof(double);
  b += (size_t)(n_chtet + 1) * sizeof(int32_t);
  b = (b + 15) & ~(size_t)15;
  b += (size_t)n_entries * sizeof(ChanEntry32);
  b += 2 * 16 * sizeof(uint32_t);
  b += (size_t)P * sizeof(uint16_t);
  b = (b + 15) & ~(size_t)15;
  if (own_in_smem) b += (size_t)P * 2 * sizeof(float4);
  if (stage) b += (size_t)3 * P * (sizeof(float4) + sizeof(float2)) + 3 * sizeof(uint64_t);
  return b;
}

namespace {

// dL/dF coefficients of the tick at step n of realization r, or null when n
// is not a tick of this segment (evaluated once per step, not per element).
__device__ __forceinline__ const double* tick_coef(const AdjArgs& a, int64_t n, int r) {
  if (a.tick_every <= 0 || n <= a.s0 || (n % a.tick_every) != 0) return nullptr;
  const int64_t slot = n / a.tick_every - a.s0 / a.tick_every - 1;
  return a.coef + ((size_t)slot * a.R + r) * a.n_samples;
}

__device__ __forceinline__ float tick_injection(const AdjArgs& a, const double* coef, int e) {
  if (!coef) return 0.0f;
  double inj = 0.0;
  for (int q = a.wt_ptr[e]; q < a.wt_ptr[e + 1]; ++q) inj += coef[a.wt_idx[q]] * a.wt_w[q];
  return (float)inj;
}


}  // namespace

// Per step t = n_steps .. 1 of the segment (x_{n-1} -> x_n, n = s0 + t), after
// one cluster barrier, every element reads the published slots of its
// neighbours (pub[cur]), forms lambda_{n-1} and publishes it into pub[cur^1]
// for the next step: lambda_ATP/CMDN/dye as they are (pub is their owner
// storage during the segment) and lambda_Ca / B(x_{n-2}), with the tick
// injection of step n-1 already added.  The last step writes lambda_{s0}
// back to the global arrays for the next segment.
template <int C>
__global__ void __launch_bounds__(512, 1) k_adjoint32(AdjArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int P = a.P;           // stride of the forward engine's partitions
  const int msub = a.m_sub;    // forward partitions per CTA
  const int Pc = msub * P;     // this CTA's element slots
  float4* pub0 = reinterpret_cast<float4*>(smem);
  float4* pub1 = pub0 + Pc;
  double* red = reinterpret_cast<double*>(pub1 + Pc);
  int32_t* s_cptr = reinterpret_cast<int32_t*>(red + 32 * NA);
  const int n_ch0 = a.n_chtet[0];
  ChanEntry32* s_clist = reinterpret_cast<ChanEntry32*>(
      (reinterpret_cast<uintptr_t>(s_cptr + n_ch0 + 1) + 15) & ~(uintptr_t)15);
  const int n_ent = a.ch_ptr[n_ch0];
  uint32_t* s_base = reinterpret_cast<uint32_t*>(s_clist + n_ent);  // [2][16]
  uint16_t* sched = reinterpret_cast<uint16_t*>(s_base + 32);         // [Pc]
  // owner state on chip: compensation terms c4, then (lambda_Ca, lambda_imm,
  // compensation of lambda_imm, unused) in one float4 per element
  float4* sm_c4 = reinterpret_cast<float4*>(
      (reinterpret_cast<uintptr_t>(sched + Pc) + 15) & ~(uintptr_t)15);
  float4* sm_o = sm_c4 + Pc;
  // trajectory staging (a.stage): slot k of the segment in buffer k % 3
  float4* st_u = reinterpret_cast<float4*>(a.own_in_smem ? reinterpret_cast<unsigned char*>(sm_o + Pc)
                                                         : reinterpret_cast<unsigned char*>(sm_c4));
  float2* st_ig = reinterpret_cast<float2*>(st_u + 3 * Pc);
  uint64_t* st_bar = reinterpret_cast<uint64_t*>(st_ig + 3 * Pc);

  uint32_t rank = 0;
  if constexpr (C > 1) asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
  const int cid = blockIdx.x / C, ncl = gridDim.x / C;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int n_ch = rank == 0 ? n_ch0 : 0;  // channel elements: forward partition 0
  const size_t NE = (size_t)C * Pc;
  const AdjRec* geo = a.geo + (size_t)rank * Pc;
  const uint32_t mask = (1u << a.off_bits) - 1u;
  const uint32_t ch_mask = (1u << a.ch_off_bits) - 1u;  // channel codes: forward layout
  // element ranges of this CTA: forward partitions rank*msub .. + msub - 1,
  // each [channel | interior | boundary] at offset j*P
  // Ranges are walked as one concatenated sequence: element k of the
  // sequence goes to thread k % nthr, so every thread gets the same count.
  auto for_range = [&](int& idx, int lo, int hi, auto&& f) {
    const int n = hi - lo;
    for (; idx < n; idx += nthr) f(lo + idx);
    idx -= n;
  };
  auto for_all = [&](auto&& f) {
    int idx = tid;
    for (int j = 0; j < msub; ++j) for_range(idx, j * P, j * P + a.n_local[rank * msub + j], f);
  };
  const Consts32& k = a.k;
  const AdjConsts& ak = a.ak;
  const int NR = a.NR, NL = a.NL, W = NR + 2 * NL + 1;

  if (rank == 0) {
    for (int i = tid; i <= n_ch; i += nthr) s_cptr[i] = a.ch_ptr[i];
    for (int i = tid; i < n_ent; i += nthr) s_clist[i] = a.ch_list[i];
  }
  if (a.stage && tid == 0) {
    for (int b = 0; b < 3; ++b) mbar_init(&st_bar[b], 1);
    fence_proxy_async();
  }
  if (tid < C) {
    s_base[tid] = (C > 1) ? map_rank(smem_addr(pub0), tid) : smem_addr(pub0);
    s_base[16 + tid] = (C > 1) ? map_rank(smem_addr(pub1), tid) : smem_addr(pub1);
  }
  // Element schedule of a step: the interior ranges of this CTA's
  // partitions, then (after the cluster wait) the channel range when it is
  // not interior and the boundary ranges.  Position q of the schedule goes
  // to thread q % nthr, so every thread gets the same count.
  int n_pre = 0, n_sched = 0;
  {
    auto put = [&](int lo, int hi) {
      for (int i = tid; i < hi - lo; i += nthr) sched[n_sched + i] = (uint16_t)(lo + i);
      n_sched += hi - lo;
    };
    for (int j = 0; j < msub; ++j) {
      const int q = rank * msub + j, nc = q == 0 ? n_ch0 : 0;
      put(j * P + (a.ch_interior ? 0 : nc), j * P + nc + a.n_int[q]);
    }
    n_pre = n_sched;
    for (int j = 0; j < msub; ++j) {
      const int q = rank * msub + j, nc = q == 0 ? n_ch0 : 0;
      if (!a.ch_interior) put(j * P, j * P + nc);
      put(j * P + nc + a.n_int[q], j * P + a.n_local[q]);
    }
  }
  step_barrier<C>();

  // Staging: thread 0 copies slot k of the trajectory (this CTA's slice) into
  // buffer k % 3 with two bulk copies completing on that buffer's mbarrier;
  // every thread waits on the mbarrier's phase before reading.  A buffer
  // receives a new slot only after the __syncthreads that ends the last step
  // reading its old one.  Uses of each buffer are counted so that all
  // threads know the phase parity of every wait.
  uint32_t use_par = 0;  // bit b: parity of the uses of buffer b so far
  uint32_t stall = 0;  // a wait that gave up (reported in the status word)
  auto slot_off = [&](int kslot, int r) {
    return ((size_t)kslot * a.R + r) * NE + (size_t)rank * Pc;
  };
  auto stage_issue = [&](int kslot, int r) {
    const int b = kslot % 3;
    const size_t o = slot_off(kslot, r);
    mbar_expect_tx(&st_bar[b], (uint32_t)(Pc * (sizeof(float4) + sizeof(float2))));
    bulk_g2s(st_u + (size_t)b * Pc, a.traj_u + o, (uint32_t)(Pc * sizeof(float4)), &st_bar[b]);
    bulk_g2s(st_ig + (size_t)b * Pc, a.traj_ig + o, (uint32_t)(Pc * sizeof(float2)), &st_bar[b]);
  };
  auto stage_wait = [&](int kslot, int len) {
    const int b = kslot % 3;
    const uint32_t parity = ((use_par >> b) ^ (uint32_t)((len - 1 - kslot) / 3)) & 1u;
    for (int it = 0; it < (1 << 22); ++it)
      if (mbar_try_wait(&st_bar[b], parity)) return;
    stall = 1;
  };

  for (int r = cid; r < a.R; r += ncl) {
    const size_t roff = (size_t)r * NE + (size_t)rank * Pc;  // lambda, this CTA
    const int len = a.n_steps;
    if (a.stage) {
      if (tid == 0) {
        fence_proxy_async();
        stage_issue(len - 1, r);
        if (len >= 2) stage_issue(len - 2, r);
      }
      stage_wait(len - 1, len);
    }
    // ---- publish lambda_{s1} (with the tick injection of step s1) ----------
    {
      const size_t xo = ((size_t)(len - 1) * a.R + r) * NE + (size_t)rank * Pc;
      const float4* xu = a.stage ? st_u + (size_t)((len - 1) % 3) * Pc : a.traj_u + xo;
      const double* coef = tick_coef(a, a.s0 + len, r);
      for_all([&](int i) {
        const float4 L = a.lam[roff + i];
        const float4 gb = __ldg(reinterpret_cast<const float4*>(geo + i) + 1);
        const bool jsr = (__float_as_uint(gb.w) >> 31) != 0;
        const float c = (jsr ? k.c0j : k.c0) + xu[i].x;
        const float inj = tick_injection(a, coef, (int)(rank * Pc + i));
        pub0[i] = make_float4(L.x * sl_inv_factor(k, fabsf(gb.z), c), L.y, L.z, L.w + inj);
        // owner state: on chip when it fits, else the global arrays themselves
        if (a.own_in_smem) {
          sm_o[i] = make_float4(L.x, a.lam_im[roff + i], a.lam_cim[roff + i], 0.0f);
          sm_c4[i] = a.lam_c4[roff + i];
        } else {
          a.lam_c[roff + i] = L.x;
        }
      });
    }
    const int warp = tid >> 5, lane = tid & 31, nw = nthr >> 5;
    // per-warp FP64 accumulators of this realization's gradient
    for (int q = tid; q < nw * NA; q += nthr) red[q] = 0.0;
    int cur = 0;
    float gstep[NA];  // this thread's contributions of the last few steps (FP32)
#pragma unroll
    for (int p = 0; p < NA; ++p) gstep[p] = 0.0f;
    // barrier phases: the arrive after the publication of step t's slots is
    // waited on after the interior elements of step t, whose neighbours'
    // slots all live in this CTA (the __syncthreads orders those)
    __syncthreads();
    cl_arrive<C>();
    // trajectory of step t (x_{t-1}, its immobile buffer and Ca rate) and
    // the Ca of x_{t-2} (for lambda_Ca / B of the next step's slot)
    struct StepPtr {
      const float4* tu;
      const float2* tig;
      const float4* cprev;
    };
    auto step_ptrs = [&](int t) {
      StepPtr sp;
      if (a.stage) {
        sp.tu = st_u + (size_t)((t - 1) % 3) * Pc;
        sp.tig = st_ig + (size_t)((t - 1) % 3) * Pc;
        sp.cprev = st_u + (size_t)((t >= 2 ? t - 2 : 0) % 3) * Pc;
      } else {
        const size_t xoff = ((size_t)(t - 1) * a.R + r) * NE + (size_t)rank * Pc;
        sp.tu = a.traj_u + xoff;
        sp.tig = a.traj_ig + xoff;
        sp.cprev = a.traj_u + ((size_t)(t >= 2 ? t - 2 : 0) * a.R + r) * NE + (size_t)rank * Pc;
      }
      return sp;
    };
    // the element's record and trajectory, loaded one element ahead (and,
    // for a thread's first element, during the previous step)
    struct Pre {
      float4 at, gb, x;
      float2 ig;
      float cp;
    };
    auto preload = [&](int i, const StepPtr& sp, int t) {
      const float4* gp = reinterpret_cast<const float4*>(geo + i);
      Pre q;
      q.at = __ldg(gp);
      q.gb = __ldg(gp + 1);
      q.x = sp.tu[i];
      q.ig = sp.tig[i];
      q.cp = t > 1 ? sp.cprev[i].x : 0.0f;
      return q;
    };
    Pre first = {};
    bool have_first = false;
    for (int t = len; t >= 1; --t) {
      const int64_t n = a.s0 + t;  // this step maps x_{n-1} to x_n
      const float4* pub = cur ? pub1 : pub0;
      float4* nxt = cur ? pub0 : pub1;
      const uint32_t* bs = s_base + 16 * cur;
      const int32_t* rec = a.traj_ch + ((size_t)(t - 1) * a.R + r) * W;
      const double* coef_next = t > 1 ? tick_coef(a, n - 1, r) : nullptr;
      if (a.stage) {
        // slot t - 3 into the buffer slot t left (read at steps t + 1, t + 2)
        if (t >= 3 && tid == 0) {
          fence_proxy_async();
          stage_issue(t - 3, r);
        }
        stage_wait(t - 1, len);
        if (t >= 2) stage_wait(t - 2, len);
      } else if (t >= 2 && tid == 0) {
        // the trajectory of the next step (slot t - 2) into L2 while this one runs
        const size_t xn = ((size_t)(t - 2) * a.R + r) * NE + (size_t)rank * Pc;
        l2_prefetch(a.traj_u + xn, (uint32_t)(Pc * sizeof(float4)));
        l2_prefetch(a.traj_ig + xn, (uint32_t)(Pc * sizeof(float2)));
      }
      const StepPtr sp = step_ptrs(t);

      // OWN: the owner state of lambda is in shared memory (else global)
      auto element = [&](int i, const Pre& pre, auto own) {
        constexpr bool OWN = decltype(own)::value;
        float lx, li, ci;
        if constexpr (OWN) {
          const float4 o = sm_o[i];
          lx = o.x;
          li = o.y;
          ci = o.z;
        } else {
          lx = a.lam_c[roff + i];
          li = a.lam_im[roff + i];
          ci = a.lam_cim[roff + i];
        }
        float4 cm = OWN ? sm_c4[i] : a.lam_c4[roff + i];
        const float4 x = pre.x;
        const float xim = pre.ig.x, G = pre.ig.y;
        const float4 at = pre.at;
        const float4 gb = pre.gb;
        const uint32_t w0 = __float_as_uint(gb.x), w1 = __float_as_uint(gb.y);
        const uint32_t c0 = w0 & 0xffffu, c1 = w0 >> 16, c2 = w1 & 0xffffu, c3 = w1 >> 16;
        const float bsl = fabsf(gb.z);
        const bool trpn = (__float_as_uint(gb.z) >> 31) != 0;
        const float sa = fabsf(gb.w);
        const bool jsr = (__float_as_uint(gb.w) >> 31) != 0;
        const float4 me = pub[i];
        float4 n0, n1, n2, n3;
        if constexpr (C == 1) {
          n0 = ld_smem_f4(bs[0] + c0 * 16u);
          n1 = ld_smem_f4(bs[0] + c1 * 16u);
          n2 = ld_smem_f4(bs[0] + c2 * 16u);
          n3 = ld_smem_f4(bs[0] + c3 * 16u);
        } else {
          n0 = ld_dsmem_f4(bs[c0 >> a.off_bits] + (c0 & mask) * 16u);
          n1 = ld_dsmem_f4(bs[c1 >> a.off_bits] + (c1 & mask) * 16u);
          n2 = ld_dsmem_f4(bs[c2 >> a.off_bits] + (c2 & mask) * 16u);
          n3 = ld_dsmem_f4(bs[c3 >> a.off_bits] + (c3 & mask) * 16u);
        }
        // transposed diffusion: S = sum_k aT_k lambda(nb_k) - (sum_k a_k) lambda(self)
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
        float* g = gstep;  // this element's terms go straight into the thread's sums
        const float w = me.x;
        const AdjTerms lt = adj_local(k, ak, x, xim, me, li, jsr, trpn, Sc, Sa, Sm, Sy, g);
        float oc = lt.oc, dG = lt.dG;
        const float oa = lt.oa, om = lt.om, oy = lt.oy, oi = lt.oi, c = lt.c;
        if (i < n_ch) {
          // channel elements and their RyR partners all sit in partition 0
          for (int q = s_cptr[i]; q < s_cptr[i + 1]; ++q) {
            const ChanEntry32 e = s_clist[q];
            if (e.kind < 2) {
              if (rec[e.ch]) {
                const uint32_t oc_code = e.kind == 0 ? a.ryr_jsr_code[e.ch] : a.ryr_cleft_code[e.ch];
                const float wo = pub[oc_code & ch_mask].x;
                const float so = e.kind == 0 ? a.ryr_s_js[e.ch] : a.ryr_s_cl[e.ch];
                const float qv = fmaf(w, e.s, wo * so);
                if (e.kind == 0) {
                  oc = fmaf(-k.jr_scale, qv, oc);
                  const float cj = k.c0j + sp.tu[oc_code & ch_mask].x;
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
        adj_rapid(k, ak, bsl, c, G, w, dG, oc, g);
        // compensated update of lambda
        float4 L = make_float4(lx, me.y, me.z, me.w);
        float lnew = li;
        kadd(L.x, cm.x, k.dt * oc);
        kadd(L.y, cm.y, k.dt * oa);
        kadd(L.z, cm.z, k.dt * om);
        kadd(L.w, cm.w, k.dt * oy);
        kadd(lnew, ci, k.dt * oi);
        if (t > 1) {
          const float cprev = (jsr ? k.c0j : k.c0) + pre.cp;
          const float inj = tick_injection(a, coef_next, (int)(rank * Pc + i));
          nxt[i] = make_float4(L.x * sl_inv_factor(k, bsl, cprev), L.y, L.z, L.w + inj);
          if constexpr (OWN) {
            sm_o[i] = make_float4(L.x, lnew, ci, 0.0f);
            sm_c4[i] = cm;
          } else {
            a.lam_c[roff + i] = L.x;
            a.lam_im[roff + i] = lnew;
            a.lam_c4[roff + i] = cm;
            a.lam_cim[roff + i] = ci;
          }
        } else {
          a.lam[roff + i] = L;
          a.lam_im[roff + i] = lnew;
          a.lam_c4[roff + i] = cm;
          a.lam_cim[roff + i] = ci;
        }
      };
      auto element_s = [&](int i, const Pre& q) { element(i, q, std::true_type{}); };
      auto element_g = [&](int i, const Pre& q) { element(i, q, std::false_type{}); };
      // the schedule in two phases around the cluster wait; the loads of a
      // thread's next element are issued before its current one is computed
      auto sweep = [&](auto&& f) {
        int q = tid;
        Pre p = first;
        if (!have_first && q < n_sched) p = preload(sched[q], sp, t);
        auto run = [&](int end) {
          for (; q < end; q += nthr) {
            Pre nx = p;
            if (q + nthr < n_sched) nx = preload(sched[q + nthr], sp, t);
            f((int)sched[q], p);
            p = nx;
          }
        };
        run(n_pre);
        cl_wait<C>();
        run(n_sched);
      };
      if (a.own_in_smem) sweep(element_s);
      else sweep(element_g);
      // the first element of the next step (its trajectory slot is resident
      // without staging; staged slots are waited on at the step's start)
      have_first = false;
      if (!a.stage && t > 1 && tid < n_sched) {
        first = preload(sched[tid], step_ptrs(t - 1), t - 1);
        have_first = true;
      }
      __syncthreads();
      cl_arrive<C>();
      // every 16 steps (and at the end) the warp's FP32 sums go into its FP64
      // accumulators: the long sum over the steps runs in double precision
      if (((t - 1) & 15) == 0) {
#pragma unroll
        for (int p = 0; p < NA; ++p) {
          float v = gstep[p];
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          if (lane == 0) red[warp * NA + p] += (double)v;
          gstep[p] = 0.0f;
        }
      }
      cur ^= 1;
    }
    cl_wait<C>();
    // ---- FP64 reduction of this realization's gradient ---------------------
    __syncthreads();
    if (tid < NA) {
      double v = 0.0;
      for (int q = 0; q < nw; ++q) v += red[q * NA + tid];
      atomicAdd(a.grad + (size_t)r * NA + tid, v * (double)k.dt);
    }
    step_barrier<C>();  // pub and red are reused by the next realization
    if (a.stage)
      for (int b = 0; b < 3; ++b)
        if (a.n_steps > b) use_par ^= (((uint32_t)((a.n_steps - 1 - b) / 3 + 1)) & 1u) << b;
  }
  if (stall) atomicOr(a.status, 1u);
}

// Line-scan loss at the ticks of a segment: F_i = base_i + sum_q w_q
// dye(col_q) with the dye deviation of the trajectory slot (base_i: pad plus
// the resting dye), e_i = F_i / F0_i - 1 - target_i, coef_i = e_i / F0_i
// (= dL/dF_i) and the loss term e_i^2 / 2, kept per sample so the host sums
// them in a fixed order.  One block per (sample, realization, tick).
__global__ void k_adj_tick(AdjTickArgs a) {
  const int i = blockIdx.x, r = blockIdx.y, z = blockIdx.z;
  // dye deviation: the fourth float of each element's state
  const float* U = reinterpret_cast<const float*>(a.traj_u + (size_t)z * a.slot_stride +
                                                  (size_t)r * a.n_state);
  double acc = 0.0;
  for (int q = a.ptr[i] + threadIdx.x; q < a.ptr[i + 1]; q += blockDim.x)
    acc += a.w[q] * (double)__ldg(U + 4 * (size_t)a.col[q] + 3);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double red[32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double F = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) F += red[q];
    F += a.base[i];
    if (a.mean_trace) {  // F itself; k_adj_tick_mean forms the loss
      a.coef[((size_t)z * a.R + r) * a.n_samples + i] = F;
      return;
    }
    const int tick = a.tick0 + z;
    const double tg = a.target ? a.target[((size_t)r * a.n_ticks + tick) * a.n_samples + i] : 0.0;
    const double e = F / a.f0[i] - 1.0 - tg;
    a.coef[((size_t)z * a.R + r) * a.n_samples + i] = e / a.f0[i];
    a.loss[((size_t)tick * a.R + r) * a.n_samples + i] = 0.5 * e * e;
  }
}

// Mean-trace loss at the ticks of a segment: coef holds F of every
// realization (k_adj_tick); the mean over the realizations (FP64, fixed
// order) against the shared target gives e_i, the loss term e_i^2 / 2 (in
// realization 0's slot) and dL/dF_ri = e_i / (R F0_i) for every r.  One
// block per (sample, tick).
__global__ void k_adj_tick_mean(AdjTickArgs a) {
  const int i = blockIdx.x, z = blockIdx.y;
  double* Fz = a.coef + (size_t)z * a.R * a.n_samples;
  double acc = 0.0;
  for (int r = threadIdx.x; r < a.R; r += blockDim.x) acc += Fz[(size_t)r * a.n_samples + i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double red[32];
  __shared__ double s_e;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  const int tick = a.tick0 + z;
  if (threadIdx.x == 0) {
    double S = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) S += red[q];
    const double tg = a.target ? a.target[(size_t)tick * a.n_samples + i] : 0.0;
    const double e = (S / a.R) / a.f0[i] - 1.0 - tg;
    a.loss[((size_t)tick * a.R) * a.n_samples + i] = 0.5 * e * e;
    s_e = e;
  }
  __syncthreads();
  const double c = s_e / ((double)a.R * a.f0[i]);
  for (int r = threadIdx.x; r < a.R; r += blockDim.x) {
    Fz[(size_t)r * a.n_samples + i] = c;
    if (r > 0) a.loss[((size_t)tick * a.R + r) * a.n_samples + i] = 0.0;
  }
}

template <int C>
static cudaError_t adj_attrs(size_t smem) {
  cudaError_t e =
      cudaFuncSetAttribute(k_adjoint32<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && C > 8)
    e = cudaFuncSetAttribute(k_adjoint32<C>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

template <int C>
static cudaLaunchConfig_t adj_cfg(int n_clusters, int threads, size_t smem, cudaStream_t st,
                                  cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(n_clusters * C);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <int C>
static int launch_adjoint_t(const AdjArgs& a, int n_clusters, int threads, size_t smem,
                            cudaStream_t st) {
  if (adj_attrs<C>(smem) != cudaSuccess) return -1;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = adj_cfg<C>(n_clusters, threads, smem, st, attr);
  return cudaLaunchKernelEx(&cfg, k_adjoint32<C>, a) == cudaSuccess ? 0 : -1;
}

template <int C>
static int adjoint_max_clusters_t(int threads, size_t smem) {
  if (adj_attrs<C>(smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = adj_cfg<C>(1, threads, smem, nullptr, attr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_adjoint32<C>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

#define SRS_ADJ_SIZES(X) X(1) X(2) X(3) X(4) X(5) X(6) X(8) X(16)

int launch_adjoint(const AdjArgs& a, int C, int n_clusters, int threads, size_t smem,
                   cudaStream_t st) {
  switch (C) {
#define SRS_L(CC) \
  case CC:        \
    return launch_adjoint_t<CC>(a, n_clusters, threads, smem, st);
    SRS_ADJ_SIZES(SRS_L)
#undef SRS_L
    default: return -1;
  }
}

int adjoint_max_clusters(int C, int threads, size_t smem) {
  switch (C) {
#define SRS_M(CC) \
  case CC:        \
    return adjoint_max_clusters_t<CC>(threads, smem);
    SRS_ADJ_SIZES(SRS_M)
#undef SRS_M
    default: return 0;
  }
}

int launch_adj_tick(const AdjTickArgs& a, cudaStream_t st) {
  constexpr int ZMAX = 65535;  // grid z limit: long segments in several launches
  for (int z0 = 0; z0 < a.n_seg_ticks; z0 += ZMAX) {
    AdjTickArgs c = a;
    c.n_seg_ticks = a.n_seg_ticks - z0 < ZMAX ? a.n_seg_ticks - z0 : ZMAX;
    c.tick0 = a.tick0 + z0;
    c.traj_u = a.traj_u + (size_t)z0 * a.slot_stride;
    c.coef = a.coef + (size_t)z0 * a.R * a.n_samples;
    k_adj_tick<<<dim3(a.n_samples, a.R, c.n_seg_ticks), 128, 0, st>>>(c);
    if (a.mean_trace) k_adj_tick_mean<<<dim3(a.n_samples, c.n_seg_ticks), 128, 0, st>>>(c);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace srs
