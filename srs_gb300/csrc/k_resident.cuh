// k_resident.cuh — the resident FP32 engine: persistent batched kernel
// k_resident32<C, TRAJ> and its launch helpers.  The kernel is instantiated
// per cluster size in the k_res_*.cu units (SRS_RESIDENT_DEFINE), which
// compile in parallel; k_fp32.cu dispatches on the cluster size.
#pragma once
#include <type_traits>

#include "srs_cluster.cuh"
#include "srs_comp.h"
#include "srs_engine.h"
#include "srs_fp32_update.cuh"
#include "srs_protocol.cuh"

namespace srs {

// ===========================================================================
// Resident FP32 engine
// ===========================================================================
// Shared-memory layout of one CTA (dynamic):
//   float4 buf[2][P]; ushort4 cm[P]; float imm[P]; ushort ci[P] (the
//   compensation terms as halves, srs_comp.h: 46 instead of 56 bytes per
//   element, so that more CTAs share an SM -- for the 10,368-element dyad two
//   of a 5-CTA cluster, or three of an 8-CTA one); then this tail (16-byte
//   aligned), then the channel block (used by rank 0).
struct ResidentSmemTail {
  RealCtl ctl;
  uint32_t base[2][16];  // cluster addresses of buf[b] in CTA rank q
  int32_t bad;
  // Termination flag published by rank 0's warp 0 in step s into slot s & 3
  // and read by every thread of the cluster after the barrier that ends step
  // s.  With speculation rank 0 can run one barrier phase ahead of a slow CTA,
  // so four slots keep a flag from being rewritten while it is read.
  int32_t done_flag[4];
};

template <int C>
__device__ __forceinline__ float4 resident_nb(const uint32_t* bs, const float4* src,
                                              uint32_t code, int off_bits, uint32_t mask) {
  if constexpr (C == 1) {
    return src[code & mask];
  } else {
    return ld_dsmem_f4(bs[code >> off_bits] + (code & mask) * 16u);
  }
}

// Absolute Ca by channel code for the protocol code.  The resident engine's
// Channels arrays hold (kind << 28 | channel) instead of element indices:
// kind 0 = RyR cleft element, 1 = RyR JSR element, 2 = LCC element.  All of
// them live in partition 0 (local shared memory of rank 0).
// Offsets in partition 0 of every channel's elements, and the LCC elements'
// resting Ca, staged in rank 0's shared memory once per launch: the channel
// group reads them every step.
struct ChanSmem {
  const uint32_t* cl;   // [NR] RyR cleft element
  const uint32_t* js;   // [NR] RyR JSR element
  const uint32_t* lc;   // [NL] LCC element
  const float* lrest;   // [NL] resting Ca of the LCC element
};

struct ResidentCa {
  const ResidentArgs* a;
  const float4* src;
  ChanSmem cs;
  __device__ double operator()(int e) const {
    int kind = e >> 28, idx = e & 0x0fffffff;
    uint32_t off;
    float rest;
    if (kind == 0) {
      off = cs.cl[idx];
      rest = a->k.c0;
    } else if (kind == 1) {
      off = cs.js[idx];
      rest = a->k.c0j;
    } else {
      off = cs.lc[idx];
      rest = cs.lrest[idx];
    }
    return (double)(src[off].x + rest);
  }
};

// Gating of every channel after time step ctl.step by one warp
// (UpdateChannelGating, cpu/RunSimulation.cpp:656-674).  `src` holds the
// state after that step; every channel element is local (partition 0).
// Named barrier of the channel group (the first `n` threads of the CTA).
__device__ __forceinline__ void group_sync(int n) {
  if (n > 32) asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory");
  else __syncwarp();
}

// Gating of every channel after time step ctl.step by the channel group of
// partition 0 (UpdateChannelGating, cpu/RunSimulation.cpp:656-674): group
// lane gl takes RyR gl, then LCC gl - NR, so with 64 lanes every channel of
// a dyad is gated in one round.  `src` holds the state after that step;
// every channel element is local (partition 0).
static __device__ void resident_gate(const ResidentArgs& a, RealCtl& ctl, const float4* src,
                              int32_t* s_ryr, int32_t* s_lcc, int32_t* s_lccv, double* s_res,
                              int32_t* s_nb, const ChanSmem& cs, int gl, int ng) {
  const int NR = a.C.NR, NL = a.C.NL;
  const srs_gate_consts* g = &a.P_.gc[ctl.vsel];
  const bool coupled = g->ryr_astar_half != 0.0f;
  if (coupled) {
    for (int i = gl; i < NR; i += ng) {
      int no = 0, nc = 0;
      for (int q = 0; q < 4; ++q) {
        int j = a.C.ryr_nb[4 * i + q];
        if (j >= 0) {
          if (s_ryr[j]) ++no;
          else ++nc;
        }
      }
      s_nb[i] = no | (nc << 16);
    }
    group_sync(ng);
  }
  for (int q = gl; q < NR + NL; q += ng) {
    if (q < NR) {
      const int i = q;
      int no = 0, nc = 0;
      if (coupled) {
        no = s_nb[i] & 0xffff;
        nc = s_nb[i] >> 16;
      }
      float ca_s = src[cs.cl[i]].x + a.k.c0;
      float ca_j = src[cs.js[i]].x + a.k.c0j;
      double rr = s_res[i];
      s_ryr[i] = srs_gate_ryr(g, s_ryr[i], ca_s, ca_j, no, nc, &rr, ctl.seed, (uint32_t)i,
                              (uint64_t)ctl.step);
      s_res[i] = rr;
    } else {
      const int i = q - NR;
      float ca_l = src[cs.lc[i]].x + cs.lrest[i];
      double rr = s_res[NR + i];
      int st = s_lcc[i], vs = s_lccv[i];
      srs_gate_lcc(g, &st, &vs, ca_l, &rr, ctl.seed, (uint32_t)(NR + i), (uint64_t)ctl.step);
      s_lcc[i] = st;
      s_lccv[i] = vs;
      s_res[NR + i] = rr;
    }
  }
  group_sync(ng);
}

// Protocol of step ctl.step (rank 0, warp 0; lane 0 does the work).
static __device__ void resident_prestep(const ResidentArgs& a, RealCtl& ctl, const float4* src,
                                 int32_t* s_ryr, int32_t* s_lcc, int32_t* s_lccv, int r,
                                 int write_row_now, int lane, const ChanSmem& cs) {
  if (lane == 0) {
    ResidentCa cab{&a, src, cs};
    float* rows = a.CS.rows + (size_t)r * a.P_.row_cap * a.P_.row_w;
    if (write_row_now && a.P_.run_protocol)
      write_row(a.P_, a.C, ctl, s_ryr, s_lcc, s_lccv, rows, ctl.t, cab);
    prestep(a.P_, a.C, ctl, s_ryr, s_lcc, s_lccv, rows, cab);
  }
  __syncwarp();
}

// TRAJ: also record, for every step of the launch, the state the step starts
// from, its Ca rate before the rapid-buffer factor and the channel states it
// uses (the trajectory the adjoint is conditioned on).
template <int C, bool TRAJ>
// At most 640 threads per CTA: two CTAs of up to 320 threads share an SM
// with up to 96 registers per thread (the tuned configurations), and
// single-CTA configurations keep the same budget.
__global__ void __launch_bounds__(SRS_RESIDENT_MAX_THREADS, 1) k_resident32(ResidentArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int P = a.P;
  float4* buf0 = reinterpret_cast<float4*>(smem);
  float4* buf1 = buf0 + P;
  ushort4* cmq = reinterpret_cast<ushort4*>(buf1 + P);
  float* immb = reinterpret_cast<float*>(cmq + P);
  uint16_t* ciq = reinterpret_cast<uint16_t*>(immb + P);
  const int NR = a.C.NR, NL = a.C.NL, NCH = NR + NL;
  ResidentSmemTail* tail = reinterpret_cast<ResidentSmemTail*>(
      (reinterpret_cast<uintptr_t>(ciq + P) + 15) & ~(uintptr_t)15);
  int32_t* s_ryr = reinterpret_cast<int32_t*>(tail + 1);
  int32_t* s_lcc = s_ryr + NR;
  int32_t* s_lccv = s_lcc + NL;
  int32_t* s_nb = s_lccv + NL;
  uint32_t* s_ccl = reinterpret_cast<uint32_t*>(s_nb + NR);
  uint32_t* s_cjs = s_ccl + NR;
  uint32_t* s_clc = s_cjs + NR;
  float* s_lrest = reinterpret_cast<float*>(s_clc + NL);
  const ChanSmem cs{s_ccl, s_cjs, s_clc, s_lrest};
  double* s_res = reinterpret_cast<double*>(
      (reinterpret_cast<uintptr_t>(s_lrest + NL) + 7) & ~(uintptr_t)7);
  // channel-entry CSR of partition 0, staged once per launch
  int32_t* s_cptr = reinterpret_cast<int32_t*>(s_res + NCH);
  ChanEntry32* s_clist = reinterpret_cast<ChanEntry32*>(
      (reinterpret_cast<uintptr_t>(s_cptr + a.n_chtet[0] + 1) + 15) & ~(uintptr_t)15);

  uint32_t rank = 0;
  if constexpr (C > 1) {
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
  }
  const int cid = blockIdx.x / C;
  const int ncl = gridDim.x / C;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int nthr = blockDim.x;
  const int n_loc = a.n_local[rank];
  const int n_ch = (rank == 0) ? a.n_chtet[0] : 0;  // channel elements: rank 0 only
  // In partition 0 the channel group (the first ng threads: two warps when
  // the CTA has at least four) owns the channel elements, gates the channels
  // right after updating them and runs the protocol; the other warps share
  // the rest.  Elsewhere every thread strides over the whole partition.
  const int ng = nthr >= 128 ? 64 : 32;
  const bool split = (rank == 0) && (n_ch > 0) && (nthr > ng);
  const bool chan_group = split && tid < ng;
  const bool chan_warp = (rank == 0) && (warp == 0);
  const int n_int = a.n_int[rank];  // interior elements follow the channel elements
  const TetRec* geo = a.geo + (size_t)rank * P;
  const uint32_t off_mask = (1u << a.off_bits) - 1u;
  const Consts32& k = a.k;
  const Protocol& P_ = a.P_;
  if (rank == 0) {
    const int nnz = a.ch_ptr[n_ch];
    for (int i = tid; i <= n_ch; i += nthr) s_cptr[i] = a.ch_ptr[i];
    for (int i = tid; i < nnz; i += nthr) s_clist[i] = a.ch_list[i];
    for (int i = tid; i < NR; i += nthr) {
      s_ccl[i] = a.ryr_cleft_code[i] & off_mask;
      s_cjs[i] = a.ryr_jsr_code[i] & off_mask;
    }
    for (int i = tid; i < NL; i += nthr) {
      s_clc[i] = a.lcc_code[i] & off_mask;
      s_lrest[i] = a.lcc_rest[i];
    }
  }

  if (tid < 32) {
    for (int q = lane; q < C; q += 32) {
      tail->base[0][q] = (C > 1) ? map_rank(smem_addr(buf0), q) : smem_addr(buf0);
      tail->base[1][q] = (C > 1) ? map_rank(smem_addr(buf1), q) : smem_addr(buf1);
    }
  }
  if (tid == 0) tail->bad = 0;
  // address of rank 0's termination flags, as seen from this CTA
  uint32_t done_addr0 = smem_addr(&tail->done_flag[0]);
  if constexpr (C > 1) done_addr0 = map_rank(done_addr0, 0);
  step_barrier<C>();  // all CTAs of the cluster are running before DSMEM use
  int bad = 0;

  for (int r = cid; r < a.R; r += ncl) {
    // ---- load the realization ----------------------------------------------
    const size_t roff = ((size_t)r * C + rank) * P;
    for (int i = tid; i < n_loc; i += nthr) {
      buf0[i] = a.M[roff + i];
      immb[i] = a.I[roff + i];
      comp_store4(cmq + i, a.CM[roff + i]);
      ciq[i] = comp_store1(a.CI[roff + i]);
    }
    if (rank == 0) {
      if (tid == 0) tail->ctl = a.CS.ctl[r];
      for (int i = tid; i < NR; i += nthr) s_ryr[i] = a.CS.ryr[(size_t)r * NR + i];
      for (int i = tid; i < NL; i += nthr) {
        s_lcc[i] = a.CS.lcc[(size_t)r * NL + i];
        s_lccv[i] = a.CS.lccv[(size_t)r * NL + i];
      }
      for (int i = tid; i < NCH; i += nthr) s_res[i] = a.CS.res[(size_t)r * NCH + i];
    }
    __syncthreads();
    if (chan_warp) {
      // protocol work that precedes the first step of a run
      if (a.prestep_first && !tail->ctl.done)
        resident_prestep(a, tail->ctl, buf0, s_ryr, s_lcc, s_lccv, r, a.initial_row, lane, cs);
      if (lane == 0) tail->done_flag[3] = tail->ctl.done;
    }
    step_barrier<C>();
    const bool skip = ((C > 1) ? ld_dsmem_s32(done_addr0 + 12u) : tail->done_flag[3]) != 0;
    int cur = 0;
    // Speculation is safe when no termination can be decided inside this
    // launch: without the protocol nothing terminates, and without the
    // fidelity criterion a run ends exactly at step n_steps.
    // (every CTA reads the step count from global memory: only partition 0
    // keeps the control block in shared memory)
    const bool spec = a.speculate && (!P_.run_protocol ||
                                      (!P_.flag_fidelity && a.CS.ctl[r].step + a.steps <= P_.n_steps));
    if (!skip) {
      // Barrier phases: the arrive that ends step s is waited on at the top of
      // step s + 1 -- after the step's interior elements when speculating
      // (their neighbours are all in this CTA, so only this CTA's writes of
      // step s are needed, which the __syncthreads below orders), before
      // them otherwise.
      cl_arrive<C>();
      bool pending = true;
      int64_t next_ev = 0;  // channel warp: next step with protocol work (0: the first)
      for (int s = 0; s < a.steps; ++s) {
        const float4* src = cur ? buf1 : buf0;
        float4* dst = cur ? buf0 : buf1;
        const uint32_t* bs = tail->base[cur];
        const uint32_t src_local = smem_addr(src);
        if constexpr (TRAJ) {
          if (chan_warp) {
            const int W = NR + 2 * NL + 1;
            int32_t* rec = a.traj_ch + ((size_t)s * a.R + r) * W;
            for (int q = lane; q < NR; q += 32) rec[q] = s_ryr[q];
            for (int q = lane; q < NL; q += 32) {
              rec[NR + q] = s_lcc[q];
              rec[NR + NL + q] = s_lccv[q];
            }
            if (lane == 0) rec[W - 1] = tail->ctl.vsel;
          }
        }
        const int v = tail->ctl.vsel;
        // one range of elements of this partition; elements that carry
        // channels (head of partition 0) add the release flux of their
        // channels, computed from the state of this step
        // Elements lo + idx, lo + idx + stride, ... below hi; idx carries
        // over to the next range, so consecutive ranges are dealt out as
        // one sequence and every thread gets the same count.
        // `local`: every neighbour of the range lies in this CTA's partition
        // (the interior range), so its state is read from this CTA's shared
        // memory directly, without the per-rank base lookup.
        // `chan`: the range of channel elements (head of partition 0), which add
        // the release flux of their channels
        auto update = [&](int& idx, int lo, int hi, int stride, auto local, auto chan) {
          const int first = lo + idx;
          // geometry of the next element is loaded one iteration ahead
          float4 ga_n = make_float4(0, 0, 0, 0), gb_n = ga_n;
          if (first < hi) {
            const float4* gp = reinterpret_cast<const float4*>(geo + first);
            ga_n = __ldg(gp);
            gb_n = __ldg(gp + 1);
          }
          int i = first;
          for (; i < hi; i += stride) {
            const float4 ga = ga_n, gb = gb_n;
            if (i + stride < hi) {
              const float4* gp = reinterpret_cast<const float4*>(geo + i + stride);
              ga_n = __ldg(gp);
              gb_n = __ldg(gp + 1);
            }
            uint32_t w0 = __float_as_uint(gb.x), w1 = __float_as_uint(gb.y);
            uint32_t c0 = w0 & 0xffffu, c1 = w0 >> 16, c2 = w1 & 0xffffu, c3 = w1 >> 16;
            const uint32_t fl = __float_as_uint(gb.w);
            float flux = 0.0f;
            if constexpr (decltype(chan)::value) {
              for (int q = s_cptr[i]; q < s_cptr[i + 1]; ++q) {
                ChanEntry32 e = s_clist[q];
                float J = 0.0f;
                if (e.kind < 2) {
                  if (s_ryr[e.ch]) {
                    float us = src[s_ccl[e.ch]].x;
                    float uj = src[s_cjs[e.ch]].x;
                    J = k.jr_scale * ((k.dc0 + uj) - us);
                  }
                } else if ((s_lcc[e.ch] == 6 || s_lcc[e.ch] == 12) && s_lccv[e.ch] == 2) {
                  float c = s_lrest[e.ch] + src[i].x;
                  J = k.lccA[v] * fmaf(c, k.lccE[v], -k.lccB);
                }
                flux = fmaf(J, e.s, flux);
              }
            }
            float4 n0, n1, n2, n3;
            if constexpr (C == 1) {
              n0 = ld_smem_f4(bs[0] + c0 * 16u);
              n1 = ld_smem_f4(bs[0] + c1 * 16u);
              n2 = ld_smem_f4(bs[0] + c2 * 16u);
              n3 = ld_smem_f4(bs[0] + c3 * 16u);
            } else if constexpr (decltype(local)::value) {
              n0 = ld_smem_f4(src_local + (c0 & off_mask) * 16u);
              n1 = ld_smem_f4(src_local + (c1 & off_mask) * 16u);
              n2 = ld_smem_f4(src_local + (c2 & off_mask) * 16u);
              n3 = ld_smem_f4(src_local + (c3 & off_mask) * 16u);
            } else {
              n0 = ld_dsmem_f4(bs[c0 >> a.off_bits] + (c0 & off_mask) * 16u);
              n1 = ld_dsmem_f4(bs[c1 >> a.off_bits] + (c1 & off_mask) * 16u);
              n2 = ld_dsmem_f4(bs[c2 >> a.off_bits] + (c2 & off_mask) * 16u);
              n3 = ld_dsmem_f4(bs[c3 >> a.off_bits] + (c3 & off_mask) * 16u);
            }
            float4 out, cm = comp_load4(cmq + i);
            float imo, ci = comp_load1(ciq[i]);
            if constexpr (TRAJ) {
              const size_t o = ((size_t)s * a.R + r) * ((size_t)C * P) + (size_t)rank * P + i;
              float g;
              a.traj_u[o] = src[i];
              const float im0 = immb[i];
              tet_update_x2(k, src[i], im0, n0, n1, n2, n3, ga, fl, gb.z, 0.0f, flux, cm, ci,
                         &out, &imo, &g);
              a.traj_ig[o] = make_float2(im0, g);
            } else {
              tet_update_x2(k, src[i], immb[i], n0, n1, n2, n3, ga, fl, gb.z, 0.0f, flux, cm, ci,
                         &out, &imo);
            }
            dst[i] = out;
            immb[i] = imo;
            comp_store4(cmq + i, cm);
            ciq[i] = comp_store1(ci);
          }
          idx = i - hi;
        };
        // channel elements, then gating of this step and the protocol of the
        // next, by warp 0 of partition 0 (split) or after the whole CTA
        auto channels = [&]() {
          if (split) {
            if (chan_group) {
              int idx = tid;
              update(idx, 0, n_ch, ng, std::false_type{}, std::true_type{});
              group_sync(ng);  // the group wrote the channel elements itself
              if (!P_.nogating) resident_gate(a, tail->ctl, dst, s_ryr, s_lcc, s_lccv, s_res, s_nb, cs, tid, ng);
            }
          } else {
            int idx = tid;
            update(idx, 0, n_ch, nthr, std::false_type{}, std::true_type{});
            __syncthreads();
            if (chan_warp && !P_.nogating)
              resident_gate(a, tail->ctl, dst, s_ryr, s_lcc, s_lccv, s_res, s_nb, cs, lane, 32);
          }
          if (chan_warp) {
            RealCtl& ctl = tail->ctl;
            if (lane == 0) {
              ctl.step += 1;
              ctl.t += P_.dt;
              // the RyR hold of this step's protocol (cpu/RunSimulation.cpp:540-542)
              if (P_.run_protocol && P_.init_ryr != -1 && ctl.step < P_.hold_end) s_ryr[P_.init_ryr] = 1;
            }
            __syncwarp();
            // the protocol runs only at the steps where it has work (the RyR
            // hold is applied above)
            if (ctl.step >= next_ev) {
              resident_prestep(a, ctl, dst, s_ryr, s_lcc, s_lccv, r, 0, lane, cs);
              if (lane == 0) next_ev = protocol_next_event(P_, ctl, !P_.nogating);
              next_ev = __shfl_sync(0xffffffffu, next_ev, 0);
            }
            if (lane == 0) {
              tail->done_flag[s & 3] = ctl.done;
              // a speculating launch must not end a run before its last step
              if (spec && ctl.done && s + 1 < a.steps) bad |= 2;
            }
          }
        };
        // termination decided at the end of step s - 1
        auto finished = [&]() -> bool {
          if (s == 0) return false;
          const uint32_t slot = (uint32_t)((s - 1) & 3);
          return ((C > 1) ? ld_dsmem_s32(done_addr0 + 4u * slot) : tail->done_flag[slot]) != 0;
        };
        const bool worker = !chan_group;  // not the channel group
        const int wt = split ? tid - ng : tid, wn = split ? nthr - ng : nthr;
        if (!spec) {
          cl_wait<C>();
          pending = false;
          if (finished()) break;
        }
        // interior elements: neighbours all in this partition
        int idx = wt;
        if (worker) update(idx, n_ch, n_ch + n_int, wn, std::true_type{}, std::false_type{});
        if (a.ch_interior && rank == 0 && n_ch > 0) channels();
        if (spec) {  // no termination inside this launch: nothing to read
          cl_wait<C>();
          pending = false;
        }
        // boundary elements: some neighbour in another partition
        if (worker) update(idx, n_ch + n_int, n_loc, wn, std::false_type{}, std::false_type{});
        if (!a.ch_interior && rank == 0 && n_ch > 0) channels();
        __syncthreads();
        cl_arrive<C>();
        pending = true;
        cur ^= 1;
      }
      if (pending) cl_wait<C>();
    }
    step_barrier<C>();
    // ---- store the realization ----------------------------------------------
    if (!skip) {
      const float4* fin = cur ? buf1 : buf0;
      // a non-finite Ca stays non-finite through every later update, so the
      // end of the launch is where it is looked for
      for (int i = tid; i < n_loc; i += nthr) {
        bad |= !isfinite(fin[i].x);
        a.M[roff + i] = fin[i];
        a.I[roff + i] = immb[i];
        a.CM[roff + i] = comp_load4(cmq + i);
        a.CI[roff + i] = comp_load1(ciq[i]);
        if constexpr (TRAJ) {
          const size_t o = ((size_t)a.steps * a.R + r) * ((size_t)C * P) + (size_t)rank * P + i;
          a.traj_u[o] = fin[i];
          a.traj_ig[o] = make_float2(immb[i], 0.0f);
        }
      }
      if (rank == 0) {
        for (int i = tid; i < NR; i += nthr) a.CS.ryr[(size_t)r * NR + i] = s_ryr[i];
        for (int i = tid; i < NL; i += nthr) {
          a.CS.lcc[(size_t)r * NL + i] = s_lcc[i];
          a.CS.lccv[(size_t)r * NL + i] = s_lccv[i];
        }
        for (int i = tid; i < NCH; i += nthr) a.CS.res[(size_t)r * NCH + i] = s_res[i];
        if (tid == 0) a.CS.ctl[r] = tail->ctl;
      }
    }
    step_barrier<C>();  // shared memory is reused by the next realization
  }
  if (bad) atomicOr(&tail->bad, bad);
  __syncthreads();
  // status bit 0: non-finite Ca; bit 3: termination inside a speculating launch
  if (tid == 0 && tail->bad) atomicOr(&a.CS.ctl[0].status, ((tail->bad & 1) ? 1u : 0u) | ((tail->bad & 2) ? 8u : 0u));
  step_barrier<C>();  // no CTA leaves while others may read its shared memory
}

template <int C, bool TRAJ>
static cudaError_t set_attrs(size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(k_resident32<C, TRAJ>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (C > 8)
    e = cudaFuncSetAttribute(k_resident32<C, TRAJ>, cudaFuncAttributeNonPortableClusterSizeAllowed,
                             1);
  return e;
}

template <int C, bool TRAJ>
static int launch_resident_t(const ResidentArgs& a, int n_clusters, int threads, size_t smem,
                             cudaStream_t st) {
  if (set_attrs<C, TRAJ>(smem) != cudaSuccess) return -1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(n_clusters * C);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, k_resident32<C, TRAJ>, a);
  return e == cudaSuccess ? 0 : -1;
}

template <int C>
static int max_clusters_t(int threads, size_t smem) {
  if (set_attrs<C, false>(smem) != cudaSuccess || set_attrs<C, true>(smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  int n2 = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_resident32<C, false>, &cfg) != cudaSuccess ||
      cudaOccupancyMaxActiveClusters(&n2, k_resident32<C, true>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n < n2 ? n : n2;
}

}  // namespace srs

// Entry points of one cluster size (declared in srs_engine.h).
#define SRS_RESIDENT_DEFINE(CC)                                                          \
  namespace srs {                                                                        \
  int launch_resident_c##CC(const ResidentArgs& a, int n_clusters, int threads, size_t smem, \
                            cudaStream_t st) {                                           \
    return a.traj_u ? launch_resident_t<CC, true>(a, n_clusters, threads, smem, st)      \
                    : launch_resident_t<CC, false>(a, n_clusters, threads, smem, st);    \
  }                                                                                      \
  int resident_max_clusters_c##CC(int threads, size_t smem) {                            \
    return max_clusters_t<CC>(threads, smem);                                            \
  }                                                                                      \
  }
