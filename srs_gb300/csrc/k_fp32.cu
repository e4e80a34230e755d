// k_fp32.cu — FP32 spark step engines.
//
// State is stored as deviations from the resting equilibrium (u = c - c_rest,
// per species; Ca relative to the resting level of its own domain), and the
// buffer reactions are written in the cancellation-free deviation form
//   r = kon*((B - b_rest)*u - c*u_b) - koff*u_b,
// which is the reference's kon*(B - b)*c - koff*b (cpu/RunSimulation.cpp:
// 78, 95, 101, 107, 115) minus its value at rest (zero at equilibrium).  At
// rest all deviations are zero, so single precision keeps full relative
// precision in the small perturbations that make up most of the domain.
//
// Two engines share the per-element update `tet_update`:
//   * k_plain32_step: one launch per time step, state in HBM, grid.y over
//     realizations, last block per realization runs gating + protocol;
//   * k_resident32<C>: persistent batched kernel.  One realization at a time
//     per thread-block cluster of C CTAs; the mobile species (Ca, ATP, CMDN,
//     dye) live in shared memory as float4, double buffered, partitioned
//     over the cluster; neighbours in another CTA's partition are read
//     through distributed shared memory.  Warp 0 of every CTA runs the
//     channel work (gating, protocol, release flux and the elements that
//     carry channels) while the other warps update all other elements, so a
//     time step costs one cluster barrier.
#include <cooperative_groups.h>

#include "srs_engine.h"
#include "srs_protocol.cuh"

namespace srs {



// flags: bit0 JSR, bit1 TropC, bit2 carries channel entries.
__device__ __forceinline__ void tet_update(const Consts32& k, float4 o, float im, float4 s1,
                                           float4 s2, float4 s3, float4 s4, float4 a,
                                           uint32_t fl, float bsl, float kb, float flux,
                                           float4* out, float* im_out) {
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
  if (bsl != 0.0f) {  // rapid SL buffer (cpu/RunSimulation.cpp:15-22)
    float kc = k.khi + c;
    rca = rca / fmaf(bsl, 1.0f / (kc * kc), 1.0f);
  }
  out->x = fmaf(k.dt, rca, o.x);
  out->y = fmaf(k.dt, ratp, o.y);
  out->z = fmaf(k.dt, rcmdn, o.z);
  out->w = fmaf(k.dt, rdye, o.w);
  *im_out = fmaf(k.dt, rim, im);
}



// ===========================================================================
// Plain FP32 engine
// ===========================================================================


__global__ void __launch_bounds__(256) k_plain32_step(Plain32Args a) {
  const int r = blockIdx.y;
  RealCtl* ctlp = a.CS.ctl + r;
  if (ctlp->done) return;
  const int N = a.N;
  const float4* M = a.M_in + (size_t)r * N;
  const float* I = a.I_in + (size_t)r * N;
  float4* Mo = a.M_out + (size_t)r * N;
  float* Io = a.I_out + (size_t)r * N;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < N) {
    const uint32_t fl = a.flags[j];
    float flux = 0.0f;
    if (fl & 4u) {
      const int32_t* ryr = a.CS.ryr + (size_t)r * a.C.NR;
      const int32_t* lcc = a.CS.lcc + (size_t)r * a.C.NL;
      const int32_t* lccv = a.CS.lccv + (size_t)r * a.C.NL;
      const int v = ctlp->vsel;
      for (int q = a.chan_ptr[j]; q < a.chan_ptr[j + 1]; ++q) {
        ChanEntry32 e = a.chan_list[q];
        if (e.kind < 2) {
          if (ryr[e.ch]) {
            float dc = (a.k.dc0 + M[a.C.ryr_jsr[e.ch]].x) - M[a.C.ryr_cleft[e.ch]].x;
            flux = fmaf(a.k.jr_scale * dc, e.s, flux);
          }
        } else if ((lcc[e.ch] == 6 || lcc[e.ch] == 12) && lccv[e.ch] == 2) {
          float c = a.rest_ca[j] + M[j].x;
          flux = fmaf(a.k.lccA[v] * fmaf(c, a.k.lccE[v], -a.k.lccB), e.s, flux);
        }
      }
    }
    const int4 nb = a.nb[j];
    float4 out;
    float imo;
    tet_update(a.k, M[j], I[j], M[nb.x], M[nb.y], M[nb.z], M[nb.w], a.a[j], fl, a.bsl[j],
               a.kb ? a.kb[j] : 0.0f, flux, &out, &imo);
    Mo[j] = out;
    Io[j] = imo;
    if (!isfinite(out.x)) atomicOr(&ctlp->status, 1u);
  }
  __shared__ int s_last;
  __shared__ int32_t s_nb[1024];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(a.counters + r, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  RealCtl ctl = *ctlp;
  const float* rest = a.rest_ca;
  auto ca = [&](int e) -> double {
    float u = ((volatile const float*)(Mo + e))[0];
    return (double)(rest[e] + u);
  };
  int32_t* ryr_w = a.CS.ryr + (size_t)r * a.C.NR;
  int32_t* lcc_w = a.CS.lcc + (size_t)r * a.C.NL;
  int32_t* lccv_w = a.CS.lccv + (size_t)r * a.C.NL;
  double* res = a.CS.res + (size_t)r * (a.C.NR + a.C.NL);
  if (!a.P.nogating) {
    gate_all(a.P, a.C, ctl.vsel, ctl.seed, ctl.step, ryr_w, lcc_w, lccv_w, res, s_nb,
             threadIdx.x, blockDim.x, ca, []() { __syncthreads(); });
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ctl.step += 1;
    ctl.t += a.P.dt;
    prestep(a.P, a.C, ctl, ryr_w, lcc_w, lccv_w,
            a.CS.rows + (size_t)r * a.P.row_cap * a.P.row_w, ca);
    *ctlp = ctl;
    a.counters[r] = 0;
    __threadfence();
  }
}

__global__ void k_plain32_prestep(Plain32Args a, int write_initial_row) {
  const int r = blockIdx.x;
  if (threadIdx.x != 0) return;
  RealCtl ctl = a.CS.ctl[r];
  const float4* M = a.M_in + (size_t)r * a.N;
  auto ca = [&](int e) -> double { return (double)(a.rest_ca[e] + M[e].x); };
  int32_t* ryr = a.CS.ryr + (size_t)r * a.C.NR;
  int32_t* lcc = a.CS.lcc + (size_t)r * a.C.NL;
  int32_t* lccv = a.CS.lccv + (size_t)r * a.C.NL;
  float* rows = a.CS.rows + (size_t)r * a.P.row_cap * a.P.row_w;
  if (write_initial_row && a.P.run_protocol) write_row(a.P, a.C, ctl, ryr, lcc, lccv, rows, ctl.t, ca);
  prestep(a.P, a.C, ctl, ryr, lcc, lccv, rows, ca);
  a.CS.ctl[r] = ctl;
}

int launch_plain32_step(const Plain32Args& a, cudaStream_t st) {
  dim3 grid((a.N + 255) / 256, a.R);
  k_plain32_step<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
int launch_plain32_prestep(const Plain32Args& a, int write_initial_row, cudaStream_t st) {
  k_plain32_prestep<<<a.R, 32, 0, st>>>(a, write_initial_row);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ===========================================================================
// Resident FP32 engine
// ===========================================================================
// Packed element record (32 bytes): neighbour slot k holds
// (cluster rank << off_bits) | local offset.




__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint32_t map_rank(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ float4 ld_dsmem_f4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr));
  return v;
}
__device__ __forceinline__ float ld_dsmem_f32(uint32_t addr) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr));
  return v;
}
__device__ __forceinline__ float4 ld_smem_f4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr));
  return v;
}
__device__ __forceinline__ void cluster_arrive_wait() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int C>
__device__ __forceinline__ void step_barrier() {
  if constexpr (C == 1) {
    __syncthreads();
  } else {
    cluster_arrive_wait();
  }
}

// Shared-memory layout of one CTA (dynamic):
//   float4 buf[2][P]; float imm[2][P];  then the channel block below.
struct ResidentSmemTail {
  RealCtl ctl;
  uint32_t base[2][16];  // cluster addresses of buf[b] in CTA rank q
  int32_t bad;
  // Termination flag published by warp 0 in iteration s into slot s & 1 and
  // read by every thread after that iteration's barrier.  Two slots, so a
  // slow warp still reading slot s & 1 never sees warp 0's write for s + 1.
  int32_t done_flag[2];
};

// Deviation u of the element with code `code` in the current buffer.
template <int C>
__device__ __forceinline__ float resident_u(const ResidentArgs& a, const uint32_t* bs,
                                            const float4* src, uint32_t code, uint32_t mask) {
  if constexpr (C == 1) {
    return src[code & mask].x;
  } else {
    return ld_dsmem_f32(bs[code >> a.off_bits] + (code & mask) * 16u);
  }
}
template <int C>
__device__ __forceinline__ float4 resident_nb(const uint32_t* bs, const float4* src,
                                              uint32_t code, int off_bits, uint32_t mask) {
  if constexpr (C == 1) {
    return src[code & mask];
  } else {
    return ld_dsmem_f4(bs[code >> off_bits] + (code & mask) * 16u);
  }
}

// Absolute Ca by channel code for the protocol code: the resident engine's
// Channels arrays hold (kind << 28 | channel) instead of element indices,
// kind 0 = RyR cleft element, 1 = RyR JSR element, 2 = LCC element.
template <int C>
struct ResidentCa {
  const ResidentArgs* a;
  const uint32_t* bs;
  const float4* src;
  uint32_t mask;
  __device__ double operator()(int e) const {
    int kind = e >> 28, idx = e & 0x0fffffff;
    uint32_t code;
    float rest;
    if (kind == 0) {
      code = a->ryr_cleft_code[idx];
      rest = a->k.c0;
    } else if (kind == 1) {
      code = a->ryr_jsr_code[idx];
      rest = a->k.c0j;
    } else {
      code = a->lcc_code[idx];
      rest = a->lcc_rest[idx];
    }
    return (double)(resident_u<C>(*a, bs, src, code, mask) + rest);
  }
};

// Gating of every channel after time step ctl.step by one warp
// (UpdateChannelGating, cpu/RunSimulation.cpp:656-674).
template <int C>
__device__ void resident_gate(const ResidentArgs& a, RealCtl& ctl, const uint32_t* bs,
                              const float4* src, int32_t* s_ryr, int32_t* s_lcc, int32_t* s_lccv,
                              double* s_res, int32_t* s_nb, int lane) {
  const int NR = a.C.NR, NL = a.C.NL;
  const uint32_t mask = (1u << a.off_bits) - 1u;
  const srs_gate_consts* g = &a.P_.gc[ctl.vsel];
  const bool coupled = g->ryr_astar_half != 0.0f;
  if (coupled) {
    for (int i = lane; i < NR; i += 32) {
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
    __syncwarp();
  }
  for (int i = lane; i < NR; i += 32) {
    int no = 0, nc = 0;
    if (coupled) {
      no = s_nb[i] & 0xffff;
      nc = s_nb[i] >> 16;
    }
    float cs = resident_u<C>(a, bs, src, a.ryr_cleft_code[i], mask) + a.k.c0;
    float cj = resident_u<C>(a, bs, src, a.ryr_jsr_code[i], mask) + a.k.c0j;
    double rr = s_res[i];
    s_ryr[i] = srs_gate_ryr(g, s_ryr[i], cs, cj, no, nc, &rr, ctl.seed, (uint32_t)i,
                            (uint64_t)ctl.step);
    s_res[i] = rr;
  }
  for (int i = lane; i < NL; i += 32) {
    float cs = resident_u<C>(a, bs, src, a.lcc_code[i], mask) + a.lcc_rest[i];
    double rr = s_res[NR + i];
    int st = s_lcc[i], vs = s_lccv[i];
    srs_gate_lcc(g, &st, &vs, cs, &rr, ctl.seed, (uint32_t)(NR + i), (uint64_t)ctl.step);
    s_lcc[i] = st;
    s_lccv[i] = vs;
    s_res[NR + i] = rr;
  }
  __syncwarp();
}

template <int C>
__global__ void __launch_bounds__(1024, 1) k_resident32(ResidentArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int P = a.P;
  float4* buf0 = reinterpret_cast<float4*>(smem);
  float4* buf1 = buf0 + P;
  float* imm0 = reinterpret_cast<float*>(buf1 + P);
  float* imm1 = imm0 + P;
  const int NR = a.C.NR, NL = a.C.NL, NCH = NR + NL;
  ResidentSmemTail* tail = reinterpret_cast<ResidentSmemTail*>(imm1 + P);
  int32_t* s_ryr = reinterpret_cast<int32_t*>(tail + 1);
  int32_t* s_lcc = s_ryr + NR;
  int32_t* s_lccv = s_lcc + NL;
  int32_t* s_nb = s_lccv + NL;
  float* s_jr = reinterpret_cast<float*>(s_nb + NR);
  float* s_jl = s_jr + NR;
  double* s_res = reinterpret_cast<double*>(
      (reinterpret_cast<uintptr_t>(s_jl + NL) + 7) & ~(uintptr_t)7);

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
  const int n_ch = a.n_chtet[rank];
  const TetRec* geo = a.geo + (size_t)rank * P;
  const uint32_t off_mask = (1u << a.off_bits) - 1u;
  const Consts32& k = a.k;
  const Protocol& P_ = a.P_;

  if (tid < 32) {
    for (int q = lane; q < C; q += 32) {
      tail->base[0][q] = (C > 1) ? map_rank(smem_addr(buf0), q) : smem_addr(buf0);
      tail->base[1][q] = (C > 1) ? map_rank(smem_addr(buf1), q) : smem_addr(buf1);
    }
  }
  if (tid == 0) tail->bad = 0;
  step_barrier<C>();  // all CTAs of the cluster are running before DSMEM use
  int bad = 0;

  for (int r = cid; r < a.R; r += ncl) {
    // ---- load the realization ----------------------------------------------
    const float4* Mg = a.M + ((size_t)r * C + rank) * P;
    const float* Ig = a.I + ((size_t)r * C + rank) * P;
    for (int i = tid; i < n_loc; i += nthr) {
      buf0[i] = Mg[i];
      imm0[i] = Ig[i];
    }
    if (tid == 0) {
      tail->ctl = a.CS.ctl[r];
      tail->done_flag[1] = tail->ctl.done;
    }
    for (int i = tid; i < NR; i += nthr) s_ryr[i] = a.CS.ryr[(size_t)r * NR + i];
    for (int i = tid; i < NL; i += nthr) {
      s_lcc[i] = a.CS.lcc[(size_t)r * NL + i];
      s_lccv[i] = a.CS.lccv[(size_t)r * NL + i];
    }
    for (int i = tid; i < NCH; i += nthr) s_res[i] = a.CS.res[(size_t)r * NCH + i];
    step_barrier<C>();
    const bool skip = tail->done_flag[1] != 0;
    int cur = 0;
    if (!skip) {
      for (int s = 0; s < a.steps; ++s) {
        const float4* src = cur ? buf1 : buf0;
        float4* dst = cur ? buf0 : buf1;
        const float* isrc = cur ? imm1 : imm0;
        float* idst = cur ? imm0 : imm1;
        const uint32_t* bs = tail->base[cur];
        if (warp == 0) {
          // ---- channel work ------------------------------------------------
          RealCtl& ctl = tail->ctl;
          if (s > 0) {
            if (!P_.nogating) resident_gate<C>(a, ctl, bs, src, s_ryr, s_lcc, s_lccv, s_res, s_nb, lane);
            if (lane == 0) {
              ctl.step += 1;
              ctl.t += P_.dt;
            }
            __syncwarp();
          }
          if (lane == 0) {
            ResidentCa<C> cab{&a, bs, src, off_mask};
            if (rank == 0) {
              prestep(P_, a.C, ctl, s_ryr, s_lcc, s_lccv,
                      a.CS.rows + (size_t)r * P_.row_cap * P_.row_w, cab);
            } else {
              // the other CTAs of the cluster track the same protocol state
              // without writing rows
              Protocol Pq = P_;
              Pq.row_cap = 0;
              const int64_t nr = ctl.n_rows;
              const uint32_t st = ctl.status;
              prestep(Pq, a.C, ctl, s_ryr, s_lcc, s_lccv, a.CS.rows, cab);
              ctl.n_rows = nr;
              ctl.status = st;
            }
            tail->done_flag[s & 1] = ctl.done;
          }
          __syncwarp();
          if (!ctl.done) {
            // release flux of every channel for this step
            const int v = ctl.vsel;
            for (int i = lane; i < NR; i += 32) {
              float J = 0.0f;
              if (s_ryr[i]) {
                float us = resident_u<C>(a, bs, src, a.ryr_cleft_code[i], off_mask);
                float uj = resident_u<C>(a, bs, src, a.ryr_jsr_code[i], off_mask);
                J = k.jr_scale * ((k.dc0 + uj) - us);
              }
              s_jr[i] = J;
            }
            for (int i = lane; i < NL; i += 32) {
              float J = 0.0f;
              if ((s_lcc[i] == 6 || s_lcc[i] == 12) && s_lccv[i] == 2) {
                float c = a.lcc_rest[i] + resident_u<C>(a, bs, src, a.lcc_code[i], off_mask);
                J = k.lccA[v] * fmaf(c, k.lccE[v], -k.lccB);
              }
              s_jl[i] = J;
            }
            __syncwarp();
            // channel elements of this partition
            const int32_t* cp = a.ch_ptr + (size_t)rank * a.ch_stride;
            for (int i = lane; i < n_ch; i += 32) {
              const TetRec g = geo[i];
              float flux = 0.0f;
              for (int q = cp[i]; q < cp[i + 1]; ++q) {
                ChanEntry32 e = a.ch_list[q];
                float J = (e.kind < 2) ? s_jr[e.ch] : s_jl[e.ch];
                flux = fmaf(J, e.s, flux);
              }
              float4 nv[4];
#pragma unroll
              for (int q = 0; q < 4; ++q) nv[q] = resident_nb<C>(bs, src, g.nb[q], a.off_bits, off_mask);
              float4 out;
              float imo;
              tet_update(k, src[i], isrc[i], nv[0], nv[1], nv[2], nv[3],
                         make_float4(g.a[0], g.a[1], g.a[2], g.a[3]), g.flags, g.bsl, 0.0f, flux,
                         &out, &imo);
              dst[i] = out;
              idst[i] = imo;
              bad |= !isfinite(out.x);
            }
          }
        } else {
          // ---- all other elements ------------------------------------------
          const int t0 = tid - 32, tstride = nthr - 32;
          for (int i = n_ch + t0; i < n_loc; i += tstride) {
            const float4* gp = reinterpret_cast<const float4*>(geo + i);
            float4 ga = __ldg(gp);
            float4 gb = __ldg(gp + 1);
            uint32_t w0 = __float_as_uint(gb.x), w1 = __float_as_uint(gb.y);
            uint32_t c0 = w0 & 0xffffu, c1 = w0 >> 16, c2 = w1 & 0xffffu, c3 = w1 >> 16;
            float4 n0, n1, n2, n3;
            if constexpr (C == 1) {
              n0 = ld_smem_f4(bs[0] + c0 * 16u);
              n1 = ld_smem_f4(bs[0] + c1 * 16u);
              n2 = ld_smem_f4(bs[0] + c2 * 16u);
              n3 = ld_smem_f4(bs[0] + c3 * 16u);
            } else {
              n0 = ld_dsmem_f4(bs[c0 >> a.off_bits] + (c0 & off_mask) * 16u);
              n1 = ld_dsmem_f4(bs[c1 >> a.off_bits] + (c1 & off_mask) * 16u);
              n2 = ld_dsmem_f4(bs[c2 >> a.off_bits] + (c2 & off_mask) * 16u);
              n3 = ld_dsmem_f4(bs[c3 >> a.off_bits] + (c3 & off_mask) * 16u);
            }
            float4 out;
            float imo;
            tet_update(k, src[i], isrc[i], n0, n1, n2, n3, ga, __float_as_uint(gb.w), gb.z, 0.0f,
                       0.0f, &out, &imo);
            dst[i] = out;
            idst[i] = imo;
            bad |= !isfinite(out.x);
          }
        }
        step_barrier<C>();
        if (tail->done_flag[s & 1]) break;
        cur ^= 1;
      }
      if (!tail->ctl.done && warp == 0) {
        // gating after the last step of this launch (the next launch starts
        // with the protocol work of the following step)
        RealCtl& ctl = tail->ctl;
        const float4* src = cur ? buf1 : buf0;
        const uint32_t* bs = tail->base[cur];
        if (!P_.nogating) resident_gate<C>(a, ctl, bs, src, s_ryr, s_lcc, s_lccv, s_res, s_nb, lane);
        if (lane == 0) {
          ctl.step += 1;
          ctl.t += P_.dt;
        }
        __syncwarp();
      }
    }
    step_barrier<C>();
    // ---- store the realization ----------------------------------------------
    {
      const float4* fin = cur ? buf1 : buf0;
      const float* ifin = cur ? imm1 : imm0;
      float4* Mw = a.M + ((size_t)r * C + rank) * P;
      float* Iw = a.I + ((size_t)r * C + rank) * P;
      if (!skip) {
        for (int i = tid; i < n_loc; i += nthr) {
          Mw[i] = fin[i];
          Iw[i] = ifin[i];
        }
      }
      if (rank == 0 && !skip) {
        for (int i = tid; i < NR; i += nthr) a.CS.ryr[(size_t)r * NR + i] = s_ryr[i];
        for (int i = tid; i < NL; i += nthr) {
          a.CS.lcc[(size_t)r * NL + i] = s_lcc[i];
          a.CS.lccv[(size_t)r * NL + i] = s_lccv[i];
        }
        for (int i = tid; i < NCH; i += nthr) a.CS.res[(size_t)r * NCH + i] = s_res[i];
        if (tid == 0) a.CS.ctl[r] = tail->ctl;
      }
    }
    step_barrier<C>();  // smem reused by the next realization
  }
  if (bad) atomicOr(&tail->bad, 1);
  __syncthreads();
  if (tid == 0 && tail->bad) atomicOr(&a.CS.ctl[0].status, 1u);
  step_barrier<C>();  // no CTA leaves while others may read its shared memory
}

size_t resident_smem_bytes(int P, int NR, int NL) {
  size_t b = (size_t)P * (2 * sizeof(float4) + 2 * sizeof(float));
  b += sizeof(ResidentSmemTail);
  b += (size_t)(NR + 2 * NL + NR) * sizeof(int32_t);
  b += (size_t)(NR + NL) * sizeof(float);
  b = (b + 7) & ~(size_t)7;
  b += (size_t)(NR + NL) * sizeof(double);
  return b;
}

template <int C>
static int launch_resident_t(const ResidentArgs& a, int n_clusters, int threads, size_t smem,
                             cudaStream_t st) {
  auto fn = k_resident32<C>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return -1;
  if (C > 8) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return -1;
  }
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
  e = cudaLaunchKernelEx(&cfg, fn, a);
  return e == cudaSuccess ? 0 : -1;
}

int launch_resident(const ResidentArgs& a, int C, int n_clusters, int threads, size_t smem,
                    cudaStream_t st) {
  switch (C) {
    case 1: return launch_resident_t<1>(a, n_clusters, threads, smem, st);
    case 2: return launch_resident_t<2>(a, n_clusters, threads, smem, st);
    case 4: return launch_resident_t<4>(a, n_clusters, threads, smem, st);
    case 8: return launch_resident_t<8>(a, n_clusters, threads, smem, st);
    case 16: return launch_resident_t<16>(a, n_clusters, threads, smem, st);
    default: return -1;
  }
}

// Largest number of co-resident clusters for a configuration (0: does not fit).
int resident_max_clusters(int C, int threads, size_t smem) {
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
  cudaError_t e;
  switch (C) {
#define SRS_MC(CC)                                                                        \
  case CC:                                                                                \
    cudaFuncSetAttribute(k_resident32<CC>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                         (int)smem);                                                      \
    if (CC > 8)                                                                           \
      cudaFuncSetAttribute(k_resident32<CC>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1); \
    e = cudaOccupancyMaxActiveClusters(&n, k_resident32<CC>, &cfg);                       \
    break;
    SRS_MC(1) SRS_MC(2) SRS_MC(4) SRS_MC(8) SRS_MC(16)
#undef SRS_MC
    default: return 0;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace srs
