// k_fp32.cu — FP32 spark step engines.
//
// State is stored as deviations from the resting equilibrium (u = c - c_rest,
// per species; Ca relative to the resting level of its own domain), and the
// buffer reactions are written in the cancellation-free deviation form
//   r = kon*((B - b_rest)*u - c*u_b) - koff*u_b,
// which is the reference's kon*(B - b)*c - koff*b (cpu/RunSimulation.cpp:
// 78, 95, 101, 107, 115) minus its value at rest (zero at equilibrium).  The
// explicit Euler update u += dt*r is compensated (Kahan summation): each
// element keeps the rounding error of its last update and feeds it back, so
// the tiny per-step increments (dt = 9 ns) do not accumulate a rounding bias
// over millions of steps.  Compensation terms are private to the element's
// owner thread and never travel to neighbours; both engines keep them as
// halves of c * 2^24 (srs_comp.h), rounded after every update.
//
// Two engines share the per-element update `tet_update`:
//   * k_plain32_step: one launch per time step, state in HBM, grid.y over
//     realizations, last block per realization runs gating + protocol;
//   * k_resident32<C>: persistent batched kernel.  One realization at a time
//     per thread-block cluster of C CTAs; the mobile species (Ca, ATP, CMDN,
//     dye) live in shared memory as float4, double buffered, partitioned over
//     the cluster; neighbours in another CTA's partition are read through
//     distributed shared memory.  Every element that carries a channel sits in
//     partition 0, where warp 0 computes the release flux, updates those
//     elements, gates the channels and runs the protocol of the next step
//     while the other warps update everything else — one cluster barrier per
//     time step, and the termination decision is known at that barrier.
#include "k_resident.cuh"
#include "srs_adjoint.cuh"
#include "srs_engine.h"
#include "srs_fp32_update.cuh"
#include "srs_protocol.cuh"

namespace srs {

// ===========================================================================
// Plain FP32 engine
// ===========================================================================
// One element of one realization: release flux of its channels, then the
// FP32 update (tet_update).  TRAJ: also record the state the step starts
// from and the Ca rate (the adjoint's trajectory).
template <bool TRAJ>
__device__ __forceinline__ void plain32_element(const Plain32Args& a, int r, int j) {
  RealCtl* ctlp = a.CS.ctl + r;
  const int N = a.N;
  const float4* M = a.M_in + (size_t)r * N;
  const float* I = a.I_in + (size_t)r * N;
  float4* Mo = a.M_out + (size_t)r * N;
  float* Io = a.I_out + (size_t)r * N;
  const uint32_t fl = a.flags[j];
  {
    float flux = 0.0f;
    if (fl & 4u) {
      const int32_t* ryr = a.CS.ryr + (size_t)r * a.C.NR;
      const int32_t* lcc = a.CS.lcc + (size_t)r * a.C.NL;
      const int32_t* lccv = a.CS.lccv + (size_t)r * a.C.NL;
      const int v = ctlp->vsel;
      for (int q = a.chan_ptr[j]; q < a.chan_ptr[j + 1]; ++q) {
        ChanEntry32 e = a.chan_list[q];
        float J = 0.0f;
        if (e.kind < 2) {
          if (ryr[e.ch]) {
            float dc = (a.k.dc0 + M[a.C.ryr_jsr[e.ch]].x) - M[a.C.ryr_cleft[e.ch]].x;
            J = a.k.jr_scale * dc;
          }
        } else if ((lcc[e.ch] == 6 || lcc[e.ch] == 12) && lccv[e.ch] == 2) {
          float c = a.rest_ca[j] + M[j].x;
          J = a.k.lccA[v] * fmaf(c, a.k.lccE[v], -a.k.lccB);
        }
        flux = fmaf(J, e.s, flux);
      }
    }
    const int4 nb = a.nb[j];
    const size_t o = (size_t)r * N + j;
    const float4 x = M[j];
    const float im = I[j];
    float4 cm;
    float ci;
    if (a.CMq) {  // compact compensation (srs_comp.h)
      cm = comp_load4(a.CMq + o);
      ci = comp_load1(a.CIq[o]);
    } else {
      cm = a.CM[o];
      ci = a.CI[o];
    }
    float4 out;
    float imo;
    if constexpr (TRAJ) {
      float g;
      tet_update(a.k, x, im, M[nb.x], M[nb.y], M[nb.z], M[nb.w], a.a[j], fl, a.bsl[j],
                 a.kb ? a.kb[j] : 0.0f, flux, cm, ci, &out, &imo, &g);
      a.traj_u[o] = x;
      a.traj_ig[o] = make_float2(im, g);
      a.traj_ib[o] = sl_inv_factor(a.k, a.bsl[j], ((fl & 1u) ? a.k.c0j : a.k.c0) + x.x);
    } else {
      tet_update(a.k, x, im, M[nb.x], M[nb.y], M[nb.z], M[nb.w], a.a[j], fl, a.bsl[j],
                 a.kb ? a.kb[j] : 0.0f, flux, cm, ci, &out, &imo);
    }
    Mo[j] = out;
    Io[j] = imo;
    if (a.CMq) {
      comp_store4(a.CMq + o, cm);
      a.CIq[o] = comp_store1(ci);
    } else {
      a.CM[o] = cm;
      a.CI[o] = ci;
    }
    if (!isfinite(out.x)) atomicOr(&ctlp->status, 1u);
  }
}

// Gating of one realization's channels from the new state, then the
// protocol of the next step (one block).  TRAJ: first record the channel
// states the step used.
template <bool TRAJ>
__device__ __forceinline__ void plain32_gate(const Plain32Args& a, int r, int32_t* s_nb) {
  RealCtl* ctlp = a.CS.ctl + r;
  float4* Mo = a.M_out + (size_t)r * a.N;
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
  if constexpr (TRAJ) {
    const int NR = a.C.NR, NL = a.C.NL, W = NR + 2 * NL + 1;
    int32_t* rec = a.traj_ch + (size_t)r * W;
    for (int q = threadIdx.x; q < NR; q += blockDim.x) rec[q] = ryr_w[q];
    for (int q = threadIdx.x; q < NL; q += blockDim.x) {
      rec[NR + q] = lcc_w[q];
      rec[NR + NL + q] = lccv_w[q];
    }
    if (threadIdx.x == 0) rec[W - 1] = ctl.vsel;
    __syncthreads();
  }
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

// Small meshes: one launch per time step.  Grid: x over realizations, y over
// blocks of 256 elements, so the blocks that run together share the geometry
// of one element range in L2; the last block of a realization gates.
template <bool TRAJ>
__global__ void __launch_bounds__(256) k_plain32_step(Plain32Args a) {
  const int r = blockIdx.x;
  if (a.CS.ctl[r].done) return;
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  const uint32_t fl = j < a.N ? a.flags[j] : 0u;
  if (j < a.N) plain32_element<TRAJ>(a, r, j);
  __shared__ int s_last;
  __shared__ int32_t s_nb[1024];
  // The last block of the realization gates its channels from the new Ca of
  // the channel elements, so blocks holding channel elements make their
  // writes visible before they count themselves in; the others need not.
  if (__syncthreads_or((fl & 4u) != 0)) {
    __threadfence();
    __syncthreads();
  }
  if (threadIdx.x == 0) s_last = (atomicAdd(a.counters + r, 1u) == gridDim.y - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  plain32_gate<TRAJ>(a, r, s_nb);
}

// Large meshes: the element update alone, without the gating code, so it
// runs at six blocks per SM; k_plain32_gate follows as its own launch.  The
// first thread of each block asks L2 for the state this realization needs
// pf_rows element blocks later (about one wave of blocks ahead), so those
// blocks find it there instead of waiting on DRAM.
template <bool TRAJ>
__global__ void __launch_bounds__(256, 6) k_plain32_update(Plain32Args a) {
  const int r = blockIdx.x;
  if (a.CS.ctl[r].done) return;
  if (threadIdx.x == 0 && a.pf_rows > 0 && blockIdx.y + a.pf_rows < gridDim.y) {
    const size_t e0 = (size_t)(blockIdx.y + a.pf_rows) * blockDim.x;
    const size_t n = min((size_t)blockDim.x, (size_t)a.N - e0);
    const size_t o = (size_t)r * a.N + e0;
    prefetch_span(a.M_in + o, n * sizeof(float4));
    prefetch_span(a.I_in + o, n * sizeof(float));
    if (a.CMq) {
      prefetch_span(a.CMq + o, n * sizeof(ushort4));
      prefetch_span(a.CIq + o, n * sizeof(uint16_t));
    } else {
      prefetch_span(a.CM + o, n * sizeof(float4));
      prefetch_span(a.CI + o, n * sizeof(float));
    }
  }
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (j < a.N) plain32_element<TRAJ>(a, r, j);
}

template <bool TRAJ>
__global__ void __launch_bounds__(256) k_plain32_gate(Plain32Args a) {
  const int r = blockIdx.x;
  if (a.CS.ctl[r].done) return;
  __shared__ int32_t s_nb[1024];
  plain32_gate<TRAJ>(a, r, s_nb);
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

int plain32_kernels_per_step(const Plain32Args& a) { return a.N >= PLAIN32_SPLIT_N ? 2 : 1; }

int launch_plain32_step(const Plain32Args& a, cudaStream_t st) {
  if ((a.N + 255) / 256 > 65535) return -1;  // grid y limit: 16.7 M elements
  dim3 grid(a.R, (a.N + 255) / 256);
  const bool traj = a.traj_u != nullptr;
  if (a.N >= PLAIN32_SPLIT_N) {
    if (traj) {
      k_plain32_update<true><<<grid, 256, 0, st>>>(a);
      k_plain32_gate<true><<<a.R, 256, 0, st>>>(a);
    } else {
      k_plain32_update<false><<<grid, 256, 0, st>>>(a);
      k_plain32_gate<false><<<a.R, 256, 0, st>>>(a);
    }
  } else {
    // few realizations: 64-thread blocks spread the step over more SMs
    const int bs = (size_t)((a.N + 255) / 256) * a.R < 304 ? 64 : 256;
    const dim3 g2(a.R, (a.N + bs - 1) / bs);
    if (traj) k_plain32_step<true><<<g2, bs, 0, st>>>(a);
    else k_plain32_step<false><<<g2, bs, 0, st>>>(a);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
int launch_plain32_prestep(const Plain32Args& a, int write_initial_row, cudaStream_t st) {
  k_plain32_prestep<<<a.R, 32, 0, st>>>(a, write_initial_row);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ===========================================================================
// Resident FP32 engine: kernel in k_resident.cuh, instantiated in k_res_*.cu
// ===========================================================================
size_t resident_smem_bytes(int P, int NR, int NL, int n_chtet, int n_entries) {
  // per element: two state buffers, the compact compensation terms of the
  // mobile species, the immobile buffer and its compact compensation term
  size_t b = (size_t)P * (2 * sizeof(float4) + sizeof(ushort4) + sizeof(float) + sizeof(uint16_t));
  b = (b + 15) & ~(size_t)15;
  b += sizeof(ResidentSmemTail);
  b += (size_t)(NR + 2 * NL + NR) * sizeof(int32_t);  // ryr, lcc, lccv, lattice counts
  b += (size_t)(2 * NR + 2 * NL) * sizeof(uint32_t);  // channel element offsets, LCC rest
  b = (b + 7) & ~(size_t)7;
  b += (size_t)(NR + NL) * sizeof(double);
  b += (size_t)(n_chtet + 1) * sizeof(int32_t);
  b = (b + 15) & ~(size_t)15;
  b += (size_t)n_entries * sizeof(ChanEntry32);
  return b;
}

#define SRS_RESIDENT_SIZES(X) X(1) X(2) X(3) X(4) X(5) X(6) X(8) X(16)

int launch_resident(const ResidentArgs& a, int C, int n_clusters, int threads, size_t smem,
                    cudaStream_t st) {
  switch (C) {
#define SRS_L(CC) \
  case CC:        \
    return launch_resident_c##CC(a, n_clusters, threads, smem, st);
    SRS_RESIDENT_SIZES(SRS_L)
#undef SRS_L
    default: return -1;
  }
}

// Largest number of co-resident clusters for a configuration (0: does not fit).
int resident_max_clusters(int C, int threads, size_t smem) {
  switch (C) {
#define SRS_M(CC) \
  case CC:        \
    return resident_max_clusters_c##CC(threads, smem);
    SRS_RESIDENT_SIZES(SRS_M)
#undef SRS_M
    default: return 0;
  }
}

bool resident_cluster_supported(int C) {
  switch (C) {
#define SRS_S(CC) \
  case CC:        \
    return true;
    SRS_RESIDENT_SIZES(SRS_S)
#undef SRS_S
    default: return false;
  }
}

}  // namespace srs
