// k_plain64.cu — FP64 spark step in the reference's operation order.
//
// One fused launch per time step: every thread advances one element of one
// realization through the whole of ExplicitStep (cpu/RunSimulation.cpp:
// 591-654) — ELL-4 diffusion of the four mobile species, buffer reactions,
// SERCA, JSR refill, RyR/LCC flux, rapid SL buffer, Euler update — reading
// the state of step n and writing step n+1 (double buffered).  The last
// block of each realization to finish then runs channel gating and the
// protocol work of the next step, so a step is a single launch.
//
// Every expression keeps the reference's association order and this file is
// compiled with -fmad=false, so with identical inputs the result matches the
// reference's FP64 step bit for bit.  This engine is the FP64 oracle run of
// the GPU path; the FP32 engines are measured against it.
#include "srs_engine.h"
#include "srs_protocol.cuh"

namespace srs {


__device__ __forceinline__ double plain64_ca(const double* S_r, int e) { return S_r[e]; }

__global__ void __launch_bounds__(256) k_plain64_step(Plain64Args a) {
  const int r = blockIdx.y;
  RealCtl* ctlp = a.CS.ctl + r;
  if (ctlp->done) return;  // uniform per realization
  const int N = a.N;
  const double* S = a.S_in + (size_t)r * 6 * N;
  double* So = a.S_out + (size_t)r * 6 * N;
  const int32_t* ryr = a.CS.ryr + (size_t)r * a.C.NR;
  const int32_t* lcc = a.CS.lcc + (size_t)r * a.C.NL;
  const int32_t* lccv = a.CS.lccv + (size_t)r * a.C.NL;
  const double* p = a.p;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < N) {
    const double* Sca = S + 0 * N;
    const double* Satp = S + 1 * N;
    const double* Scmdn = S + 2 * N;
    const double* Strpn = S + 3 * N;
    const double* Scsqn = S + 4 * N;
    const double* Sdye = S + 5 * N;
    double c_ca = Sca[j];
    double a0 = a.aij[5 * j], a1 = a.aij[5 * j + 1], a2 = a.aij[5 * j + 2];
    double a3 = a.aij[5 * j + 3], a4 = a.aij[5 * j + 4];
    int n1 = a.nij[4 * j], n2 = a.nij[4 * j + 1], n3 = a.nij[4 * j + 2], n4 = a.nij[4 * j + 3];
    // UpdateReactionTerms (cpu/RunSimulation.cpp:25-125)
    double b_ca = p[5] * (c_ca * a0 + Sca[n1] * a1 + Sca[n2] * a2 + Sca[n3] * a3 + Sca[n4] * a4) +
                  a.br[0 * N + j];
    double b_dye = p[11] * (Sdye[j] * a0 + Sdye[n1] * a1 + Sdye[n2] * a2 + Sdye[n3] * a3 +
                            Sdye[n4] * a4) + a.br[3 * N + j];
    double b_atp = p[7] * (Satp[j] * a0 + Satp[n1] * a1 + Satp[n2] * a2 + Satp[n3] * a3 +
                           Satp[n4] * a4) + a.br[1 * N + j];
    double b_cmdn = p[8] * (Scmdn[j] * a0 + Scmdn[n1] * a1 + Scmdn[n2] * a2 + Scmdn[n3] * a3 +
                            Scmdn[n4] * a4) + a.br[2 * N + j];
    double b_trpn = 0, b_csqn = 0;
    const int fl = a.flags[j];
    double r_net, c_b;
    if (!(fl & 1)) {
      if (fl & 2) {
        c_b = Strpn[j];
        r_net = p[26] * (p[24] - c_b) * c_ca - p[25] * c_b;
        b_ca += -r_net;
        b_trpn = r_net;
        double K_i = c_ca / p[49];
        K_i = K_i * K_i;
        double K_sr = a.nsr / p[50];
        K_sr = K_sr * K_sr;
        double D_cycle = 0.104217 + 17.923 * K_sr + K_i * (1.75583e6 + K_sr * 7.61673e6) +
                         K_i * K_i * (6.08463e11 + K_sr * 4.50544e11);
        double v_cycle =
            (K_i * K_i * 3.24873e12 + K_i * (9.17846e6 - 11478.2 * K_sr) - 0.329904 * K_sr) /
            D_cycle;
        double d_ca = (2e-3) * v_cycle * p[51];
        b_ca -= d_ca;
      }
      c_b = Sdye[j];
      r_net = p[33] * (p[31] - c_b) * c_ca - p[32] * c_b;
      b_ca += -r_net;
      b_dye += r_net;
      c_b = Satp[j];
      r_net = p[20] * (p[18] - c_b) * c_ca - p[19] * c_b;
      b_ca += -r_net;
      b_atp += r_net;
      c_b = Scmdn[j];
      r_net = p[23] * (p[21] - c_b) * c_ca - p[22] * c_b;
      b_ca += -r_net;
      b_cmdn += r_net;
    } else {
      c_b = Scsqn[j];
      r_net = p[39] * (p[34] - c_b) * c_ca - p[40] * c_b;
      b_ca += -r_net;
      b_csqn = r_net;
      b_ca += (a.nsr - c_ca) * p[36];
    }
    // Channel fluxes (UpdateRyRFlux / UpdateLCCFlux, :127-164), in order.
    if (fl & 4) {
      const int v = ctlp->vsel;
      for (int q = a.chan_ptr[j]; q < a.chan_ptr[j + 1]; ++q) {
        ChanEntry e = a.chan_list[q];
        if (e.kind == 0) {
          if (ryr[e.ch]) {
            double J = a.P.v_ryr * (Sca[a.C.ryr_jsr[e.ch]] - Sca[a.C.ryr_cleft[e.ch]]) * a.P.v_cell;
            b_ca += J / a.v0[j];
          }
        } else if (e.kind == 1) {
          if (ryr[e.ch]) {
            double J = a.P.v_ryr * (Sca[a.C.ryr_jsr[e.ch]] - Sca[a.C.ryr_cleft[e.ch]]) * a.P.v_cell;
            b_ca -= J / a.v0[j];
          }
        } else {
          if ((lcc[e.ch] == 6 || lcc[e.ch] == 12) && lccv[e.ch] == 2) {
            double J = a.P.lccA[v] * (c_ca * a.P.lccE[v] - a.P.lccB) / a.P.lccEm1[v] / a.v0[j];
            b_ca += J;
          }
        }
      }
    }
    // UpdateFastBuffer (:15-22)
    {
      double khi = p[28], klo = p[30];
      double B = 1 + (a.bhi[j] * khi / ((khi + c_ca) * (khi + c_ca))) +
                 (a.blo[j] * klo / ((klo + c_ca) * (klo + c_ca)));
      b_ca /= B;
    }
    // Euler update (:640-644)
    const double dt = a.P.dt;
    double* O = So;
    O[0 * N + j] = c_ca + b_ca * dt;
    O[1 * N + j] = Satp[j] + b_atp * dt;
    O[2 * N + j] = Scmdn[j] + b_cmdn * dt;
    O[3 * N + j] = Strpn[j] + b_trpn * dt;
    O[4 * N + j] = Scsqn[j] + b_csqn * dt;
    O[5 * N + j] = Sdye[j] + b_dye * dt;
    if (!isfinite(O[j])) atomicOr(&ctlp->status, 1u);
  }
  // ---- last block of this realization: gating + next step's protocol ----
  __shared__ int s_last;
  __shared__ int32_t s_nb[1024];
  // the last block gates from the new Ca of the channel elements: blocks
  // holding channel elements make their writes visible before counting in
  if (__syncthreads_or(j < N && (a.flags[j] & 4) != 0)) {
    __threadfence();
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    unsigned int done = atomicAdd(a.counters + r, 1u);
    s_last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  RealCtl ctl = *ctlp;
  const double* Sn = So;  // Ca after the update
  auto ca = [&](int e) -> double { return *((volatile const double*)(Sn + e)); };
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

// Protocol work before the first step of a run (and the t = 0 row).
__global__ void k_plain64_prestep(Plain64Args a, int write_initial_row) {
  const int r = blockIdx.x;
  if (threadIdx.x != 0) return;
  RealCtl ctl = a.CS.ctl[r];
  const double* S = a.S_in + (size_t)r * 6 * a.N;
  auto ca = [&](int e) -> double { return S[e]; };
  int32_t* ryr = a.CS.ryr + (size_t)r * a.C.NR;
  int32_t* lcc = a.CS.lcc + (size_t)r * a.C.NL;
  int32_t* lccv = a.CS.lccv + (size_t)r * a.C.NL;
  float* rows = a.CS.rows + (size_t)r * a.P.row_cap * a.P.row_w;
  if (write_initial_row && a.P.run_protocol) write_row(a.P, a.C, ctl, ryr, lcc, lccv, rows, ctl.t, ca);
  prestep(a.P, a.C, ctl, ryr, lcc, lccv, rows, ca);
  a.CS.ctl[r] = ctl;
}

int launch_plain64_step(const Plain64Args& a, cudaStream_t st) {
  // Few realizations: 64-thread blocks spread the element updates (and their
  // FP64 arithmetic) over more SMs than 256-thread blocks would.
  const int bs = (size_t)((a.N + 255) / 256) * a.R < 304 ? 64 : 256;
  dim3 grid((a.N + bs - 1) / bs, a.R);
  k_plain64_step<<<grid, bs, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
int launch_plain64_prestep(const Plain64Args& a, int write_initial_row, cudaStream_t st) {
  k_plain64_prestep<<<a.R, 32, 0, st>>>(a, write_initial_row);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace srs
