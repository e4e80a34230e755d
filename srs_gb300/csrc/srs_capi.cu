// srs_capi.cu — the C ABI (include/srs_gb300.h): grids, simulations, engine
// set-up and launch sequencing.  All numerics run in the sm_103a kernels of
// k_plain64.cu / k_fp32.cu; this file packs data, moves it and orders work.
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "srs_engine.h"
#include "srs_host.h"

using namespace srs;

namespace {
thread_local std::string g_err;
int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
#define SRS_CUDA(call)                                                               \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return fail(SRS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
}  // namespace

namespace srs {
// Records an error for srs_last_error() from other translation units.
int set_last_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace srs

struct srs_grid {
  Mesh m;
  Operator op;
  srs_params p;
};

struct srs_sim {
  Mesh m;
  Operator op;
  srs_params p;
  srs_sim_desc d;
  std::vector<uint64_t> seeds;
  int R = 0, N = 0, NR = 0, NL = 0, NCH = 0;
  cudaStream_t st = nullptr;
  std::vector<void*> allocs;
  // element numbering of the engine
  std::vector<int> eng_of_ref, ref_of_eng;
  // FP32 rest values per engine element
  std::vector<double> rest_ca, rest_imm;
  RestValues rv;
  double vm = 0, nsr = 0;
  // channel state (device)
  int32_t *d_ryr = nullptr, *d_lcc = nullptr, *d_lccv = nullptr;
  double* d_res = nullptr;
  RealCtl* d_ctl = nullptr;
  float* d_rows = nullptr;
  int64_t rows_cap_alloc = 0;
  int rows_w_alloc = 0;
  int64_t* d_ticks = nullptr;
  double* d_tick_t = nullptr;
  size_t ticks_cap = 0;  // capacity of d_ticks / d_tick_t (reused across runs)
  unsigned int* d_counters = nullptr;
  Channels ch{};
  Protocol P{};
  // engines
  Plain64Args a64{};
  Plain32Args a32{};
  ResidentArgs ar{};
  double* d_S[2] = {nullptr, nullptr};
  float4* d_M[2] = {nullptr, nullptr};
  float* d_I[2] = {nullptr, nullptr};
  float4* d_CM = nullptr;  // resident FP32 engine: Euler compensation terms
  float* d_CI = nullptr;
  // the plain FP32 engine keeps them compact (srs_comp.h) in these instead
  ushort4* d_CMq = nullptr;
  uint16_t* d_CIq = nullptr;
  int C = 1, threads = 0, n_clusters = 0, P_stride = 0, off_bits = 0;
  int pf_override = -1;  // plain FP32 split form: L2 prefetch distance (-1: one wave)
  size_t smem = 0;
  std::vector<int> part_start, part_len, part_nch, part_nint;  // resident partitions
  int ch_interior = 0;
  int64_t launches = 0;
  cudaGraphExec_t graph_plain = nullptr;
  int graph_plain_len = 0;
  void* h_stage = nullptr;  // pinned host staging for state uploads
  size_t h_stage_bytes = 0;
  // the FP32 staging holds this many copies of one realization's state
  // (the last upload_state_range); 0: unknown content
  int stage_copies = 0;
  // line scan
  LinescanArgs ls{};
  std::vector<double> ls_rest;  // F at the equilibrium state
  double* d_ls_out = nullptr;
  std::vector<int32_t> ls_ptr_h, ls_col_h;  // host copy of the line-scan CSR
  std::vector<double> ls_w_h;
  std::vector<double> ls_pad_h;
  int ls_version = 0;
  // adjoint (built on first use)
  std::vector<float4> aT_h;  // transposed coefficients, engine order (host)
  float* d_ryr_s_cl = nullptr;
  float* d_ryr_s_js = nullptr;
  int32_t* d_wt_ptr = nullptr;
  double* d_ls_base = nullptr;  // resting part of each line-scan sample
  int32_t* d_wt_idx = nullptr;
  double* d_wt_w = nullptr;
  int adj_ls_version = -1;
  AdjRec* d_adj_geo = nullptr;  // reverse-sweep records of the CTA grouping
  int adj_geo_m = 0;
  float4* d_adjp_aT = nullptr;  // plain engine: transposed coefficients [N]
  float2* d_adjp_bs = nullptr;  // plain engine: (bsl, sum a + kb) with the domain flags
  // total Ca (built on first use)
  MassArgs mass{};
  // adjoint work buffers, kept between calls (name -> allocation)
  std::vector<std::pair<void*, size_t>> adj_bufs;
};

namespace {

template <class T>
int dev_upload(srs_sim* s, T** dst, const T* src, size_t n) {
  void* p = nullptr;
  size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  SRS_CUDA(cudaMalloc(&p, bytes));
  s->allocs.push_back(p);
  if (n) SRS_CUDA(cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice));
  *dst = (T*)p;
  return SRS_OK;
}
template <class T>
int dev_alloc(srs_sim* s, T** dst, size_t n) {
  void* p = nullptr;
  SRS_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
  SRS_CUDA(cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T)));
  s->allocs.push_back(p);
  *dst = (T*)p;
  return SRS_OK;
}
#define SRS_TRY(x)          \
  do {                      \
    int rc_ = (x);          \
    if (rc_ != SRS_OK) return rc_; \
  } while (0)

}  // namespace

namespace srs {
// Gating and flux constants for membrane potential V (cpu/RunSimulation.cpp:
// 149-161, 185-197, 239-375), evaluated in double precision on the host.
void gate_consts(const srs_params& p, double V, srs_gate_consts* g) {
  const double* R = p.reals;
  g->ryr_kplus = (float)R[R_RYR_K_PLUS];
  g->ryr_kminus = (float)R[R_RYR_K_MINUS];
  g->ryr_eta = (float)R[R_RYR_ETA];
  g->ryr_phi0 = (float)(1.0 - std::pow(1000.0 / R[R_RYR_PHI_B], R[R_RYR_PHI_M]));
  g->ryr_inv_kphi = (float)(1.0 / R[R_RYR_PHI_B]);
  g->ryr_phin = (float)R[R_RYR_PHI_M];
  g->ryr_astar_half = (float)(0.5 * R[R_RYR_A_STAR]);
  g->ryr_eps_cc = (float)R[R_RYR_EPS_CC];
  g->ryr_eps_oo = (float)R[R_RYR_EPS_OO];
  const double alphacf = 4.0 * 1.2 * 0.416;
  const double betacf = 4.0 * 0.45 * 0.049;
  const double gammacf = 0.83 * 1.9 * 1.3 * 0.31 * 7.5 * 0.09233 / 1000.0;
  g->alpha = (float)(alphacf * std::exp(0.012 * (V - 35.0)));
  g->beta = (float)(betacf * std::exp(-0.05 * (V - 35.0)));
  g->gamma_cf = (float)gammacf;
  const double yCa_frac = 0.4;
  double yCa_inf = yCa_frac / (1.0 + std::exp((V + 12.5) / 5.0)) + (1.0 - yCa_frac);
  double tau_yCa = 60.0 + 340.0 / (1.0 + std::exp((V + 30.0) / 12.0));
  g->lccv_rate_inact_to_act = (float)(yCa_inf / tau_yCa);
  g->lccv_rate_act_to_inact = (float)((1.0 - yCa_inf) / tau_yCa);
  g->dt = R[R_T_STEP];
}

void lcc_flux_consts(const srs_params& p, double V, double* A, double* E, double* Em1, double* B,
                     double* Vg) {
  const double P_CaL = (9.13e-13) * (1e12) * (1e-3);
  const double F = 96.5;
  const double RT = 310 * 8.314;
  const double F_over_RT = F / RT;
  if (std::fabs(V) < 1e-6) V = 1e-6;
  *Vg = V;
  *A = -P_CaL * V * (2 * F_over_RT);
  *E = std::exp(2 * V * F_over_RT);
  *Em1 = std::exp(2 * V * F_over_RT) - 1;
  *B = 0.34 * p.reals[R_CA_0];
}

}  // namespace srs

namespace {

void fill_protocol_consts(srs_sim* s) {
  Protocol& P = s->P;
  const double* R = s->p.reals;
  const int* I = s->p.ints;
  double Vs[2] = {s->vm, R[R_V_CLAMP]};
  for (int v = 0; v < 2; ++v) {
    gate_consts(s->p, Vs[v], &P.gc[v]);
    double Vg;
    lcc_flux_consts(s->p, Vs[v], &P.lccA[v], &P.lccE[v], &P.lccEm1[v], &P.lccB, &Vg);
    P.Vm[v] = Vg;
  }
  P.dt = R[R_T_STEP];
  P.v_ryr = R[R_V_RYR];
  P.v_cell = R[R_V_CELL];
  P.c_min = R[R_C_MIN];
  P.flag_vclamp = I[I_FLAG_V_CLAMP];
  P.flag_lcc = I[I_FLAG_LCC];
  P.lcc_index = I[I_LCC_INDEX];
  P.init_ryr = I[I_INIT_RYR];
  P.flag_fidelity = I[I_FLAG_FIDELITY_SIM];
  P.n_open_max = I[I_N_RYR_FIDELITY];
  P.nogating = I[I_FLAG_NO_GATING];
  P.ryr_out = I[I_FLAG_RYR_OUT];
  P.row_w = SRS_STATES_ROW_BASE + (P.ryr_out ? s->NR : 0);
}

Consts32 make_consts32(const srs_sim* s) {
  const double* R = s->p.reals;
  const RestValues& rv = s->rv;
  Consts32 k{};
  k.D[0] = (float)R[R_D_CA];
  k.D[1] = (float)R[R_D_ATP];
  k.D[2] = (float)R[R_D_CMDN];
  k.D[3] = (float)R[R_D_DYE];
  const int ion[5] = {R_K_ON_DYE, R_K_ON_ATP, R_K_ON_CMDN, R_K_ON_TRPN, R_K_ON_CSQN};
  const int ioff[5] = {R_K_OFF_DYE, R_K_OFF_ATP, R_K_OFF_CMDN, R_K_OFF_TRPN, R_K_OFF_CSQN};
  const double btot[5] = {R[R_B_TOT_DYE], R[R_B_TOT_ATP], R[R_B_TOT_CMDN], R[R_B_TOT_TRPN],
                          R[R_B_T_JSR]};
  const double brest[5] = {rv.dye, rv.atp, rv.cmdn, rv.trpn, rv.csqn};
  for (int q = 0; q < 5; ++q) {
    k.kon[q] = (float)R[ion[q]];
    k.koff[q] = (float)R[ioff[q]];
    k.bfree[q] = (float)(btot[q] - brest[q]);
  }
  k.c0 = (float)rv.ca0;
  k.c0j = (float)rv.ca0_jsr;
  k.inv_kdi = (float)(1.0 / R[R_K_D_i]);
  double Ksr = s->nsr / R[R_K_D_SR];
  Ksr = Ksr * Ksr;
  k.sd0 = (float)(0.104217 + 17.923 * Ksr);
  k.sd1 = (float)(1.75583e6 + Ksr * 7.61673e6);
  k.sd2 = (float)(6.08463e11 + Ksr * 4.50544e11);
  k.sn1 = (float)(9.17846e6 - 11478.2 * Ksr);
  k.sn0 = (float)(0.329904 * Ksr);
  k.serca_scale = (float)(2e-3 * R[R_A_P]);
  k.refill_v = (float)R[R_V_REFILL];
  k.refill0 = (float)((s->nsr - rv.ca0_jsr) * R[R_V_REFILL]);
  k.khi = (float)R[R_K_D_SL_HI];
  k.dt = (float)R[R_T_STEP];
  k.jr_scale = (float)(R[R_V_RYR] * R[R_V_CELL]);
  k.dc0 = (float)(rv.ca0_jsr - rv.ca0);
  for (int v = 0; v < 2; ++v) {
    k.lccA[v] = (float)(s->P.lccA[v] / s->P.lccEm1[v]);
    k.lccE[v] = (float)s->P.lccE[v];
  }
  k.lccB = (float)s->P.lccB;
  return k;
}

// Channel contributions per element in the reference's order, engine numbering.
void chan_lists(const srs_sim* s, std::vector<int32_t>* ptr, std::vector<ChanEntry>* list) {
  const Mesh& m = s->m;
  std::vector<std::vector<ChanEntry>> per(s->N);
  for (int i = 0; i < m.NR; ++i) {
    per[s->eng_of_ref[m.ryr_ele[i]]].push_back({0, i});
    per[s->eng_of_ref[m.ryr_jsr[i]]].push_back({1, i});
  }
  for (int i = 0; i < m.NL; ++i) per[s->eng_of_ref[m.lcc_ele[i]]].push_back({2, i});
  ptr->assign(s->N + 1, 0);
  list->clear();
  for (int e = 0; e < s->N; ++e) {
    (*ptr)[e] = (int32_t)list->size();
    list->insert(list->end(), per[e].begin(), per[e].end());
  }
  (*ptr)[s->N] = (int32_t)list->size();
}

int alloc_channel_state(srs_sim* s) {
  SRS_TRY(dev_alloc(s, &s->d_ryr, (size_t)s->R * s->NR));
  SRS_TRY(dev_alloc(s, &s->d_lcc, (size_t)s->R * s->NL));
  SRS_TRY(dev_alloc(s, &s->d_lccv, (size_t)s->R * s->NL));
  SRS_TRY(dev_alloc(s, &s->d_res, (size_t)s->R * s->NCH));
  SRS_TRY(dev_alloc(s, &s->d_ctl, (size_t)s->R));
  SRS_TRY(dev_alloc(s, &s->d_counters, (size_t)s->R));
  SRS_TRY(dev_alloc(s, &s->d_rows, 8));
  s->rows_cap_alloc = 0;
  s->rows_w_alloc = 0;
  return SRS_OK;
}

ChanState chan_state(const srs_sim* s) {
  ChanState cs;
  cs.ryr = s->d_ryr;
  cs.lcc = s->d_lcc;
  cs.lccv = s->d_lccv;
  cs.res = s->d_res;
  cs.ctl = s->d_ctl;
  cs.rows = s->d_rows;
  return cs;
}

int upload_channels_engine_order(srs_sim* s) {
  std::vector<int32_t> rc(s->NR), rj(s->NR), lc(s->NL);
  for (int i = 0; i < s->NR; ++i) {
    rc[i] = s->eng_of_ref[s->m.ryr_ele[i]];
    rj[i] = s->eng_of_ref[s->m.ryr_jsr[i]];
  }
  for (int i = 0; i < s->NL; ++i) lc[i] = s->eng_of_ref[s->m.lcc_ele[i]];
  int32_t *a, *b, *c, *d;
  SRS_TRY(dev_upload(s, &a, rc.data(), rc.size()));
  SRS_TRY(dev_upload(s, &b, rj.data(), rj.size()));
  SRS_TRY(dev_upload(s, &c, s->m.ryr_nb.data(), s->m.ryr_nb.size()));
  SRS_TRY(dev_upload(s, &d, lc.data(), lc.size()));
  s->ch.NR = s->NR;
  s->ch.NL = s->NL;
  s->ch.ryr_cleft = a;
  s->ch.ryr_jsr = b;
  s->ch.ryr_nb = c;
  s->ch.lcc_ele = d;
  return SRS_OK;
}

// ---- FP64 plain engine (reference numbering) --------------------------------
int setup_plain64(srs_sim* s) {
  const int N = s->N;
  s->eng_of_ref.resize(N);
  s->ref_of_eng.resize(N);
  for (int i = 0; i < N; ++i) s->eng_of_ref[i] = s->ref_of_eng[i] = i;
  Plain64Args& a = s->a64;
  a.N = N;
  a.R = s->R;
  const double* R = s->p.reals;
  std::vector<double> br4(4 * (size_t)N), bhi(N), blo(N);
  for (int j = 0; j < N; ++j) {
    br4[0 * (size_t)N + j] = s->op.br[SP_CA * (size_t)N + j];
    br4[1 * (size_t)N + j] = s->op.br[SP_ATP * (size_t)N + j];
    br4[2 * (size_t)N + j] = s->op.br[SP_CMDN * (size_t)N + j];
    br4[3 * (size_t)N + j] = s->op.br[SP_DYE * (size_t)N + j];
    // btothi / btotlo exactly as UpdateFastBuffer forms them (:17-18)
    bhi[j] = s->m.TT[j] * R[R_B_TOT_SL_HI] / (s->m.V0[j] * (1e-15));
    blo[j] = s->m.TT[j] * R[R_B_TOT_SL_LO] / (s->m.V0[j] * (1e-15));
  }
  std::vector<int32_t> ptr;
  std::vector<ChanEntry> list;
  chan_lists(s, &ptr, &list);
  std::vector<int32_t> flags(N);
  for (int j = 0; j < N; ++j)
    flags[j] = (s->m.domain[j] == DOMAIN_JSR ? 1 : 0) | (s->m.tropc[j] ? 2 : 0) |
               (ptr[j + 1] > ptr[j] ? 4 : 0);
  SRS_TRY(dev_upload(s, (double**)&a.aij, s->op.aij.data(), s->op.aij.size()));
  SRS_TRY(dev_upload(s, (int32_t**)&a.nij, s->op.nij.data(), s->op.nij.size()));
  SRS_TRY(dev_upload(s, (double**)&a.br, br4.data(), br4.size()));
  SRS_TRY(dev_upload(s, (double**)&a.v0, s->m.V0.data(), s->m.V0.size()));
  SRS_TRY(dev_upload(s, (double**)&a.bhi, bhi.data(), bhi.size()));
  SRS_TRY(dev_upload(s, (double**)&a.blo, blo.data(), blo.size()));
  SRS_TRY(dev_upload(s, (int32_t**)&a.flags, flags.data(), flags.size()));
  SRS_TRY(dev_upload(s, (int32_t**)&a.chan_ptr, ptr.data(), ptr.size()));
  SRS_TRY(dev_upload(s, (ChanEntry**)&a.chan_list, list.data(), list.size()));
  for (int b = 0; b < 2; ++b) SRS_TRY(dev_alloc(s, &s->d_S[b], (size_t)s->R * 6 * N));
  for (int q = 0; q < 56; ++q) a.p[q] = R[q];
  SRS_TRY(upload_channels_engine_order(s));
  return SRS_OK;
}

// ---- FP32 engines: checks shared by both ------------------------------------
int check_fp32_supported(const srs_sim* s, bool resident) {
  const Mesh& m = s->m;
  const Operator& op = s->op;
  if (s->p.reals[R_B_TOT_SL_LO] != 0.0)
    return fail(SRS_ERR_UNSUPPORTED, "FP32 engines model only the high-affinity SL buffer");
  for (int i = 0; i < m.NR; ++i)
    if (m.domain[m.ryr_ele[i]] != DOMAIN_CYTO || m.domain[m.ryr_jsr[i]] != DOMAIN_JSR)
      return fail(SRS_ERR_MESH, "RyR " + std::to_string(i) +
                                    ": the FP32 engines need its cleft element in the cytosol and "
                                    "its JSR element in the JSR");
  for (int j = 0; j < m.N; ++j) {
    for (int k = 0; k < 4; ++k) {
      int n = op.nij[4 * (size_t)j + k];
      if (op.aij[5 * (size_t)j + 1 + k] != 0 && m.domain[n] != m.domain[j])
        return fail(SRS_ERR_UNSUPPORTED,
                    "FP32 engines need cytosol and JSR uncoupled by diffusion faces");
    }
    if (op.kb[j] != 0 && (resident || m.domain[j] == DOMAIN_JSR))
      return fail(SRS_ERR_UNSUPPORTED,
                  resident ? "resident engine needs no-flux boundaries (flag_noflux)"
                           : "FP32 engines need Dirichlet faces on cytosolic elements only");
  }
  return SRS_OK;
}

void fp32_rest(srs_sim* s) {
  const int N = s->N;
  s->rest_ca.resize(N);
  s->rest_imm.resize(N);
  for (int e = 0; e < N; ++e) {
    int j = s->ref_of_eng[e];
    bool jsr = s->m.domain[j] == DOMAIN_JSR;
    s->rest_ca[e] = jsr ? s->rv.ca0_jsr : s->rv.ca0;
    s->rest_imm[e] = jsr ? s->rv.csqn : (s->m.tropc[j] ? s->rv.trpn : 0.0);
  }
}

float bsl_of(const srs_sim* s, int j) {
  const double* R = s->p.reals;
  double bhi = s->m.TT[j] * R[R_B_TOT_SL_HI] / (s->m.V0[j] * (1e-15));
  return (float)(bhi * R[R_K_D_SL_HI]);
}

int setup_plain32(srs_sim* s) {
  SRS_TRY(check_fp32_supported(s, false));
  const int N = s->N;
  s->ref_of_eng = rcm_order_by_domain(s->m, s->op);
  s->eng_of_ref.resize(N);
  for (int e = 0; e < N; ++e) s->eng_of_ref[s->ref_of_eng[e]] = e;
  fp32_rest(s);
  Plain32Args& a = s->a32;
  a.N = N;
  a.R = s->R;
  std::vector<float4> A(N);
  std::vector<int4> NB(N);
  std::vector<float> bsl(N), kb(N), rest(N);
  std::vector<uint32_t> flags(N);
  std::vector<int32_t> ptr;
  std::vector<ChanEntry> list;
  chan_lists(s, &ptr, &list);
  bool any_kb = false;
  for (int e = 0; e < N; ++e) {
    int j = s->ref_of_eng[e];
    const double* aj = &s->op.aij[5 * (size_t)j];
    const int* nj = &s->op.nij[4 * (size_t)j];
    A[e] = make_float4((float)aj[1], (float)aj[2], (float)aj[3], (float)aj[4]);
    NB[e] = make_int4(s->eng_of_ref[nj[0]], s->eng_of_ref[nj[1]], s->eng_of_ref[nj[2]],
                      s->eng_of_ref[nj[3]]);
    bsl[e] = bsl_of(s, j);
    kb[e] = (float)s->op.kb[j];
    any_kb |= kb[e] != 0.0f;
    rest[e] = (float)s->rest_ca[e];
    flags[e] = (s->m.domain[j] == DOMAIN_JSR ? 1u : 0u) | (s->m.tropc[j] ? 2u : 0u) |
               (ptr[e + 1] > ptr[e] ? 4u : 0u);
  }
  std::vector<ChanEntry32> l32(list.size());
  for (int e = 0; e < N; ++e) {
    double iv = 1.0 / s->m.V0[s->ref_of_eng[e]];
    for (int q = ptr[e]; q < ptr[e + 1]; ++q) {
      l32[q].kind = list[q].kind;
      l32[q].ch = list[q].ch;
      l32[q].s = (float)(list[q].kind == 1 ? -iv : iv);
      l32[q].pad = 0;
    }
  }
  SRS_TRY(dev_upload(s, (float4**)&a.a, A.data(), A.size()));
  SRS_TRY(dev_upload(s, (int4**)&a.nb, NB.data(), NB.size()));
  SRS_TRY(dev_upload(s, (float**)&a.bsl, bsl.data(), bsl.size()));
  if (any_kb) SRS_TRY(dev_upload(s, (float**)&a.kb, kb.data(), kb.size()));
  else a.kb = nullptr;
  SRS_TRY(dev_upload(s, (uint32_t**)&a.flags, flags.data(), flags.size()));
  SRS_TRY(dev_upload(s, (int32_t**)&a.chan_ptr, ptr.data(), ptr.size()));
  SRS_TRY(dev_upload(s, (ChanEntry32**)&a.chan_list, l32.data(), l32.size()));
  SRS_TRY(dev_upload(s, (float**)&a.rest_ca, rest.data(), rest.size()));
  for (int b = 0; b < 2; ++b) {
    SRS_TRY(dev_alloc(s, &s->d_M[b], (size_t)s->R * N));
    SRS_TRY(dev_alloc(s, &s->d_I[b], (size_t)s->R * N));
  }
  // compensation terms as halves (srs_comp.h), as in the resident engine
  SRS_TRY(dev_alloc(s, &s->d_CMq, (size_t)s->R * N));
  SRS_TRY(dev_alloc(s, &s->d_CIq, (size_t)s->R * N));
  SRS_TRY(upload_channels_engine_order(s));
  return SRS_OK;
}

// ---- FP32 resident engine ----------------------------------------------------
int resident_partition(srs_sim* s, int C, int threads) {
  // Order: the elements that carry channels, then breadth-first layers
  // outward from them over the diffusion faces (so partition 0 holds the
  // channels' neighbourhood and partitions are cut between layers); the
  // sequence is cut into C contiguous partitions that give every element
  // thread the same number of elements (in partition 0 the channel group of
  // 64 threads -- 32 in small CTAs -- takes the channel elements and the
  // gating instead).  Inside each
  // partition: channel elements (partition 0 only), then interior elements
  // (every neighbour in the same partition), then boundary elements.
  const int N = s->N;
  const Mesh& m = s->m;
  const Operator& op = s->op;
  std::vector<int> base = rcm_order_by_domain(m, op);
  std::vector<char> has_ch(N, 0);
  for (int i = 0; i < m.NR; ++i) has_ch[m.ryr_ele[i]] = has_ch[m.ryr_jsr[i]] = 1;
  for (int i = 0; i < m.NL; ++i) has_ch[m.lcc_ele[i]] = 1;
  auto nbr = [&](int j, int k) -> int {
    const int u = op.nij[4 * (size_t)j + k];
    return (u != j && op.aij[5 * (size_t)j + 1 + k] != 0) ? u : -1;
  };
  std::vector<int> seq;
  seq.reserve(N);
  std::vector<char> seen(N, 0);
  auto grow = [&](size_t h) {
    for (; h < seq.size(); ++h)
      for (int k = 0; k < 4; ++k) {
        const int u = nbr(seq[h], k);
        if (u >= 0 && !seen[u]) {
          seen[u] = 1;
          seq.push_back(u);
        }
      }
  };
  for (int j : base)
    if (has_ch[j]) {
      seen[j] = 1;
      seq.push_back(j);
    }
  const int n_ch = (int)seq.size();
  grow(0);
  for (int j : base)
    if (!seen[j]) {
      seen[j] = 1;
      const size_t h = seq.size();
      seq.push_back(j);
      grow(h);
    }
  s->part_start.assign(C, 0);
  s->part_len.assign(C, 0);
  s->part_nch.assign(C, 0);
  s->part_nint.assign(C, 0);
  int Pmax = 0;
  {
    const int ng = threads >= 128 ? 64 : 32;
    const bool split = C > 1 && n_ch > 0 && threads > ng;
    int len0 = (int)((int64_t)N / C);
    if (split) {
      const double lam = (double)(N - n_ch) / ((double)C * threads - ng);
      len0 = std::min(N, std::max(n_ch, n_ch + (int)std::lround(lam * (threads - ng))));
    }
    if (C == 1) len0 = N;
    s->part_start[0] = 0;
    s->part_len[0] = len0;
    for (int q = 1; q < C; ++q) {
      const int b0 = len0 + (int)((int64_t)(N - len0) * (q - 1) / (C - 1));
      const int e0 = len0 + (int)((int64_t)(N - len0) * q / (C - 1));
      s->part_start[q] = b0;
      s->part_len[q] = e0 - b0;
    }
    for (int q = 0; q < C; ++q) Pmax = std::max(Pmax, s->part_len[q]);
  }
  if (n_ch > s->part_len[0])
    return fail(SRS_ERR_UNSUPPORTED, "channel elements do not fit in one partition");
  s->part_nch[0] = n_ch;
  std::vector<int> part_of(N);
  for (int q = 0; q < C; ++q)
    for (int i = 0; i < s->part_len[q]; ++i) part_of[seq[s->part_start[q] + i]] = q;
  auto interior = [&](int j) {
    for (int k = 0; k < 4; ++k) {
      const int u = nbr(j, k);
      if (u >= 0 && part_of[u] != part_of[j]) return false;
    }
    return true;
  };
  s->ch_interior = 1;
  for (int i = 0; i < n_ch; ++i) s->ch_interior &= interior(seq[i]) ? 1 : 0;
  std::vector<int> order;
  order.reserve(N);
  for (int q = 0; q < C; ++q) {
    const int b0 = s->part_start[q], e0 = b0 + s->part_len[q];
    const int c0 = q == 0 ? n_ch : 0;
    for (int i = b0; i < b0 + c0; ++i) order.push_back(seq[i]);
    for (int i = b0 + c0; i < e0; ++i)
      if (interior(seq[i])) order.push_back(seq[i]);
    s->part_nint[q] = (int)order.size() - b0 - c0;
    for (int i = b0 + c0; i < e0; ++i)
      if (!interior(seq[i])) order.push_back(seq[i]);
  }
  int bits = 1;
  while ((1 << bits) < Pmax) ++bits;
  int rank_bits = 0;
  while ((1 << rank_bits) < C) ++rank_bits;
  if (bits + rank_bits > 16) return fail(SRS_ERR_UNSUPPORTED, "partition too large for 16-bit element codes");
  s->off_bits = bits;
  s->P_stride = (Pmax + 3) & ~3;
  s->ref_of_eng.assign((size_t)C * s->P_stride, -1);
  s->eng_of_ref.assign(N, -1);
  for (int q = 0; q < C; ++q)
    for (int i = 0; i < s->part_len[q]; ++i) {
      int j = order[s->part_start[q] + i];
      s->ref_of_eng[(size_t)q * s->P_stride + i] = j;
      s->eng_of_ref[j] = q * s->P_stride + i;
    }
  return SRS_OK;
}

uint16_t code_of(const srs_sim* s, int eng) {
  int q = eng / s->P_stride, off = eng % s->P_stride;
  return (uint16_t)((q << s->off_bits) | off);
}

int setup_resident(srs_sim* s, int C, int threads) {
  SRS_TRY(check_fp32_supported(s, true));
  SRS_TRY(resident_partition(s, C, threads));
  const int N = s->N;
  const int NE = C * s->P_stride;
  // rest arrays over the padded engine numbering
  s->rest_ca.assign(NE, 0.0);
  s->rest_imm.assign(NE, 0.0);
  for (int e = 0; e < NE; ++e) {
    int j = s->ref_of_eng[e];
    if (j < 0) continue;
    bool jsr = s->m.domain[j] == DOMAIN_JSR;
    s->rest_ca[e] = jsr ? s->rv.ca0_jsr : s->rv.ca0;
    s->rest_imm[e] = jsr ? s->rv.csqn : (s->m.tropc[j] ? s->rv.trpn : 0.0);
  }
  std::vector<TetRec> geo(NE);
  std::memset(geo.data(), 0, geo.size() * sizeof(TetRec));
  std::vector<int32_t> ptr_all;
  std::vector<ChanEntry> list_all;
  {
    // per-element lists in engine numbering (N here is the padded count)
    std::vector<std::vector<ChanEntry>> per(NE);
    for (int i = 0; i < s->m.NR; ++i) {
      per[s->eng_of_ref[s->m.ryr_ele[i]]].push_back({0, i});
      per[s->eng_of_ref[s->m.ryr_jsr[i]]].push_back({1, i});
    }
    for (int i = 0; i < s->m.NL; ++i) per[s->eng_of_ref[s->m.lcc_ele[i]]].push_back({2, i});
    const int n_ch = s->part_nch[0];
    std::vector<int32_t> cptr(n_ch + 1, 0);
    std::vector<ChanEntry32> clist;
    for (int i = 0; i < n_ch; ++i) {
      cptr[i] = (int32_t)clist.size();
      double iv = 1.0 / s->m.V0[s->ref_of_eng[i]];
      for (auto& ce : per[i]) clist.push_back({ce.kind, ce.ch, (float)(ce.kind == 1 ? -iv : iv), 0});
    }
    cptr[n_ch] = (int32_t)clist.size();
    SRS_TRY(dev_upload(s, (int32_t**)&s->ar.ch_ptr, cptr.data(), cptr.size()));
    SRS_TRY(dev_upload(s, (ChanEntry32**)&s->ar.ch_list, clist.data(), clist.size()));
    for (int e = 0; e < NE; ++e) {
      int j = s->ref_of_eng[e];
      if (j < 0) {
        // padding slot: isolated element with zero coefficients
        for (int k = 0; k < 4; ++k) geo[e].nb[k] = code_of(s, e);
        continue;
      }
      const double* aj = &s->op.aij[5 * (size_t)j];
      const int* nj = &s->op.nij[4 * (size_t)j];
      for (int k = 0; k < 4; ++k) {
        geo[e].a[k] = (float)aj[1 + k];
        geo[e].nb[k] = code_of(s, s->eng_of_ref[nj[k]]);
      }
      geo[e].bsl = bsl_of(s, j);
      geo[e].flags = (s->m.domain[j] == DOMAIN_JSR ? 1u : 0u) | (s->m.tropc[j] ? 2u : 0u) |
                     (per[e].empty() ? 0u : 4u);
    }
  }
  (void)N;
  ResidentArgs& a = s->ar;
  a.R = s->R;
  a.P = s->P_stride;
  a.off_bits = s->off_bits;
  SRS_TRY(dev_upload(s, (TetRec**)&a.geo, geo.data(), geo.size()));
  SRS_TRY(dev_upload(s, (int32_t**)&a.n_local, s->part_len.data(), s->part_len.size()));
  SRS_TRY(dev_upload(s, (int32_t**)&a.n_chtet, s->part_nch.data(), s->part_nch.size()));
  SRS_TRY(dev_upload(s, (int32_t**)&a.n_int, s->part_nint.data(), s->part_nint.size()));
  a.ch_interior = s->ch_interior;
  std::vector<uint16_t> rc(s->NR), rj(s->NR), lc(s->NL);
  std::vector<float> lrest(s->NL);
  for (int i = 0; i < s->NR; ++i) {
    rc[i] = code_of(s, s->eng_of_ref[s->m.ryr_ele[i]]);
    rj[i] = code_of(s, s->eng_of_ref[s->m.ryr_jsr[i]]);
  }
  for (int i = 0; i < s->NL; ++i) {
    lc[i] = code_of(s, s->eng_of_ref[s->m.lcc_ele[i]]);
    lrest[i] = (float)s->rest_ca[s->eng_of_ref[s->m.lcc_ele[i]]];
  }
  SRS_TRY(dev_upload(s, (uint16_t**)&a.ryr_cleft_code, rc.data(), rc.size()));
  SRS_TRY(dev_upload(s, (uint16_t**)&a.ryr_jsr_code, rj.data(), rj.size()));
  SRS_TRY(dev_upload(s, (uint16_t**)&a.lcc_code, lc.data(), lc.size()));
  SRS_TRY(dev_upload(s, (float**)&a.lcc_rest, lrest.data(), lrest.size()));
  // Channels for the protocol code: codes by kind (see ResidentCa)
  std::vector<int32_t> kc(s->NR), kj(s->NR), kl(s->NL);
  for (int i = 0; i < s->NR; ++i) {
    kc[i] = i;
    kj[i] = (1 << 28) | i;
  }
  for (int i = 0; i < s->NL; ++i) kl[i] = (2 << 28) | i;
  int32_t *p1, *p2, *p3, *p4;
  SRS_TRY(dev_upload(s, &p1, kc.data(), kc.size()));
  SRS_TRY(dev_upload(s, &p2, kj.data(), kj.size()));
  SRS_TRY(dev_upload(s, &p3, s->m.ryr_nb.data(), s->m.ryr_nb.size()));
  SRS_TRY(dev_upload(s, &p4, kl.data(), kl.size()));
  s->ch.NR = s->NR;
  s->ch.NL = s->NL;
  s->ch.ryr_cleft = p1;
  s->ch.ryr_jsr = p2;
  s->ch.ryr_nb = p3;
  s->ch.lcc_ele = p4;
  SRS_TRY(dev_alloc(s, &s->d_M[0], (size_t)s->R * NE));
  SRS_TRY(dev_alloc(s, &s->d_I[0], (size_t)s->R * NE));
  SRS_TRY(dev_alloc(s, &s->d_CM, (size_t)s->R * NE));
  SRS_TRY(dev_alloc(s, &s->d_CI, (size_t)s->R * NE));
  if (!resident_cluster_supported(C)) return fail(SRS_ERR_UNSUPPORTED, "unsupported cluster size");
  s->C = C;
  s->threads = threads;
  s->smem = resident_smem_bytes(s->P_stride, s->NR, s->NL, s->part_nch[0], 2 * s->NR + s->NL);
  int maxc = resident_max_clusters(C, threads, s->smem);
  if (maxc <= 0) return fail(SRS_ERR_UNSUPPORTED, "resident configuration does not fit on the device");
  s->n_clusters = std::min(maxc, s->R);
  return SRS_OK;
}

// Engine-layout offsets of realization r.
size_t eng_count(const srs_sim* s) {
  return s->d.engine == SRS_ENGINE_RESIDENT ? (size_t)s->C * s->P_stride : (size_t)s->N;
}

// ---- state conversion ---------------------------------------------------------
void* stage(srs_sim* s, size_t bytes) {
  s->stage_copies = 0;
  if (bytes > s->h_stage_bytes) {
    if (s->h_stage) cudaFreeHost(s->h_stage);
    s->h_stage = nullptr;
    s->h_stage_bytes = 0;
    if (cudaMallocHost(&s->h_stage, bytes) != cudaSuccess) return nullptr;
    s->h_stage_bytes = bytes;
  }
  return s->h_stage;
}

// Reference-numbered absolute state -> engine layout of one realization.
void to_engine_fp32(const srs_sim* s, const double* S6, float4* M, float* I) {
  const int N = s->N;
  const size_t NE = eng_count(s);
  const RestValues& rv = s->rv;
  for (size_t e = 0; e < NE; ++e) {
    int j = s->ref_of_eng[e];
    if (j < 0) {
      M[e] = make_float4(0, 0, 0, 0);
      I[e] = 0.0f;
      continue;
    }
    // mobile buffers rest at their cytosolic equilibrium; JSR elements carry
    // none (they are never coupled to the cytosol by diffusion)
    bool jsr = s->m.domain[j] == DOMAIN_JSR;
    double f = jsr ? 0.0 : 1.0;
    M[e] = make_float4((float)(S6[SP_CA * (size_t)N + j] - s->rest_ca[e]),
                       (float)(S6[SP_ATP * (size_t)N + j] - f * rv.atp),
                       (float)(S6[SP_CMDN * (size_t)N + j] - f * rv.cmdn),
                       (float)(S6[SP_DYE * (size_t)N + j] - f * rv.dye));
    double imm = jsr ? S6[SP_CSQN * (size_t)N + j] : S6[SP_TRPN * (size_t)N + j];
    I[e] = (float)(imm - s->rest_imm[e]);
  }
}

// Uploads one state to realizations [r0, r1) through pinned staging.
int upload_state_range(srs_sim* s, int r0, int r1, const double* S6) {
  const int N = s->N;
  const int nr = r1 - r0;
  if (s->d.precision == SRS_FP64) {
    const size_t per = (size_t)6 * N;
    double* h = (double*)stage(s, per * nr * sizeof(double));
    if (!h) return fail(SRS_ERR_NOMEM, "pinned staging allocation failed");
    for (int r = 0; r < nr; ++r) std::memcpy(h + r * per, S6, per * sizeof(double));
    SRS_CUDA(cudaMemcpyAsync(s->d_S[0] + (size_t)r0 * per, h, per * nr * sizeof(double),
                             cudaMemcpyHostToDevice, s->st));
    SRS_CUDA(cudaStreamSynchronize(s->st));
    return SRS_OK;
  }
  const size_t NE = eng_count(s);
  const int copies = s->stage_copies;
  float4* hM = (float4*)stage(s, NE * nr * (sizeof(float4) + sizeof(float)));
  if (!hM) return fail(SRS_ERR_NOMEM, "pinned staging allocation failed");
  float* hI = (float*)(hM + NE * nr);
  // A reset that repeats the previous one (same state, same realizations)
  // finds the copies already staged: only the upload below is repeated.
  bool staged = false;
  if (copies == nr && nr > 1) {
    std::vector<float4> m0(NE);
    std::vector<float> i0(NE);
    to_engine_fp32(s, S6, m0.data(), i0.data());
    staged = std::memcmp(m0.data(), hM, NE * sizeof(float4)) == 0 &&
             std::memcmp(i0.data(), hI, NE * sizeof(float)) == 0;
  }
  if (!staged) to_engine_fp32(s, S6, hM, hI);
  // realization 0's state copied into the others' staging slots by up to 8
  // host threads (the copy is memory-bound: one thread does not saturate it)
  auto fill = [&](int ra, int rb) {
    for (int r = ra; r < rb; ++r) {
      std::memcpy(hM + r * NE, hM, NE * sizeof(float4));
      std::memcpy(hI + r * NE, hI, NE * sizeof(float));
    }
  };
  const int nt = std::max(1, std::min({8, (int)std::thread::hardware_concurrency(), (nr - 1) / 16}));
  if (!staged && nt <= 1) {
    fill(1, nr);
  } else if (!staged) {
    std::vector<std::thread> pool;
    const int chunk = (nr - 1 + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) {
      const int ra = 1 + t * chunk, rb = std::min(nr, ra + chunk);
      if (ra < rb) pool.emplace_back(fill, ra, rb);
    }
    for (auto& th : pool) th.join();
  }
  SRS_CUDA(cudaMemcpyAsync(s->d_M[0] + (size_t)r0 * NE, hM, NE * nr * sizeof(float4),
                           cudaMemcpyHostToDevice, s->st));
  SRS_CUDA(cudaMemcpyAsync(s->d_I[0] + (size_t)r0 * NE, hI, NE * nr * sizeof(float),
                           cudaMemcpyHostToDevice, s->st));
  if (s->d_CMq) {  // q = 0 is c = 0
    SRS_CUDA(cudaMemsetAsync(s->d_CMq + (size_t)r0 * NE, 0, NE * nr * sizeof(ushort4), s->st));
    SRS_CUDA(cudaMemsetAsync(s->d_CIq + (size_t)r0 * NE, 0, NE * nr * sizeof(uint16_t), s->st));
  } else {
    SRS_CUDA(cudaMemsetAsync(s->d_CM + (size_t)r0 * NE, 0, NE * nr * sizeof(float4), s->st));
    SRS_CUDA(cudaMemsetAsync(s->d_CI + (size_t)r0 * NE, 0, NE * nr * sizeof(float), s->st));
  }
  SRS_CUDA(cudaStreamSynchronize(s->st));
  s->stage_copies = nr;
  return SRS_OK;
}

int upload_state(srs_sim* s, int r, const double* S6) { return upload_state_range(s, r, r + 1, S6); }

int download_state(srs_sim* s, int r, double* S6) {
  const int N = s->N;
  if (s->d.precision == SRS_FP64) {
    SRS_CUDA(cudaMemcpy(S6, s->d_S[0] + (size_t)r * 6 * N, sizeof(double) * 6 * N,
                        cudaMemcpyDeviceToHost));
    return SRS_OK;
  }
  size_t NE = eng_count(s);
  std::vector<float4> M(NE), CMh(NE);
  std::vector<float> I(NE), CIh(NE);
  SRS_CUDA(cudaMemcpy(M.data(), s->d_M[0] + r * NE, NE * sizeof(float4), cudaMemcpyDeviceToHost));
  SRS_CUDA(cudaMemcpy(I.data(), s->d_I[0] + r * NE, NE * sizeof(float), cudaMemcpyDeviceToHost));
  if (s->d_CMq) {
    std::vector<ushort4> Q(NE);
    std::vector<uint16_t> QI(NE);
    SRS_CUDA(cudaMemcpy(Q.data(), s->d_CMq + r * NE, NE * sizeof(ushort4), cudaMemcpyDeviceToHost));
    SRS_CUDA(cudaMemcpy(QI.data(), s->d_CIq + r * NE, NE * sizeof(uint16_t), cudaMemcpyDeviceToHost));
    for (size_t e = 0; e < NE; ++e) {
      CMh[e] = make_float4(comp_decode_host(Q[e].x), comp_decode_host(Q[e].y), comp_decode_host(Q[e].z),
                           comp_decode_host(Q[e].w));
      CIh[e] = comp_decode_host(QI[e]);
    }
  } else {
    SRS_CUDA(cudaMemcpy(CMh.data(), s->d_CM + r * NE, NE * sizeof(float4), cudaMemcpyDeviceToHost));
    SRS_CUDA(cudaMemcpy(CIh.data(), s->d_CI + r * NE, NE * sizeof(float), cudaMemcpyDeviceToHost));
  }
  const RestValues& rv = s->rv;
  for (size_t e = 0; e < NE; ++e) {
    int j = s->ref_of_eng[e];
    if (j < 0) continue;
    bool jsr = s->m.domain[j] == DOMAIN_JSR;
    double f = jsr ? 0.0 : 1.0;
    // compensated sum: the state is u - comp (the comp term holds the
    // rounding error of the last update)
    S6[SP_CA * (size_t)N + j] = s->rest_ca[e] + ((double)M[e].x - (double)CMh[e].x);
    S6[SP_ATP * (size_t)N + j] = f * rv.atp + ((double)M[e].y - (double)CMh[e].y);
    S6[SP_CMDN * (size_t)N + j] = f * rv.cmdn + ((double)M[e].z - (double)CMh[e].z);
    S6[SP_DYE * (size_t)N + j] = f * rv.dye + ((double)M[e].w - (double)CMh[e].w);
    double imm = s->rest_imm[e] + ((double)I[e] - (double)CIh[e]);
    S6[SP_TRPN * (size_t)N + j] = jsr ? 0.0 : imm;
    S6[SP_CSQN * (size_t)N + j] = jsr ? imm : 0.0;
  }
  return SRS_OK;
}

// After a run of the plain engines realization r's state sits in buffer
// (steps taken) % 2; move it to buffer 0.
int normalize_buffers(srs_sim* s, const std::vector<int64_t>& steps_before) {
  if (s->d.engine == SRS_ENGINE_RESIDENT) return SRS_OK;
  std::vector<RealCtl> ctl(s->R);
  SRS_CUDA(cudaMemcpy(ctl.data(), s->d_ctl, sizeof(RealCtl) * s->R, cudaMemcpyDeviceToHost));
  const size_t N = s->N;
  for (int r = 0; r < s->R; ++r) {
    if (((ctl[r].step - steps_before[r]) & 1) == 0) continue;
    if (s->d.precision == SRS_FP64) {
      SRS_CUDA(cudaMemcpyAsync(s->d_S[0] + r * 6 * N, s->d_S[1] + r * 6 * N, sizeof(double) * 6 * N,
                               cudaMemcpyDeviceToDevice, s->st));
    } else {
      SRS_CUDA(cudaMemcpyAsync(s->d_M[0] + r * N, s->d_M[1] + r * N, sizeof(float4) * N,
                               cudaMemcpyDeviceToDevice, s->st));
      SRS_CUDA(cudaMemcpyAsync(s->d_I[0] + r * N, s->d_I[1] + r * N, sizeof(float) * N,
                               cudaMemcpyDeviceToDevice, s->st));
    }
  }
  SRS_CUDA(cudaStreamSynchronize(s->st));
  return SRS_OK;
}

std::vector<int64_t> ctl_steps(srs_sim* s) {
  std::vector<RealCtl> ctl(s->R);
  cudaMemcpy(ctl.data(), s->d_ctl, sizeof(RealCtl) * s->R, cudaMemcpyDeviceToHost);
  std::vector<int64_t> v(s->R);
  for (int r = 0; r < s->R; ++r) v[r] = ctl[r].step;
  return v;
}

// ---- launches -----------------------------------------------------------------
void refresh_args(srs_sim* s) {
  ChanState cs = chan_state(s);
  if (s->d.precision == SRS_FP64) {
    s->a64.P = s->P;
    s->a64.C = s->ch;
    s->a64.CS = cs;
    s->a64.counters = s->d_counters;
    s->a64.nsr = s->nsr;
  } else if (s->d.engine == SRS_ENGINE_PLAIN) {
    s->a32.P = s->P;
    s->a32.C = s->ch;
    s->a32.CS = cs;
    s->a32.counters = s->d_counters;
    {
      // one wave of update blocks (six per SM) ahead, counted in element blocks
      int dev = 0, n_sm = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
      s->a32.pf_rows = s->pf_override >= 0 ? s->pf_override : std::max(1, (n_sm * 6 + s->R - 1) / s->R);
    }
    s->a32.k = make_consts32(s);
    s->a32.CM = s->d_CM;
    s->a32.CI = s->d_CI;
    s->a32.CMq = s->d_CMq;
    s->a32.CIq = s->d_CIq;
  } else {
    s->ar.P_ = s->P;
    s->ar.C = s->ch;
    s->ar.CS = cs;
    s->ar.k = make_consts32(s);
    s->ar.M = s->d_M[0];
    s->ar.I = s->d_I[0];
    s->ar.CM = s->d_CM;
    s->ar.CI = s->d_CI;
  }
  if (s->graph_plain) {
    cudaGraphExecDestroy(s->graph_plain);
    s->graph_plain = nullptr;
  }
}

int plain_launch(srs_sim* s, int parity) {
  int rc;
  if (s->d.precision == SRS_FP64) {
    Plain64Args a = s->a64;
    a.S_in = s->d_S[parity];
    a.S_out = s->d_S[parity ^ 1];
    rc = launch_plain64_step(a, s->st);
  } else {
    Plain32Args a = s->a32;
    a.M_in = s->d_M[parity];
    a.I_in = s->d_I[parity];
    a.M_out = s->d_M[parity ^ 1];
    a.I_out = s->d_I[parity ^ 1];
    rc = launch_plain32_step(a, s->st);
    s->launches += plain32_kernels_per_step(a) - 1;
  }
  s->launches++;
  if (rc) return fail(SRS_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString(cudaGetLastError()));
  return SRS_OK;
}

int plain_prestep(srs_sim* s, int write_initial_row) {
  int rc;
  if (s->d.precision == SRS_FP64) {
    Plain64Args a = s->a64;
    a.S_in = s->d_S[0];
    rc = launch_plain64_prestep(a, write_initial_row, s->st);
  } else {
    Plain32Args a = s->a32;
    a.M_in = s->d_M[0];
    rc = launch_plain32_prestep(a, write_initial_row, s->st);
  }
  s->launches++;
  if (rc) return fail(SRS_ERR_CUDA, "prestep launch failed");
  return SRS_OK;
}

// n plain steps starting from buffer 0 (graph-replayed in pairs).
int plain_steps(srs_sim* s, int64_t n) {
  const int G = 32;  // launches per graph replay (even)
  int64_t done = 0;
  if (n >= G) {
    if (!s->graph_plain) {
      cudaGraph_t g;
      SRS_CUDA(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
      int64_t l0 = s->launches;
      for (int i = 0; i < G; ++i) {
        int rc = plain_launch(s, i & 1);
        if (rc) {
          cudaStreamEndCapture(s->st, &g);
          return rc;
        }
      }
      s->launches = l0;
      SRS_CUDA(cudaStreamEndCapture(s->st, &g));
      SRS_CUDA(cudaGraphInstantiate(&s->graph_plain, g, 0));
      cudaGraphDestroy(g);
      s->graph_plain_len = G;
    }
    const int per = s->d.precision == SRS_FP64 ? 1 : plain32_kernels_per_step(s->a32);
    while (n - done >= G) {
      SRS_CUDA(cudaGraphLaunch(s->graph_plain, s->st));
      s->launches += (int64_t)G * per;
      done += G;
    }
  }
  for (; done < n; ++done) SRS_TRY(plain_launch(s, (int)(done & 1)));
  return SRS_OK;
}

int resident_launch(srs_sim* s, int steps, int prestep_first = 0) {
  ResidentArgs a = s->ar;
  a.steps = steps;
  a.prestep_first = prestep_first;
  a.initial_row = prestep_first;
  a.speculate = 1;
  int rc = launch_resident(a, s->C, s->n_clusters, s->threads, s->smem, s->st);
  s->launches++;
  if (rc) return fail(SRS_ERR_CUDA, std::string("resident launch: ") + cudaGetErrorString(cudaGetLastError()));
  return SRS_OK;
}

int advance(srs_sim* s, int64_t n) {
  if (s->d.engine == SRS_ENGINE_RESIDENT) {
    const int S = s->d.steps_per_launch > 0 ? s->d.steps_per_launch : 1000;
    for (int64_t done = 0; done < n;) {
      int k = (int)std::min<int64_t>(S, n - done);
      SRS_TRY(resident_launch(s, k));
      done += k;
    }
    return SRS_OK;
  }
  return plain_steps(s, n);
}

int ensure_rows(srs_sim* s, int64_t cap, int w) {
  if (cap <= s->rows_cap_alloc && w == s->rows_w_alloc) return SRS_OK;
  void* p = nullptr;
  SRS_CUDA(cudaMalloc(&p, std::max<size_t>(1, (size_t)s->R * cap * w) * sizeof(float)));
  s->allocs.push_back(p);
  s->d_rows = (float*)p;
  s->rows_cap_alloc = cap;
  s->rows_w_alloc = w;
  return SRS_OK;
}

int set_schedule(srs_sim* s, const Schedule& sc) {
  std::vector<int64_t> ticks = sc.tick_steps;
  std::vector<double> tt = sc.tick_times;
  if (ticks.empty()) {
    ticks.push_back(-1);
    tt.push_back(0.0);
  }
  if (ticks.size() > s->ticks_cap) {
    SRS_TRY(dev_upload(s, &s->d_ticks, ticks.data(), ticks.size()));
    SRS_TRY(dev_upload(s, &s->d_tick_t, tt.data(), tt.size()));
    s->ticks_cap = ticks.size();
  } else {
    SRS_CUDA(cudaMemcpy(s->d_ticks, ticks.data(), ticks.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
    SRS_CUDA(cudaMemcpy(s->d_tick_t, tt.data(), tt.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  s->P.ticks = s->d_ticks;
  s->P.tick_t = s->d_tick_t;
  s->P.sched_ver = s->P.sched_ver + 1;  // invalidates the per-realization tick caches
  s->P.n_ticks = (int32_t)sc.tick_steps.size();
  s->P.n_steps = sc.n_steps;
  s->P.clamp_end = sc.clamp_end_step;
  s->P.hold_end = sc.hold_end_step;
  return SRS_OK;
}

int check_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(SRS_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  SRS_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3)
    return fail(SRS_ERR_CUDA, "the library targets sm_103a (GB300); device is sm_" +
                                  std::to_string(prop.major) + std::to_string(prop.minor));
  return SRS_OK;
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" {

const char* srs_status_string(int status) {
  switch (status) {
    case SRS_OK: return "ok";
    case SRS_ERR_INPUT: return "invalid input";
    case SRS_ERR_IO: return "i/o error";
    case SRS_ERR_MESH: return "invalid mesh";
    case SRS_ERR_UNSTABLE: return "unstable time step";
    case SRS_ERR_CUDA: return "cuda error";
    case SRS_ERR_UNSUPPORTED: return "unsupported configuration";
    case SRS_ERR_NONFINITE: return "non-finite state";
    case SRS_ERR_TIMEOUT: return "device wait timed out";
    case SRS_ERR_STATE: return "call out of order";
    case SRS_ERR_NOMEM: return "out of memory";
    default: return "unknown status";
  }
}
const char* srs_last_error(void) { return g_err.c_str(); }
const char* srs_version(void) { return "srs_gb300 0.1 (sm_103a)"; }

void srs_default_parameters(srs_params* ps) { params_default(ps); }

int srs_read_parameters(srs_params* ps, const char* param_file) {
  if (!ps || !param_file) return fail(SRS_ERR_INPUT, "null argument");
  std::string err;
  int rc = params_read_xml(param_file, ps, &err);
  if (rc) return fail(rc, err);
  return SRS_OK;
}

int srs_read_grid(const srs_params* ps, const char* mesh_base, srs_grid** out) {
  if (!ps || !mesh_base || !out) return fail(SRS_ERR_INPUT, "null argument");
  srs_grid* g = new srs_grid();
  g->p = *ps;
  std::string err;
  int rc = mesh_read(mesh_base, ps->ints[I_FLAG_NO_FLUX_BOUNDARY], &g->m, &err);
  if (!rc) rc = assemble_operator(g->m, g->p, &g->op, &err);
  if (rc) {
    delete g;
    return fail(rc, err);
  }
  *out = g;
  return SRS_OK;
}

void srs_free_grid(srs_grid* g) { delete g; }

int srs_grid_get_info(const srs_grid* g, srs_grid_info* info) {
  if (!g || !info) return fail(SRS_ERR_INPUT, "null argument");
  info->n_ele = g->m.N;
  info->n_face = g->m.NF;
  info->n_nodes = g->m.NN;
  info->n_ryr = g->m.NR;
  info->n_lcc = g->m.NL;
  int nj = 0;
  double vj = 0;
  for (int i = 0; i < g->m.N; ++i)
    if (g->m.domain[i] == DOMAIN_JSR) {
      ++nj;
      vj += g->m.V0[i];
    }
  info->n_jsr = nj;
  info->vol_jsr = vj;
  info->max_diag = g->op.max_diag;
  return SRS_OK;
}

int srs_grid_get_operator(const srs_grid* g, double* aij, int* nij, double* br) {
  if (!g) return fail(SRS_ERR_INPUT, "null argument");
  if (aij) std::memcpy(aij, g->op.aij.data(), g->op.aij.size() * sizeof(double));
  if (nij) std::memcpy(nij, g->op.nij.data(), g->op.nij.size() * sizeof(int));
  if (br) std::memcpy(br, g->op.br.data(), g->op.br.size() * sizeof(double));
  return SRS_OK;
}

int srs_grid_get_elements(const srs_grid* g, double* v0, double* tt, int* domain, int* tropc,
                          int* file_index) {
  if (!g) return fail(SRS_ERR_INPUT, "null argument");
  const int N = g->m.N;
  if (v0) std::memcpy(v0, g->m.V0.data(), N * sizeof(double));
  if (tt) std::memcpy(tt, g->m.TT.data(), N * sizeof(double));
  if (domain) std::memcpy(domain, g->m.domain.data(), N * sizeof(int));
  if (tropc) std::memcpy(tropc, g->m.tropc.data(), N * sizeof(int));
  if (file_index) std::memcpy(file_index, g->m.order.data(), N * sizeof(int));
  return SRS_OK;
}

int srs_grid_get_channels(const srs_grid* g, int* ryr_ele, int* ryr_jsr, int* ryr_nb, int* lcc) {
  if (!g) return fail(SRS_ERR_INPUT, "null argument");
  if (ryr_ele) std::memcpy(ryr_ele, g->m.ryr_ele.data(), g->m.NR * sizeof(int));
  if (ryr_jsr) std::memcpy(ryr_jsr, g->m.ryr_jsr.data(), g->m.NR * sizeof(int));
  if (ryr_nb) std::memcpy(ryr_nb, g->m.ryr_nb.data(), 4 * g->m.NR * sizeof(int));
  if (lcc) std::memcpy(lcc, g->m.lcc_ele.data(), g->m.NL * sizeof(int));
  return SRS_OK;
}

int srs_initial_states(const srs_grid* g, const srs_params* ps, double* states) {
  if (!g || !ps || !states) return fail(SRS_ERR_INPUT, "null argument");
  std::vector<double> S;
  initial_states(g->m, *ps, &S);
  std::memcpy(states, S.data(), S.size() * sizeof(double));
  return SRS_OK;
}

int srs_sim_create(const srs_grid* g, const srs_params* ps, const srs_sim_desc* d, srs_sim** out) {
  if (!g || !ps || !d || !out) return fail(SRS_ERR_INPUT, "null argument");
  if (d->n_realizations <= 0 || d->n_realizations > SRS_MAX_REALIZATIONS)
    return fail(SRS_ERR_INPUT, "n_realizations must be in [1, " +
                                   std::to_string(SRS_MAX_REALIZATIONS) + "]");
  if (d->precision != SRS_FP64 && d->precision != SRS_FP32)
    return fail(SRS_ERR_INPUT, "precision must be 64 or 32");
  if (d->engine != SRS_ENGINE_PLAIN && d->engine != SRS_ENGINE_RESIDENT)
    return fail(SRS_ERR_INPUT, "unknown engine");
  if (d->engine == SRS_ENGINE_RESIDENT && d->precision != SRS_FP32)
    return fail(SRS_ERR_UNSUPPORTED, "the resident engine runs in FP32");
  if (ps->ints[I_GATING_FFWD])
    return fail(SRS_ERR_UNSUPPORTED, "flag_ffwd (steady-state gating fast-forward) is not supported");
  if (g->m.NR <= 0) return fail(SRS_ERR_MESH, "mesh has no RyRs");
  if (g->m.NR > 1024 && ps->reals[R_RYR_A_STAR] != 0)
    return fail(SRS_ERR_UNSUPPORTED, "coupled gating supports at most 1024 RyRs");
  // explicit stability: D_max * dt * max|a0| <= 1
  double Dmax = std::max(std::max(ps->reals[R_D_CA], ps->reals[R_D_ATP]),
                         std::max(ps->reals[R_D_CMDN], ps->reals[R_D_DYE]));
  double cfl = Dmax * ps->reals[R_T_STEP] * g->op.max_diag;
  if (!(cfl <= 1.0))
    return fail(SRS_ERR_UNSTABLE, "explicit step unstable: D*dt*max|a0| = " + std::to_string(cfl));
  SRS_TRY(check_device());
  srs_sim* s = new srs_sim();
  s->m = g->m;
  s->op = g->op;
  s->p = *ps;
  s->d = *d;
  s->R = d->n_realizations;
  s->N = g->m.N;
  s->NR = g->m.NR;
  s->NL = g->m.NL;
  s->NCH = s->NR + s->NL;
  s->rv = rest_values(*ps);
  s->vm = ps->reals[R_DEFAULT_VM];
  s->nsr = ps->reals[R_DEFAULT_CA_NSR];
  s->seeds.resize(s->R);
  for (int r = 0; r < s->R; ++r) s->seeds[r] = d->seeds ? d->seeds[r] : (uint64_t)(r + 1);
  s->d.seeds = nullptr;
  int rc = SRS_OK;
  if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(SRS_ERR_CUDA, "stream creation failed");
  if (!rc) rc = alloc_channel_state(s);
  if (!rc) fill_protocol_consts(s);
  if (!rc) {
    if (d->precision == SRS_FP64) rc = setup_plain64(s);
    else if (d->engine == SRS_ENGINE_PLAIN) rc = setup_plain32(s);
    else {
      // resident: smallest cluster whose partition fits in shared memory
      int threads = d->threads_per_cta > 0 ? d->threads_per_cta : 512;
      if (threads > SRS_RESIDENT_MAX_THREADS || threads % 32)
        rc = fail(SRS_ERR_INPUT, "resident engine: threads_per_cta must be a multiple of 32, <= " +
                                     std::to_string(SRS_RESIDENT_MAX_THREADS));
      int C = d->cluster_size;
      if (C <= 0) {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        for (int c : {1, 2, 3, 4, 5, 6, 8, 16}) {
          int Pm = (s->N + c - 1) / c;
          Pm = (Pm + 3) & ~3;
          if (resident_smem_bytes(Pm, s->NR, s->NL, 2 * s->NR + s->NL, 2 * s->NR + s->NL) <=
              (size_t)optin) {
            C = c;
            break;
          }
        }
        if (C <= 0) rc = fail(SRS_ERR_UNSUPPORTED, "mesh too large for the resident engine");
      }
      if (!rc) rc = setup_resident(s, C, threads);
    }
  }
  if (rc) {
    srs_sim_destroy(s);
    return rc;
  }
  s->d.cluster_size = s->C;
  s->d.threads_per_cta = s->threads;
  s->P.run_protocol = 0;
  s->P.row_cap = 0;
  refresh_args(s);
  rc = srs_sim_reset(s);
  if (rc) {
    srs_sim_destroy(s);
    return rc;
  }
  *out = s;
  return SRS_OK;
}

void srs_sim_destroy(srs_sim* s) {
  if (!s) return;
  if (s->graph_plain) cudaGraphExecDestroy(s->graph_plain);
  if (s->st) cudaStreamSynchronize(s->st);
  for (void* p : s->allocs) cudaFree(p);
  for (auto& b : s->adj_bufs) cudaFree(b.first);
  if (s->h_stage) cudaFreeHost(s->h_stage);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
}

int srs_sim_get_desc(const srs_sim* s, srs_sim_desc* d) {
  if (!s || !d) return fail(SRS_ERR_INPUT, "null argument");
  *d = s->d;
  return SRS_OK;
}

int srs_sim_set_prefetch(srs_sim* s, int element_blocks) {
  if (!s) return fail(SRS_ERR_INPUT, "null argument");
  if (s->d.engine != SRS_ENGINE_PLAIN || s->d.precision != SRS_FP32 || s->N < PLAIN32_SPLIT_N)
    return fail(SRS_ERR_UNSUPPORTED, "the prefetch distance applies to the plain FP32 engine's large-mesh form");
  s->pf_override = element_blocks < 0 ? -1 : element_blocks;
  refresh_args(s);
  return SRS_OK;
}

int srs_sim_get_config(const srs_sim* s, srs_sim_config* c) {
  if (!s || !c) return fail(SRS_ERR_INPUT, "null argument");
  c->engine = s->d.engine;
  c->precision = s->d.precision;
  c->threads_per_cta = s->d.engine == SRS_ENGINE_RESIDENT ? s->threads : 256;
  c->cluster_size = s->d.engine == SRS_ENGINE_RESIDENT ? s->C : 1;
  c->steps_per_launch =
      s->d.engine == SRS_ENGINE_RESIDENT ? (s->d.steps_per_launch > 0 ? s->d.steps_per_launch : 1000) : 1;
  c->smem_bytes = (int)s->smem;
  c->kernel_launches = s->launches;
  const int64_t NE = (int64_t)eng_count(s);
  const int64_t per_state = s->d.precision == SRS_FP64 ? (int64_t)6 * s->N * 8 : NE * 20;
  c->ctl_bytes = (int64_t)s->R * (int64_t)sizeof(RealCtl);
  c->reset_h2d_bytes = (int64_t)s->R * (per_state + (int64_t)(s->NR + 2 * s->NL) * 4 +
                                         (int64_t)s->NCH * 8) + c->ctl_bytes;
  c->engine_elements = NE;
  return SRS_OK;
}

int srs_sim_reset(srs_sim* s) {
  if (!s) return fail(SRS_ERR_INPUT, "null argument");
  const Mesh& m = s->m;
  const srs_params& p = s->p;
  const int* I = p.ints;
  const double* Rr = p.reals;
  std::vector<double> S6;
  initial_states(m, p, &S6);
  const int NR = s->NR, NL = s->NL, NCH = s->NCH;
  std::vector<int32_t> ryr((size_t)s->R * NR, 0), lcc((size_t)s->R * NL, 1), lccv((size_t)s->R * NL, 2);
  std::vector<double> res((size_t)s->R * NCH);
  std::vector<RealCtl> ctl(s->R);
  // The RyR hold of RunSimulation indexes RyR_States[INIT_RYR] under every
  // protocol (cpu/RunSimulation.cpp:540), so the index is checked always.
  if (I[I_INIT_RYR] != -1 && (I[I_INIT_RYR] < 0 || I[I_INIT_RYR] >= NR))
    return fail(SRS_ERR_INPUT, "Invalid initial RyR index (" + std::to_string(I[I_INIT_RYR]) +
                                   "), must be -1 to ignore, or between 0 and the number of RyRs");
  if (I[I_FLAG_LCC] && (I[I_LCC_INDEX] < 0 || I[I_LCC_INDEX] >= NL))
    return fail(SRS_ERR_INPUT, "LCC trigger index out of range");
  for (int r = 0; r < s->R; ++r) {
    const uint64_t seed = s->seeds[r];
    int32_t* ry = &ryr[(size_t)r * NR];
    int32_t* lc = &lcc[(size_t)r * NL];
    // initial channel opening (cpu/main.cpp:217-250)
    if (I[I_FLAG_LCC]) {
      lc[I[I_LCC_INDEX]] = 6;
    } else if (I[I_FLAG_V_CLAMP]) {
    } else if (I[I_INIT_RYR] != -1) {
      ry[I[I_INIT_RYR]] = 1;
    } else {
      // OpenRandomRyR (cpu/InitFuncs.cpp:1420-1475): rate-weighted choice with
      // the linear luminal factor it uses, drawn from protocol stream 1.
      std::vector<double> rate(NR);
      double tot = 0;
      for (int i = 0; i < NR; ++i) {
        int no = 0, nc = 0;
        for (int k = 0; k < 4; ++k) {
          int j = m.ryr_nb[4 * i + k];
          if (j >= 0) (ry[j] ? no : nc)++;
        }
        double ca_ss = S6[SP_CA * (size_t)m.N + m.ryr_ele[i]];
        double phi = Rr[R_RYR_PHI_M] * S6[SP_CA * (size_t)m.N + m.ryr_jsr[i]] + Rr[R_RYR_PHI_B];
        double X = std::exp(0.5 * Rr[R_RYR_A_STAR] * (nc * Rr[R_RYR_EPS_CC] - no * Rr[R_RYR_EPS_OO]));
        rate[i] = X * phi * Rr[R_RYR_K_PLUS] * std::pow(ca_ss, Rr[R_RYR_ETA]);
        tot += rate[i];
      }
      double u = tot * srs_protocol_uniform(seed, 1);
      int pick = 0;
      double sum = 0;
      for (int i = 0; i < NR; ++i) {
        sum += rate[i];
        if (sum >= u) {
          pick = i;
          break;
        }
      }
      ry[pick] = 1;
    }
    for (int i = 0; i < NCH; ++i) res[(size_t)r * NCH + i] = srs_initial_residual(seed, (uint32_t)i);
    RealCtl& c = ctl[r];
    std::memset(&c, 0, sizeof(c));
    c.seed = seed;
    c.lcc_open = I[I_FLAG_LCC];
    c.lcc_close_step = -1;
    if (I[I_FLAG_LCC]) {
      double T = -Rr[R_LCC_DURATION] * srs_log(srs_protocol_uniform(seed, 0));
      c.lcc_close_step = first_step_at_or_after(p, T);
    }
    int n_open = 0;
    for (int i = 0; i < NR; ++i) n_open += ry[i];
    c.n_open_tick = n_open;
  }
  SRS_TRY(upload_state_range(s, 0, s->R, S6.data()));
  SRS_CUDA(cudaMemcpy(s->d_ryr, ryr.data(), ryr.size() * 4, cudaMemcpyHostToDevice));
  SRS_CUDA(cudaMemcpy(s->d_lcc, lcc.data(), lcc.size() * 4, cudaMemcpyHostToDevice));
  SRS_CUDA(cudaMemcpy(s->d_lccv, lccv.data(), lccv.size() * 4, cudaMemcpyHostToDevice));
  SRS_CUDA(cudaMemcpy(s->d_res, res.data(), res.size() * 8, cudaMemcpyHostToDevice));
  SRS_CUDA(cudaMemcpy(s->d_ctl, ctl.data(), ctl.size() * sizeof(RealCtl), cudaMemcpyHostToDevice));
  SRS_CUDA(cudaMemset(s->d_counters, 0, sizeof(unsigned) * s->R));
  return SRS_OK;
}

int srs_sim_set_state(srs_sim* s, int r, const double* states, const int* ryr, const int* lcc,
                      const int* lccv, const double* res) {
  if (!s || r < 0 || r >= s->R) return fail(SRS_ERR_INPUT, "bad realization index");
  if (states) SRS_TRY(upload_state(s, r, states));
  if (ryr) SRS_CUDA(cudaMemcpy(s->d_ryr + (size_t)r * s->NR, ryr, s->NR * 4, cudaMemcpyHostToDevice));
  if (lcc) SRS_CUDA(cudaMemcpy(s->d_lcc + (size_t)r * s->NL, lcc, s->NL * 4, cudaMemcpyHostToDevice));
  if (lccv) SRS_CUDA(cudaMemcpy(s->d_lccv + (size_t)r * s->NL, lccv, s->NL * 4, cudaMemcpyHostToDevice));
  if (res) SRS_CUDA(cudaMemcpy(s->d_res + (size_t)r * s->NCH, res, s->NCH * 8, cudaMemcpyHostToDevice));
  return SRS_OK;
}

int srs_sim_get_state(srs_sim* s, int r, double* states, int* ryr, int* lcc, int* lccv, double* res) {
  if (!s || r < 0 || r >= s->R) return fail(SRS_ERR_INPUT, "bad realization index");
  SRS_CUDA(cudaStreamSynchronize(s->st));
  if (states) SRS_TRY(download_state(s, r, states));
  if (ryr) SRS_CUDA(cudaMemcpy(ryr, s->d_ryr + (size_t)r * s->NR, s->NR * 4, cudaMemcpyDeviceToHost));
  if (lcc) SRS_CUDA(cudaMemcpy(lcc, s->d_lcc + (size_t)r * s->NL, s->NL * 4, cudaMemcpyDeviceToHost));
  if (lccv) SRS_CUDA(cudaMemcpy(lccv, s->d_lccv + (size_t)r * s->NL, s->NL * 4, cudaMemcpyDeviceToHost));
  if (res) SRS_CUDA(cudaMemcpy(res, s->d_res + (size_t)r * s->NCH, s->NCH * 8, cudaMemcpyDeviceToHost));
  return SRS_OK;
}

int srs_sim_set_globals(srs_sim* s, double v_m, double ca_nsr) {
  if (!s) return fail(SRS_ERR_INPUT, "null argument");
  s->vm = v_m;
  s->nsr = ca_nsr;
  fill_protocol_consts(s);
  refresh_args(s);
  return SRS_OK;
}

int srs_explicit_step(srs_sim* s, int64_t n_steps) {
  if (!s || n_steps < 0) return fail(SRS_ERR_INPUT, "bad argument");
  std::vector<int64_t> before = ctl_steps(s);
  s->P.run_protocol = 0;
  refresh_args(s);
  SRS_TRY(advance(s, n_steps));
  SRS_CUDA(cudaStreamSynchronize(s->st));
  SRS_TRY(normalize_buffers(s, before));
  return SRS_OK;
}

int srs_sim_advance_async(srs_sim* s, int64_t n_steps) {
  if (!s || n_steps < 0) return fail(SRS_ERR_INPUT, "bad argument");
  if (s->d.engine != SRS_ENGINE_RESIDENT && (n_steps & 1))
    return fail(SRS_ERR_INPUT, "plain engines advance asynchronously by an even number of steps");
  if (s->P.run_protocol) {
    s->P.run_protocol = 0;
    refresh_args(s);
  }
  return advance(s, n_steps);
}

int srs_sim_synchronize(srs_sim* s) {
  if (!s) return fail(SRS_ERR_INPUT, "null argument");
  SRS_CUDA(cudaStreamSynchronize(s->st));
  return SRS_OK;
}

int srs_sim_time_advance(srs_sim* s, int64_t n_steps, float* ms) {
  if (!s || !ms) return fail(SRS_ERR_INPUT, "null argument");
  cudaEvent_t e0, e1;
  SRS_CUDA(cudaEventCreate(&e0));
  SRS_CUDA(cudaEventCreate(&e1));
  SRS_CUDA(cudaStreamSynchronize(s->st));
  SRS_CUDA(cudaEventRecord(e0, s->st));
  int rc = srs_sim_advance_async(s, n_steps);
  SRS_CUDA(cudaEventRecord(e1, s->st));
  SRS_CUDA(cudaEventSynchronize(e1));
  SRS_CUDA(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int srs_sim_status(srs_sim* s, int* bits) {
  if (!s || !bits) return fail(SRS_ERR_INPUT, "null argument");
  std::vector<RealCtl> ctl(s->R);
  SRS_CUDA(cudaStreamSynchronize(s->st));
  SRS_CUDA(cudaMemcpy(ctl.data(), s->d_ctl, sizeof(RealCtl) * s->R, cudaMemcpyDeviceToHost));
  int b = 0;
  for (auto& c : ctl) b |= (int)c.status;
  *bits = b;
  return SRS_OK;
}

}  // extern "C"

namespace {

// RunSimulation set-up: schedule, rows buffer, protocol mode.
int run_prepare(srs_sim* s, const srs_run_output* out, Schedule* sc, std::vector<int64_t>* before) {
  if (!out || !out->rows || out->row_capacity <= 0) return fail(SRS_ERR_INPUT, "bad output");
  *sc = make_schedule(s->p);
  fill_protocol_consts(s);
  if (out->row_width != s->P.row_w)
    return fail(SRS_ERR_INPUT, "row_width must be " + std::to_string(s->P.row_w));
  SRS_TRY(set_schedule(s, *sc));
  SRS_TRY(ensure_rows(s, out->row_capacity, s->P.row_w));
  s->P.row_cap = out->row_capacity;
  s->P.run_protocol = 1;
  refresh_args(s);
  *before = ctl_steps(s);
  return SRS_OK;
}

int all_done(srs_sim* s, bool* done) {
  std::vector<RealCtl> ctl(s->R);
  SRS_CUDA(cudaMemcpyAsync(ctl.data(), s->d_ctl, sizeof(RealCtl) * s->R, cudaMemcpyDeviceToHost, s->st));
  SRS_CUDA(cudaStreamSynchronize(s->st));
  bool all = true;
  for (auto& c : ctl) all &= c.done != 0;
  *done = all;
  return SRS_OK;
}

// RunSimulation results: rows and per-realization summary to the host.
int run_finish(srs_sim* s, srs_run_output* out, const std::vector<int64_t>& before) {
  std::vector<RealCtl> ctl(s->R);
  SRS_CUDA(cudaStreamSynchronize(s->st));
  SRS_TRY(normalize_buffers(s, before));
  SRS_CUDA(cudaMemcpy(ctl.data(), s->d_ctl, sizeof(RealCtl) * s->R, cudaMemcpyDeviceToHost));
  const size_t rw = (size_t)s->P.row_w;
  SRS_CUDA(cudaMemcpy(out->rows, s->d_rows, (size_t)s->R * out->row_capacity * rw * sizeof(float),
                      cudaMemcpyDeviceToHost));
  int st_bits = 0;
  for (int r = 0; r < s->R; ++r) {
    if (out->n_rows) out->n_rows[r] = ctl[r].n_rows;
    if (out->t_end) out->t_end[r] = ctl[r].t;
    if (out->n_steps) out->n_steps[r] = ctl[r].step;
    st_bits |= (int)ctl[r].status;
  }
  s->P.run_protocol = 0;
  s->P.row_cap = 0;
  refresh_args(s);
  if (st_bits & 1) return fail(SRS_ERR_NONFINITE, "a realization produced a non-finite Ca value");
  if (st_bits & 4) return fail(SRS_ERR_INPUT, "row_capacity too small for the run");
  if (st_bits & 8) return fail(SRS_ERR_STATE, "internal: termination inside a speculating launch");
  return SRS_OK;
}

}  // namespace

extern "C" {

int srs_run_simulation(srs_sim* s, srs_run_output* out) {
  return srs_run_simulation_grid(s, out, nullptr, nullptr, nullptr, 0, nullptr);
}

int srs_run_simulation_timed(srs_sim* s, srs_run_output* out, float* launch_ms, int max_launches,
                             int* n_launches) {
  return srs_run_simulation_grid(s, out, nullptr, nullptr, launch_ms, max_launches, n_launches);
}

int srs_run_simulation_grid(srs_sim* s, srs_run_output* out, srs_grid_callback cb, void* user,
                            float* launch_ms, int max_launches, int* n_launches) {
  if (launch_ms && max_launches < 0) return fail(SRS_ERR_INPUT, "max_launches must be >= 0");
  if (!s) return fail(SRS_ERR_INPUT, "bad output");
  Schedule sc;
  std::vector<int64_t> before;
  SRS_TRY(run_prepare(s, out, &sc, &before));
  struct Events {  // destroyed on every return path
    cudaEvent_t e[2] = {nullptr, nullptr};
    ~Events() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
    }
  } evs;
  cudaEvent_t* ev = evs.e;
  int n_timed = 0;
  if (launch_ms) {
    SRS_CUDA(cudaEventCreate(&ev[0]));
    SRS_CUDA(cudaEventCreate(&ev[1]));
  }
  // device time of the launches between two all-done checks
  auto t_begin = [&]() -> int {
    if (launch_ms) SRS_CUDA(cudaEventRecord(ev[0], s->st));
    return SRS_OK;
  };
  auto t_end = [&]() -> int {
    if (!launch_ms) return SRS_OK;
    SRS_CUDA(cudaEventRecord(ev[1], s->st));
    SRS_CUDA(cudaEventSynchronize(ev[1]));
    float ms = 0.0f;
    SRS_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    if (n_timed < max_launches) launch_ms[n_timed] = ms;
    n_timed++;
    return SRS_OK;
  };
  // Grid-file steps (OUTPUT_GRID_FLAG): the launches end there and the
  // callback sees the state before that step, as WriteToGridFiles does
  // (cpu/RunSimulation.cpp:545-549).  Realizations advance in lock step, so
  // they must start from the same step.
  const bool grid = cb != nullptr && !sc.grid_steps.empty();
  const int64_t base = before.empty() ? 0 : before[0];
  if (grid)
    for (int64_t b : before)
      if (b != base) return fail(SRS_ERR_STATE, "grid snapshots need every realization at the same step");
  size_t gi = 0;
  while (grid && gi < sc.grid_steps.size() && sc.grid_steps[gi] <= base) ++gi;
  const size_t G = grid ? sc.grid_steps.size() : 0;
  std::vector<int64_t> since = before;  // steps at the last buffer normalisation
  auto deliver = [&]() -> int {
    SRS_TRY(normalize_buffers(s, since));  // the state in buffer 0 for every realization
    since = ctl_steps(s);
    std::vector<RealCtl> ctl(s->R);
    SRS_CUDA(cudaMemcpy(ctl.data(), s->d_ctl, sizeof(RealCtl) * s->R, cudaMemcpyDeviceToHost));
    std::vector<int> dn(s->R);
    for (int r = 0; r < s->R; ++r) dn[r] = ctl[r].done != 0;
    cb(user, (int64_t)gi + 1, sc.grid_times[gi], dn.data());
    ++gi;
    return SRS_OK;
  };
  bool done = false;
  int64_t cur = base;  // step of the realizations still running
  if (s->d.engine != SRS_ENGINE_RESIDENT) {
    SRS_TRY(plain_prestep(s, 1));
    int64_t total = 0;  // steps since the last normalisation (buffer parity)
    const int64_t chunk = 4096;
    while (true) {
      int64_t n = std::min<int64_t>(chunk, sc.n_steps + 1 - (cur - base));
      if (n <= 0) break;
      bool stop = false;
      if (gi < G && sc.grid_steps[gi] - cur <= n) {
        n = sc.grid_steps[gi] - cur;
        stop = true;
      } else {
        n += n & 1;  // whole chunks keep the double-buffer parity
      }
      // plain_steps assumes buffer 0 at the start: alternate by the count
      if (total & 1) return fail(SRS_ERR_STATE, "internal: odd chunk");
      if (n > 0) {
        SRS_TRY(t_begin());
        SRS_TRY(plain_steps(s, n));
        SRS_TRY(t_end());
        total += n;
        cur += n;
      }
      SRS_TRY(all_done(s, &done));
      if (stop) {
        SRS_TRY(deliver());
        total = 0;
      }
      if (done) break;
    }
  } else {
    // the first launch writes the t = 0 row and runs the protocol of step 0
    const int S = s->d.steps_per_launch > 0 ? s->d.steps_per_launch : 1000;
    int first = 1;
    while (!done) {
      int steps = S;
      if (gi < G && sc.grid_steps[gi] - cur < steps) steps = (int)(sc.grid_steps[gi] - cur);
      if (steps > 0) {
        SRS_TRY(t_begin());
        SRS_TRY(resident_launch(s, steps, first));
        SRS_TRY(t_end());
        first = 0;
        cur += steps;
      }
      SRS_TRY(all_done(s, &done));
      if (gi < G && cur == sc.grid_steps[gi]) SRS_TRY(deliver());
    }
  }
  if (n_launches) *n_launches = n_timed;
  return run_finish(s, out, since);
}

}  // extern "C"

// ---- multi-mesh batch ----------------------------------------------------------
struct srs_batch {
  std::vector<srs_sim*> sims;
  std::vector<size_t> order;  // enqueue order: decreasing elements x realizations
  int S = 1000;  // steps per member launch in one graph replay
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t graph = nullptr;
  int graph_mode = -1;  // run_protocol the graph was captured with
  int64_t replays = 0;
};

namespace {

void batch_drop_graph(srs_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_mode = -1;
}

// One replay: every member advances S steps on its own stream; the members'
// launches are branches of one graph forked from and joined into b->st.
// Members are enqueued by decreasing work (elements x realizations), so the
// longest clusters are dispatched first and the small members fill the SMs
// around them.
int batch_enqueue(srs_batch* b, int steps, int first) {
  SRS_CUDA(cudaEventRecord(b->fork, b->st));
  for (size_t i : b->order) {
    srs_sim* s = b->sims[i];
    SRS_CUDA(cudaStreamWaitEvent(s->st, b->fork, 0));
    SRS_TRY(resident_launch(s, steps, first));
    SRS_CUDA(cudaEventRecord(b->join[i], s->st));
    SRS_CUDA(cudaStreamWaitEvent(b->st, b->join[i], 0));
  }
  return SRS_OK;
}

int batch_graph(srs_batch* b) {
  const int mode = b->sims[0]->P.run_protocol;
  if (b->graph && b->graph_mode == mode) return SRS_OK;
  batch_drop_graph(b);
  cudaGraph_t g;
  SRS_CUDA(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  int rc = batch_enqueue(b, b->S, 0);
  cudaError_t e = cudaStreamEndCapture(b->st, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(SRS_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(SRS_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
  for (srs_sim* s : b->sims) s->launches--;  // counted per replay instead
  b->graph_mode = mode;
  return SRS_OK;
}

int batch_replay(srs_batch* b) {
  SRS_CUDA(cudaGraphLaunch(b->graph, b->st));
  for (srs_sim* s : b->sims) s->launches++;
  b->replays++;
  return SRS_OK;
}

}  // namespace

extern "C" {

int srs_batch_create(srs_sim* const* sims, int n, int steps_per_launch, srs_batch** out) {
  if (!sims || n <= 0 || !out) return fail(SRS_ERR_INPUT, "bad argument");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!sims[i]) return fail(SRS_ERR_INPUT, "null simulation");
    if (sims[i]->d.precision != SRS_FP32 || sims[i]->d.engine != SRS_ENGINE_RESIDENT)
      return fail(SRS_ERR_UNSUPPORTED, "batch members are FP32 resident simulations");
    for (int j = 0; j < i; ++j)
      if (sims[j] == sims[i]) return fail(SRS_ERR_INPUT, "a simulation appears twice in the batch");
  }
  srs_batch* b = new srs_batch();
  b->sims.assign(sims, sims + n);
  b->order.resize(n);
  for (int i = 0; i < n; ++i) b->order[i] = (size_t)i;
  std::stable_sort(b->order.begin(), b->order.end(), [&](size_t x, size_t y) {
    return (int64_t)sims[x]->N * sims[x]->R > (int64_t)sims[y]->N * sims[y]->R;
  });
  b->S = steps_per_launch > 0 ? steps_per_launch : 1000;
  b->join.assign(n, nullptr);
  bool ok = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; ok && i < n; ++i)
    ok = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    srs_batch_destroy(b);
    return fail(SRS_ERR_CUDA, "batch stream/event creation failed");
  }
  *out = b;
  return SRS_OK;
}

void srs_batch_destroy(srs_batch* b) {
  if (!b) return;
  if (b->st) cudaStreamSynchronize(b->st);
  batch_drop_graph(b);
  for (auto e : b->join)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

int srs_batch_advance(srs_batch* b, int64_t n_steps) {
  if (!b || n_steps < 0) return fail(SRS_ERR_INPUT, "bad argument");
  for (srs_sim* s : b->sims)
    if (s->P.run_protocol) {
      s->P.run_protocol = 0;
      refresh_args(s);
    }
  if (n_steps >= b->S) SRS_TRY(batch_graph(b));
  int64_t done = 0;
  for (; n_steps - done >= b->S; done += b->S) SRS_TRY(batch_replay(b));
  if (n_steps > done) SRS_TRY(batch_enqueue(b, (int)(n_steps - done), 0));
  return SRS_OK;
}

int srs_batch_synchronize(srs_batch* b) {
  if (!b) return fail(SRS_ERR_INPUT, "null argument");
  SRS_CUDA(cudaStreamSynchronize(b->st));
  return SRS_OK;
}

int srs_batch_time_advance(srs_batch* b, int64_t n_steps, float* ms) {
  if (!b || !ms) return fail(SRS_ERR_INPUT, "null argument");
  cudaEvent_t e0, e1;
  SRS_CUDA(cudaEventCreate(&e0));
  SRS_CUDA(cudaEventCreate(&e1));
  for (srs_sim* s : b->sims) SRS_CUDA(cudaStreamSynchronize(s->st));
  SRS_CUDA(cudaStreamSynchronize(b->st));
  SRS_CUDA(cudaEventRecord(e0, b->st));
  int rc = srs_batch_advance(b, n_steps);
  SRS_CUDA(cudaEventRecord(e1, b->st));
  SRS_CUDA(cudaEventSynchronize(e1));
  SRS_CUDA(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int srs_batch_run_simulation(srs_batch* b, srs_run_output* outs) {
  if (!b || !outs) return fail(SRS_ERR_INPUT, "null argument");
  const size_t n = b->sims.size();
  std::vector<Schedule> sc(n);
  std::vector<std::vector<int64_t>> before(n);
  for (size_t i = 0; i < n; ++i) SRS_TRY(run_prepare(b->sims[i], &outs[i], &sc[i], &before[i]));
  batch_drop_graph(b);  // run-mode arguments (rows, schedule) are captured afresh
  // the first launch of every member writes its t = 0 row
  SRS_TRY(batch_enqueue(b, b->S, 1));
  SRS_TRY(batch_graph(b));
  while (true) {
    SRS_CUDA(cudaStreamSynchronize(b->st));
    bool all = true;
    for (srs_sim* s : b->sims) {
      bool d = false;
      SRS_TRY(all_done(s, &d));
      all &= d;
    }
    if (all) break;
    SRS_TRY(batch_replay(b));
  }
  SRS_CUDA(cudaStreamSynchronize(b->st));
  batch_drop_graph(b);
  int rc = SRS_OK;
  for (size_t i = 0; i < n; ++i) {
    int r = run_finish(b->sims[i], &outs[i], before[i]);
    if (r && !rc) rc = r;
  }
  return rc;
}


int srs_linescan_setup(srs_sim* s, const srs_linescan_desc* d, int* n_samples) {
  if (!s || !d || d->res <= 0 || d->r_thresh <= 0) return fail(SRS_ERR_INPUT, "bad line-scan description");
  // linescan/main.cpp:160-190: line position and PSF widths by scan axis
  double sx = std::sqrt(d->var_x), sy = std::sqrt(d->var_y), sz = std::sqrt(d->var_z);
  if (d->axis == 2) {
    sx = std::sqrt(d->var_z);
    sy = std::sqrt(d->var_x);
    sz = std::sqrt(d->var_y);
  } else if (d->axis != 0 && d->axis != 1) {
    return fail(SRS_ERR_INPUT, "axis must be 0, 1 or 2");
  }
  const int ns = (int)((d->x_max - d->x_min) / d->res);
  if (ns <= 0) return fail(SRS_ERR_INPUT, "no line-scan samples");
  // normpdf3d with the tool's own constant (linescan/parameters.h: PI = 3.14159)
  const double alpha = 1.0 / std::pow(2 * 3.14159, 1.5);
  auto pdf = [&](double rx, double ry, double rz) {
    return alpha * std::exp(-0.5 * ((rx * rx / (sx * sx)) + (ry * ry / (sy * sy)) + (rz * rz / (sz * sz)))) /
           (sx * sy * sz);
  };
  auto center = [&](int i, double* c) {
    double xi = d->x_min + i * d->res;
    if (d->axis == 0) { c[0] = xi; c[1] = d->offset1; c[2] = d->offset2; }
    else if (d->axis == 1) { c[0] = d->offset1; c[1] = xi; c[2] = d->offset2; }
    else { c[0] = d->offset1; c[1] = d->offset2; c[2] = xi; }
  };
  // element centroids and volumes from the nodes (linescan/main.cpp:95-109:
  // the mean of the four nodes, |(c1-c4) . ((c2-c4) x (c3-c4))| / 6)
  const Mesh& m = s->m;
  std::vector<double> cx(m.N), cy(m.N), cz(m.N), vol(m.N);
  for (int j = 0; j < m.N; ++j) {
    double px[4], py[4], pz[4];
    for (int k = 0; k < 4; ++k) {
      int v = m.ele_nodes[4 * (size_t)j + k];
      px[k] = m.node_x[v];
      py[k] = m.node_y[v];
      pz[k] = m.node_z[v];
    }
    cx[j] = (px[0] + px[1] + px[2] + px[3]) / 4.0;
    cy[j] = (py[0] + py[1] + py[2] + py[3]) / 4.0;
    cz[j] = (pz[0] + pz[1] + pz[2] + pz[3]) / 4.0;
    double ax = px[0] - px[3], ay = py[0] - py[3], az = pz[0] - pz[3];
    double bx = px[1] - px[3], by = py[1] - py[3], bz = pz[1] - pz[3];
    double qx = px[2] - px[3], qy = py[2] - py[3], qz = pz[2] - pz[3];
    double nx = by * qz - bz * qy, ny = bz * qx - bx * qz, nz = bx * qy - by * qx;
    vol[j] = std::fabs((ax * nx + ay * ny + az * nz) / 6.0);
  }
  // padding voxels at the resting fluorescence (AddPointGrid, :275-313)
  std::vector<double> px, py, pz, pv;
  auto add_grid = [&](double x0, double x1, double y0, double y1, double z0, double z1) {
    double dx = d->pad_res, dy = d->pad_res, dz = d->pad_res;
    if (x0 > x1) dx = -dx;
    if (y0 > y1) dy = -dy;
    if (z0 > z1) dz = -dz;
    int nx = (int)((x1 - x0) / dx), ny = (int)((y1 - y0) / dy), nz = (int)((z1 - z0) / dz);
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) {
          px.push_back(x0 + i * dx + 0.5 * dx);
          py.push_back(y0 + j * dy + 0.5 * dy);
          pz.push_back(z0 + k * dz + 0.5 * dz);
          pv.push_back(std::fabs(dx * dy * dz));
        }
  };
  if (d->pad_res > 0) {
    const double* D = d->domain;
    double a0 = d->pad_min, a1 = d->pad_max;
    add_grid(a0, a1, a0, a1, D[5], a1);
    add_grid(a0, a1, a0, a1, D[4], a0);
    add_grid(D[0], a0, a0, a1, D[4], D[5]);
    add_grid(D[1], a1, a0, a1, D[4], D[5]);
    add_grid(D[0], D[1], D[2], a0, D[4], D[5]);
    add_grid(D[0], D[1], D[3], a1, D[4], D[5]);
  }
  std::vector<int32_t> ptr(ns + 1, 0), col;
  std::vector<double> w, pad(ns, 0.0);
  s->ls_rest.assign(ns, 0.0);
  std::vector<double> S6;
  initial_states(m, s->p, &S6);
  for (int i = 0; i < ns; ++i) {
    double c[3];
    center(i, c);
    ptr[i] = (int32_t)col.size();
    double rest = 0.0;
    for (int j = 0; j < m.N; ++j) {
      double rx = cx[j] - c[0], ry = cy[j] - c[1], rz = cz[j] - c[2];
      if (rx * rx + ry * ry + rz * rz < d->r_thresh) {
        double wj = vol[j] * pdf(rx, ry, rz);
        col.push_back(s->eng_of_ref[j]);
        w.push_back(wj);
        rest += wj * S6[SP_DYE * (size_t)m.N + j];
      }
    }
    double pd = 0.0;
    for (size_t q = 0; q < px.size(); ++q) {
      double rx = px[q] - c[0], ry = py[q] - c[1], rz = pz[q] - c[2];
      if (rx * rx + ry * ry + rz * rz < d->r_thresh) pd += pv[q] * d->f0_pad * pdf(rx, ry, rz);
    }
    pad[i] = pd;
    s->ls_rest[i] = pd + rest;
  }
  ptr[ns] = (int32_t)col.size();
  s->ls_ptr_h = ptr;
  s->ls_col_h = col;
  s->ls_w_h = w;
  s->ls_pad_h = pad;
  s->ls_version++;
  LinescanArgs& a = s->ls;
  a.n_samples = ns;
  a.n_state = (int32_t)eng_count(s);
  SRS_TRY(dev_upload(s, (int32_t**)&a.ptr, ptr.data(), ptr.size()));
  SRS_TRY(dev_upload(s, (int32_t**)&a.col, col.data(), col.size()));
  SRS_TRY(dev_upload(s, (double**)&a.w, w.data(), w.size()));
  SRS_TRY(dev_upload(s, (double**)&a.pad, pad.data(), pad.size()));
  if (s->d.precision != SRS_FP64) {
    std::vector<double> rd(eng_count(s), 0.0);
    for (size_t e = 0; e < rd.size(); ++e) {
      int j = s->ref_of_eng[e];
      if (j >= 0 && s->m.domain[j] == DOMAIN_CYTO) rd[e] = s->rv.dye;
    }
    SRS_TRY(dev_upload(s, (double**)&a.rest_dye, rd.data(), rd.size()));
  }
  SRS_TRY(dev_alloc(s, &s->d_ls_out, (size_t)s->R * ns));
  a.out = s->d_ls_out;
  if (n_samples) *n_samples = ns;
  return SRS_OK;
}

int srs_linescan(srs_sim* s, double* out, double* rest) {
  if (!s || !s->ls.ptr) return fail(SRS_ERR_STATE, "call srs_linescan_setup first");
  LinescanArgs a = s->ls;
  if (s->d.precision == SRS_FP64) {
    a.S64 = s->d_S[0];
  } else {
    a.M = s->d_M[0];
    a.CM = s->d_CM;
    a.CMq = s->d_CMq;
  }
  if (launch_linescan(a, s->R, s->st)) return fail(SRS_ERR_CUDA, "line-scan launch failed");
  s->launches++;
  if (out)
    SRS_CUDA(cudaMemcpyAsync(out, s->d_ls_out, sizeof(double) * s->R * a.n_samples,
                             cudaMemcpyDeviceToHost, s->st));
  SRS_CUDA(cudaStreamSynchronize(s->st));
  if (rest) std::memcpy(rest, s->ls_rest.data(), sizeof(double) * a.n_samples);
  return SRS_OK;
}

static const int kAdjParam[SRS_N_ADJ] = {
    R_D_CA,      R_D_DYE,       R_K_ON_CMDN, R_K_OFF_CMDN, R_K_ON_TRPN, R_K_OFF_TRPN,
    R_K_ON_CSQN, R_K_OFF_CSQN,  R_K_ON_DYE,  R_K_OFF_DYE,  R_V_RYR,     R_A_P,
    R_B_TOT_SL_HI, R_K_D_SL_HI, R_D_ATP,     R_D_CMDN,     R_K_ON_ATP,  R_K_OFF_ATP};

int srs_adjoint_param_index(int k) { return (k >= 0 && k < SRS_N_ADJ) ? kAdjParam[k] : -1; }

}  // extern "C"

namespace {

// Device work buffers of srs_adjoint, numbered in request order and kept in
// the simulation between calls (grown when a call needs more).
struct Scratch {
  srs_sim* s;
  size_t next = 0;
  template <class T>
  int get(T** out, size_t n) {
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    if (next == s->adj_bufs.size()) s->adj_bufs.push_back({nullptr, 0});
    auto& b = s->adj_bufs[next++];
    if (b.second < bytes) {
      if (b.first) cudaFree(b.first);
      b = {nullptr, 0};
      void* q = nullptr;
      cudaError_t e = cudaMalloc(&q, bytes);
      if (e != cudaSuccess)
        return fail(SRS_ERR_NOMEM, std::string("adjoint buffers: ") + cudaGetErrorString(e));
      b = {q, bytes};
    }
    *out = (T*)b.first;
    return SRS_OK;
  }
};

// Transposed coefficients, RyR volume factors and the element -> sample map
// of the line scan, in the resident engine layout.
int adjoint_setup(srs_sim* s) {
  if (!s->aT_h.empty() && s->adj_ls_version == s->ls_version) return SRS_OK;
  const int NE = (int)eng_count(s);
  if (s->aT_h.empty()) {
    std::vector<float4>& aT = s->aT_h;
    aT.assign(NE, make_float4(0, 0, 0, 0));
    for (int e = 0; e < NE; ++e) {
      const int j = s->ref_of_eng[e];
      if (j < 0) continue;
      float v[4] = {0, 0, 0, 0};
      for (int k = 0; k < 4; ++k) {
        const int nj = s->op.nij[4 * (size_t)j + k];
        if (nj == j || s->op.aij[5 * (size_t)j + 1 + k] == 0.0) continue;
        for (int l = 0; l < 4; ++l)
          if (s->op.nij[4 * (size_t)nj + l] == j) {
            v[k] = (float)s->op.aij[5 * (size_t)nj + 1 + l];
            break;
          }
      }
      aT[e] = make_float4(v[0], v[1], v[2], v[3]);
    }
    std::vector<float> scl(s->NR), sjs(s->NR);
    for (int i = 0; i < s->NR; ++i) {
      scl[i] = (float)(1.0 / s->m.V0[s->m.ryr_ele[i]]);
      sjs[i] = (float)(-(1.0 / s->m.V0[s->m.ryr_jsr[i]]));
    }
    SRS_TRY(dev_upload(s, &s->d_ryr_s_cl, scl.data(), scl.size()));
    SRS_TRY(dev_upload(s, &s->d_ryr_s_js, sjs.data(), sjs.size()));
  }
  const int ns = s->ls.n_samples;
  std::vector<int32_t> cnt(NE + 1, 0);
  for (size_t q = 0; q < s->ls_col_h.size(); ++q) cnt[s->ls_col_h[q] + 1]++;
  for (int e = 0; e < NE; ++e) cnt[e + 1] += cnt[e];
  std::vector<int32_t> idx(s->ls_col_h.size());
  std::vector<double> wv(s->ls_col_h.size());
  std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
  for (int i = 0; i < ns; ++i)
    for (int q = s->ls_ptr_h[i]; q < s->ls_ptr_h[i + 1]; ++q) {
      const int e = s->ls_col_h[q];
      idx[fill[e]] = i;
      wv[fill[e]] = s->ls_w_h[q];
      fill[e]++;
    }
  SRS_TRY(dev_upload(s, &s->d_wt_ptr, cnt.data(), cnt.size()));
  SRS_TRY(dev_upload(s, &s->d_wt_idx, idx.data(), idx.size()));
  SRS_TRY(dev_upload(s, &s->d_wt_w, wv.data(), wv.size()));
  // the resting part of every sample, pad + sum_q w_q dye_rest(col_q): the
  // tick kernels add the trajectory's dye deviations to it
  std::vector<double> base(ns);
  for (int i = 0; i < ns; ++i) {
    double acc = 0.0;
    for (int q = s->ls_ptr_h[i]; q < s->ls_ptr_h[i + 1]; ++q) {
      const int j = s->ref_of_eng[s->ls_col_h[q]];
      if (j >= 0 && s->m.domain[j] == DOMAIN_CYTO) acc += s->ls_w_h[q] * s->rv.dye;
    }
    base[i] = s->ls_pad_h[i] + acc;
  }
  SRS_TRY(dev_upload(s, &s->d_ls_base, base.data(), base.size()));
  s->adj_ls_version = s->ls_version;
  return SRS_OK;
}

// Device copies of the complete engine state of all realizations.
struct StateSnap {
  float4* M = nullptr;
  float* I = nullptr;
  float4* CM = nullptr;  // compensation: float, or compact (srs_comp.h) in CMq / CIq
  float* CI = nullptr;
  ushort4* CMq = nullptr;
  uint16_t* CIq = nullptr;
  int32_t *ryr = nullptr, *lcc = nullptr, *lccv = nullptr;
  double* res = nullptr;
  RealCtl* ctl = nullptr;
};

// Reverse-sweep records with neighbour codes for CTAs that each hold m
// consecutive partitions of the forward layout (same element order, so every
// per-element array keeps its index).  The two domain flags ride in sign
// bits: bsl and sa are never negative.
int adjoint_geometry(srs_sim* s, int m, int bits) {
  if (s->d_adj_geo && s->adj_geo_m == m) return SRS_OK;
  const int Pf = s->P_stride, NE = (int)eng_count(s);
  auto mcode = [&](int e) -> uint16_t {
    const int q = e / Pf, off = e % Pf;
    return (uint16_t)(((q / m) << bits) | ((q % m) * Pf + off));
  };
  std::vector<AdjRec> geo(NE);
  std::memset(geo.data(), 0, geo.size() * sizeof(AdjRec));
  for (int e = 0; e < NE; ++e) {
    const int j = s->ref_of_eng[e];
    if (j < 0) {
      for (int k = 0; k < 4; ++k) geo[e].nb[k] = mcode(e);
      continue;
    }
    float a[4];
    for (int k = 0; k < 4; ++k) {
      a[k] = (float)s->op.aij[5 * (size_t)j + 1 + k];
      geo[e].nb[k] = mcode(s->eng_of_ref[s->op.nij[4 * (size_t)j + k]]);
    }
    const float4 t = s->aT_h[e];
    geo[e].aT[0] = t.x;
    geo[e].aT[1] = t.y;
    geo[e].aT[2] = t.z;
    geo[e].aT[3] = t.w;
    const float sa = (a[0] + a[1]) + (a[2] + a[3]);
    const float bsl = bsl_of(s, j);
    geo[e].bsl = s->m.tropc[j] ? -bsl : bsl;
    geo[e].sa = s->m.domain[j] == DOMAIN_JSR ? -sa : sa;
    if (bsl < 0.0f || sa < 0.0f || std::signbit(bsl) || std::signbit(sa))
      return fail(SRS_ERR_MESH, "negative SL capacity or coupling coefficient");
  }
  if (s->d_adj_geo) {
    SRS_CUDA(cudaMemcpy(s->d_adj_geo, geo.data(), geo.size() * sizeof(AdjRec), cudaMemcpyHostToDevice));
  } else {
    SRS_TRY(dev_upload(s, &s->d_adj_geo, geo.data(), geo.size()));
  }
  s->adj_geo_m = m;
  return SRS_OK;
}

// Reverse-step records of the plain engine: aT in engine order and (bsl,
// sum a + kb) with TropC and JSR in the sign bits.
int adjoint_plain_geometry(srs_sim* s) {
  if (s->d_adjp_aT) return SRS_OK;
  const int N = s->N;
  std::vector<float2> bs(N);
  for (int e = 0; e < N; ++e) {
    const int j = s->ref_of_eng[e];
    float a[4];
    for (int k = 0; k < 4; ++k) a[k] = (float)s->op.aij[5 * (size_t)j + 1 + k];
    const float sa = ((a[0] + a[1]) + (a[2] + a[3])) + (float)s->op.kb[j];
    const float bsl = bsl_of(s, j);
    if (bsl < 0.0f || sa < 0.0f || std::signbit(bsl) || std::signbit(sa))
      return fail(SRS_ERR_MESH, "negative SL capacity or coupling coefficient");
    bs[e] = make_float2(s->m.tropc[j] ? -bsl : bsl, s->m.domain[j] == DOMAIN_JSR ? -sa : sa);
  }
  SRS_TRY(dev_upload(s, &s->d_adjp_aT, s->aT_h.data(), s->aT_h.size()));
  SRS_TRY(dev_upload(s, &s->d_adjp_bs, bs.data(), bs.size()));
  return SRS_OK;
}

// Checkpoint plan of a reverse sweep over nseg trajectory segments: L levels
// of at most f - 1 snapshots each (f^L >= nseg), plus the final state.  The
// sweep recomputes the forward run L times at most; one level is the plain
// "checkpoint every K steps" scheme.  Returns false when max_snaps snapshots
// cannot hold any plan.
bool checkpoint_plan(int64_t nseg, int64_t max_snaps, int* L, int64_t* f) {
  for (int l = 1; l <= 12; ++l) {
    int64_t g = (int64_t)std::ceil(std::pow((double)nseg, 1.0 / l));
    while (g > 1) {  // the smallest fan-out with g^l >= nseg
      int64_t p = 1;
      for (int i = 0; i < l && p < nseg; ++i) p *= g - 1;
      if (p >= nseg) --g;
      else break;
    }
    for (;;) {
      int64_t p = 1;
      for (int i = 0; i < l && p < nseg; ++i) p *= g;
      if (p >= nseg) break;
      ++g;
    }
    if ((int64_t)l * std::max<int64_t>(g - 1, 0) + 1 <= max_snaps) {
      *L = l;
      *f = std::max<int64_t>(g, 1);
      return true;
    }
  }
  return false;
}

// Segment length and checkpoint plan of srs_adjoint for the device memory
// free now (buffers the previous calls keep count as free).
struct AdjPlan {
  int K;        // steps of a recorded segment
  int L;        // checkpoint levels (forward recomputations)
  int64_t fan;  // pieces per level
  int64_t forward_steps;  // forward steps the sweep runs (advance and record)
};

int adjoint_plan(srs_sim* s, const srs_adjoint_desc* d, AdjPlan* pl) {
  if (s->d.precision != SRS_FP32)
    return fail(SRS_ERR_UNSUPPORTED, "the adjoint runs on the FP32 engines");
  if (d->n_steps < 1 || d->tick_every < 1 || d->checkpoint_every < 0 || d->max_checkpoints < 0)
    return fail(SRS_ERR_INPUT, "n_steps and tick_every must be positive");
  const bool plain = s->d.engine != SRS_ENGINE_RESIDENT;
  const int R = s->R, NR = s->NR, NL = s->NL, W = NR + 2 * NL + 1, te = d->tick_every;
  const size_t NE = eng_count(s);
  const int ns = s->ls.n_samples;
  const int64_t n_steps = d->n_steps, n_ticks = n_steps / te;
  // bytes: one recorded step, one snapshot of the whole state, lambda
  const size_t step_b = (size_t)R * (NE * (plain ? 28 : 24) + (size_t)W * 4);
  // state 20 B per element, compensation 20 B (10 B compact)
  const size_t snap_b = (size_t)R * NE * (s->d_CMq ? 30 : 40) + (size_t)R * (NR + 2 * NL) * 4 +
                        (size_t)R * s->NCH * 8 + (size_t)R * sizeof(RealCtl);
  const size_t lam_b = (size_t)R * NE * (plain ? 76 : 44);
  size_t free_b = 0, total_b = 0, held = 0;
  for (auto& b : s->adj_bufs) held += b.second;
  SRS_CUDA(cudaMemGetInfo(&free_b, &total_b));
  free_b += held;
  int K = d->checkpoint_every;
  if (K == 0) {
    // automatic: keep the whole trajectory (no recomputation) when it takes
    // at most half of the free device memory, else segments of 256 steps
    // (fewer when 256 recorded steps would take more than a quarter)
    const size_t whole = (size_t)(n_steps + 1) * step_b;
    if (n_steps <= INT32_MAX && whole <= free_b / 2) {
      K = (int)n_steps;
    } else {
      K = 256;
      while (K > 8 && (size_t)(K + 1) * step_b > free_b / 4) K /= 2;
    }
  }
  const int64_t nseg = (n_steps + K - 1) / K;
  // memory: snapshots, one segment of trajectory, lambda, tick coefficients
  const size_t traj_b = (size_t)(K + 1) * R * NE * 24 + (size_t)K * R * (W + (plain ? NE : 0)) * 4;
  const size_t fixed = traj_b + lam_b + (size_t)(K / te + 2) * R * ns * 8 +
                       (size_t)R * std::max<int64_t>(n_ticks, 1) * ns * 16;
  const size_t usable = free_b / 10 * 9;
  int64_t max_snaps = usable > fixed ? (int64_t)((usable - fixed) / snap_b) : 0;
  if (d->max_checkpoints > 0) max_snaps = std::min<int64_t>(max_snaps, d->max_checkpoints + 1);
  int L = 1;
  int64_t fan = 1;
  if (!checkpoint_plan(nseg, max_snaps, &L, &fan))
    return fail(SRS_ERR_NOMEM, "adjoint needs " + std::to_string((fixed + 2 * snap_b) >> 20) +
                                   " MiB of device memory at least (" + std::to_string(free_b >> 20) +
                                   " MiB free): lower checkpoint_every or the realizations");
  pl->K = K;
  pl->L = L;
  pl->fan = fan;
  // forward steps of the recursion (see srs_adjoint)
  std::vector<int64_t> q(L + 1);
  q[L] = K;
  for (int l = L - 1; l >= 0; --l) q[l] = l == L - 1 ? K : std::min<int64_t>(INT64_MAX / 2, q[l + 1] * fan);
  std::function<int64_t(int, int64_t)> cnt = [&](int l, int64_t len) -> int64_t {
    if (l == L) return len;
    const int64_t p = (len + q[l] - 1) / q[l];
    return (p - 1) * q[l] + cnt(l + 1, len - (p - 1) * q[l]) + (p - 1) * cnt(l + 1, q[l]);
  };
  pl->forward_steps = cnt(0, n_steps);
  return SRS_OK;
}

int snap_alloc(srs_sim* s, Scratch& sc, StateSnap* o) {
  const size_t n = (size_t)s->R * eng_count(s);
  SRS_TRY(sc.get(&o->M, n));
  SRS_TRY(sc.get(&o->I, n));
  if (s->d_CMq) {
    SRS_TRY(sc.get(&o->CMq, n));
    SRS_TRY(sc.get(&o->CIq, n));
  } else {
    SRS_TRY(sc.get(&o->CM, n));
    SRS_TRY(sc.get(&o->CI, n));
  }
  SRS_TRY(sc.get(&o->ryr, (size_t)s->R * s->NR));
  SRS_TRY(sc.get(&o->lcc, (size_t)s->R * s->NL));
  SRS_TRY(sc.get(&o->lccv, (size_t)s->R * s->NL));
  SRS_TRY(sc.get(&o->res, (size_t)s->R * s->NCH));
  SRS_TRY(sc.get(&o->ctl, (size_t)s->R));
  return SRS_OK;
}

int snap_copy(srs_sim* s, const StateSnap& o, bool save) {
  const size_t n = (size_t)s->R * eng_count(s);
  auto cp = [&](void* snap, void* live, size_t bytes) -> cudaError_t {
    return save ? cudaMemcpyAsync(snap, live, bytes, cudaMemcpyDeviceToDevice, s->st)
                : cudaMemcpyAsync(live, snap, bytes, cudaMemcpyDeviceToDevice, s->st);
  };
  SRS_CUDA(cp(o.M, s->d_M[0], n * sizeof(float4)));
  SRS_CUDA(cp(o.I, s->d_I[0], n * sizeof(float)));
  if (s->d_CMq) {
    SRS_CUDA(cp(o.CMq, s->d_CMq, n * sizeof(ushort4)));
    SRS_CUDA(cp(o.CIq, s->d_CIq, n * sizeof(uint16_t)));
  } else {
    SRS_CUDA(cp(o.CM, s->d_CM, n * sizeof(float4)));
    SRS_CUDA(cp(o.CI, s->d_CI, n * sizeof(float)));
  }
  SRS_CUDA(cp(o.ryr, s->d_ryr, (size_t)s->R * s->NR * 4));
  SRS_CUDA(cp(o.lcc, s->d_lcc, (size_t)s->R * s->NL * 4));
  SRS_CUDA(cp(o.lccv, s->d_lccv, (size_t)s->R * s->NL * 4));
  SRS_CUDA(cp(o.res, s->d_res, (size_t)s->R * s->NCH * 8));
  SRS_CUDA(cp(o.ctl, s->d_ctl, (size_t)s->R * sizeof(RealCtl)));
  return SRS_OK;
}

}  // namespace

extern "C" {

int srs_adjoint(srs_sim* s, const srs_adjoint_desc* d, srs_adjoint_out* out) {
  if (!s || !d || !out || !out->loss || !out->grad || !d->f0) return fail(SRS_ERR_INPUT, "null argument");
  if (!s->ls.ptr) return fail(SRS_ERR_STATE, "call srs_linescan_setup first");
  AdjPlan pl;
  SRS_TRY(adjoint_plan(s, d, &pl));  // also checks the descriptor
  const bool plain = s->d.engine != SRS_ENGINE_RESIDENT;
  const int R = s->R, NR = s->NR, NL = s->NL, W = NR + 2 * NL + 1, te = d->tick_every;
  const size_t NE = eng_count(s);
  const int ns = s->ls.n_samples;
  const int64_t n_steps = d->n_steps, n_ticks = n_steps / te;
  const int K = pl.K, L = pl.L;
  const int64_t fan = pl.fan;
  SRS_TRY(adjoint_setup(s));
  Scratch sc{s};
  // level l holds the starts of its pieces but the last; then the final state
  std::vector<std::vector<StateSnap>> lv(L, std::vector<StateSnap>(std::max<int64_t>(fan - 1, 0)));
  for (auto& l : lv)
    for (auto& c : l) SRS_TRY(snap_alloc(s, sc, &c));
  StateSnap fin;
  SRS_TRY(snap_alloc(s, sc, &fin));
  float4* traj_u;
  float2* traj_ig;
  int32_t* traj_ch;
  float* traj_ib = nullptr;  // plain engine: 1 / B of every recorded state
  SRS_TRY(sc.get(&traj_u, (size_t)(K + 1) * R * NE));
  SRS_TRY(sc.get(&traj_ig, (size_t)(K + 1) * R * NE));
  SRS_TRY(sc.get(&traj_ch, (size_t)K * R * W));
  if (plain) SRS_TRY(sc.get(&traj_ib, (size_t)K * R * NE));
  float4 *lam, *lam_c4;
  float *lam_im, *lam_cim;
  SRS_TRY(sc.get(&lam, (size_t)R * NE));
  SRS_TRY(sc.get(&lam_c4, (size_t)R * NE));
  SRS_TRY(sc.get(&lam_im, (size_t)R * NE));
  SRS_TRY(sc.get(&lam_cim, (size_t)R * NE));
  float* lam_c;
  SRS_TRY(sc.get(&lam_c, (size_t)R * NE));
  double *coef, *grad, *loss, *f0, *target = nullptr;
  SRS_TRY(sc.get(&coef, (size_t)(K / te + 2) * R * ns));
  SRS_TRY(sc.get(&grad, (size_t)R * SRS_N_ADJ));
  SRS_TRY(sc.get(&loss, (size_t)std::max<int64_t>(n_ticks, 1) * R * ns));  // [tick][R][sample]
  SRS_TRY(sc.get(&f0, (size_t)ns));
  SRS_CUDA(cudaMemcpyAsync(f0, d->f0, sizeof(double) * ns, cudaMemcpyHostToDevice, s->st));
  const bool mean_trace = (d->flags & SRS_ADJ_MEAN_TRACE) != 0;
  const size_t tg_rows = mean_trace ? 1 : (size_t)R;  // target per realization or shared
  {
    double* tg;
    SRS_TRY(sc.get(&tg, tg_rows * std::max<int64_t>(n_ticks, 1) * ns));
    if (d->target && n_ticks > 0) target = tg;
  }
  if (target) {
    SRS_CUDA(cudaMemcpyAsync(target, d->target, sizeof(double) * tg_rows * n_ticks * ns,
                             cudaMemcpyHostToDevice, s->st));
  }
  s->P.run_protocol = 0;
  refresh_args(s);
  // plain engine: the published slots (double buffered) and the gradient
  // rows of the reverse-step blocks
  float4* pub[2] = {nullptr, nullptr};
  double* part = nullptr;
  int adjp_by = 0;
  if (plain) {
    int dev = 0, n_sm = 0;
    SRS_CUDA(cudaGetDevice(&dev));
    SRS_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    adjp_by = adjp_blocks_per_realization((int)NE, R, n_sm);
    SRS_TRY(sc.get(&pub[0], (size_t)R * NE));
    SRS_TRY(sc.get(&pub[1], (size_t)R * NE));
    SRS_TRY(sc.get(&part, (size_t)R * adjp_by * SRS_N_ADJ));
    SRS_TRY(adjoint_plain_geometry(s));
  }

  // ---- engine operations on the live state ----------------------------------
  // advance: len steps without recording (the plain engine's state returns
  // to buffer 0)
  auto advance_live = [&](int64_t len) -> int {
    if (!plain) {
      for (int64_t done = 0; done < len;) {
        const int k = (int)std::min<int64_t>(K, len - done);
        SRS_TRY(resident_launch(s, k));
        done += k;
      }
      return SRS_OK;
    }
    SRS_TRY(plain_steps(s, len));
    if (len & 1) {
      SRS_CUDA(cudaMemcpyAsync(s->d_M[0], s->d_M[1], sizeof(float4) * R * NE, cudaMemcpyDeviceToDevice, s->st));
      SRS_CUDA(cudaMemcpyAsync(s->d_I[0], s->d_I[1], sizeof(float) * R * NE, cudaMemcpyDeviceToDevice, s->st));
    }
    return SRS_OK;
  };
  // record: len steps writing trajectory slots 0 .. len (slot t = x_{s0+t})
  auto record_live = [&](int len) -> int {
    if (!plain) {
      ResidentArgs ra = s->ar;
      ra.steps = len;
      ra.prestep_first = 0;
      ra.initial_row = 0;
      ra.speculate = 1;
      ra.traj_u = traj_u;
      ra.traj_ig = traj_ig;
      ra.traj_ch = traj_ch;
      if (launch_resident(ra, s->C, s->n_clusters, s->threads, s->smem, s->st))
        return fail(SRS_ERR_CUDA, std::string("trajectory launch: ") + cudaGetErrorString(cudaGetLastError()));
      s->launches++;
      return SRS_OK;
    }
    for (int t = 0; t < len; ++t) {
      Plain32Args a = s->a32;
      const int par = t & 1;
      a.M_in = s->d_M[par];
      a.I_in = s->d_I[par];
      a.M_out = s->d_M[par ^ 1];
      a.I_out = s->d_I[par ^ 1];
      a.traj_u = traj_u + (size_t)t * R * NE;
      a.traj_ig = traj_ig + (size_t)t * R * NE;
      a.traj_ch = traj_ch + (size_t)t * R * W;
      a.traj_ib = traj_ib + (size_t)t * R * NE;
      if (launch_plain32_step(a, s->st))
        return fail(SRS_ERR_CUDA, std::string("trajectory step: ") + cudaGetErrorString(cudaGetLastError()));
      s->launches += plain32_kernels_per_step(a);
    }
    const int par = len & 1;
    SRS_CUDA(cudaMemcpyAsync(traj_u + (size_t)len * R * NE, s->d_M[par], sizeof(float4) * R * NE,
                             cudaMemcpyDeviceToDevice, s->st));
    if (par) {
      SRS_CUDA(cudaMemcpyAsync(s->d_M[0], s->d_M[1], sizeof(float4) * R * NE, cudaMemcpyDeviceToDevice, s->st));
      SRS_CUDA(cudaMemcpyAsync(s->d_I[0], s->d_I[1], sizeof(float) * R * NE, cudaMemcpyDeviceToDevice, s->st));
    }
    return SRS_OK;
  };

  // ---- reverse-sweep arguments ------------------------------------------------
  AdjConsts ak{};
  {
    const RestValues& rv = s->rv;
    const double brest[5] = {rv.dye, rv.atp, rv.cmdn, rv.trpn, rv.csqn};
    for (int q = 0; q < 5; ++q) ak.brest[q] = (float)brest[q];
    const double bt = s->p.reals[R_B_TOT_SL_HI];
    ak.inv_btot_sl = bt != 0.0 ? (float)(1.0 / bt) : 0.0f;
    ak.serca_per_ap = 2e-3f;
    ak.v_cell = (float)s->p.reals[R_V_CELL];
    ak.inv_khi = (float)(1.0 / s->p.reals[R_K_D_SL_HI]);
    // Dirichlet sources D kb Bv of dye, ATP, CMDN, Bv = c0 B / (Kd + c0)
    const double* Rr = s->p.reals;
    const int dq[3] = {R_D_DYE, R_D_ATP, R_D_CMDN}, onq[3] = {R_K_ON_DYE, R_K_ON_ATP, R_K_ON_CMDN},
              offq[3] = {R_K_OFF_DYE, R_K_OFF_ATP, R_K_OFF_CMDN};
    const double bv[3] = {rv.dye, rv.atp, rv.cmdn};
    for (int q = 0; q < 3; ++q) {
      const double kon = Rr[onq[q]], Kd = Rr[offq[q]] / kon, den = Kd + Rr[R_C_0_CA];
      ak.kb_on[q] = (float)(Rr[dq[q]] * bv[q] * Kd / (kon * den));
      ak.kb_off[q] = (float)(-Rr[dq[q]] * bv[q] / (kon * den));
    }
  }
  SRS_CUDA(cudaMemsetAsync(lam, 0, sizeof(float4) * R * NE, s->st));
  SRS_CUDA(cudaMemsetAsync(lam_c4, 0, sizeof(float4) * R * NE, s->st));
  SRS_CUDA(cudaMemsetAsync(lam_im, 0, sizeof(float) * R * NE, s->st));
  SRS_CUDA(cudaMemsetAsync(lam_cim, 0, sizeof(float) * R * NE, s->st));
  SRS_CUDA(cudaMemsetAsync(grad, 0, sizeof(double) * R * SRS_N_ADJ, s->st));
  if (part) SRS_CUDA(cudaMemsetAsync(part, 0, sizeof(double) * R * adjp_by * SRS_N_ADJ, s->st));
  SRS_CUDA(cudaMemsetAsync(loss, 0, sizeof(double) * std::max<int64_t>(n_ticks, 1) * R * ns, s->st));
  AdjArgs aa{};
  int best_C = 0, adj_ncl = 0, adj_threads = 0;
  size_t adj_smem = 0;
  unsigned int* d_status;
  SRS_TRY(sc.get(&d_status, 1));
  SRS_CUDA(cudaMemsetAsync(d_status, 0, sizeof(unsigned int), s->st));
  if (!plain) {
    aa.R = R;
    aa.P = s->P_stride;
    aa.n_local = s->ar.n_local;
    aa.n_chtet = s->ar.n_chtet;
    aa.n_int = s->ar.n_int;
    aa.ch_interior = s->ar.ch_interior;
    aa.ch_ptr = s->ar.ch_ptr;
    aa.ch_list = s->ar.ch_list;
    aa.ryr_cleft_code = s->ar.ryr_cleft_code;
    aa.ryr_jsr_code = s->ar.ryr_jsr_code;
    aa.ryr_s_cl = s->d_ryr_s_cl;
    aa.ryr_s_js = s->d_ryr_s_js;
    aa.NR = NR;
    aa.NL = NL;
    aa.traj_u = traj_u;
    aa.traj_ig = traj_ig;
    aa.traj_ch = traj_ch;
    aa.tick_every = te;
    aa.n_samples = ns;
    aa.coef = coef;
    aa.wt_ptr = s->d_wt_ptr;
    aa.wt_idx = s->d_wt_idx;
    aa.wt_w = s->d_wt_w;
    aa.lam = lam;
    aa.lam_im = lam_im;
    aa.lam_c4 = lam_c4;
    aa.lam_cim = lam_cim;
    aa.lam_c = lam_c;
    aa.grad = grad;
    aa.k = s->ar.k;
    aa.ak = ak;
    const int n_ent = 2 * NR + NL;
    if (d->threads_per_cta != 0 &&
        (d->threads_per_cta % 32 || d->threads_per_cta < 64 || d->threads_per_cta > 512))
      return fail(SRS_ERR_INPUT, "threads_per_cta must be a multiple of 32 in [64, 512]");
    if (d->cta_partitions < 0 || (d->cta_partitions > 0 && s->C % d->cta_partitions))
      return fail(SRS_ERR_INPUT, "cta_partitions must divide the cluster size");
    // CTA grouping: m forward partitions per CTA (clusters of C/m CTAs), the
    // owner state of lambda on chip when it fits next to the published slots,
    // 256 or 512 threads.  Chosen by the estimated time, rounds of clusters x
    // slots per thread; at equal estimate the 256-thread CTA wins (two CTAs per
    // SM overlap each other's barrier waits).
    int best_m = 0, best_bits = 0;
    bool best_own = false, best_stage = false;
    double best_cost = 1e300;
    const std::vector<int> thr_list =
        d->threads_per_cta ? std::vector<int>{d->threads_per_cta} : std::vector<int>{256, 512};
    for (int thr : thr_list) {
      for (int m = 1; m <= s->C; ++m) {
        if (s->C % m || (d->cta_partitions && m != d->cta_partitions)) continue;
        const int Ca = s->C / m, Pc = m * s->P_stride;
        int bits = 1, rbits = 0;
        while ((1 << bits) < Pc) ++bits;
        while ((1 << rbits) < Ca) ++rbits;
        if (bits + rbits > 16) continue;
        for (int stage = 1; stage >= 0; --stage) {
          if (stage && (d->flags & SRS_ADJ_NO_STAGE)) continue;
          if (!stage && (d->flags & SRS_ADJ_STAGE)) continue;
          for (int own = 1; own >= 0; --own) {
            if (own && (d->flags & SRS_ADJ_LAMBDA_GLOBAL)) continue;
            const size_t sm = adjoint_smem_bytes(Pc, s->part_nch[0], n_ent, own != 0, stage != 0);
            const int ncl = std::min(adjoint_max_clusters(Ca, thr, sm), R);
            if (ncl <= 0) continue;
            const double cost = std::ceil((double)R / ncl) * std::ceil((double)Pc / thr) *
                                (own ? 1.0 : 1.15) * (stage ? 1.01 : 1.0) * (thr == 512 ? 1.02 : 1.0);
            if (cost < best_cost) {
              best_cost = cost;
              best_m = m;
              best_C = Ca;
              adj_ncl = ncl;
              adj_smem = sm;
              best_own = own != 0;
              best_stage = stage != 0;
              best_bits = bits;
              adj_threads = thr;
            }
            break;  // the on-chip variant when it fits
          }
        }
      }
    }
    if (adj_ncl <= 0) return fail(SRS_ERR_UNSUPPORTED, "adjoint configuration does not fit on the device");
    SRS_TRY(adjoint_geometry(s, best_m, best_bits));
    aa.own_in_smem = best_own;
    aa.stage = best_stage;
    aa.status = d_status;
    aa.m_sub = best_m;
    aa.off_bits = best_bits;
    aa.ch_off_bits = s->off_bits;
    aa.geo = s->d_adj_geo;
  }
  AdjPlainArgs pa{};
  if (plain) {
    pa.N = (int32_t)NE;
    pa.R = R;
    pa.NR = NR;
    pa.NL = NL;
    pa.n_samples = ns;
    pa.aT = s->d_adjp_aT;
    pa.nb = s->a32.nb;
    pa.bs = s->d_adjp_bs;
    pa.kb = s->a32.kb;
    pa.flags = s->a32.flags;
    pa.ch_ptr = s->a32.chan_ptr;
    pa.ch_list = s->a32.chan_list;
    pa.ryr_cleft = s->ch.ryr_cleft;
    pa.ryr_jsr = s->ch.ryr_jsr;
    pa.ryr_s_cl = s->d_ryr_s_cl;
    pa.ryr_s_js = s->d_ryr_s_js;
    pa.wt_ptr = s->d_wt_ptr;
    pa.wt_idx = s->d_wt_idx;
    pa.wt_w = s->d_wt_w;
    pa.lam_c = lam_c;
    pa.lam_im = lam_im;
    // lambda's compensation as halves, like the forward's (the buffers are
    // big enough)
    pa.lam_c4q = reinterpret_cast<ushort4*>(lam_c4);
    pa.lam_cimq = reinterpret_cast<uint16_t*>(lam_cim);
    pa.lam = lam;
    pa.part = part;
    pa.k = s->a32.k;
    pa.ak = ak;
  }
  AdjTickArgs ta{};
  ta.n_samples = ns;
  ta.n_state = (int32_t)NE;
  ta.n_ticks = (int32_t)n_ticks;
  ta.ptr = s->ls.ptr;
  ta.col = s->ls.col;
  ta.w = s->ls.w;
  ta.f0 = f0;
  ta.target = target;
  ta.base = s->d_ls_base;
  ta.R = R;
  ta.loss = loss;
  ta.mean_trace = mean_trace ? 1 : 0;
  // the reverse sweep over the recorded segment [s0, s0 + len)
  auto reverse_segment = [&](int64_t s0, int len) -> int {
    // every tick of the segment in one launch
    const int64_t n1 = (s0 / te + 1) * te;
    if (n1 <= s0 + len) {
      ta.tick0 = (int32_t)(n1 / te - 1);
      ta.n_seg_ticks = (int32_t)((s0 + len - n1) / te + 1);
      ta.traj_u = traj_u + (size_t)(n1 - s0) * R * NE;
      ta.slot_stride = (int64_t)te * R * (int64_t)NE;
      ta.coef = coef + (size_t)(n1 / te - s0 / te - 1) * R * ns;
      if (launch_adj_tick(ta, s->st)) return fail(SRS_ERR_CUDA, "tick launch failed");
      s->launches++;
    }
    if (!plain) {
      aa.n_steps = len;
      aa.s0 = s0;
      if (launch_adjoint(aa, best_C, adj_ncl, adj_threads, adj_smem, s->st))
        return fail(SRS_ERR_CUDA, std::string("adjoint launch: ") + cudaGetErrorString(cudaGetLastError()));
      s->launches++;
      return SRS_OK;
    }
    // dL/dF of the tick at global step n of this segment, or null
    auto coef_at = [&](int64_t n) -> const double* {
      if (n <= s0 || n % te) return nullptr;
      return coef + (size_t)(n / te - s0 / te - 1) * R * ns;
    };
    auto slot = [&](int t) { return (size_t)t * R * NE; };
    int cur = 0;
    pa.ib = traj_ib + slot(len - 1);
    pa.coef_cur = coef_at(s0 + len);
    pa.nxt = pub[cur];
    if (launch_adjp_publish(pa, adjp_by, s->st)) return fail(SRS_ERR_CUDA, "adjoint publish launch failed");
    s->launches++;
    for (int t = len; t >= 1; --t) {
      pa.pub = pub[cur];
      pa.nxt = pub[cur ^ 1];
      pa.tu = traj_u + slot(t - 1);
      pa.tig = traj_ig + slot(t - 1);
      pa.ib = t > 1 ? traj_ib + slot(t - 2) : nullptr;
      pa.rec = traj_ch + (size_t)(t - 1) * R * W;
      pa.coef_next = t > 1 ? coef_at(s0 + t - 1) : nullptr;
      pa.last = t == 1;
      if (launch_adjp_step(pa, adjp_by, s->st))
        return fail(SRS_ERR_CUDA, std::string("adjoint step launch: ") + cudaGetErrorString(cudaGetLastError()));
      s->launches++;
      cur ^= 1;
    }
    return SRS_OK;
  };

  // ---- forward with checkpoints, reverse sweep ---------------------------------
  // rev(l, a, b): reverses steps [a, b) from the live state x_a.  Level l
  // cuts the range into pieces of K * fan^(L-1-l) steps, runs forward to the
  // start of its last piece keeping the starts of the others, recurses into
  // the last piece from the live state, then restores and recurses into the
  // others from last to first.  At level L a piece is one segment: recorded,
  // then reversed.  The first segment recorded is the last of the run, whose
  // end state is kept as the final state (restored at the end).
  int64_t piece_steps[16];
  {
    int64_t q = K;
    for (int l = L - 1; l >= 0; --l) {
      piece_steps[l] = q;
      if (l > 0) q = (q > INT64_MAX / fan) ? INT64_MAX : q * fan;
    }
  }
  bool fin_saved = false;
  std::function<int(int, int64_t, int64_t)> rev = [&](int l, int64_t a, int64_t b) -> int {
    if (l == L) {
      const int len = (int)(b - a);
      SRS_TRY(record_live(len));
      if (!fin_saved) {
        SRS_TRY(snap_copy(s, fin, true));
        std::vector<RealCtl> ctl(R);
        SRS_CUDA(cudaMemcpyAsync(ctl.data(), fin.ctl, sizeof(RealCtl) * R, cudaMemcpyDeviceToHost, s->st));
        SRS_CUDA(cudaStreamSynchronize(s->st));
        for (auto& c : ctl) {
          if (c.status & 1u) return fail(SRS_ERR_NONFINITE, "a realization produced a non-finite Ca value");
          if (c.done) return fail(SRS_ERR_STATE, "a realization is finished; reset it before the adjoint");
        }
        fin_saved = true;
      }
      return reverse_segment(a, len);
    }
    const int64_t q = piece_steps[l];
    const int64_t p = (b - a + q - 1) / q;
    for (int64_t i = 0; i + 1 < p; ++i) {
      SRS_TRY(snap_copy(s, lv[l][i], true));
      SRS_TRY(advance_live(q));
    }
    SRS_TRY(rev(l + 1, a + (p - 1) * q, b));
    for (int64_t i = p - 2; i >= 0; --i) {
      SRS_TRY(snap_copy(s, lv[l][i], false));
      SRS_TRY(rev(l + 1, a + i * q, a + (i + 1) * q));
    }
    return SRS_OK;
  };
  SRS_TRY(rev(0, 0, n_steps));
  SRS_TRY(snap_copy(s, fin, false));
  std::vector<double> loss_t((size_t)std::max<int64_t>(n_ticks, 1) * R * ns);
  SRS_CUDA(cudaMemcpyAsync(loss_t.data(), loss, sizeof(double) * loss_t.size(), cudaMemcpyDeviceToHost,
                           s->st));
  std::vector<double> part_h;
  if (plain) {
    part_h.resize((size_t)R * adjp_by * SRS_N_ADJ);
    SRS_CUDA(cudaMemcpyAsync(part_h.data(), part, sizeof(double) * part_h.size(), cudaMemcpyDeviceToHost,
                             s->st));
  } else {
    SRS_CUDA(cudaMemcpyAsync(out->grad, grad, sizeof(double) * R * SRS_N_ADJ, cudaMemcpyDeviceToHost, s->st));
  }
  std::vector<float4> hl, hc;
  std::vector<float> hi, hci;
  if (out->grad_state) {
    hl.resize((size_t)R * NE);
    hc.resize((size_t)R * NE);
    hi.resize((size_t)R * NE);
    hci.resize((size_t)R * NE);
    SRS_CUDA(cudaMemcpyAsync(hl.data(), lam, sizeof(float4) * R * NE, cudaMemcpyDeviceToHost, s->st));
    SRS_CUDA(cudaMemcpyAsync(hi.data(), lam_im, sizeof(float) * R * NE, cudaMemcpyDeviceToHost, s->st));
    if (plain) {
      std::vector<ushort4> q4((size_t)R * NE);
      std::vector<uint16_t> q1((size_t)R * NE);
      SRS_CUDA(cudaMemcpyAsync(q4.data(), lam_c4, sizeof(ushort4) * R * NE, cudaMemcpyDeviceToHost, s->st));
      SRS_CUDA(cudaMemcpyAsync(q1.data(), lam_cim, sizeof(uint16_t) * R * NE, cudaMemcpyDeviceToHost, s->st));
      SRS_CUDA(cudaStreamSynchronize(s->st));
      for (size_t e = 0; e < q4.size(); ++e) {
        hc[e] = make_float4(comp_decode_host(q4[e].x), comp_decode_host(q4[e].y), comp_decode_host(q4[e].z),
                            comp_decode_host(q4[e].w));
        hci[e] = comp_decode_host(q1[e]);
      }
    } else {
      SRS_CUDA(cudaMemcpyAsync(hc.data(), lam_c4, sizeof(float4) * R * NE, cudaMemcpyDeviceToHost, s->st));
      SRS_CUDA(cudaMemcpyAsync(hci.data(), lam_cim, sizeof(float) * R * NE, cudaMemcpyDeviceToHost, s->st));
    }
  }
  SRS_CUDA(cudaStreamSynchronize(s->st));
  SRS_CUDA(cudaGetLastError());
  if (plain) {  // the blocks' rows in a fixed order
    const double dt = (double)pa.k.dt;
    for (int r = 0; r < R; ++r)
      for (int p = 0; p < SRS_N_ADJ; ++p) {
        double v = 0.0;
        for (int b = 0; b < adjp_by; ++b) v += part_h[((size_t)r * adjp_by + b) * SRS_N_ADJ + p];
        out->grad[(size_t)r * SRS_N_ADJ + p] = v * dt;
      }
  }
  for (int r = 0; r < R; ++r) {  // ticks in time order: the same sum for any segmentation
    double Ls = 0.0;
    for (int64_t t = 0; t < n_ticks; ++t)
      for (int i = 0; i < ns; ++i) Ls += loss_t[((size_t)t * R + r) * ns + i];
    out->loss[r] = Ls;
  }
  if (out->grad_state) {
    const int N = s->N;
    for (int r = 0; r < R; ++r) {
      double* g = out->grad_state + (size_t)r * 6 * N;
      for (int j = 0; j < N; ++j) {
        const size_t e = (size_t)r * NE + s->eng_of_ref[j];
        const float4 Lv = hl[e], Cc = hc[e];
        const double li = (double)hi[e] - (double)hci[e];
        const bool jsr = s->m.domain[j] == DOMAIN_JSR;
        g[SP_CA * (size_t)N + j] = (double)Lv.x - (double)Cc.x;
        g[SP_ATP * (size_t)N + j] = (double)Lv.y - (double)Cc.y;
        g[SP_CMDN * (size_t)N + j] = (double)Lv.z - (double)Cc.z;
        g[SP_DYE * (size_t)N + j] = (double)Lv.w - (double)Cc.w;
        g[SP_TRPN * (size_t)N + j] = (!jsr && s->m.tropc[j]) ? li : 0.0;
        g[SP_CSQN * (size_t)N + j] = jsr ? li : 0.0;
      }
    }
  }
  {
    unsigned int st_bits = 0;
    SRS_CUDA(cudaMemcpy(&st_bits, d_status, sizeof(st_bits), cudaMemcpyDeviceToHost));
    if (st_bits & 1u) return fail(SRS_ERR_TIMEOUT, "adjoint: a trajectory copy did not complete");
  }
  for (int r = 0; r < R; ++r)
    for (int p = 0; p < SRS_N_ADJ; ++p)
      if (!std::isfinite(out->grad[(size_t)r * SRS_N_ADJ + p]))
        return fail(SRS_ERR_NONFINITE, "non-finite adjoint gradient");
  return SRS_OK;
}

int srs_adjoint_plan(srs_sim* s, const srs_adjoint_desc* d, int* segment_steps, int* levels,
                     int64_t* forward_steps) {
  if (!s || !d) return fail(SRS_ERR_INPUT, "null argument");
  AdjPlan pl;
  SRS_TRY(adjoint_plan(s, d, &pl));
  if (segment_steps) *segment_steps = pl.K;
  if (levels) *levels = pl.L;
  if (forward_steps) *forward_steps = pl.forward_steps;
  return SRS_OK;
}

int srs_sim_total_ca(srs_sim* s, double* out) {
  if (!s || !out) return fail(SRS_ERR_INPUT, "null argument");
  MassArgs& a = s->mass;
  const size_t NE = eng_count(s);
  if (!a.v0) {
    const double* Rr = s->p.reals;
    std::vector<double> v0(NE, 0.0), bhi(NE, 0.0), blo(NE, 0.0), rest4(4 * NE, 0.0), rimm(NE, 0.0);
    std::vector<uint8_t> jsr(NE, 0);
    for (size_t e = 0; e < NE; ++e) {
      const int j = s->ref_of_eng[e];
      if (j < 0) continue;
      v0[e] = s->m.V0[j];
      jsr[e] = s->m.domain[j] == DOMAIN_JSR;
      bhi[e] = s->m.TT[j] * Rr[R_B_TOT_SL_HI] / (s->m.V0[j] * (1e-15));
      blo[e] = s->m.TT[j] * Rr[R_B_TOT_SL_LO] / (s->m.V0[j] * (1e-15));
      if (s->d.precision != SRS_FP64) {
        const double f = jsr[e] ? 0.0 : 1.0;
        rest4[4 * e] = s->rest_ca[e];
        rest4[4 * e + 1] = f * s->rv.atp;
        rest4[4 * e + 2] = f * s->rv.cmdn;
        rest4[4 * e + 3] = f * s->rv.dye;
        rimm[e] = s->rest_imm[e];
      }
    }
    a.n_state = (int32_t)NE;
    a.khi = Rr[R_K_D_SL_HI];
    a.klo = Rr[R_K_D_SL_LO];
    SRS_TRY(dev_upload(s, (double**)&a.v0, v0.data(), v0.size()));
    SRS_TRY(dev_upload(s, (uint8_t**)&a.jsr, jsr.data(), jsr.size()));
    SRS_TRY(dev_upload(s, (double**)&a.bhi, bhi.data(), bhi.size()));
    SRS_TRY(dev_upload(s, (double**)&a.blo, blo.data(), blo.size()));
    SRS_TRY(dev_upload(s, (double**)&a.rest4, rest4.data(), rest4.size()));
    SRS_TRY(dev_upload(s, (double**)&a.rest_imm, rimm.data(), rimm.size()));
    SRS_TRY(dev_alloc(s, &a.out, (size_t)2 * s->R));
  }
  MassArgs m = a;
  if (s->d.precision == SRS_FP64) {
    m.S64 = s->d_S[0];
  } else {
    m.M = s->d_M[0];
    m.CM = s->d_CM;
    m.I = s->d_I[0];
    m.CI = s->d_CI;
    m.CMq = s->d_CMq;
    m.CIq = s->d_CIq;
  }
  SRS_CUDA(cudaStreamSynchronize(s->st));
  if (launch_total_ca(m, s->R, s->st)) return fail(SRS_ERR_CUDA, "total-Ca launch failed");
  s->launches++;
  SRS_CUDA(cudaMemcpyAsync(out, m.out, sizeof(double) * 2 * s->R, cudaMemcpyDeviceToHost, s->st));
  SRS_CUDA(cudaStreamSynchronize(s->st));
  return SRS_OK;
}

int srs_write_grid_vtk(srs_sim* s, int r, const char* path, int run, int rank, int n, double t) {
  if (!s || !path || r < 0 || r >= s->R) return fail(SRS_ERR_INPUT, "bad argument");
  std::vector<double> S6((size_t)6 * s->N);
  SRS_TRY(download_state(s, r, S6.data()));
  std::vector<int32_t> ryr(s->NR);
  SRS_CUDA(cudaMemcpy(ryr.data(), s->d_ryr + (size_t)r * s->NR, s->NR * 4, cudaMemcpyDeviceToHost));
  return write_grid_vtk(path, s->m, run, rank, n, t, &S6[0], &S6[(size_t)SP_DYE * s->N], ryr.data());
}

int srs_grid_write_vtk(const srs_grid* g, const double* states, const int* ryr_states,
                       const char* path, int run, int rank, int n, double t) {
  if (!g || !states || !path || (g->m.NR > 0 && !ryr_states)) return fail(SRS_ERR_INPUT, "null argument");
  int rc = write_grid_vtk(path, g->m, run, rank, n, t, states, states + (size_t)SP_DYE * g->m.N, ryr_states);
  return rc ? fail(rc, std::string("cannot write ") + path) : SRS_OK;
}

void srs_box_mesh_default(srs_box_mesh_spec* spec) {
  MeshGenSpec s;
  meshgen_default_spec(&s);
  static_assert(sizeof(MeshGenSpec) == sizeof(srs_box_mesh_spec), "spec layouts differ");
  std::memcpy(spec, &s, sizeof(s));
}

int srs_multisite_mesh_write(const srs_multisite_spec* spec, const char* base, int* rep_i,
                             double* rep_a0) {
  if (!spec || !base) return fail(SRS_ERR_INPUT, "null argument");
  static_assert(sizeof(MultiSiteSpec) == sizeof(srs_multisite_spec), "spec layouts differ");
  MultiSiteSpec s;
  std::memcpy(&s, spec, sizeof(s));
  MeshGenReport rep;
  int rc = meshgen_multisite(s, base, &rep);
  if (rc) return fail(rc, "multi-site mesh generation failed");
  if (rep_i) {
    rep_i[0] = rep.n_tets;
    rep_i[1] = rep.n_faces;
    rep_i[2] = rep.n_nodes;
    rep_i[3] = rep.n_ryr;
    rep_i[4] = rep.n_lcc;
    rep_i[5] = rep.n_jsr_tets;
  }
  if (rep_a0) *rep_a0 = rep.max_a0;
  return SRS_OK;
}

int srs_comp_round_trip(const float* in, float* out, int64_t n, int packed) {
  if (!in || !out || n < 0) return fail(SRS_ERR_INPUT, "bad argument");
  if (n == 0) return SRS_OK;
  struct Bufs {  // freed on every return path
    float* d[2] = {nullptr, nullptr};
    ~Bufs() {
      for (float* p : d)
        if (p) cudaFree(p);
    }
  } b;
  SRS_CUDA(cudaMalloc(&b.d[0], n * sizeof(float)));
  SRS_CUDA(cudaMalloc(&b.d[1], n * sizeof(float)));
  SRS_CUDA(cudaMemcpy(b.d[0], in, n * sizeof(float), cudaMemcpyHostToDevice));
  if (launch_comp_round_trip(b.d[0], b.d[1], n, packed ? 1 : 0, 0))
    return fail(SRS_ERR_CUDA, "codec kernel launch failed");
  SRS_CUDA(cudaMemcpy(out, b.d[1], n * sizeof(float), cudaMemcpyDeviceToHost));
  return SRS_OK;
}

int srs_box_mesh_write(const srs_box_mesh_spec* spec, const char* base, int* rep_i, double* rep_a0) {
  if (!spec || !base) return fail(SRS_ERR_INPUT, "null argument");
  MeshGenSpec s;
  std::memcpy(&s, spec, sizeof(s));
  MeshGenReport rep;
  int rc = meshgen_box(s, base, &rep);
  if (rc) return fail(rc, "mesh generation failed");
  if (rep_i) {
    rep_i[0] = rep.n_tets;
    rep_i[1] = rep.n_faces;
    rep_i[2] = rep.n_nodes;
    rep_i[3] = rep.n_ryr;
    rep_i[4] = rep.n_lcc;
    rep_i[5] = rep.n_jsr_tets;
  }
  if (rep_a0) *rep_a0 = rep.max_a0;
  return SRS_OK;
}

}  // extern "C"
