// ref_harness.cpp — drives the reference's own cpu/RunSimulation.cpp.
// TEST INFRASTRUCTURE: built into oracle/_ref/ by oracle/build_ref.sh from
// the reference sources where they lie; never shipped, never copied.
//
// cpu/RunSimulation.cpp compiles on its own (it needs only parameters.h and
// libm).  Its callers in cpu/main.cpp / cpu/InitFuncs.cpp need Xerces-C and
// MPI, so this harness takes their place: it fills the reference structures
// (GridStruct, SimData, ParamStruct of cpu/parameters.h) from arrays the
// caller provides and supplies the three output hooks RunSimulation calls.
// WriteToStateFiles below writes the same float32 row as
// cpu/OutputFuncs.cpp:241-350 into a capture buffer instead of a file.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "parameters.h"

namespace {
float* g_rows = nullptr;
int64_t g_row_cap = 0, g_nrows = 0;
int g_row_w = 0;

// line scan of the bound dye taken at every grid-file call: F_i = pad_i +
// sum_q w_q [CaDye]_{col_q} over row i of a CSR weight matrix (the PSF sum
// of linescan/main.cpp:197-225 with the cell volumes folded into w)
int g_ls_n = 0;
const int* g_ls_ptr = nullptr;
const int* g_ls_col = nullptr;
const double* g_ls_w = nullptr;
const double* g_ls_pad = nullptr;
double* g_ls_out = nullptr;
int64_t g_ls_cap = 0, g_ls_rows = 0;
}  // namespace

void CreateOutputFiles(int, int, ParamStruct*) {}

// Called by RunSimulation at t = 0, at every grid-file step when
// OUTPUT_GRID_FLAG is set, and at the end (cpu/RunSimulation.cpp:421-586).
// Writes one line-scan row [t, F_0 .. F_{n-1}] when a capture is set.
void WriteToGridFiles(int, double t, GridStruct* g, SimData*, ParamStruct*) {
  if (!g_ls_out || g_ls_rows >= g_ls_cap) return;
  double* o = g_ls_out + g_ls_rows * (int64_t)(g_ls_n + 1);
  o[0] = t;
  const double* dye = g->States[INDEX_DYE];
  for (int i = 0; i < g_ls_n; ++i) {
    double acc = 0.0;
    for (int q = g_ls_ptr[i]; q < g_ls_ptr[i + 1]; ++q) acc += g_ls_w[q] * dye[g_ls_col[q]];
    o[1 + i] = g_ls_pad[i] + acc;
  }
  ++g_ls_rows;
}
void WriteToStateFiles(double t, SimData* sd, ParamStruct* ps) {
  if (g_nrows >= g_row_cap) return;
  float* row = g_rows + g_nrows * g_row_w;
  int k = 0;
  row[k++] = (float)t;
  double i_ryr = 0;
  for (int i = 0; i < sd->N_RyR; i++) {
    double CaJSR = sd->Grid.States[INDEX_CA][sd->RyR_JSR_Ele[i]];
    double CaSS = sd->Grid.States[INDEX_CA][sd->RyR_Ele[i]];
    i_ryr += sd->RyR_States[i] * ps->Reals[I_V_RYR] * (CaJSR - CaSS) * (ps->Reals[I_V_CELL]) * 96485 * 2 * (1e-6);
  }
  row[k++] = (float)i_ryr;
  int n_open = 0;
  for (int i = 0; i < sd->N_RyR; i++) n_open += sd->RyR_States[i];
  row[k++] = (float)n_open;
  int n_lcc = 0;
  for (int i = 0; i < sd->N_LCC; i++)
    if (sd->LCCV_States[i] == 2 && (sd->LCC_States[i] == 6 || sd->LCC_States[i] == 12)) n_lcc++;
  row[k++] = (float)n_lcc;
  const double P_CaL = (9.13e-13) * (1e12) * (1e-3);
  const double F = 96.5;
  const double RT = 310 * 8.314;
  const double F_over_RT = F / RT;
  double V = sd->Global_Vars[GLOBAL_VM];
  if (fabs(V) < 1e-6) V = 1e-6;
  double i_lcc = 0;
  for (int i = 0; i < sd->N_LCC; i++) {
    double CA_DYAD = sd->Grid.States[INDEX_CA][sd->LCC_Ele[i]];
    if ((sd->LCC_States[i] == STATE_LCC_OPEN_1 || sd->LCC_States[i] == STATE_LCC_OPEN_2) &&
        (sd->LCCV_States[i] == STATE_LCCV_OPEN))
      i_lcc += -P_CaL * V * (2 * F_over_RT) * (CA_DYAD * exp(2 * V * F_over_RT) - 0.34 * ps->Reals[I_CA_0]) /
               (exp(2 * V * F_over_RT) - 1) * 96485 * 2 * (1e-6);
  }
  row[k++] = (float)i_lcc;
  double m_sr = 0, m_i = 0;
  for (int i = 0; i < sd->N_RyR; i++) m_sr += sd->Grid.States[INDEX_CA][sd->RyR_JSR_Ele[i]];
  m_sr /= sd->N_RyR;
  row[k++] = (float)m_sr;
  for (int i = 0; i < sd->N_RyR; i++) m_i += sd->Grid.States[INDEX_CA][sd->RyR_Ele[i]];
  m_i /= sd->N_RyR;
  row[k++] = (float)m_i;
  if (ps->Integers[I_FLAG_RYR_OUT])
    for (int i = 0; i < sd->N_RyR; i++) row[k++] = (float)sd->RyR_States[i];
  ++g_nrows;
}

namespace {

struct Holder {
  SimData sd;
  ParamStruct ps;
  std::vector<std::vector<double>> states, br;
  std::vector<double*> sp, bp;
  std::vector<double> buf, aij, v0, tt, sr;
  std::vector<int> nij, tropc, domain, ryr_ele, ryr_jsr, ryr_nb, lcc_ele, ryr_state, lcc_state, lccv_state;
  std::vector<double> res;
};

void fill(Holder* h, int N, int NR, int NL, const double* aij, const int* nij, const double* br,
          const double* v0, const double* tt, const int* domain, const int* tropc, const int* ryr_ele,
          const int* ryr_jsr, const int* ryr_nb, const int* lcc_ele, const int* ints, const double* reals,
          const double* states) {
  memset(&h->sd, 0, sizeof(h->sd));
  memset(&h->ps, 0, sizeof(h->ps));
  for (int i = 0; i < N_PARAMETERS_INT; ++i) h->ps.Integers[i] = ints[i];
  for (int i = 0; i < N_PARAMETERS_REAL; ++i) h->ps.Reals[i] = reals[i];
  h->ps.Diff[0] = reals[I_D_CA];
  h->ps.Diff[1] = reals[I_D_ATP];
  h->ps.Diff[2] = reals[I_D_CMDN];
  h->ps.Diff[3] = reals[I_D_TRPN];
  h->ps.Diff[4] = reals[I_D_CSQN];
  h->ps.Diff[5] = reals[I_D_DYE];
  h->ps.Default_Globals[0] = reals[I_DEFAULT_VM];
  h->ps.Default_Globals[1] = reals[I_DEFAULT_CA_NSR];
  GridStruct& g = h->sd.Grid;
  g.N_States = N_STATES;
  g.N_Ele = N;
  h->states.assign(N_STATES, std::vector<double>(N));
  h->br.assign(N_STATES, std::vector<double>(N));
  h->sp.resize(N_STATES);
  h->bp.resize(N_STATES);
  for (int k = 0; k < N_STATES; ++k) {
    for (int j = 0; j < N; ++j) {
      h->states[k][j] = states[k * N + j];
      h->br[k][j] = br[k * N + j];
    }
    h->sp[k] = h->states[k].data();
    h->bp[k] = h->br[k].data();
  }
  g.States = h->sp.data();
  g.Boundary_Rates = h->bp.data();
  h->buf.assign(N_STATES * (size_t)N, 0.0);
  g.States_Buffer = h->buf.data();
  h->aij.assign(aij, aij + 5 * (size_t)N);
  h->nij.assign(nij, nij + 4 * (size_t)N);
  h->v0.assign(v0, v0 + N);
  h->tt.assign(tt, tt + N);
  h->sr.assign(N, 0.0);
  h->domain.assign(domain, domain + N);
  h->tropc.assign(tropc, tropc + N);
  g.aij = h->aij.data();
  g.nij = h->nij.data();
  g.V0 = h->v0.data();
  g.TTSurfaceArea = h->tt.data();
  g.SRSurfaceArea = h->sr.data();
  g.Domain = h->domain.data();
  g.TropC = h->tropc.data();
  g.Vol_JSR = 0;
  for (int j = 0; j < N; ++j)
    if (domain[j] == DOMAIN_JSR) g.Vol_JSR += v0[j];
  h->ryr_ele.assign(ryr_ele, ryr_ele + NR);
  h->ryr_jsr.assign(ryr_jsr, ryr_jsr + NR);
  h->ryr_nb.assign(ryr_nb, ryr_nb + 4 * NR);
  h->lcc_ele.assign(lcc_ele, lcc_ele + NL);
  h->ryr_state.assign(NR, DEFAULT_STATE_RYR);
  h->lcc_state.assign(NL, DEFAULT_STATE_LCC);
  h->lccv_state.assign(NL, DEFAULT_STATE_LCCV);
  h->res.assign(NR + NL, 0.0);
  SimData& sd = h->sd;
  sd.N_RyR = NR;
  sd.N_LCC = NL;
  sd.N_Channels = NR + NL;
  sd.RyR_Ele = h->ryr_ele.data();
  sd.RyR_JSR_Ele = h->ryr_jsr.data();
  sd.RyR_Neighb = h->ryr_nb.data();
  sd.LCC_Ele = h->lcc_ele.data();
  sd.RyR_States = h->ryr_state.data();
  sd.LCC_States = h->lcc_state.data();
  sd.LCCV_States = h->lccv_state.data();
  sd.R = h->res.data();
  sd.Global_Vars[GLOBAL_VM] = reals[I_DEFAULT_VM];
  sd.Global_Vars[GLOBAL_CA_NSR] = reals[I_DEFAULT_CA_NSR];
}

void unload(Holder* h, int N, double* states) {
  for (int k = 0; k < N_STATES; ++k)
    for (int j = 0; j < N; ++j) states[k * N + j] = h->states[k][j];
}

}  // namespace

extern "C" {

// ExplicitStep (cpu/RunSimulation.cpp:591) n times, gating as the flags say.
// Channel states and residuals are taken from and returned to the caller.
int ref_explicit_steps(int N, int NR, int NL, const double* aij, const int* nij, const double* br,
                       const double* v0, const double* tt, const int* domain, const int* tropc,
                       const int* ryr_ele, const int* ryr_jsr, const int* ryr_nb, const int* lcc_ele,
                       const int* ints, const double* reals, double* states, int* ryr, int* lcc, int* lccv,
                       double* res, int64_t n, unsigned int srand_seed) {
  Holder h;
  fill(&h, N, NR, NL, aij, nij, br, v0, tt, domain, tropc, ryr_ele, ryr_jsr, ryr_nb, lcc_ele, ints, reals,
       states);
  for (int i = 0; i < NR; ++i) h.ryr_state[i] = ryr[i];
  for (int i = 0; i < NL; ++i) {
    h.lcc_state[i] = lcc[i];
    h.lccv_state[i] = lccv[i];
  }
  for (int i = 0; i < NR + NL; ++i) h.res[i] = res[i];
  srand(srand_seed);
  for (int64_t s = 0; s < n; ++s) ExplicitStep(reals[I_T_STEP], &h.sd, &h.ps);
  unload(&h, N, states);
  for (int i = 0; i < NR; ++i) ryr[i] = h.ryr_state[i];
  for (int i = 0; i < NL; ++i) {
    lcc[i] = h.lcc_state[i];
    lccv[i] = h.lccv_state[i];
  }
  for (int i = 0; i < NR + NL; ++i) res[i] = h.res[i];
  return 0;
}

// cpu/main.cpp:216-253 for one realization (without OpenRandomRyR, which
// lives in the unbuildable InitFuncs.cpp: the parameter set must name the
// initial RyR, trigger an LCC or clamp), then RunSimulation.
int64_t ref_run_simulation(int N, int NR, int NL, const double* aij, const int* nij, const double* br,
                           const double* v0, const double* tt, const int* domain, const int* tropc,
                           const int* ryr_ele, const int* ryr_jsr, const int* ryr_nb, const int* lcc_ele,
                           const int* ints, const double* reals, const double* states0, int rank, int index,
                           float* rows, int64_t row_cap, int row_w, double* states_out) {
  Holder h;
  fill(&h, N, NR, NL, aij, nij, br, v0, tt, domain, tropc, ryr_ele, ryr_jsr, ryr_nb, lcc_ele, ints, reals,
       states0);
  h.sd.device = rank;
  h.sd.ensemble_index = index;
  if (h.ps.Integers[I_FLAG_LCC]) {
    h.sd.LCC_States[h.ps.Integers[I_LCC_INDEX]] = STATE_LCC_OPEN_1;
  } else if (h.ps.Integers[I_FLAG_V_CLAMP]) {
  } else if (h.ps.Integers[I_INIT_RYR] >= 0 && h.ps.Integers[I_INIT_RYR] < NR) {
    h.sd.RyR_States[h.ps.Integers[I_INIT_RYR]] = 1;
  } else {
    return -1;
  }
  g_rows = rows;
  g_row_cap = row_cap;
  g_row_w = row_w;
  g_nrows = 0;
  g_ls_rows = 0;
  RunSimulation(&h.sd, &h.ps);
  fflush(stdout);  // the reference's progress output, while the caller still captures it
  if (states_out) unload(&h, N, states_out);
  return g_nrows;
}

// Line-scan capture for the next ref_run_simulation calls (n_samples rows
// of CSR weights in the reference's element numbering; out holds cap rows
// of n_samples + 1 doubles).  n_samples = 0 switches it off.
void ref_set_linescan(int n_samples, const int* ptr, const int* col, const double* w, const double* pad,
                      double* out, int64_t cap) {
  g_ls_n = n_samples;
  g_ls_ptr = ptr;
  g_ls_col = col;
  g_ls_w = w;
  g_ls_pad = pad;
  g_ls_out = n_samples > 0 ? out : nullptr;
  g_ls_cap = cap;
  g_ls_rows = 0;
}

int64_t ref_linescan_rows() { return g_ls_rows; }

}  // extern "C"
