// ref_io_harness.cpp — drives the reference's own input/output code:
// cpu/InitFuncs.cpp (ReadParameters, ReadGrid, ResetGlobals,
// InitializeDefaultGrid, InitializeDefaultChannels, InitializeDomainStruct,
// ResetDefaultGridStates, OpenRandomRyR) and cpu/OutputFuncs.cpp
// (CreateOutputFiles, WriteToGridFiles, WriteToStateFiles).
// TEST INFRASTRUCTURE: built into oracle/_ref/libsrsref_io.so by
// oracle/build_ref.sh from the reference sources where they lie, with the
// single-rank MPI stand-in and the Xerces DOM subset of oracle/shim/ in place
// of those libraries; never shipped, never copied.
//
// Each entry point returns plain arrays so that tests can compare them with
// the product's C ABI.  The set-up order is cpu/main.cpp:170-189.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "parameters.h"

namespace {

struct RefIo {
  SimData sd;
  ParamStruct ps;
};

void fill_params(ParamStruct* ps, const int* ints, const double* reals) {
  for (int i = 0; i < N_PARAMETERS_INT; ++i) ps->Integers[i] = ints[i];
  for (int i = 0; i < N_PARAMETERS_REAL; ++i) ps->Reals[i] = reals[i];
  // the tail of ReadParameters (cpu/InitFuncs.cpp:356-368)
  ps->Diff[0] = ps->Reals[I_D_CA];
  ps->Diff[1] = ps->Reals[I_D_ATP];
  ps->Diff[2] = ps->Reals[I_D_CMDN];
  ps->Diff[3] = ps->Reals[I_D_TRPN];
  ps->Diff[4] = ps->Reals[I_D_CSQN];
  ps->Diff[5] = ps->Reals[I_D_DYE];
  ps->Default_Globals[0] = ps->Reals[I_DEFAULT_VM];
  ps->Default_Globals[1] = ps->Reals[I_DEFAULT_CA_NSR];
}

}  // namespace

extern "C" {

// ReadParameters: the reference defaults overridden by the XML file.
// chars receives Chars[4][255].
int refio_read_parameters(const char* path, int* ints, double* reals, char* chars) {
  ParamStruct* ps = (ParamStruct*)calloc(1, sizeof(ParamStruct));
  ReadParameters(ps, path);
  for (int i = 0; i < N_PARAMETERS_INT; ++i) ints[i] = ps->Integers[i];
  for (int i = 0; i < N_PARAMETERS_REAL; ++i) reals[i] = ps->Reals[i];
  if (chars) memcpy(chars, ps->Chars, sizeof(ps->Chars));
  free(ps);
  fflush(stdout);  // the reference's progress output, while the caller still captures it
  return 0;
}

// cpu/main.cpp:170-189 for the mesh `base`: ReadGrid, ResetGlobals,
// InitializeDefaultGrid, InitializeDefaultChannels, InitializeDomainStruct.
void* refio_load(const char* base, const int* ints, const double* reals) {
  RefIo* h = new RefIo();
  memset(&h->sd, 0, sizeof(h->sd));
  memset(&h->ps, 0, sizeof(h->ps));
  fill_params(&h->ps, ints, reals);
  snprintf(h->ps.Chars[I_FILE_BASE], sizeof(h->ps.Chars[I_FILE_BASE]), "%s", base);
  ReadGrid(&h->sd, &h->sd.Grid, &h->ps);
  ResetGlobals(&h->sd, &h->ps);
  InitializeDefaultGrid(&h->sd, &h->ps);
  InitializeDefaultChannels(&h->sd);
  InitializeDomainStruct(&h->sd.Grid, h->ps.Integers[I_FLAG_SECONDARY_GRADIENT], &h->ps);
  fflush(stdout);
  fflush(stderr);
  return h;
}

// N, faces, nodes, RyRs, LCCs
void refio_counts(void* p, int* out) {
  RefIo* h = (RefIo*)p;
  out[0] = h->sd.Grid.N_Ele;
  out[1] = h->sd.Grid.N_Face;
  out[2] = h->sd.Grid.N_Nodes;
  out[3] = h->sd.N_RyR;
  out[4] = h->sd.N_LCC;
}

// aij[5N], nij[4N], Boundary_Rates[6][N]
void refio_operator(void* p, double* aij, int* nij, double* br) {
  GridStruct& g = ((RefIo*)p)->sd.Grid;
  memcpy(aij, g.aij, sizeof(double) * 5 * (size_t)g.N_Ele);
  memcpy(nij, g.nij, sizeof(int) * 4 * (size_t)g.N_Ele);
  for (int k = 0; k < N_STATES; ++k) memcpy(br + (size_t)k * g.N_Ele, g.Boundary_Rates[k], sizeof(double) * g.N_Ele);
}

void refio_elements(void* p, double* v0, double* tt, int* domain, int* tropc) {
  GridStruct& g = ((RefIo*)p)->sd.Grid;
  memcpy(v0, g.V0, sizeof(double) * g.N_Ele);
  memcpy(tt, g.TTSurfaceArea, sizeof(double) * g.N_Ele);
  memcpy(domain, g.Domain, sizeof(int) * g.N_Ele);
  memcpy(tropc, g.TropC, sizeof(int) * g.N_Ele);
}

void refio_channels(void* p, int* ryr_ele, int* ryr_jsr, int* ryr_nb, int* lcc_ele) {
  SimData& sd = ((RefIo*)p)->sd;
  memcpy(ryr_ele, sd.RyR_Ele, sizeof(int) * sd.N_RyR);
  memcpy(ryr_jsr, sd.RyR_JSR_Ele, sizeof(int) * sd.N_RyR);
  memcpy(ryr_nb, sd.RyR_Neighb, sizeof(int) * 4 * sd.N_RyR);
  memcpy(lcc_ele, sd.LCC_Ele, sizeof(int) * sd.N_LCC);
}

// States[6][N] as they are now
void refio_get_states(void* p, double* S) {
  GridStruct& g = ((RefIo*)p)->sd.Grid;
  for (int k = 0; k < N_STATES; ++k) memcpy(S + (size_t)k * g.N_Ele, g.States[k], sizeof(double) * g.N_Ele);
}

void refio_set_states(void* p, const double* S) {
  GridStruct& g = ((RefIo*)p)->sd.Grid;
  for (int k = 0; k < N_STATES; ++k) memcpy(g.States[k], S + (size_t)k * g.N_Ele, sizeof(double) * g.N_Ele);
}

// ResetDefaultGridStates, then States[6][N]
void refio_reset_states(void* p, double* S) {
  RefIo* h = (RefIo*)p;
  ResetDefaultGridStates(&h->sd, &h->ps);
  refio_get_states(p, S);
}

// OpenRandomRyR for (rank, ensemble index) from the channel states given
// (and the current grid states); returns the RyR it opened.
int refio_open_random_ryr(void* p, int rank, int index, int* ryr_states) {
  SimData& sd = ((RefIo*)p)->sd;
  memcpy(sd.RyR_States, ryr_states, sizeof(int) * sd.N_RyR);
  sd.device = rank;
  sd.ensemble_index = index;
  int before[4096];
  int n = sd.N_RyR < 4096 ? sd.N_RyR : 4096;
  memcpy(before, sd.RyR_States, sizeof(int) * n);
  OpenRandomRyR(&((RefIo*)p)->ps, &sd);
  int opened = -1;
  for (int i = 0; i < n; ++i)
    if (sd.RyR_States[i] != before[i]) opened = i;
  memcpy(ryr_states, sd.RyR_States, sizeof(int) * sd.N_RyR);
  return opened;
}

void refio_set_ryr(void* p, const int* ryr_states) {
  SimData& sd = ((RefIo*)p)->sd;
  memcpy(sd.RyR_States, ryr_states, sizeof(int) * sd.N_RyR);
}

// CreateOutputFiles + WriteToGridFiles(n, t) of the current states into
// `dir` (grid files <dir>/grid_<rank>_<run>_<n>.vtk, cpu/OutputFuncs.cpp:42-220).
void refio_write_grid(void* p, const char* dir, int rank, int run, int n, double t) {
  RefIo* h = (RefIo*)p;
  snprintf(h->ps.Chars[I_OUTPUT_GRID], sizeof(h->ps.Chars[I_OUTPUT_GRID]), "%s", dir);
  snprintf(h->ps.Chars[I_OUTPUT_STATE], sizeof(h->ps.Chars[I_OUTPUT_STATE]), "%s", dir);
  h->sd.device = rank;
  h->sd.ensemble_index = run;
  CreateOutputFiles(run, rank, &h->ps);
  WriteToGridFiles(n, t, &h->sd.Grid, &h->sd, &h->ps);
  fflush(stdout);
}

void refio_free(void* p) { delete (RefIo*)p; }

}  // extern "C"
