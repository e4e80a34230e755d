// srs_host.h — host-side model of the reference's input path: parameter
// sets, mesh files, element renumbering, diffusion-operator assembly and the
// equilibrium initial state.  The layouts mirror the reference structures
// (ParamStruct / GridStruct / SimData, cpu/parameters.h:161-246) so that the
// C ABI can speak the reference's numbering and units.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/srs_gb300.h"

namespace srs {

// Parameter indices (cpu/parameters.h:18-96).
enum IntParam {
  I_OUTPUT_GRID_FLAG = 0, I_FLAG_FIDELITY_SIM = 1, I_FLAG_CLOCK_SEED = 2, I_RAND_SEED_0 = 3,
  I_RAND_ADD_A = 4, I_RAND_ADD_B = 5, I_INITIALIZE_FROM_FILE = 6, I_CUDA_DEVICE = 7,
  I_FLAG_SECONDARY_GRADIENT = 8, I_FLAG_NO_FLUX_BOUNDARY = 9, I_N_RYR_FIDELITY = 10,
  I_FLAG_LCC = 11, I_LCC_INDEX = 12, I_FLAG_V_CLAMP = 13, I_FLAG_NO_GATING = 14,
  I_GATING_FFWD = 15, I_FLAG_RYR_OUT = 16, I_N_SIMS = 17, I_INIT_RYR = 18
};
enum RealParam {
  R_T_FINAL = 0, R_T_STEP = 1, R_OUTPUT_STATES_INTERVAL = 2, R_OUTPUT_GRID_INTERVAL = 3,
  R_C_MIN = 4, R_D_CA = 5, R_D_CA_JSR = 6, R_D_ATP = 7, R_D_CMDN = 8, R_D_TRPN = 9,
  R_D_CSQN = 10, R_D_DYE = 11, R_D_EGTA = 12, R_C_0_CA = 13, R_C_0_CA_JSR = 14,
  R_DEFAULT_VM = 15, R_DEFAULT_CA_NSR = 16, R_CA_0 = 17, R_B_TOT_ATP = 18, R_K_OFF_ATP = 19,
  R_K_ON_ATP = 20, R_B_TOT_CMDN = 21, R_K_OFF_CMDN = 22, R_K_ON_CMDN = 23, R_B_TOT_TRPN = 24,
  R_K_OFF_TRPN = 25, R_K_ON_TRPN = 26, R_B_TOT_SL_HI = 27, R_K_D_SL_HI = 28,
  R_B_TOT_SL_LO = 29, R_K_D_SL_LO = 30, R_B_TOT_DYE = 31, R_K_OFF_DYE = 32, R_K_ON_DYE = 33,
  R_B_T_JSR = 34, R_K_M_JSR = 35, R_V_REFILL = 36, R_V_RYR = 37, R_V_CELL = 38,
  R_K_ON_CSQN = 39, R_K_OFF_CSQN = 40, R_RYR_ETA = 41, R_RYR_A_STAR = 42, R_RYR_EPS_CC = 43,
  R_RYR_EPS_OO = 44, R_RYR_K_PLUS = 45, R_RYR_K_MINUS = 46, R_RYR_PHI_M = 47,
  R_RYR_PHI_B = 48, R_K_D_i = 49, R_K_D_SR = 50, R_A_P = 51, R_LCC_DURATION = 52,
  R_T_CLAMP = 53, R_V_CLAMP = 54, R_INIT_RYR_HOLD = 55
};
enum CharParam { C_FILE_BASE = 0, C_OUTPUT_STATE = 1, C_OUTPUT_GRID = 2, C_PARAM_TITLE = 3 };

// Species (cpu/parameters.h:136-144) and other constants.
enum { SP_CA = 0, SP_ATP = 1, SP_CMDN = 2, SP_TRPN = 3, SP_CSQN = 4, SP_DYE = 5, N_SPECIES = 6 };
enum { FACE_DEFAULT = 0, FACE_BOUND = 1, FACE_NOFLUX = 2 };
enum { DOMAIN_CYTO = 0, DOMAIN_JSR = 1 };

// Diffusion coefficients by species index (cpu/InitFuncs.cpp:359-364).
void diffusion_by_species(const srs_params& p, double D[N_SPECIES]);

// Fills the reference defaults (cpu/InitFuncs.cpp:28-108).
void params_default(srs_params* p);
// Parses <parameter><symbol/><value/></parameter> entries into p
// (cpu/InitFuncs.cpp:157-350).  Unknown symbols are ignored like the reference.
int params_read_xml(const char* path, srs_params* p, std::string* err);

// Mesh as read from the reference file set, in file order, then renumbered.
struct Mesh {
  int N = 0, NF = 0, NN = 0, NR = 0, NL = 0;
  std::vector<double> V0, TT, SR;       // per tet
  std::vector<int> tropc, domain;       // per tet
  std::vector<int> ele1, ele2, ftype;   // per face; ftype = simulation face type
  std::vector<double> faceC;            // per face lumped coefficient
  std::vector<double> node_x, node_y, node_z;
  std::vector<int> ele_nodes;           // 4 per tet, 0-based
  std::vector<int> ryr_ele, ryr_jsr, ryr_nb, lcc_ele;
  std::vector<int> order;               // order[new] = file index of that tet
};
// Reads the six mesh files (ReadGrid, cpu/InitFuncs.cpp:384-676) and applies
// the reference's breadth-first renumbering (cpu/InitFuncs.cpp:679-793) in
// linear time.  flag_noflux selects how boundary faces are treated.
int mesh_read(const char* base, int flag_noflux, Mesh* m, std::string* err);

// ELL-4 explicit diffusion operator with D factored out plus boundary rates
// (InitializeExplicitSparseMatrixFast, cpu/InitFuncs.cpp:1058-1418, and
// InitializeDomainStruct, cpu/InitFuncs.cpp:1005-1039).
struct Operator {
  std::vector<double> aij;  // 5 per tet: diagonal, then 4 off-diagonals
  std::vector<int> nij;     // 4 per tet; padding slots point at the tet itself
  std::vector<double> br;   // N_SPECIES x N boundary source rates
  std::vector<double> kb;   // per tet: sum of boundary-face coefficients (FACE_BOUND)
  double boundary_value[N_SPECIES];
  double max_diag = 0.0;    // max |aij diagonal|
};
int assemble_operator(const Mesh& m, const srs_params& p, Operator* op, std::string* err);

// Equilibrium initial state (ResetDefaultGridStates, cpu/InitFuncs.cpp:890-955):
// states is N_SPECIES x N, species-major.
struct RestValues {
  double ca0, ca0_jsr, trpn, csqn, atp, cmdn, dye;
};
RestValues rest_values(const srs_params& p);
void initial_states(const Mesh& m, const srs_params& p, std::vector<double>* states);

// Reverse Cuthill-McKee order of the face graph restricted to each domain,
// cytosol first.  Returns perm[new] = old (old = reference numbering).
std::vector<int> rcm_order_by_domain(const Mesh& m, const Operator& op);

// Step schedule: the reference advances t += dt in double precision and
// tests its protocol predicates on that t (cpu/RunSimulation.cpp:522-575).
// The schedule replays that arithmetic on the host.
struct Schedule {
  int64_t n_steps = 0;             // steps taken while t <= T_FINAL
  std::vector<int64_t> tick_steps; // steps before which a states row is written
  std::vector<double> tick_times;  // t at those steps
  std::vector<int64_t> grid_steps; // steps before which a grid file is written (OUTPUT_GRID_FLAG)
  std::vector<double> grid_times;  // t at those steps
  int64_t clamp_end_step = -1;     // first step with t > T_CLAMP (clamp protocol)
  int64_t hold_end_step = -1;      // first step with t >= INIT_RYR_HOLD
  double t_end = 0.0;              // t after the last step
};
Schedule make_schedule(const srs_params& p, double t0 = 0.0);
// First step whose pre-step time t satisfies t >= T (T_LCC_Close test).
int64_t first_step_at_or_after(const srs_params& p, double T);

// Mesh generator (box dyad), writing the reference mesh file set.
struct MeshGenSpec {
  double box_x, box_y, box_z;
  double foot_half_x, foot_half_y;
  int n_foot_x, n_foot_y, n_out_x, n_out_y;
  double cleft_h, jsr_h;
  int n_cleft_z, n_jsr_z, n_above_z;
  double r_trpn;
  int flag_tt;
  int ryr_mode;  // 0 lattice, 1 Poisson disk
  int ryr_nx, ryr_ny;
  double ryr_pitch, ryr_depth, ryr_cx, ryr_cy;
  int ryr_count;
  double ryr_radius;
  int n_lcc;
  double lcc_half;
  uint64_t lcc_seed, seed;
};
struct MeshGenReport {
  int n_tets, n_faces, n_nodes, n_ryr, n_lcc, n_jsr_tets;
  double max_a0;
  int n_face_type[4];
};
void meshgen_default_spec(MeshGenSpec* s);
int meshgen_box(const MeshGenSpec& s, const char* base, MeshGenReport* rep);

// Multi-site release unit: several cleft footprints with Poisson-disk RyR
// clusters over one box (same layout as srs_multisite_spec).
#ifndef SRS_MAX_SITES
#define SRS_MAX_SITES 8
#endif
struct MultiSiteSpec {
  double box_x, box_y, box_z;
  double h_fine, h_max, growth;
  double cleft_h, jsr_h;
  int n_cleft_z, n_jsr_z;
  double r_trpn;
  int flag_tt;
  int n_sites;
  double site_x[SRS_MAX_SITES], site_y[SRS_MAX_SITES];
  int site_ryr[SRS_MAX_SITES];
  double site_radius[SRS_MAX_SITES];
  double foot_margin, ryr_pitch, ryr_depth, sheet_half;
  uint64_t seed;
};
int meshgen_multisite(const MultiSiteSpec& s, const char* base, MeshGenReport* rep);

// Output formats (cpu/OutputFuncs.cpp): one states row and one VTK snapshot.
int states_row(const Mesh& m, const srs_params& p, const double* ca, const int* ryr_state,
               const int* lcc_state, const int* lccv_state, double V, double t, float* row,
               int row_cap);
int write_grid_vtk(const char* path, const Mesh& m, int run, int rank, int n, double t,
                   const double* ca, const double* dye, const int* ryr_state);

}  // namespace srs
