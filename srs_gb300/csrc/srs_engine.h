// srs_engine.h — host-side declarations of the kernel launchers and the
// argument blocks they take (definitions in k_plain64.cu and k_fp32.cu).
#pragma once
#include "srs_comp.h"
#include <cuda_runtime.h>

#include "../../include/srs_gb300.h"
#include "srs_sim.cuh"

namespace srs {

struct Plain64Args {
  int32_t N, R;
  const double* aij;
  const int32_t* nij;
  const double* br;
  const double* v0;
  const double* bhi;
  const double* blo;
  const int32_t* flags;
  const int32_t* chan_ptr;
  const ChanEntry* chan_list;
  const double* S_in;
  double* S_out;
  double p[56];
  double nsr;
  Protocol P;
  Channels C;
  ChanState CS;
  unsigned int* counters;
};
int launch_plain64_step(const Plain64Args& a, cudaStream_t st);
int launch_plain64_prestep(const Plain64Args& a, int write_initial_row, cudaStream_t st);

struct Consts32 {
  float D[4];
  float kon[5], koff[5], bfree[5];
  float c0, c0j;
  float inv_kdi;
  float sd0, sd1, sd2;
  float sn1, sn0;
  float serca_scale;
  float refill_v, refill0;
  float khi;
  float dt;
  float jr_scale;
  float dc0;
  float lccA[2], lccE[2], lccB;
};

struct ChanEntry32 {
  int32_t kind;
  int32_t ch;
  float s;
  int32_t pad;
};

struct Plain32Args {
  int32_t N, R;
  const float4* a;
  const int4* nb;
  const float* bsl;
  const float* kb;
  const uint32_t* flags;
  const int32_t* chan_ptr;
  const ChanEntry32* chan_list;
  const float* rest_ca;
  const float4* M_in;
  const float* I_in;
  float4* M_out;
  float* I_out;
  float4* CM;  // [R][N] compensation of the Euler update (mobile species)
  float* CI;   // [R][N] compensation (immobile buffer)
  // compact compensation (srs_comp.h): when set (always, in the plain
  // engine), these hold the compensation and CM / CI are unused.  The
  // kernels keep the float branch: without it the 40-register update
  // measured 6 % slower (0.472 against 0.445 ms per large-mesh step).
  ushort4* CMq;  // [R][N]
  uint16_t* CIq;  // [R][N]
  Consts32 k;
  Protocol P;
  Channels C;
  ChanState CS;
  unsigned int* counters;
  int32_t pf_rows;  // split form: element blocks ahead whose state is prefetched into L2
  // trajectory recording for the adjoint (null: none): the slot of this
  // step, [R][N] x_{n-1} and (immobile buffer, Ca rate before the
  // rapid-buffer factor), and [R][NR + 2 NL + 1] the channel states the step
  // used (RyR, LCC, LCC voltage state, voltage selector)
  float4* traj_u;
  float2* traj_ig;
  int32_t* traj_ch;
  float* traj_ib;  // [R][N] 1 / B(x_{n-1}), B the rapid-buffer factor
};
// Meshes of at least this many elements take the split form of the plain
// FP32 step (element update, then gating, as two launches).
constexpr int PLAIN32_SPLIT_N = 65536;
int plain32_kernels_per_step(const Plain32Args& a);
int launch_plain32_step(const Plain32Args& a, cudaStream_t st);
int launch_plain32_prestep(const Plain32Args& a, int write_initial_row, cudaStream_t st);

struct __align__(16) TetRec {
  float a[4];
  uint16_t nb[4];
  float bsl;
  uint32_t flags;
};

// Per-element record of the reverse sweep (32 bytes, two vector loads).
struct __align__(16) AdjRec {
  float aT[4];     // coefficient of this element in each neighbour's row
  uint16_t nb[4];  // neighbour codes of the adjoint's CTA grouping
  float bsl;       // SL capacity x K_D; sign bit set: the element has troponin C
  float sa;        // sum of the element's own off-diagonal coefficients; sign bit
                   // set: JSR element
};

// Largest CTA of the resident engine (its kernel's launch bound).
#define SRS_RESIDENT_MAX_THREADS 640

struct ResidentArgs {
  int32_t R;
  int32_t P;
  int32_t off_bits;
  int32_t steps;
  const TetRec* geo;
  int32_t prestep_first;  // run the protocol of the first step before it
  int32_t initial_row;    // ... and write the t = 0 states row
  const int32_t* n_local; // [C] elements in each partition
  const int32_t* n_chtet; // [1] channel elements (partition 0, offsets 0..n-1)
  const int32_t* n_int;   // [C] interior elements (all neighbours in the same
                          // partition), right after the channel elements
  int32_t ch_interior;    // every channel element is interior to partition 0
  int32_t speculate;      // allow updating interior elements before the
                          // barrier completes where no realization can
                          // finish inside the launch (decided per realization)
  const int32_t* ch_ptr;  // [n_chtet+1] CSR of channel entries per channel element
  const ChanEntry32* ch_list;
  const uint16_t* ryr_cleft_code;
  const uint16_t* ryr_jsr_code;
  const uint16_t* lcc_code;
  const float* lcc_rest;
  float4* M;   // [R][C][P] state
  float* I;
  float4* CM;  // [R][C][P] compensation
  float* CI;
  Consts32 k;
  Protocol P_;
  Channels C;
  ChanState CS;
  // Trajectory recording (null: off).  Step s of the launch stores the state
  // it starts from (traj_u slot s and traj_ig.x), its Ca rate before the
  // rapid-buffer factor (traj_ig.y) and the channel states it uses (traj_ch
  // slot s: RyR[NR], LCC[NL], LCC V-gate[NL], voltage selector); slot
  // `steps` of traj_u/traj_ig holds the final state.  Layout [slot][R][C*P].
  float4* traj_u;
  float2* traj_ig;
  int32_t* traj_ch;
  float* traj_ib;  // [R][N] 1 / B(x_{n-1}), B the rapid-buffer factor
};
// Line scan: F[r][i] = pad[i] + sum_q w[q] * dye(col[q]) over ptr[i]..ptr[i+1].
struct LinescanArgs {
  int32_t n_samples;
  int32_t n_state;       // elements per realization in the engine layout
  const int32_t* ptr;    // [n_samples + 1]
  const int32_t* col;    // engine element indices
  const double* w;       // V0 * PSF weight
  const double* pad;     // [n_samples] padding-voxel contribution
  const double* S64;     // FP64 engine state [R][6][N] (or null)
  const float4* M;       // FP32 engines: deviations [R][n_state]
  const float4* CM;      //   and their compensation terms
  const ushort4* CMq;    //   (or in compact form, srs_comp.h)
  const double* rest_dye;  // [n_state] resting bound dye per element
  double* out;           // [R][n_samples]
};
int launch_linescan(const LinescanArgs& a, int R, cudaStream_t st);

// ---- total Ca per compartment (k_mass.cu) ------------------------------------
struct MassArgs {
  int32_t n_state;        // elements per realization in the engine layout
  const double* v0;       // [n_state] volume (0 for padding slots)
  const uint8_t* jsr;     // [n_state] 1 for JSR elements
  const double* bhi;      // [n_state] rapid SL buffer capacities (uM)
  const double* blo;
  double khi, klo;
  const double* S64;      // FP64 engine state [R][6][n_state], or null
  const float4* M;        // FP32 engines: deviations and compensation
  const float4* CM;
  const float* I;
  const float* CI;
  const ushort4* CMq;     // compact compensation (srs_comp.h), when set
  const uint16_t* CIq;
  const double* rest4;    // [n_state][4] rest of Ca, ATP, CMDN, dye
  const double* rest_imm; // [n_state]
  double* out;            // [R][2]: cytosol, JSR
};
int launch_total_ca(const MassArgs& a, int R, cudaStream_t st);
int launch_comp_round_trip(const float* in, float* out, int64_t n, int packed, cudaStream_t st);

// ---- pathwise adjoint (k_adjoint.cu) ---------------------------------------
// FP32 constants of the Jacobian beyond Consts32.
struct AdjConsts {
  float brest[5];      // resting bound buffer: dye, ATP, CMDN, TRPN, CSQN
  float inv_btot_sl;   // 1 / B_TOT_SL_HI (0 when B_TOT_SL_HI = 0)
  float serca_per_ap;  // dF_Ca/dA_P = -serca_per_ap * v_cycle / B
  float v_cell;        // V_CELL
  float inv_khi;       // 1 / K_D_SL_HI
  // Dirichlet faces hold the mobile buffers at their resting bound level
  // c0 B / (Kd + c0), Kd = koff / kon, so their source D kb Bv depends on kon
  // and koff: d(source)/dkon = kb * kb_on[q], d(source)/dkoff = kb * kb_off[q]
  // (q: dye, ATP, CMDN)
  float kb_on[3];
  float kb_off[3];
};

struct AdjArgs {
  int32_t R, P, off_bits;  // P: forward partition stride; off_bits of the codes in geo
  int32_t m_sub;           // forward partitions per CTA (CTA slots m_sub * P)
  int32_t ch_off_bits;     // off_bits of the forward layout (channel codes)
  int32_t n_steps;  // steps of the segment; the kernel runs t = n_steps .. 1
  int64_t s0;       // global index of the state the segment starts from
  const AdjRec* geo;  // [C*P] per-element records of the CTA grouping
  const int32_t* n_local;
  const int32_t* n_chtet;
  const int32_t* n_int;    // [C] interior elements after the channel elements
  int32_t ch_interior;     // every channel element is interior to partition 0
  const int32_t* ch_ptr;
  const ChanEntry32* ch_list;
  const uint16_t* ryr_cleft_code;
  const uint16_t* ryr_jsr_code;
  const float* ryr_s_cl;  // +1/V0 of each RyR's cleft element
  const float* ryr_s_js;  // -1/V0 of each RyR's JSR element
  int32_t NR, NL;
  const float4* traj_u;    // trajectory of the segment (ResidentArgs layout)
  const float2* traj_ig;  // (immobile buffer, Ca rate before the rapid-buffer factor)
  const int32_t* traj_ch;
  int32_t tick_every;      // loss ticks at global steps that are multiples
  int32_t n_samples;
  const double* coef;      // [tick slot][R][n_samples] dL/dF at the ticks of the segment
  const int32_t* wt_ptr;   // [C*P + 1] element -> line-scan samples
  const int32_t* wt_idx;
  const double* wt_w;
  float4* lam;   // [R][C*P] (Ca, ATP, CMDN, dye) at segment boundaries
  float* lam_im; // [R][C*P] immobile buffer
  float4* lam_c4;  // Kahan compensation
  float* lam_cim;
  float* lam_c;    // [R][C*P] lambda_Ca within a segment (when not on chip)
  int32_t own_in_smem;  // owner state of lambda in shared memory
  int32_t stage;        // trajectory staged in shared memory by bulk copies
  unsigned int* status; // bit 0: a staging wait gave up
  double* grad;  // [R][SRS_N_ADJ]
  Consts32 k;
  AdjConsts ak;
};

struct AdjTickArgs {
  int32_t n_samples, n_state, n_ticks, R;
  int32_t tick0;        // global index of the segment's first tick
  int32_t n_seg_ticks;  // ticks of the segment (grid z)
  int64_t slot_stride;  // trajectory elements between consecutive ticks
  const int32_t* ptr;
  const int32_t* col;
  const double* w;
  const double* base;    // [n_samples] pad + resting dye part
  const double* f0;
  const double* target;  // [R][n_ticks][n_samples] or null
  const float4* traj_u;  // trajectory slot of the first tick [R][n_state]
  double* coef;          // [n_seg_ticks][R][n_samples]
  double* loss;          // [n_ticks][R][n_samples]: loss terms of every tick
  int32_t mean_trace;    // loss on the realizations' mean trace (target [n_ticks][n_samples])
};

// Reverse step of the plain FP32 engine's adjoint (k_adjoint_plain.cu); all
// arrays [R][N] in the plain engine's numbering unless noted.
struct AdjPlainArgs {
  int32_t N, R, NR, NL, n_samples;
  int32_t last;            // t == 1: write the boundary lambda instead of nxt
  const float4* aT;        // [N] coefficient of this element in each neighbour's row
  const int4* nb;          // [N] neighbours
  const float2* bs;        // [N] (bsl, TropC in the sign bit; sum a + kb, JSR in the sign bit)
  const float* kb;         // [N] Dirichlet rate kb, or null when the mesh has none
  const uint32_t* flags;   // [N] bit 2: the element carries channel entries
  const int32_t* ch_ptr;
  const ChanEntry32* ch_list;
  const int32_t* ryr_cleft;
  const int32_t* ryr_jsr;
  const float* ryr_s_cl;   // +1/V0 of each RyR's cleft element
  const float* ryr_s_js;   // -1/V0 of each RyR's JSR element
  const float4* tu;        // trajectory slot of x_{n-1}
  const float2* tig;       // (immobile buffer, Ca rate) of x_{n-1}
  const float* ib;         // [R][N] 1 / B of the state the published slots divide by:
                           // x_{n-2} (step, t > 1) or x_{s1-1} (publish)
  const int32_t* rec;      // [R][NR + 2 NL + 1] channel states of step n
  const double* coef_cur;  // publish: dL/dF of the tick at s1 ([R][n_samples]) or null
  const double* coef_next; // step: dL/dF of the tick at n - 1 or null
  const int32_t* wt_ptr;   // [N + 1] element -> line-scan samples
  const int32_t* wt_idx;
  const double* wt_w;
  const float4* pub;
  float4* nxt;
  float* lam_c;
  float* lam_im;
  // Kahan compensation of lambda as halves (srs_comp.h), like the forward
  // state's
  ushort4* lam_c4q;
  uint16_t* lam_cimq;
  float4* lam;             // boundary lambda (Ca, ATP, CMDN, dye)
  double* part;            // [R][blocks][SRS_N_ADJ] FP64 gradient rows of the blocks
  Consts32 k;
  AdjConsts ak;
};
int adjp_blocks_per_realization(int N, int R, int n_sm);
int launch_adjp_publish(const AdjPlainArgs& a, int blocks, cudaStream_t st);
int launch_adjp_step(const AdjPlainArgs& a, int blocks, cudaStream_t st);

size_t adjoint_smem_bytes(int P, int n_chtet, int n_entries, bool own_in_smem, bool stage);
int launch_adjoint(const AdjArgs& a, int C, int n_clusters, int threads, size_t smem,
                   cudaStream_t st);
int adjoint_max_clusters(int C, int threads, size_t smem);
int launch_adj_tick(const AdjTickArgs& a, cudaStream_t st);

// Host-side constants (double precision, from the parameter set and the
// membrane potential V): gating rates and the LCC flux terms.
void gate_consts(const srs_params& p, double V, srs_gate_consts* g);
void lcc_flux_consts(const srs_params& p, double V, double* A, double* E, double* Em1, double* B,
                     double* Vg);

size_t resident_smem_bytes(int P, int NR, int NL, int n_chtet, int n_entries);
// per cluster size (k_res_*.cu)
#define SRS_RESIDENT_DECLARE(CC)                                                            \
  int launch_resident_c##CC(const ResidentArgs& a, int n_clusters, int threads, size_t smem, \
                            cudaStream_t st);                                              \
  int resident_max_clusters_c##CC(int threads, size_t smem);
SRS_RESIDENT_DECLARE(1)
SRS_RESIDENT_DECLARE(2)
SRS_RESIDENT_DECLARE(3)
SRS_RESIDENT_DECLARE(4)
SRS_RESIDENT_DECLARE(5)
SRS_RESIDENT_DECLARE(6)
SRS_RESIDENT_DECLARE(8)
SRS_RESIDENT_DECLARE(16)
#undef SRS_RESIDENT_DECLARE
int launch_resident(const ResidentArgs& a, int C, int n_clusters, int threads, size_t smem,
                    cudaStream_t st);
int resident_max_clusters(int C, int threads, size_t smem);
bool resident_cluster_supported(int C);

}  // namespace srs
