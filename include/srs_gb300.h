/*
 * srs_gb300.h — C ABI of the GB300-native (sm_103a) spark timestep.
 *
 * The reference (mwalker174/srs) has no plugin or FFI layer: its seam is the
 * C++ function set declared in cpu/parameters.h:252-275 (ReadParameters,
 * ReadGrid, InitializeDomainStruct, ResetDefaultGridStates, RunSimulation,
 * ExplicitStep, UpdateChannelGating, WriteToStateFiles, ...), plus the
 * on-disk mesh / XML / states formats.  Each entry point below replaces one
 * of those functions; the comment names the reference definition.
 *
 * Conventions: every call returns an int status (SRS_OK == 0, negative on
 * failure; srs_last_error() gives the message).  Host buffers are owned by
 * the caller; device buffers are owned by the library.  Element indices,
 * state arrays and channel arrays use the reference's numbering (the
 * breadth-first renumbering of cpu/InitFuncs.cpp:679-793) and absolute
 * concentrations in uM.  One CUDA stream per simulation; a simulation is not
 * thread-safe.  No entry point falls back to the CPU: without a usable
 * sm_103a device, srs_sim_create fails with SRS_ERR_CUDA.
 */
#ifndef SRS_GB300_H
#define SRS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SRS_N_INT_PARAMS 19
#define SRS_N_REAL_PARAMS 56
#define SRS_N_CHAR_PARAMS 4
#define SRS_N_SPECIES 6
#define SRS_STATES_ROW_BASE 7

enum srs_status {
  SRS_OK = 0,
  SRS_ERR_INPUT = -1,       /* bad argument or parameter value */
  SRS_ERR_IO = -2,          /* file missing or malformed */
  SRS_ERR_MESH = -3,        /* mesh not connected / inconsistent */
  SRS_ERR_UNSTABLE = -4,    /* explicit step violates D*dt*max|a0| <= 1 */
  SRS_ERR_CUDA = -5,        /* no sm_103a device or a CUDA call failed */
  SRS_ERR_UNSUPPORTED = -6, /* configuration outside what the engine supports */
  SRS_ERR_NONFINITE = -7,   /* a realization produced NaN/Inf (status word) */
  SRS_ERR_TIMEOUT = -8,     /* a bounded device wait gave up */
  SRS_ERR_STATE = -9,       /* call out of order */
  SRS_ERR_NOMEM = -10
};

enum srs_precision { SRS_FP64 = 64, SRS_FP32 = 32 };
enum srs_engine {
  SRS_ENGINE_PLAIN = 0,   /* one fused step kernel launch per time step */
  SRS_ENGINE_RESIDENT = 1 /* persistent batched kernel, state held on chip */
};

/* ParamStruct (cpu/parameters.h:234-246): Integers[19], Reals[56], Chars[4][255]. */
typedef struct srs_params {
  int ints[SRS_N_INT_PARAMS];
  double reals[SRS_N_REAL_PARAMS];
  char chars[SRS_N_CHAR_PARAMS][255];
} srs_params;

const char* srs_status_string(int status);
const char* srs_last_error(void);
const char* srs_version(void);

/* ---- parameters: ReadParameters (cpu/InitFuncs.cpp:25-381) ------------- */
void srs_default_parameters(srs_params* ps);                 /* :28-108 */
int srs_read_parameters(srs_params* ps, const char* param_file); /* :110-364 */

/* ---- mesh: ReadGrid (cpu/InitFuncs.cpp:384-813) + InitializeDomainStruct
 *      (cpu/InitFuncs.cpp:1005-1039) / InitializeExplicitSparseMatrixFast
 *      (cpu/InitFuncs.cpp:1058-1418) ------------------------------------ */
typedef struct srs_grid srs_grid;
int srs_read_grid(const srs_params* ps, const char* mesh_base, srs_grid** out);
void srs_free_grid(srs_grid* g); /* FreeGridStruct (cpu/main.cpp:298-338) */

typedef struct srs_grid_info {
  int n_ele, n_face, n_nodes, n_ryr, n_lcc, n_jsr;
  double vol_jsr;   /* GridStruct::Vol_JSR (cpu/InitFuncs.cpp:1032-1037) */
  double max_diag;  /* max |a0| over elements (explicit stability bound) */
} srs_grid_info;
int srs_grid_get_info(const srs_grid* g, srs_grid_info* info);
/* aij[5N], nij[4N], boundary_rates[6N] exactly as GridStruct holds them. */
int srs_grid_get_operator(const srs_grid* g, double* aij, int* nij, double* boundary_rates);
/* V0[N], tt_area[N], domain[N], tropc[N], file_index[N] (file order of each element). */
int srs_grid_get_elements(const srs_grid* g, double* v0, double* tt_area, int* domain,
                          int* tropc, int* file_index);
/* RyR_Ele[NR], RyR_JSR_Ele[NR], RyR_Neighb[4 NR], LCC_Ele[NL] (renumbered). */
int srs_grid_get_channels(const srs_grid* g, int* ryr_ele, int* ryr_jsr_ele, int* ryr_neighb,
                          int* lcc_ele);
/* ResetDefaultGridStates (cpu/InitFuncs.cpp:890-955): states[6N], species-major. */
int srs_initial_states(const srs_grid* g, const srs_params* ps, double* states);

/* ---- simulation ---------------------------------------------------------- */
typedef struct srs_sim srs_sim;
/* Realizations per simulation: kernels put them on a grid dimension limited
 * to 65535 blocks. */
#define SRS_MAX_REALIZATIONS 65535
typedef struct srs_sim_desc {
  int n_realizations;   /* independent realizations sharing the grid */
  int precision;        /* SRS_FP64 or SRS_FP32 */
  int engine;           /* SRS_ENGINE_PLAIN or SRS_ENGINE_RESIDENT */
  int threads_per_cta;  /* resident engine: a multiple of 32 up to 640 (0: 512) */
  int cluster_size;     /* resident engine: CTAs sharing one realization, 0: tuner */
  int steps_per_launch; /* resident engine: time steps per persistent launch, 0: tuner */
  const uint64_t* seeds;/* n_realizations Philox keys; NULL: 1..n_realizations */
} srs_sim_desc;

/* InitializeDefaultGrid + InitializeDefaultChannels + ResetGlobals + the
 * device upload of gpu/InitFuncs.cu:1001-1105, for R realizations. */
int srs_sim_create(const srs_grid* g, const srs_params* ps, const srs_sim_desc* d,
                   srs_sim** out);
void srs_sim_destroy(srs_sim* s);
int srs_sim_get_desc(const srs_sim* s, srs_sim_desc* d);

/* Per-realization reset (cpu/main.cpp:216-257): equilibrium grid state,
 * default channels, globals, initial channel opening by protocol (LCC
 * trigger / clamp / fixed RyR / rate-weighted random RyR as OpenRandomRyR,
 * cpu/InitFuncs.cpp:1420-1475) and initial residuals (Philox). */
int srs_sim_reset(srs_sim* s);

/* State exchange for realization r, reference numbering, absolute units.
 * Any pointer may be NULL to skip that array.  states: 6N doubles. */
int srs_sim_set_state(srs_sim* s, int r, const double* states, const int* ryr_states,
                      const int* lcc_states, const int* lccv_states, const double* residuals);
int srs_sim_get_state(srs_sim* s, int r, double* states, int* ryr_states, int* lcc_states,
                      int* lccv_states, double* residuals);
/* Global_Vars (V_m, Ca_NSR) for every realization. */
int srs_sim_set_globals(srs_sim* s, double v_m, double ca_nsr);

/* ExplicitStep (cpu/RunSimulation.cpp:591-654) repeated n_steps times for
 * every realization: reactions, RyR/LCC flux, fast SL buffer, Euler update,
 * then UpdateChannelGating (:656-674) unless I_FLAG_NO_GATING.  No protocol
 * events and no output. */
int srs_explicit_step(srs_sim* s, int64_t n_steps);

/* RunSimulation (cpu/RunSimulation.cpp:402-589) for every realization:
 * protocol events, termination predicate and states rows (the float32 row
 * layout of WriteToStateFiles, cpu/OutputFuncs.cpp:223-350).  rows must hold
 * n_realizations * row_capacity * row_width floats where row_width is
 * SRS_STATES_ROW_BASE (+ n_ryr when I_FLAG_RYR_OUT).  n_rows[r] receives the
 * number of rows written for realization r, t_end[r] its final time. */
typedef struct srs_run_output {
  float* rows;
  int64_t row_capacity;
  int row_width;
  int64_t* n_rows;
  double* t_end;
  int64_t* n_steps;
} srs_run_output;
int srs_run_simulation(srs_sim* s, srs_run_output* out);
/* srs_run_simulation that also returns the device time of each of its
 * time-step launches (CUDA events on the engine's stream around the launch;
 * set-up and the read-back of rows are outside): launch_ms[i] for the first
 * max_launches launches, their count in *n_launches.  A launch advances
 * steps_per_launch steps (resident engine) or up to 4096 (plain engines). */
int srs_run_simulation_timed(srs_sim* s, srs_run_output* out, float* launch_ms, int max_launches,
                             int* n_launches);
/* srs_run_simulation with the grid files of WriteToGridFiles
 * (cpu/RunSimulation.cpp:545-549): when OUTPUT_GRID_FLAG is set, the run
 * stops at every step where the reference writes a grid file and calls
 * cb(user, n, t, done) with the file index n (1, 2, ...; the initial file is
 * 0), the time t and done[r] != 0 for realizations already finished (the
 * reference writes none for them).  The callback may read any realization
 * (srs_sim_get_state, srs_write_grid_vtk).  Every realization must start at
 * the same step.  launch_ms / max_launches / n_launches as in
 * srs_run_simulation_timed (NULL: not timed). */
typedef void (*srs_grid_callback)(void* user, int64_t n, double t, const int* done);
int srs_run_simulation_grid(srs_sim* s, srs_run_output* out, srs_grid_callback cb, void* user,
                            float* launch_ms, int max_launches, int* n_launches);

/* Time-stepping without protocol, for throughput measurement: advances every
 * realization by n_steps (gating on), device-resident, stream-ordered; the
 * call returns after the work is enqueued.  srs_sim_synchronize waits. */
int srs_sim_advance_async(srs_sim* s, int64_t n_steps);
int srs_sim_synchronize(srs_sim* s);
/* srs_sim_advance_async bracketed by CUDA events recorded on the
 * simulation's stream; *ms receives the device time of the advance. */
int srs_sim_time_advance(srs_sim* s, int64_t n_steps, float* ms);
/* Device status word OR-ed over realizations (bit 0: non-finite value,
 * bit 1: bounded wait timed out). */
int srs_sim_status(srs_sim* s, int* status_bits);
/* Kernel configuration actually used (engine, threads, cluster, steps/launch,
 * dynamic shared memory bytes, kernels launched so far). */
typedef struct srs_sim_config {
  int engine, precision, threads_per_cta, cluster_size, steps_per_launch;
  int smem_bytes;
  int64_t kernel_launches;
  int64_t reset_h2d_bytes;  /* host->device bytes of one srs_sim_reset */
  int64_t ctl_bytes;        /* bytes of the per-realization control blocks */
  int64_t engine_elements;  /* element slots per realization in the engine layout */
} srs_sim_config;
int srs_sim_get_config(const srs_sim* s, srs_sim_config* c);
/* Plain FP32 engine on meshes of 65,536 elements and more (the split form):
 * how many element blocks of 256 ahead each update block asks L2 to prefetch
 * (0: none; negative: the default, one wave of blocks).  A tuning knob of
 * this implementation, no counterpart in the reference; srs_gb300/tuner.py
 * searches it. */
int srs_sim_set_prefetch(srs_sim* s, int element_blocks);

/* ---- line scan (linescan/main.cpp:160-225) --------------------------------
 * PSF-weighted bound-dye fluorescence at sample points on a line, from the
 * current state of every realization:
 *   F_i = sum_j V0_j [CaDye]_j N(r_ij; sigma) + padding voxels at f0_pad,
 * restricted to |r_ij|^2 < r_thresh.  axis 0/1/2 scans x/y/z; the line
 * passes through (offset1, offset2) in the other two coordinates in the
 * reference's convention (X: (y,z) = (o1,o2); Y: (x,z) = (o1,o2);
 * Z: (x,y) = (o1,o2), with the PSF variances rotated as the reference does).
 * Samples sit at x_min + i*res for i < (int)((x_max - x_min)/res).  Padding
 * voxels of edge pad_res fill [pad_min, pad_max]^3 outside `domain`
 * (xmin, xmax, ymin, ymax, zmin, zmax). */
typedef struct srs_linescan_desc {
  int axis;
  double offset1, offset2;
  double x_min, x_max, res;
  double var_x, var_y, var_z;
  double r_thresh;
  double f0_pad, pad_res, pad_min, pad_max;
  double domain[6];
} srs_linescan_desc;
int srs_linescan_setup(srs_sim* s, const srs_linescan_desc* d, int* n_samples);
/* out[R][n_samples]: F of every realization now; rest[n_samples] (optional):
 * F of the equilibrium state (for dF/F0). */
int srs_linescan(srs_sim* s, double* out, double* rest);

/* ---- multi-mesh batch ----------------------------------------------------------
 * No reference counterpart (the reference runs one mesh per process and one
 * realization at a time).  Several FP32 resident simulations -- different
 * grids, parameter sets, protocols, realization counts and launch
 * configurations -- advanced as one unit: one replay of a CUDA graph runs a
 * launch of steps_per_launch steps (0: 1000) of every member, each member on
 * its own stream as a concurrent branch of the graph.  The members stay
 * ordinary simulations (state exchange, line scan, adjoint ...) between batch
 * calls; their results equal those of running them one by one. */
typedef struct srs_batch srs_batch;
int srs_batch_create(srs_sim* const* sims, int n, int steps_per_launch, srs_batch** out);
void srs_batch_destroy(srs_batch* b);
/* Every member advances n_steps (the srs_explicit_step loop); enqueued on the
 * batch's stream and returns. */
int srs_batch_advance(srs_batch* b, int64_t n_steps);
int srs_batch_synchronize(srs_batch* b);
/* srs_batch_advance bracketed by CUDA events; *ms = elapsed device time. */
int srs_batch_time_advance(srs_batch* b, int64_t n_steps, float* ms);
/* srs_run_simulation of every member (outs[i] for member i), replaying the
 * graph until every realization of every member has finished. */
int srs_batch_run_simulation(srs_batch* b, srs_run_output* outs);

/* ---- total Ca per compartment ---------------------------------------------
 * No reference counterpart (the reference keeps no mass balance).  For every
 * realization, out[2r] / out[2r+1] = sum over the cytosol / JSR elements of
 * V0 * (free Ca + Ca bound to every buffer state + Ca bound to the rapid SL
 * buffers at equilibrium), in uM um^3, accumulated in double precision from
 * the current state (FP64 or FP32 engine).  Without sources (no SERCA, no
 * refill, no LCC current, no-flux boundaries) the sum over both compartments
 * is conserved by the explicit step. */
int srs_sim_total_ca(srs_sim* s, double* out);

/* ---- pathwise adjoint -------------------------------------------------------
 * No reference counterpart: the reference has no derivatives.  Gradient of a
 * line-scan dF/F0 loss with respect to the parameters of the deterministic
 * integrator (the diffusion / buffer / pump / release terms of
 * cpu/RunSimulation.cpp:25-164), conditioned on the recorded gating
 * trajectory (pathwise sensitivity: channel states are held at the values
 * the forward run drew).
 *
 * From the current state, every realization runs n_steps explicit steps
 * (the srs_explicit_step loop, no protocol events).  At the ticks
 * k*tick_every (k = 1 .. n_steps/tick_every) the line scan of
 * srs_linescan_setup gives F_ki, and
 *   L_r = 1/2 sum_k sum_i (F_ki / f0_i - 1 - target_rki)^2.
 * Returned: loss[r], grad[r][SRS_N_ADJ] = dL_r/dtheta (parameter order
 * below, each the derivative with respect to that ParamStruct::Reals entry)
 * and optionally grad_state[r][6][N] = dL_r/d(initial state), reference
 * numbering and species order.  The run is cut into segments of
 * checkpoint_every steps; each segment's trajectory is recorded by a forward
 * pass from a snapshot of its start, then swept in reverse.  With a snapshot
 * for every segment start (when device memory holds them) each segment but
 * the last is recomputed once; otherwise snapshots are taken on several
 * levels (the first forward pass keeps every f^(L-1)-th segment start, the
 * pass over one such piece every f^(L-2)-th, ...) and the run is recomputed
 * up to L times.  checkpoint_every = 0 keeps the whole trajectory of the
 * forward pass (no recomputation) when it takes at most half of the free
 * device memory, else segments of 256 steps (fewer when 256 recorded steps
 * would take more than a quarter).  The simulation is left at the state after
 * n_steps.  FP32 engines: the resident engine, and the plain engine for
 * meshes too large for it (SRS_ERR_UNSUPPORTED for FP64). */
#define SRS_N_ADJ 18
enum {
  SRS_ADJ_D_CA = 0,
  SRS_ADJ_D_DYE = 1,
  SRS_ADJ_K_ON_CMDN = 2,
  SRS_ADJ_K_OFF_CMDN = 3,
  SRS_ADJ_K_ON_TRPN = 4,
  SRS_ADJ_K_OFF_TRPN = 5,
  SRS_ADJ_K_ON_CSQN = 6,
  SRS_ADJ_K_OFF_CSQN = 7,
  SRS_ADJ_K_ON_DYE = 8,
  SRS_ADJ_K_OFF_DYE = 9,
  SRS_ADJ_V_RYR = 10,
  SRS_ADJ_A_P = 11,
  SRS_ADJ_B_TOT_SL = 12,
  SRS_ADJ_K_D_SL = 13,
  SRS_ADJ_D_ATP = 14,
  SRS_ADJ_D_CMDN = 15,
  SRS_ADJ_K_ON_ATP = 16,
  SRS_ADJ_K_OFF_ATP = 17
};
/* flags: SRS_ADJ_LAMBDA_GLOBAL keeps the adjoint state in global memory even
 * where it fits on chip (the path taken for partitions too large for it). */
#define SRS_ADJ_LAMBDA_GLOBAL 1
/* SRS_ADJ_NO_STAGE reads the recorded trajectory straight from global memory
 * instead of staging each step's slice in shared memory by bulk copies. */
#define SRS_ADJ_NO_STAGE 2
/* SRS_ADJ_STAGE always stages the slices (the library does not choose it by
 * itself: on the measured meshes it is not faster). */
#define SRS_ADJ_STAGE 4
/* SRS_ADJ_MEAN_TRACE: the loss is the misfit of the realizations' mean
 * trace, L = 1/2 sum_ticks sum_i (mean_r(F_ri) / F0_i - 1 - target_i)^2,
 * with target [n_steps/tick_every][n_samples] shared by all realizations;
 * loss[0] receives L (the other entries 0) and grad[r] the part of dL/dtheta
 * that flows through realization r (their sum is dL/dtheta).  Without it
 * each realization has its own loss against target[r]. */
#define SRS_ADJ_MEAN_TRACE 8
typedef struct srs_adjoint_desc {
  int64_t n_steps;
  int tick_every;
  int checkpoint_every;
  const double* f0;      /* [n_samples] reference fluorescence F0 */
  const double* target;  /* [R][n_steps/tick_every][n_samples] ([n_steps/tick_every]
                            [n_samples] with SRS_ADJ_MEAN_TRACE), or NULL (zero) */
  int flags;
  int threads_per_cta;   /* reverse-sweep kernel: a multiple of 32 in [64, 512] (0: chosen
                            by the library) */
  int cta_partitions;    /* forward partitions per reverse-sweep CTA, a divisor of the
                            cluster size (0: chosen by the library) */
  int max_checkpoints;   /* at most this many state snapshots besides the final state
                            (0: as many as the free device memory holds); fewer
                            snapshots than segments make the sweep recompute the forward
                            run on more levels */
} srs_adjoint_desc;
typedef struct srs_adjoint_out {
  double* loss;        /* [R] */
  double* grad;        /* [R][SRS_N_ADJ] */
  double* grad_state;  /* [R][6][N] or NULL */
} srs_adjoint_out;
/* ParamStruct::Reals index of each gradient entry. */
int srs_adjoint_param_index(int k);
int srs_adjoint(srs_sim* s, const srs_adjoint_desc* d, srs_adjoint_out* out);
/* The plan srs_adjoint would take for d with the device memory free now: the
 * steps of one recorded segment, the checkpoint levels, and the forward steps
 * the sweep runs in all (n_steps with one level and the whole trajectory). */
int srs_adjoint_plan(srs_sim* s, const srs_adjoint_desc* d, int* segment_steps, int* levels,
                     int64_t* forward_steps);

/* ---- output formats (cpu/OutputFuncs.cpp) -------------------------------- */
/* WriteToGridFiles (cpu/OutputFuncs.cpp:42-220): legacy ASCII VTK of the
 * current state of realization r at time t. */
int srs_write_grid_vtk(srs_sim* s, int r, const char* path, int run, int rank, int n, double t);
/* The same file from host arrays (no device needed): states[6N] species-major
 * in the grid's numbering (C_CA and C_DYE are written) and ryr_states[NR]
 * (B_RYR marks open RyRs with 2); WriteToGridFiles (cpu/OutputFuncs.cpp:42-220). */
int srs_grid_write_vtk(const srs_grid* g, const double* states, const int* ryr_states,
                       const char* path, int run, int rank, int n, double t);

/* ---- numerics check (no reference counterpart) ------------------------------
 * The FP32 engines keep their Euler compensation terms as IEEE halves of
 * c * 2^24 (round to nearest even, saturated to +-65504, a NaN stays a NaN).
 * out[i] = in[i] after that round trip on the device, through the
 * four-species form of the forward engines (packed = 0) or of the plain
 * engine's adjoint (packed = 1); every fifth value through the single form.
 * For tests of the device codec against a restatement. */
int srs_comp_round_trip(const float* in, float* out, int64_t n, int packed);

/* ---- synthetic meshes (no reference counterpart beyond the file format of
 * mesh/main.cpp:1305-1364): box dyad, see the generator for the geometry. */
typedef struct srs_box_mesh_spec {
  double box_x, box_y, box_z;
  double foot_half_x, foot_half_y;
  int n_foot_x, n_foot_y, n_out_x, n_out_y;
  double cleft_h, jsr_h;
  int n_cleft_z, n_jsr_z, n_above_z;
  double r_trpn;
  int flag_tt;
  int ryr_mode; /* 0: square lattice, 1: Poisson disk */
  int ryr_nx, ryr_ny;
  double ryr_pitch, ryr_depth, ryr_cx, ryr_cy;
  int ryr_count;
  double ryr_radius;
  int n_lcc;
  double lcc_half;
  uint64_t lcc_seed, seed;
} srs_box_mesh_spec;
void srs_box_mesh_default(srs_box_mesh_spec* spec);
/* report: n_tets, n_faces, n_nodes, n_ryr, n_lcc, n_jsr (6 ints); max_a0 (1 double) */
int srs_box_mesh_write(const srs_box_mesh_spec* spec, const char* base, int* report_ints,
                       double* report_max_a0);

/* Multi-site release unit: n_sites cleft footprints over one box, each with a
 * Poisson-disk RyR cluster of site_ryr[k] channels at least ryr_pitch apart
 * in a disc of site_radius[k] around (site_x[k], site_y[k]) and one LCC per
 * 7 RyRs in its footprint (half width site_radius[k] + foot_margin).  JSR
 * caps over the footprints are joined by JSR sheets (half width sheet_half)
 * along L-shaped paths between consecutive sites.  In-plane cells are about
 * h_fine over the footprints and grow by `growth` up to h_max elsewhere; the
 * cleft and the JSR take n_cleft_z and n_jsr_z layers.  Same six files and
 * report as srs_box_mesh_write. */
#define SRS_MAX_SITES 8
typedef struct srs_multisite_spec {
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
  uint64_t seed; /* site k places its RyRs with seed + k, its LCCs with seed + 100 + k */
} srs_multisite_spec;
int srs_multisite_mesh_write(const srs_multisite_spec* spec, const char* base, int* report_ints,
                             double* report_max_a0);

/* ---- allocation-free step ---------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory — a host application that owns every device allocation through its
 * own pool or budget, or a real-time loop in which cudaMalloc/cudaFree (which
 * may synchronise the device) must not run — srs_explicit_step_fp64_noalloc
 * performs one
 * ExplicitStep (cpu/RunSimulation.cpp:591-654, FP64, reference operation
 * order, followed by gating unless `nogating`) for up to
 * SRS_NOALLOC_MAX_REALIZATIONS realizations, reading states_in and writing
 * states_out, with every array a device buffer owned by the caller.  It calls
 * no cudaMalloc/cudaFree.  Its only other device memory is a fixed array
 * compiled into the library (per GPU, held until the process exits, about
 * 22 KB), shared by all calls and reused without reallocation: each call
 * clears it first, and calls whose work overlaps on the GPU race on it, so
 * serialise them.  The first call on a device, with that device current,
 * looks up that array's device address (cudaGetSymbolAddress) and caches it;
 * make that first call before any stream capture.  The cache is not
 * refreshed, so cudaDeviceReset between calls is not supported.  Arrays use the reference numbering and the layouts returned by
 * srs_grid_get_operator / srs_grid_get_elements / srs_grid_get_channels:
 *   aij[5N], nij[4N]; br4[4N] = boundary rates of Ca, ATP, CMDN, dye;
 *   bhi[N] = TTArea*B_TOT_SL_HI/(V0*1e-15), blo[N] the same with B_TOT_SL_LO;
 *   flags[N]: bit0 JSR, bit1 troponin C, bit2 element has channel entries;
 *   chan_ptr[N+1], chan_list[2*nnz] = (kind, channel) per entry, RyRs in
 *   index order (kind 0 cleft side, 1 JSR side) then LCCs (kind 2);
 *   states_in/out[R][6N]; ryr_states[R][NR], lcc/lccv_states[R][NL],
 *   residuals[R][NR+NL] updated in place.  `reals` (ParamStruct::Reals) and
 *   `seeds` (Philox key per realization) are host arrays; `step` is the time
 *   step index that keys the draws; `status` (optional, device) receives bit
 *   0 on a non-finite value; `stream` is a cudaStream_t (NULL: default). */
#define SRS_NOALLOC_MAX_REALIZATIONS 256
typedef struct srs_noalloc_step {
  int n_ele, n_realizations, n_ryr, n_lcc;
  const double* aij;
  const int* nij;
  const double* br4;
  const double* v0;
  const double* bhi;
  const double* blo;
  const int* flags;
  const int* chan_ptr;
  const int* chan_list;
  const int* ryr_ele;
  const int* ryr_jsr;
  const int* ryr_nb;
  const int* lcc_ele;
  const double* states_in;
  double* states_out;
  int* ryr_states;
  int* lcc_states;
  int* lccv_states;
  double* residuals;
  unsigned int* status;
  const double* reals;
  const uint64_t* seeds;
  int64_t step;
  double v_m, ca_nsr;
  int nogating;
  void* stream;
} srs_noalloc_step;
int srs_explicit_step_fp64_noalloc(const srs_noalloc_step* d);

#ifdef __cplusplus
}
#endif
#endif /* SRS_GB300_H */
