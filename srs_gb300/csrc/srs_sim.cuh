// srs_sim.cuh — device-side data structures shared by the step kernels and
// the host driver of the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "srs_math.h"

namespace srs {

// Per-realization control block: the reference's RunSimulation loop
// variables (cpu/RunSimulation.cpp:410-443) kept on the device.
struct RealCtl {
  int64_t step;            // index of the next time step
  int64_t lcc_close_step;  // first step with t >= T_LCC_Close (-1: never)
  int64_t n_rows;          // states rows written
  double t;                // simulated time before the next step (ms)
  double ca_max_tick;      // ca_ss_max refreshed at output ticks
  uint64_t seed;           // Philox key of this realization
  int32_t done;            // loop predicate failed (or run finished)
  int32_t lcc_open;        // bLCC_Open
  int32_t n_open_tick;     // N_RyR_Open refreshed at output ticks
  int32_t tick_idx;        // next entry of the tick list
  int32_t vsel;            // 0: default potential, 1: clamp potential
  uint32_t status;         // bit 0: non-finite state seen, bit 1: wait timeout
  int64_t next_tick;       // ticks[tick_cache_idx] of schedule tick_cache_ver
  int32_t tick_cache_idx;
  int32_t tick_cache_ver;  // 0: nothing cached (schedule versions start at 1)
};

// Protocol and channel constants (cpu/RunSimulation.cpp:436-575, 143-400).
struct Protocol {
  int64_t n_steps;          // steps while t <= T_FINAL
  const int64_t* ticks;     // output steps (ascending)
  const double* tick_t;     // t at those steps
  int32_t n_ticks;
  int32_t run_protocol;     // 0: plain ExplicitStep loop (no events / rows)
  int64_t clamp_end;        // steps < clamp_end use the clamp potential
  int64_t hold_end;         // steps < hold_end force INIT_RYR open
  int32_t flag_vclamp, flag_lcc, lcc_index, init_ryr;
  int32_t flag_fidelity, n_open_max, nogating, ryr_out;
  int32_t row_w;
  int32_t sched_ver;        // version of ticks / tick_t (incremented per upload)
  int64_t row_cap;
  double c_min;
  double dt;
  double Vm[2];             // potential (after the |V| < 1e-6 guard) per vsel
  // LCC GHK flux: J = ((A*(c*E - B))/Em1)/V0 (cpu/RunSimulation.cpp:149-162)
  double lccA[2], lccE[2], lccEm1[2], lccB;
  // RyR flux: J = (V_RYR*(c_jsr - c_cleft))*V_CELL (cpu/RunSimulation.cpp:135)
  double v_ryr, v_cell;
  srs_gate_consts gc[2];    // gating constants per vsel
};

// Channel topology in the engine's element numbering.
struct Channels {
  int32_t NR, NL;
  const int32_t* ryr_cleft;  // [NR]
  const int32_t* ryr_jsr;    // [NR]
  const int32_t* ryr_nb;     // [4 NR], -1 = none
  const int32_t* lcc_ele;    // [NL]
};

// Per-realization channel state, realization-major.
struct ChanState {
  int32_t* ryr;   // [R][NR]
  int32_t* lcc;   // [R][NL]
  int32_t* lccv;  // [R][NL]
  double* res;    // [R][NR+NL]
  RealCtl* ctl;   // [R]
  float* rows;    // [R][row_cap][row_w]
};

// Channel contributions to one element's Ca rate, in the reference's order
// (all RyRs by index, then LCCs by index; cpu/RunSimulation.cpp:619-632).
// kind 0: RyR cleft side (+J/V0), 1: RyR JSR side (-J/V0), 2: LCC.
struct ChanEntry {
  int32_t kind;
  int32_t ch;
};

}  // namespace srs
