// srs_protocol.cuh — per-realization protocol, output rows and channel
// gating, shared by every engine.  `CaAt` is a callable returning the Ca
// concentration (double, uM) of an element of the current realization, so
// the same code reads global memory (plain engines) or distributed shared
// memory (resident engine).
#pragma once
#include "srs_sim.cuh"

namespace srs {

// One states row (WriteToStateFiles, cpu/OutputFuncs.cpp:241-350), computed
// serially in double precision in the reference's summation order.
template <class CaAt>
__device__ void write_row(const Protocol& P, const Channels& C, RealCtl& ctl,
                          const int32_t* ryr, const int32_t* lcc, const int32_t* lccv,
                          float* rows_r, double t, CaAt ca) {
  if (ctl.n_rows >= P.row_cap) {
    ctl.status |= 4u;  // row buffer full
    return;
  }
  float* row = rows_r + ctl.n_rows * (int64_t)P.row_w;
  int k = 0;
  row[k++] = (float)t;
  double i_ryr = 0;
  for (int i = 0; i < C.NR; ++i) {
    double CaJSR = ca(C.ryr_jsr[i]);
    double CaSS = ca(C.ryr_cleft[i]);
    i_ryr += ryr[i] * P.v_ryr * (CaJSR - CaSS) * (P.v_cell) * 96485 * 2 * (1e-6);
  }
  row[k++] = (float)i_ryr;
  int n_open = 0;
  for (int i = 0; i < C.NR; ++i) n_open += ryr[i];
  row[k++] = (float)n_open;
  int n_lcc = 0;
  for (int i = 0; i < C.NL; ++i)
    if (lccv[i] == 2 && (lcc[i] == 6 || lcc[i] == 12)) n_lcc++;
  row[k++] = (float)n_lcc;
  const int v = ctl.vsel;
  double i_lcc = 0;
  for (int i = 0; i < C.NL; ++i) {
    double c = ca(C.lcc_ele[i]);
    if ((lcc[i] == 6 || lcc[i] == 12) && lccv[i] == 2)
      i_lcc += P.lccA[v] * (c * P.lccE[v] - P.lccB) / P.lccEm1[v] * 96485 * 2 * (1e-6);
  }
  row[k++] = (float)i_lcc;
  double mean_sr = 0;
  for (int i = 0; i < C.NR; ++i) mean_sr += ca(C.ryr_jsr[i]);
  mean_sr /= C.NR;
  row[k++] = (float)mean_sr;
  double mean_i = 0;
  for (int i = 0; i < C.NR; ++i) mean_i += ca(C.ryr_cleft[i]);
  mean_i /= C.NR;
  row[k++] = (float)mean_i;
  if (P.ryr_out)
    for (int i = 0; i < C.NR; ++i) row[k++] = (float)ryr[i];
  ctl.n_rows++;
}

// Protocol work that precedes time step ctl.step (one thread):
// termination predicate, LCC closing, voltage clamp, RyR hold and the states
// row at output ticks (cpu/RunSimulation.cpp:522-566).
template <class CaAt>
__device__ void prestep(const Protocol& P, const Channels& C, RealCtl& ctl, int32_t* ryr,
                        int32_t* lcc, const int32_t* lccv, float* rows_r, CaAt ca) {
  if (ctl.done || !P.run_protocol) return;
  const int64_t n = ctl.step;
  bool go = n < P.n_steps &&
            (!P.flag_fidelity ||
             ((ctl.lcc_open || ctl.n_open_tick > 0 || ctl.ca_max_tick > P.c_min) &&
              ctl.n_open_tick < P.n_open_max));
  if (!go) {
    ctl.done = 1;
    write_row(P, C, ctl, ryr, lcc, lccv, rows_r, ctl.t, ca);  // final row (:584)
    return;
  }
  if (P.flag_lcc && ctl.lcc_open && ctl.lcc_close_step >= 0 && n >= ctl.lcc_close_step) {
    ctl.lcc_open = 0;
    lcc[P.lcc_index] = 1;  // DEFAULT_STATE_LCC
  }
  if (P.flag_vclamp) ctl.vsel = (n < P.clamp_end) ? 1 : 0;
  if (P.init_ryr != -1 && n < P.hold_end && !ryr[P.init_ryr]) ryr[P.init_ryr] = 1;
  // the step of the next tick, read from the schedule once per tick rather
  // than once per step (a global load on the protocol thread's path)
  if (ctl.tick_idx < P.n_ticks &&
      (ctl.tick_cache_ver != P.sched_ver || ctl.tick_cache_idx != ctl.tick_idx)) {
    ctl.next_tick = P.ticks[ctl.tick_idx];
    ctl.tick_cache_idx = ctl.tick_idx;
    ctl.tick_cache_ver = P.sched_ver;
  }
  if (ctl.tick_idx < P.n_ticks && ctl.next_tick == n) {
    int n_open = 0;
    double ca_max = 0;
    for (int i = 0; i < C.NR; ++i) {
      n_open += ryr[i];
      double c = ca(C.ryr_cleft[i]);
      if (c > ca_max) ca_max = c;
    }
    ctl.n_open_tick = n_open;
    ctl.ca_max_tick = ca_max;
    write_row(P, C, ctl, ryr, lcc, lccv, rows_r, P.tick_t[ctl.tick_idx], ca);
    ctl.tick_idx++;
  }
}

// The next step at which prestep has work for this realization: the end of
// the run (and every later step once done: never), the next output tick, the
// LCC closing, the end of the voltage clamp, and -- unless the caller forces
// the initial RyR open itself -- every step of the RyR hold.  Between two
// such steps prestep changes nothing.
__device__ __forceinline__ int64_t protocol_next_event(const Protocol& P, const RealCtl& ctl,
                                                       bool hold_elsewhere) {
  const int64_t never = INT64_MAX;
  if (ctl.done || !P.run_protocol) return never;
  const int64_t n = ctl.step;
  int64_t e = P.n_steps;
  if (ctl.tick_idx < P.n_ticks) {
    // a cache entry for another tick or schedule: look again next step
    const bool fresh = ctl.tick_cache_ver == P.sched_ver && ctl.tick_cache_idx == ctl.tick_idx;
    e = min(e, fresh ? ctl.next_tick : n + 1);
  }
  if (P.flag_lcc && ctl.lcc_open && ctl.lcc_close_step >= 0) e = min(e, ctl.lcc_close_step);
  if (P.flag_vclamp && n < P.clamp_end) e = min(e, P.clamp_end);
  if (!hold_elsewhere && P.init_ryr != -1 && n < P.hold_end) e = min(e, n + 1);
  return max(e, n + 1);
}

// Gating of every channel of one realization after time step `step`
// (UpdateChannelGating, cpu/RunSimulation.cpp:656-674), spread over
// `nlanes` cooperating threads.  Lattice coupling counts are taken from the
// states before this update (all RyRs see the same snapshot); with
// RYR_A_STAR == 0, as in every shipped parameter set, they do not enter.
// `nb_scratch` holds NR ints; `sync` synchronises the cooperating threads.
template <class CaAt, class Sync>
__device__ void gate_all(const Protocol& P, const Channels& C, int vsel, uint64_t seed,
                         int64_t step, int32_t* ryr, int32_t* lcc, int32_t* lccv, double* res,
                         int32_t* nb_scratch, int lane, int nlanes, CaAt ca, Sync sync) {
  const srs_gate_consts* g = &P.gc[vsel];
  const bool coupled = g->ryr_astar_half != 0.0f;
  if (coupled) {
    for (int i = lane; i < C.NR; i += nlanes) {
      int no = 0, nc = 0;
      for (int k = 0; k < 4; ++k) {
        int j = C.ryr_nb[4 * i + k];
        if (j >= 0) {
          if (ryr[j]) ++no;
          else ++nc;
        }
      }
      nb_scratch[i] = no | (nc << 16);
    }
    sync();
  }
  for (int i = lane; i < C.NR; i += nlanes) {
    int no = 0, nc = 0;
    if (coupled) {
      no = nb_scratch[i] & 0xffff;
      nc = nb_scratch[i] >> 16;
    }
    float ca_ss = (float)ca(C.ryr_cleft[i]);
    float ca_jsr = (float)ca(C.ryr_jsr[i]);
    double r = res[i];
    ryr[i] = srs_gate_ryr(g, ryr[i], ca_ss, ca_jsr, no, nc, &r, seed, (uint32_t)i, (uint64_t)step);
    res[i] = r;
  }
  for (int i = lane; i < C.NL; i += nlanes) {
    float ca_ss = (float)ca(C.lcc_ele[i]);
    double r = res[C.NR + i];
    int s = lcc[i], vs = lccv[i];
    srs_gate_lcc(g, &s, &vs, ca_ss, &r, seed, (uint32_t)(C.NR + i), (uint64_t)step);
    lcc[i] = s;
    lccv[i] = vs;
    res[C.NR + i] = r;
  }
}

}  // namespace srs
