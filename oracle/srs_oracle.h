/*
 * srs_oracle.h — CPU oracle of the spark timestep (test infrastructure only).
 *
 * A plain-C restatement of the reference path, used by tests/, by the smoke
 * check and by the CPU baseline of bench.py, to compare against.  The product
 * (srs_gb300/) never links, imports or calls it.
 *
 * Two gating modes:
 *   OR_RNG_REFERENCE  glibc rand() and libm exactly as cpu/RunSimulation.cpp
 *                     (pinned bit-for-bit against the reference's own
 *                     RunSimulation.cpp compiled in oracle/_ref);
 *   OR_RNG_PHILOX     counter-based Philox4x32-10 draws keyed by
 *                     (realization seed, channel, step) and the FP32 rate
 *                     arithmetic the GPU engines use, restated independently,
 *                     so GPU gating decisions can be checked bit-for-bit.
 */
#ifndef SRS_ORACLE_H
#define SRS_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { OR_RNG_REFERENCE = 0, OR_RNG_PHILOX = 1 };

typedef struct or_mesh or_mesh;

/* ReadGrid (cpu/InitFuncs.cpp:384-813) restated, including the quadratic
 * breadth-first renumbering, then the operator of
 * InitializeExplicitSparseMatrixFast / InitializeDomainStruct
 * (cpu/InitFuncs.cpp:1005-1418).  reals: ParamStruct::Reals[56]. */
int or_mesh_load(const char* base, int flag_noflux, const double* reals, or_mesh** out);
void or_mesh_free(or_mesh* m);
/* counts[6]: N, NF, NN, NR, NL, n_jsr */
void or_mesh_counts(const or_mesh* m, int* counts);
void or_mesh_operator(const or_mesh* m, double* aij, int* nij, double* br);
void or_mesh_elements(const or_mesh* m, double* v0, double* tt, int* domain, int* tropc, int* order);
void or_mesh_channels(const or_mesh* m, int* ryr_ele, int* ryr_jsr, int* ryr_nb, int* lcc_ele);

/* ResetDefaultGridStates (cpu/InitFuncs.cpp:890-955). */
void or_initial_states(const or_mesh* m, const double* reals, double* states);

/* One ExplicitStep (cpu/RunSimulation.cpp:591-647) without gating.
 * globals[2] = {V_m, Ca_NSR}.  states is updated in place. */
void or_explicit_step(const or_mesh* m, const double* reals, const double* globals, double* states,
                      const int* ryr, const int* lcc, const int* lccv);

/* Gating after step `step` in PHILOX mode (the GPU's update rule). */
void or_gating_philox(const or_mesh* m, const double* reals, double V, const double* ca,
                      uint64_t seed, int64_t step, int* ryr, int* lcc, int* lccv, double* res);

/* n steps with gating (PHILOX mode, no protocol): srs_explicit_step's contract. */
void or_steps_philox(const or_mesh* m, const double* reals, const double* globals, double* states,
                     uint64_t seed, int64_t step0, int64_t n, int* ryr, int* lcc, int* lccv,
                     double* res);

/* Per-realization reset used by the GPU engines in PHILOX mode. */
void or_reset_philox(const or_mesh* m, const int* ints, const double* reals, uint64_t seed,
                     double* states, int* ryr, int* lcc, int* lccv, double* res,
                     int64_t* lcc_close_step);

/* RunSimulation (cpu/RunSimulation.cpp:402-589) with states rows.  In
 * REFERENCE mode `seed_or_rank` is sd->device (rank) and `index` the
 * ensemble index, and the initial channel opening of cpu/main.cpp:217-250 is
 * applied; in PHILOX mode `seed_or_rank` is the Philox key.  Returns rows
 * written; *t_end, *n_steps receive the final time and step count. */
int64_t or_run_simulation(const or_mesh* m, const int* ints, const double* reals, int mode,
                          uint64_t seed_or_rank, int index, float* rows, int64_t row_cap,
                          int row_w, double* states_out, double* t_end, int64_t* n_steps);

/* The FP32 engines restated: deviation-form state u = c - c_rest (4 mobile
 * species per element, AoS, plus the immobile buffer), each element updated
 * with the same operation order as the GPU.  Reference numbering. */
void or_fp32_to_dev(const or_mesh* m, const double* reals, const double* states, float* U, float* Im);
void or_fp32_from_dev(const or_mesh* m, const double* reals, const float* U, const float* Im,
                      const float* CM, const float* CI, double* states);
/* The compact compensation term's round trip: float(half(clamp(c 2^24))) 2^-24. */
float or_comp_round_trip(float c);
/* CM (4N) and CI (N) hold the compensation terms of the Euler update.
 * flags: bit 0 gating, bit 1 compact (16-bit) compensation terms. */
void or_steps_fp32(const or_mesh* m, const double* reals, const double* globals, float* U, float* Im,
                   float* CM, float* CI, uint64_t seed, int64_t step0, int64_t n, int* ryr, int* lcc,
                   int* lccv, double* res, int flags);

/* Bit-reproducible arithmetic restated (for direct tests). */
float or_logf(float x);
float or_exp2f(float y);
double or_log(double x);
void or_philox4x32_10(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
