/*
 * rdsim_oracle.h -- CPU float64 restatement of PyRDSim's step (TEST
 * INFRASTRUCTURE ONLY: used by tests/, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg as the checker; never by the product path).
 *
 * It takes the same rdsim_system description as the GPU engine and follows
 * pyrdsim/pyrdsim.pyx operation by operation (order of float64 operations,
 * C round/floor/fmod semantics, no FMA contraction when compiled with
 * -ffp-contract=off).  Random numbers come either from the reference's own
 * stream (std::mt19937 with a fresh normal_distribution / uniform_real_
 * distribution per draw, pyrdsim.pyx:51-109) or from injected arrays.
 */
#ifndef RDSIM_ORACLE_H
#define RDSIM_ORACLE_H
#include "../include/rdsim.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_handle oracle_handle;

enum {
  ORACLE_NO_NOISE = 1,     /* random_force = False                          */
  ORACLE_INJECT = 2,       /* xi/u1/u2 host arrays like rdsim_step          */
  ORACLE_STREAM = 8        /* the reference's mt19937 stream, seeded by seed */
};

/* history_quirk != 0 reproduces the shallow dict copy of pyrdsim.pyx:1513:
 * every candidate pair ever listed stays a candidate at later rebuilds. */
int oracle_create(const rdsim_system* sys, int32_t history_quirk,
                  oracle_handle** out);
int oracle_destroy(oracle_handle* h);
int oracle_step(oracle_handle* h, int32_t n_steps, int32_t flags,
                const double* xi, const double* u1, const double* u2);
int oracle_set_state(oracle_handle* h, const double* x, const int32_t* types);
int oracle_get_state(oracle_handle* h, double* x, int32_t* types);
int oracle_get_drift(oracle_handle* h, double* a);
/* total_reaction_rates: those of the last reaction step, or (recompute != 0)
 * recomputed from the current positions, types and neighbour list. */
int oracle_get_reaction_rates(oracle_handle* h, int32_t recompute, double* total);
int oracle_get_pairs(oracle_handle* h, int32_t* pairs, int64_t cap,
                     int64_t* n_pairs);
int oracle_get_cell_ids(oracle_handle* h, int32_t* cell_ids);
int oracle_get_min_dist(oracle_handle* h, double* min_dist);
int oracle_get_error(oracle_handle* h, int32_t* code, int64_t* particle,
                     int32_t* dim, double* value, int64_t* step);
int oracle_set_step(oracle_handle* h, int64_t step);
/* rdsim_get_observables / rdsim_get_rdf restated over the oracle's state and
 * neighbour list (min_distance: min_dist of the last calculate_distances). */
int oracle_get_observables(oracle_handle* h, rdsim_observables* out);
int oracle_get_rdf(oracle_handle* h, int32_t type_a, int32_t type_b, double r_max,
                   int32_t n_bins, int32_t flags, int64_t* counts);
const char* oracle_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
