/* CPU oracle for loopy belief propagation, restating PGMax 0.6.1 (google-deepmind/PGMax).
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA engine: it is loaded by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline / reference arm, never by the
 * product package. It follows the reference's float32 operation order exactly (serial scatters in
 * index order, sum-then-subtract-own, max-shifted logsumexp divided by T); see bp_oracle.c for the
 * file:line of each step.
 *
 * Wiring arrays are the flat arrays of pgmax/infer/inferer.py:76-118 (InfererContext): per edge
 * state its variable state and edge; per factor type (Enum, OR, AND, Pool, in the registry order of
 * pgmax/factor/__init__.py:37-44) its message / potential ranges and its inference arguments. Every
 * per-type index array is relative to that type's message range, as in the reference.
 */
#ifndef BP_ORACLE_H_
#define BP_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int64_t num_edge_states;
  int64_t num_var_states;
  int64_t num_edges;
  const int32_t* var_states_for_edge_states;   /* [num_edge_states] */
  const int32_t* edge_indices_for_edge_states; /* [num_edge_states] */
  int64_t msgs_range[4][2];                    /* Enum, OR, AND, Pool */
  int64_t potentials_range[4][2];
  /* Enum (pgmax/factor/enum.py:54-72) */
  int64_t enum_num_rows;
  const int32_t* enum_factor_configs_indices;
  const int32_t* enum_factor_configs_edge_states;
  int64_t enum_num_val_configs;
  /* OR / AND (pgmax/factor/logical.py:76-104); index 0 = OR, 1 = AND */
  int64_t logical_num_parents[2];
  const int32_t* logical_parents_factor_indices[2];
  const int32_t* logical_parents_msg_indices[2];
  int64_t logical_num_factors[2];
  const int32_t* logical_children_edge_states[2];
  /* Pool (pgmax/factor/pool.py:62-83) */
  int64_t pool_num_choices;
  const int32_t* pool_choices_factor_indices;
  const int32_t* pool_choices_msg_indices;
  int64_t pool_num_factors;
  const int32_t* pool_indicators_edge_states;
} bpo_wiring;

/* One factor-type update, FAC_TO_VAR_UPDATES[type](vtof, lp, T, normalize) of
 * pgmax/factor/__init__.py:37-44. `vtof` and `out` are the type's message slice, `lp` its
 * potential slice. type: 0 Enum, 1 OR, 2 AND, 3 Pool. Returns 0 on success. */
int bpo_factor_update(const bpo_wiring* w, int type, const float* vtof, const float* lp,
                      double temperature, int normalize, float* out);

/* run_with_diffs of pgmax/infer/bp.py:63-155 for one instance. deltas has max(num_iters, 1)
 * entries. Returns 0 on success. */
int bpo_run(const bpo_wiring* w, const float* log_potentials, const float* evidence,
            const float* msgs_in, int64_t num_iters, double damping, double temperature,
            float* msgs_out, float* deltas);

/* The same over a batch of independent instances, one OpenMP thread per instance.
 * Per-instance strides are in floats (0 broadcasts one array to every instance); msgs_out is
 * [batch, num_edge_states], deltas [batch, max(num_iters, 1)]. */
int bpo_run_batch(const bpo_wiring* w, int64_t batch, const float* log_potentials,
                  int64_t lp_stride, const float* evidence, int64_t ev_stride,
                  const float* msgs_in, int64_t msgs_stride, int64_t num_iters, double damping,
                  double temperature, float* msgs_out, float* deltas, int num_threads);

/* Flat beliefs evidence.at[var_states_for_edge_states].add(msgs), pgmax/infer/inferer.py:218-222. */
int bpo_beliefs(const bpo_wiring* w, const float* evidence, const float* msgs, float* beliefs);

/* Draws first .. first + count - 1 of the Gumbel(0, 1) stream of `seed` that the engine's
 * perturb-and-MAP runs add to the evidence (pgbp_gumbel / pgbp_run_perturbed of include/pgbp.h),
 * restated from its specification: SplitMix64 output c + 1 from state mix64(seed), 23 bits to
 * u = (2k + 1) 2^-24, then -ln(-ln(u)) with ln by range reduction and the atanh series in
 * float32 (no fused operations). */
void bpo_gumbel(uint64_t seed, int64_t first, int64_t count, float* out);

#ifdef __cplusplus
}
#endif

#endif /* BP_ORACLE_H_ */
