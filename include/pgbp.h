/* pgbp: GB300-native loopy belief propagation behind PGMax's BP interface.
 *
 * A thin C ABI over hand-written sm_103a CUDA kernels. Plain pointers and sizes only: any host
 * binding (ctypes, jax.ffi, a torch extension) can call it. All float data is float32 and all
 * indices int32, as PGMax computes without jax_enable_x64.
 *
 * Entry points and the PGMax interface each one replaces (paths relative to the PGMax tree):
 *   pgbp_plan_create    InfererContext.__post_init__   pgmax/infer/inferer.py:65-118
 *                       (the flat wiring it compiles becomes an immutable device plan)
 *   pgbp_run            BP(...).run_with_diffs / run / run_bp   pgmax/infer/bp.py:63-176
 *   pgbp_factor_update  FAC_TO_VAR_UPDATES[type](vtof, lp, T, normalize, **args)
 *                       pgmax/factor/__init__.py:37-44 -> enum.py:398-475, logical.py:492-779,
 *                       pool.py:276-474
 *   pgbp_beliefs        InfererContext.get_beliefs (flat part)   pgmax/infer/inferer.py:211-222
 *   pgbp_decode         decode_map_states                        pgmax/infer/inferer.py:251-264
 *   pgbp_marginals      get_marginals                            pgmax/infer/bp.py:263-288
 *   pgbp_softmax_rows / pgbp_argmax_rows   get_marginals / decode_map_states of any belief arrays
 *   pgbp_energy         compute_energy                           pgmax/infer/energy.py:53-148
 *   pgbp_energy_terms   compute_energy(debug_mode=True)          pgmax/infer/energy.py:151-204
 *   pgbp_sdlp_run       SDLP(...).run_with_objvals               pgmax/infer/dual_lp.py:238-313
 *   pgbp_sdlp_objective smooth_dual_objval_and_grad / get_bp_updates  dual_lp.py:65-236, 419-448
 *
 * Conventions
 *   - Every call returns PGBP_OK (0) or an error code; nothing aborts or traps.
 *     pgbp_last_error() gives a message for the calling thread's last failure.
 *   - Device pointers are CUDA global memory on the plan's device; `stream` is a cudaStream_t
 *     (NULL = legacy default stream). Calls only enqueue work; they do not synchronise, except
 *     pgbp_plan_create / pgbp_plan_destroy.
 *   - Batches follow jax.vmap over BPArrays: arrays are [batch, n] with a per-instance stride in
 *     floats; stride 0 broadcasts one array to every instance.
 *   - pgbp_run allocates nothing: its scratch comes from the caller (pgbp_workspace_size bytes).
 *   - A plan is immutable after creation, so concurrent calls on different streams are safe as
 *     long as their workspaces and outputs differ.
 */
#ifndef PGBP_H_
#define PGBP_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PGBP_OK = 0,
  PGBP_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, bad stride */
  PGBP_ERR_INVALID_WIRING = 2,   /* index out of range, inconsistent flat arrays */
  PGBP_ERR_UNSUPPORTED = 3,      /* wiring layout the engine cannot schedule */
  PGBP_ERR_CUDA = 4,             /* a CUDA runtime call failed */
  PGBP_ERR_WORKSPACE = 5,        /* workspace missing or too small */
  PGBP_ERR_TIMEOUT = 6           /* a bounded device-side wait gave up */
};

/* Factor types, in the order of PGMax's FAC_TO_VAR_UPDATES registry. */
enum { PGBP_ENUM = 0, PGBP_OR = 1, PGBP_AND = 2, PGBP_POOL = 3 };

/* The flat wiring of InfererContext (pgmax/infer/inferer.py:76-118) and of each wiring's
 * get_inference_arguments() (enum.py:54-72, logical.py:76-104, pool.py:62-83). Host pointers.
 * Per-type index arrays are relative to that type's message range, exactly as PGMax passes them.
 * Arrays of an absent factor type may be NULL with length 0. */
typedef struct {
  int64_t num_edge_states;                     /* len(ftov_msgs) */
  int64_t num_var_states;                      /* len(evidence) */
  int64_t num_edges;
  const int32_t* var_states_for_edge_states;     /* [num_edge_states] */
  const int32_t* edge_indices_for_edge_states;   /* [num_edge_states] */
  const int32_t* factor_indices_for_edge_states; /* [num_edge_states] */
  int64_t msgs_range[4][2];                    /* factor_type_to_msgs_range, registry order */
  int64_t potentials_range[4][2];              /* factor_type_to_potentials_range */
  /* EnumFactor */
  int64_t enum_num_rows;
  const int32_t* enum_factor_configs_indices;     /* [enum_num_rows] */
  const int32_t* enum_factor_configs_edge_states; /* [enum_num_rows] */
  int64_t enum_num_val_configs;
  /* ORFactor (index 0) and ANDFactor (index 1) */
  int64_t logical_num_parents[2];
  const int32_t* logical_parents_factor_indices[2];
  const int32_t* logical_parents_msg_indices[2];
  int64_t logical_num_factors[2];
  const int32_t* logical_children_edge_states[2];
  /* PoolFactor */
  int64_t pool_num_choices;
  const int32_t* pool_choices_factor_indices;
  const int32_t* pool_choices_msg_indices;
  int64_t pool_num_factors;
  const int32_t* pool_indicators_edge_states;
  /* Variables: evidence_to_vars (FactorGraphState.evidence_to_vars, fgraph.py:317-326), needed
   * only by pgbp_decode / pgbp_marginals / pgbp_energy / pgbp_sdlp_*; may be NULL. */
  int64_t num_variables;
  const int32_t* evidence_to_vars;             /* [num_var_states] */
  /* Execution options, 0 = automatic. Three execution paths exist: multi-kernel (one launch per
   * kernel class per iteration, any size), one CTA per instance with its state in shared memory,
   * and one thread-block cluster per instance; the last two run every iteration in one launch and
   * exist for graphs whose state fits in shared memory. Automatic mode times the eligible paths
   * once per (batch, temperature == 0) on the first pgbp_run and keeps the fastest (the timing
   * synchronises the stream once; under stream capture the single-CTA path is used). The flags
   * force a path instead (a forced path the graph is not eligible for falls back to
   * multi-kernel); results are identical on every path. */
  int64_t flags;
  /* Shared potential tables (no counterpart in PGMax, which stores one table per factor). When
   * non-NULL, EnumFactor k (k-th Enum factor in factor order) reads the potential of its config c
   * at log_potentials[potentials_range[PGBP_ENUM][0] + enum_factor_potential_offsets[k] + c], so
   * factors (and graphs of a batch) may share one table and log_potentials may be compact;
   * enum_num_val_configs then only counts configs, not potentials. NULL: PGMax's layout (factor k
   * reads its own configs' potentials). Plans with shared tables have no adjoint. */
  int64_t enum_num_factors;                    /* length of enum_factor_potential_offsets */
  const int32_t* enum_factor_potential_offsets;
} pgbp_wiring_desc;

#define PGBP_FLAG_NO_SMALL_GRAPH 1 /* multi-kernel only; the other paths are not even prepared */
#define PGBP_FLAG_PATH_SMALL 2
#define PGBP_FLAG_PATH_CLUSTER 4
#define PGBP_FLAG_PATH_MULTI 8
/* The Enum config rows are implied, not passed (enum_num_rows = 0, the row arrays NULL): every
 * Enum factor is unary (configs = its states) or pairwise (all K1 * K2 configs, row-major: the
 * PairwiseFactorGroup layout, fgroup/enum.py:303-310), each factor's configs following the
 * previous factor's. For large dense pairwise graphs, whose rows (2 * K1 * K2 per factor) would
 * dwarf the messages. No counterpart in PGMax, which always materialises the rows. */
#define PGBP_FLAG_ENUM_IMPLICIT_ROWS 16

typedef struct pgbp_plan pgbp_plan;

typedef struct {
  int64_t num_edge_states, num_var_states, num_edges, num_variables;
  int64_t num_potentials;        /* end of the last potentials range */
  int64_t num_enum_factors, num_enum_pairwise_factors, num_or_factors, num_and_factors,
      num_pool_factors;
  int64_t num_pairwise_buckets;  /* (n1, n2) classes run by the dense pairwise kernel */
  int64_t device_bytes;          /* device memory owned by the plan */
  int64_t num_slots;             /* message slots per instance: 1 per binary edge, else 1 per state */
  int64_t small_graph_smem_bytes; /* shared memory of the one-CTA-per-instance path, 0 if unused */
} pgbp_plan_info;

/* Compiles the wiring into device-resident schedules on `device`. Validates every index. */
int pgbp_plan_create(const pgbp_wiring_desc* desc, int device, pgbp_plan** plan);
int pgbp_plan_destroy(pgbp_plan* plan);
int pgbp_plan_get_info(const pgbp_plan* plan, pgbp_plan_info* info);

/* Bytes of scratch pgbp_run needs for `batch` instances and `num_iters` iterations. */
size_t pgbp_workspace_size(const pgbp_plan* plan, int64_t batch, int64_t num_iters);

/* run_with_diffs (pgmax/infer/bp.py:63-155) over `batch` instances:
 *   log potentials clipped to +-1e6, initial messages normalised and clipped, then
 *   max(num_iters, 1) damped iterations (num_iters <= 1 runs exactly one, as the reference does).
 * log_potentials [batch, P] (lp_stride floats apart, 0 = shared), evidence [batch, N_vs],
 * msgs_in / msgs_out [batch, E_s] (msgs_out rows are contiguous), deltas [batch, max(iters,1)]
 * or NULL. damping and temperature are the Python floats of the reference call: the
 * temperature == 0 and temperature < 0.5 branches are taken on the double values and the
 * arithmetic uses their float32 roundings (1 - damping is rounded after the subtraction). */
int pgbp_run(const pgbp_plan* plan, void* stream, int64_t batch,
             const float* log_potentials, int64_t lp_stride,
             const float* evidence, int64_t ev_stride,
             const float* msgs_in, int64_t msgs_stride,
             float* msgs_out, float* deltas,
             int64_t num_iters, double damping, double temperature,
             void* workspace, size_t workspace_bytes);

/* pgbp_run without any device allocation, for callers that cannot call cudaMalloc while they run
 * inference and cannot pass a workspace either (code inside a host framework that owns all device
 * memory and hands it only inputs and outputs; services with a fixed memory budget reserved at
 * start-up). No counterpart in the reference, which leaves memory to XLA.
 * Scratch is one static device array of PGBP_STATIC_SCRATCH_BYTES per GPU that loads this library,
 * held until the process exits; a run needing more (pgbp_workspace_size) fails with
 * PGBP_ERR_WORKSPACE. The first call on a device looks up the array's address and keeps it: make
 * that call before any stream capture. A device reset (cudaDeviceReset) frees the array with
 * every plan, so neither this entry point nor any plan may be used across one. All calls share
 * the array, so calls that overlap on the GPU race; each call clears what must start at zero.
 * Arguments and results are those of pgbp_run, bit for bit. */
#define PGBP_STATIC_SCRATCH_BYTES (32u << 20)
int pgbp_run_static_scratch(const pgbp_plan* plan, void* stream, int64_t batch,
                            const float* log_potentials, int64_t lp_stride,
                            const float* evidence, int64_t ev_stride,
                            const float* msgs_in, int64_t msgs_stride,
                            float* msgs_out, float* deltas,
                            int64_t num_iters, double damping, double temperature);

/* Perturb-and-MAP without a noise array: pgbp_run with the evidence of instance b
 *   evidence[b][i] = evidence_base[b * ev_stride + i] + (float)noise_scale * G[b * N_vs + i]
 * where G is the Gumbel(0, 1) stream of `seed` (pgbp_gumbel), generated inside the run's evidence
 * transpose: nothing is copied from the host and no noise array is stored. evidence_base may be
 * NULL (a zero base, ev_stride 0) or [batch, N_vs] (ev_stride 0 shares one base). evidence_out
 * (NULL or [batch, N_vs], contiguous) receives the perturbed evidence, for pgbp_beliefs. The same
 * result, bit for bit, as pgbp_run on that evidence. This is the loop the reference's perturb-and-MAP
 * users write around run (fresh Gumbel evidence per sample through update_evidence under
 * jax.vmap: benchmark/rbm_lib.py:173-184, pgmax/infer/bp_state.py:292-342), fused into the run. */
int pgbp_run_perturbed(const pgbp_plan* plan, void* stream, int64_t batch,
                       const float* log_potentials, int64_t lp_stride,
                       const float* evidence_base, int64_t ev_stride,
                       uint64_t seed, double noise_scale,
                       const float* msgs_in, int64_t msgs_stride,
                       float* msgs_out, float* deltas, float* evidence_out,
                       int64_t num_iters, double damping, double temperature,
                       void* workspace, size_t workspace_bytes);

/* The noise stream of pgbp_run_perturbed: out[c] = G[c] for c < count, on the current device.
 * G[c] = -ln(-ln(u_c)), u_c in (0, 1) from output c + 1 of SplitMix64 seeded with mix64(seed)
 * (23 bits, u = (2k + 1) 2^-24), ln evaluated with correctly rounded float32 operations only (the
 * exact steps are in pgmax_gb300/csrc/pgbp_gumbel.h), so the stream can be reproduced bit for bit
 * on a host. No reference counterpart (jax.random.gumbel uses its own generator). */
int pgbp_gumbel(void* stream, uint64_t seed, int64_t count, float* out);

/* Runs BP until every instance's max message residual is below `tolerance` (the convergence loop
 * PGMax users write around run_with_diffs, bp.py:63-155, checking its msgs_deltas), or
 * max_iters iterations. The residual is tested every `check_every` iterations (the stream is
 * synchronised there, so this call cannot be captured); all instances keep iterating until the
 * last one converges. Outputs: msgs_out [batch, E_s]; first_below (device, [batch]) the first
 * iteration (1-based) whose residual was below the tolerance, -1 if none; *iters_run (host) the
 * iterations run. Workspace: pgbp_workspace_size(plan, batch, check_every). No counterpart in the
 * reference's API. */
int pgbp_run_to_tolerance(const pgbp_plan* plan, void* stream, int64_t batch,
                          const float* log_potentials, int64_t lp_stride,
                          const float* evidence, int64_t ev_stride,
                          const float* msgs_in, int64_t msgs_stride, float* msgs_out,
                          double tolerance, int64_t max_iters, int64_t check_every,
                          double damping, double temperature, int32_t* first_below,
                          int64_t* iters_run, void* workspace, size_t workspace_bytes);

/* pgbp_run that also keeps the messages every `checkpoint_every` iterations, for pgbp_run_vjp:
 * checkpoints [ceil(iters / k)][batch][E_s] contiguous (k = min(checkpoint_every, iters), iters =
 * max(num_iters, 1)); checkpoint 0 is msgs_in as given, checkpoint c the messages after c * k
 * iterations. msgs_out and deltas are those of pgbp_run (bit for bit); the workspace is
 * pgbp_workspace_size's. No reference counterpart: the reference's jax.grad stores every
 * iteration's messages (its scan body is wrapped in jax.checkpoint, bp.py:98). */
int pgbp_run_checkpointed(const pgbp_plan* plan, void* stream, int64_t batch,
                          const float* log_potentials, int64_t lp_stride,
                          const float* evidence, int64_t ev_stride,
                          const float* msgs_in, int64_t msgs_stride,
                          float* msgs_out, float* deltas,
                          int64_t num_iters, int64_t checkpoint_every,
                          double damping, double temperature, float* checkpoints,
                          void* workspace, size_t workspace_bytes);

/* Reverse mode of pgbp_run: the gradients that jax.grad gives through bp.run in the reference
 * (its learning example, examples/grid_mrf.ipynb cells 15-16, differentiates
 * pgmax/infer/bp.py:63-155 this way), computed by a hand-written adjoint instead of autodiff.
 * Covers graphs of EnumFactors (dense pairwise and any other config table, each with its own
 * potentials), OR and AND factors, at temperature > 0; Pool factors, shared tables or
 * temperature 0 give PGBP_ERR_UNSUPPORTED.
 * checkpoints: those of pgbp_run_checkpointed with the same k = checkpoint_every (or, the same
 *   values, msgs_in followed by the msgs_out of pgbp_run called k iterations at a time). Each
 *   chunk is recomputed with the engine's arithmetic and walked backwards.
 * g_msgs_out [batch, E_s]: dL/d(msgs_out). Outputs: g_log_potentials [batch, P] when lp_stride
 *   != 0, else [P] summed over the batch; g_evidence likewise; g_msgs_in [batch, E_s] or NULL.
 *   Potentials clipped by the forward (|lp| > 1e6) get zero gradient. */
size_t pgbp_vjp_workspace_size(const pgbp_plan* plan, int64_t batch, int64_t num_iters,
                               int64_t checkpoint_every);
int pgbp_run_vjp(const pgbp_plan* plan, void* stream, int64_t batch,
                 const float* log_potentials, int64_t lp_stride,
                 const float* evidence, int64_t ev_stride,
                 const float* checkpoints, int64_t num_iters, int64_t checkpoint_every,
                 double damping, double temperature,
                 const float* g_msgs_out, float* g_log_potentials, float* g_evidence,
                 float* g_msgs_in, void* workspace, size_t workspace_bytes);

/* Reverse mode of pgbp_beliefs with respect to the messages (jax.grad of get_beliefs,
 * pgmax/infer/inferer.py:211-225): g_msgs[b, e] = g_beliefs[b, var_states_for_edge_states[e]];
 * the evidence gradient is g_beliefs itself. g_msgs rows are contiguous. */
int pgbp_beliefs_vjp(const pgbp_plan* plan, void* stream, int64_t batch, const float* g_beliefs,
                     int64_t gb_stride, float* g_msgs);

/* One factor type's un-fused update: out = FAC_TO_VAR_UPDATES[type](vtof, lp, T, normalize).
 * vtof / out are that type's message slice [batch, n_type] (stride floats apart), lp its
 * potential slice [batch, p_type] (lp_stride, 0 = shared). No workspace is needed. */
int pgbp_factor_update(const pgbp_plan* plan, void* stream, int type, int64_t batch,
                       const float* vtof, int64_t vtof_stride,
                       const float* log_potentials, int64_t lp_stride,
                       double temperature, int normalize, float* out, int64_t out_stride);

/* beliefs[b] = evidence[b].at[var_states_for_edge_states].add(msgs[b]); [batch, N_vs]. */
int pgbp_beliefs(const pgbp_plan* plan, void* stream, int64_t batch,
                 const float* evidence, int64_t ev_stride, const float* msgs,
                 int64_t msgs_stride, float* beliefs);

/* MAP decode: map[b, v] = argmax of variable v's states in beliefs[b] (first maximum wins).
 * Needs evidence_to_vars in the plan. */
int pgbp_decode(const pgbp_plan* plan, void* stream, int64_t batch, const float* beliefs,
                int64_t beliefs_stride, int32_t* map);

/* Per-variable softmax of the flat beliefs: marginals[b] has the layout of beliefs[b]. */
int pgbp_marginals(const pgbp_plan* plan, void* stream, int64_t batch, const float* beliefs,
                   int64_t beliefs_stride, float* marginals);

/* get_marginals (pgmax/infer/bp.py:263-288) and decode_map_states (pgmax/infer/inferer.py:251-264)
 * of belief arrays that did not come from a plan: `in` is a dense [rows, k] float32 array on the
 * current device (a VarGroup's unflattened beliefs, padded states at -inf). pgbp_softmax_rows writes
 * exp(x - logsumexp(x)) of every row ([rows, k]; padded states get 0, a row of -inf gets nan, as in
 * the reference); pgbp_argmax_rows the index of each row's first maximum, or of its first NaN
 * ([rows] int32). */
int pgbp_softmax_rows(void* stream, int64_t rows, int64_t k, const float* in, float* out);
int pgbp_argmax_rows(void* stream, int64_t rows, int64_t k, const float* in, int32_t* out);

/* Autotuner decisions. pgbp_run times, once per (batch, temperature == 0), the eligible execution
 * paths and then, on the multi-kernel path, the kernel variants of each launch site (the binary
 * variable sums: 1, 4 or 2 instances per thread, variants 0, 1, 2; the other variable sums: per
 * state or by variable; each dense 2 x 2 pairwise bucket: 1 or 4 instances per thread; OR and AND: a thread
 * or a warp per factor; the generic EnumFactors: a thread per (factor, instance) or a CTA per
 * factor staged in shared memory). Those variants give bit-identical results. A site of shared K x K tables
 * at temperature > 0 is not timed (the exp-domain tensor-core kernel, variant 1, agrees with the
 * direct kernel, variant 0, within float32 accuracy only) but may be set here. These calls export
 * and import the decision table so that a host can cache it across processes: sites are site[0]
 * the binary variable sums, site[1] the other variable sums, site[2 .. P + 1] the P pairwise
 * buckets in plan order, then OR, AND, the generic EnumFactors (per-thread or staged kernel)
 * (num_sites = 5 + P); -1 = the built-in rule; path -1 = not tuned. pgbp_plan_signature writes a string identifying the plan's structure
 * and the device's SM count: the key under which a table may be reused. */
#define PGBP_TUNE_MAX_SITES 64
typedef struct {
  int64_t batch;
  int32_t temperature0;
  int32_t path;        /* 0 multi-kernel, 1 one CTA per instance, 2 one cluster per instance */
  int32_t num_sites;   /* 0 when the sites are not tuned */
  int32_t site[PGBP_TUNE_MAX_SITES];
} pgbp_tuning_entry;
int64_t pgbp_plan_tuning_count(const pgbp_plan* plan);
int pgbp_plan_tuning_get(const pgbp_plan* plan, pgbp_tuning_entry* entries, int64_t max_entries);
int pgbp_plan_tuning_set(const pgbp_plan* plan, const pgbp_tuning_entry* entries,
                         int64_t num_entries);
int pgbp_plan_signature(const pgbp_plan* plan, char* buf, size_t len);

/* Smooth dual LP-MAP solver (SDLP): pgmax.infer.SDLP (pgmax/infer/dual_lp.py:60-463), the dual of
 * the LP relaxation of MAP smoothed by a log-sum-exp at temperature logsumexp_temp in [0, 1]
 * (0: the non-smooth dual and its subgradient). Messages are the dual variables, [batch, E_s]
 * rows msgs_stride floats apart (msgs_out contiguous); evidence and potentials as in pgbp_run.
 * pgbp_sdlp_objective: smooth_dual_objval_and_grad (dual_lp.py:65-236) at msgs: objval [batch];
 *   optionally the gradient grad [batch, E_s], the un-normalised factor updates at -msgs
 *   bp_updates [batch, E_s] and the per-edge log-sum-exp (max at temperature 0) of
 *   bp_updates - msgs, edge_lse [batch, num_edges] (get_bp_updates, dual_lp.py:419-448;
 *   get_primal_upper_bound is objval at temperature 0).
 * pgbp_sdlp_run: run_with_objvals (dual_lp.py:238-313): num_iters steps of accelerated gradient
 *   descent (temperature > 0, learning rate lr <= temperature) or of subgradient descent with
 *   step lr / sqrt(it + 1) (temperature 0); lr <= 0 takes the reference's default (the
 *   temperature, or 0.01 at 0). objvals [batch, num_iters] (may be NULL): the objective before
 *   each step. Objective sums are double, added in a fixed order.
 * Workspace: pgbp_sdlp_workspace_size(plan, batch) bytes, 256-byte aligned, for both. Needs
 * evidence_to_vars in the plan. */
size_t pgbp_sdlp_workspace_size(const pgbp_plan* plan, int64_t batch);
int pgbp_sdlp_objective(const pgbp_plan* plan, void* stream, int64_t batch,
                        const float* log_potentials, int64_t lp_stride,
                        const float* evidence, int64_t ev_stride,
                        const float* msgs, int64_t msgs_stride, double logsumexp_temp,
                        float* objval, float* grad, float* bp_updates, float* edge_lse,
                        void* workspace, size_t workspace_bytes);
int pgbp_sdlp_run(const pgbp_plan* plan, void* stream, int64_t batch,
                  const float* log_potentials, int64_t lp_stride,
                  const float* evidence, int64_t ev_stride,
                  const float* msgs_in, int64_t msgs_stride, float* msgs_out, float* objvals,
                  int64_t num_iters, double logsumexp_temp, double lr,
                  void* workspace, size_t workspace_bytes);

/* Energy of decodings, lower is better: pgmax.infer.compute_energy (pgmax/infer/energy.py:53-148,
 * debug_mode=False) for `batch` decodings at once. map [batch, num_variables] (map_stride ints
 * apart, 0 = one decoding for all) holds each variable's state as pgbp_decode writes it; a negative
 * state s of a K-state variable counts as s + K, a state outside [0, K) decodes no state.
 * log_potentials and evidence as the reference's BPArrays hold them (not clipped; stride 0 =
 * shared); energy [batch]:
 *   -sum(onehot * evidence) - sum of the decoded Enum configs' potentials, or +inf when the number
 *   of decoded Enum configs differs from the number of Enum factors (enum.py:276-323) or a
 *   decoding violates an OR / AND (logical.py:295-358) or Pool (pool.py:184-239) factor.
 * The partial sums are in double and added in a fixed order (deterministic); the reference sums in
 * float32. With shared potential tables an Enum config's potential is its table's entry.
 * Workspace: pgbp_energy_workspace_size(plan, batch) bytes, 256-byte aligned. Needs
 * evidence_to_vars in the plan. */
size_t pgbp_energy_workspace_size(const pgbp_plan* plan, int64_t batch);
int pgbp_energy(const pgbp_plan* plan, void* stream, int64_t batch,
                const float* log_potentials, int64_t lp_stride,
                const float* evidence, int64_t ev_stride,
                const int32_t* map, int64_t map_stride, float* energy,
                void* workspace, size_t workspace_bytes);

/* The per-variable and per-factor terms of the energy of `batch` decodings: compute_energy's
 * debug mode (pgmax/infer/energy.py:151-204), on the device. evidence and map as for pgbp_energy.
 * Outputs, no workspace:
 *   var_energy [batch, num_variables] (evidence_to_vars order): -evidence[state] of the decoded
 *     state (a negative state s of a K-state variable is s + K), NaN when no state is decoded;
 *   factor_config [batch, num_factors] (the flat wiring's factor order): for an EnumFactor the
 *     index of the decoded config among the factor's configs (the last of equal configs, as the
 *     reference's lookup keeps it), -1 when its variables decode no config (enum.py:326-360);
 *     for an OR / AND / Pool factor 0 when the decoding satisfies it, -1 when it violates it
 *     (logical.py:378-406, pool.py:242-272). The reference's factor energy is then
 *     -potentials[config] of the factor object's own potentials (in their own precision), or
 *     +inf for -1, 0 for a satisfied logical or Pool factor. */
int pgbp_energy_terms(const pgbp_plan* plan, void* stream, int64_t batch,
                      const float* evidence, int64_t ev_stride,
                      const int32_t* map, int64_t map_stride,
                      float* var_energy, int32_t* factor_config);

/* Kernel timing. While enabled, pgbp_run brackets every kernel launch with CUDA events on its
 * stream (no synchronisation is added). pgbp_profile_read waits for the recorded events, returns
 * per-class launch counts and total device milliseconds, and clears the record. Classes:
 * 0 variable sums, 1 dense pairwise Enum, 2 generic Enum, 3 OR, 4 AND, 5 Pool,
 * 6 layout (transposes, potential clipping, initial normalisation, residual copy-out),
 * 7 read-out (pgbp_beliefs, pgbp_decode, pgbp_marginals, pgbp_beliefs_vjp, pgbp_energy, the
 * SDLP per-variable and per-factor kernels; the SDLP factor passes count in classes 1-5), 8 the
 * one-CTA-per-instance small-graph kernel (all iterations in one launch), 9 the adjoint kernels of
 * pgbp_run_vjp (its forward recomputation is counted in the classes above), 10 the tcgen05
 * kernel of shared 64 x 64 tables of one instance (class 1 counts every other dense pairwise
 * launch, class 6 the building of the exp-domain run-time tables). Process-wide, not
 * thread-safe. */
#define PGBP_PROFILE_CLASSES 11
typedef struct {
  int64_t launches[PGBP_PROFILE_CLASSES];
  double milliseconds[PGBP_PROFILE_CLASSES];
} pgbp_profile;
int pgbp_profile_enable(int enable);
int pgbp_profile_read(pgbp_profile* out);

/* Bounded device-side waits. Kernels that wait for their own asynchronous copies (the shared
 * K x K table of the exp-domain pairwise kernels arrives by one bulk copy on an mbarrier) give up
 * after 2 s instead of hanging: the CTA that gave up stops (its part of the messages is left
 * unwritten, so the launch's results are invalid), counts the wait on the device and sets the
 * plan's fault word, which lives in mapped host memory.
 *   pgbp_plan_check     PGBP_ERR_TIMEOUT when a completed launch on `plan` gave up a wait since
 *                       the last report, else PGBP_OK; clears the word. It reads host memory
 *                       only and does not synchronise: synchronise the stream first to cover the
 *                       launches in it. Every entry point that enqueues work on a plan makes
 *                       the same check first and fails with PGBP_ERR_TIMEOUT, enqueueing
 *                       nothing, while the word is set.
 *   pgbp_wait_timeouts  the device-wide count since the last call in *count, reset to zero:
 *                       PGBP_OK when it is zero, PGBP_ERR_TIMEOUT otherwise. Synchronises the
 *                       current device.
 * No reference counterpart (JAX has no device-side waits to bound). */
int pgbp_plan_check(const pgbp_plan* plan);
int pgbp_wait_timeouts(int64_t* count);

/* Debug settings, process-wide, read when a launch is enqueued. No reference counterpart.
 *   PGBP_DEBUG_WAIT_LIMIT_NS     limit of the bounded device waits in ns (0 = the built-in 2 s;
 *                                at most 10 s)
 *   PGBP_DEBUG_SKIP_TABLE_COPY   1: the exp-domain pairwise kernels arm their table barrier for
 *                                the copy's bytes but issue no copy, so their wait runs out with
 *                                nothing in flight (tests the timeout path); 0: normal
 *   PGBP_DEBUG_LEGACY_MMA        1: shared 64 x 64 tables of a single instance run on the
 *                                warp-level mma.sync kernel instead of the tcgen05 one (for
 *                                comparison); 0: normal
 *   PGBP_DEBUG_ENUM_KERNEL       generic EnumFactors (not dense pairwise) in run() and
 *                                pgbp_factor_update: 1 = the per-thread kernel, 2 = the kernel
 *                                staging each factor in shared memory (bit-identical results);
 *                                0: the tuned choice, else the built-in rule */
#define PGBP_DEBUG_WAIT_LIMIT_NS 1
#define PGBP_DEBUG_SKIP_TABLE_COPY 2
#define PGBP_DEBUG_LEGACY_MMA 3
#define PGBP_DEBUG_ENUM_KERNEL 4
int pgbp_debug_set(int knob, int64_t value);

const char* pgbp_last_error(void);
int pgbp_version(void); /* major * 10000 + minor * 100 + patch */

#ifdef __cplusplus
}
#endif

#endif /* PGBP_H_ */
