// Internal structures shared by the plan compiler (pgbp_plan.cpp) and the kernels (pgbp_kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pgbp.h"

namespace pgbp {

// Message storage during a run ("slots"). Every edge of the graph owns a run of slots, in edge
// order: an edge of a binary variable owns ONE slot holding its normalised message compressed to
// a float (after normalisation one of the two states is exactly +0, see encode/decode in
// pgbp_kernels.cu); any other edge owns one slot per state. Slot s of instance b is at s * B + b.

// Dense pairwise EnumFactors with an n1 x n2 table listing every config in row-major order
// (PairwiseFactorGroup, pgmax/fgroup/enum.py:303-310). rec[u] = (first edge state, first slot,
// first variable state of variable 0, first variable state of variable 1); cfg_begin[u] is the
// absolute index of its first potential.
struct PairwiseBucket {
  int n1 = 0, n2 = 0;
  int64_t count = 0;
  int4* rec = nullptr;
  int32_t* cfg_begin = nullptr;
  // Shared-table exp-domain schedule (plans with shared tables, n1 == n2 in {16, 32, 64}): the
  // factors are sorted by table and group g is factors grp_first[g] .. + grp_count[g] - 1, all
  // reading the table at potential grp_table[g]. Run-time tables (exp of the potentials, split
  // for the tensor cores) take gemm_floats floats of the run workspace.
  int n_groups = 0;
  int32_t* grp_first = nullptr;
  int32_t* grp_count = nullptr;
  int32_t* grp_table = nullptr;
  std::vector<int64_t> grp_count_host;
  int64_t gemm_floats = 0;
  bool rows16 = false;  // every factor's message pair starts at a multiple of 4 slots
  int32_t* fac = nullptr;  // [count] the record's factor index in the flat wiring
};

// Floats of run-time tables one group of a shared-table bucket with K x K tables needs: E and E'
// as K rows of K + 8 floats each (the exp-domain kernel's shared-memory layout, copied there as
// one block) plus the row and column maxima (2 K).
#ifdef __CUDACC__
__host__ __device__
#endif
inline int64_t expgemm_table_floats(int K) { return 2LL * K * (K + 8) + 2LL * K; }
// Floats of the tcgen05 path's tables of one group (K = 64 only, else 0): E and E' split into
// tf32 high and low parts in the 128-byte swizzled layout of its shared memory, then the row
// and column maxima. A K = 64 bucket keeps both layouts (n_groups blocks of each).
int64_t expgemm_tc_table_floats(int K);

// Every other EnumFactor: per factor its edge-state range, edges and config rows. Rows of config
// k of factor f are row_begin[f] + k * n_vars[f] + i (i = variable), holding the edge state local to
// the factor (row_les), the layout of _compile_enumeration_wiring_numba (enum.py:364-394).
// Per factor-edge j (edge_off[f] <= j < edge_off[f + 1]): its size, first slot, first var state.
struct EnumGeneric {
  int64_t count = 0;
  int max_es = 0;                 // largest number of edge states of one factor
  int max_nv = 0;                 // largest number of variables of one factor
  int64_t max_cfg = 0;            // largest number of configs of one factor
  int32_t* fac = nullptr;         // [count] factor index in the flat wiring
  int32_t* es_begin = nullptr;    // [count] absolute edge-state index
  int32_t* n_es = nullptr;        // [count]
  int32_t* edge_off = nullptr;    // [count + 1]
  int32_t* edge_size = nullptr;
  int32_t* edge_slot = nullptr;
  int32_t* edge_vs = nullptr;
  int32_t* row_begin = nullptr;   // [count] into row_les
  int32_t* n_cfg = nullptr;       // [count]
  int32_t* n_vars = nullptr;      // [count]
  int32_t* cfg_begin = nullptr;   // [count] absolute potential index
  int32_t* row_les = nullptr;     // [rows] edge state local to its factor
  // configs by edge state: local edge state e of factor f is held by the local configs
  // inv_cfg[inv_off[inv_begin[f] + e]] .. inv_cfg[inv_off[inv_begin[f] + e + 1] - 1], increasing
  int32_t* inv_begin = nullptr;   // [count]
  int32_t* inv_off = nullptr;     // [sum of (n_es + 1)] absolute positions in inv_cfg
  int32_t* inv_cfg = nullptr;     // [rows]
};

// OR (off = +1) / AND (off = -1) factors: parents par_begin[f] .. par_begin[f + 1] - 1. Every edge
// is binary: (lower edge state, slot, first variable state) per parent and per child. The
// relevant state is state 1 for OR and state 0 for AND (logical.py:262-279).
struct LogicalSet {
  int64_t count = 0, num_parents = 0;
  int off = 1;
  int32_t* par_begin = nullptr;  // [count + 1]
  int4* par = nullptr;           // [num_parents] (es0, slot, vs0, 0)
  int4* child = nullptr;         // [count]
  int32_t* fac = nullptr;        // [count] factor index in the flat wiring
};

// Pool factors: choices ch_begin[f] .. ch_begin[f + 1] - 1, binary edges as above (pool.py:62-83).
struct PoolSet {
  int64_t count = 0, num_choices = 0;
  int32_t* ch_begin = nullptr;
  int4* ch = nullptr;            // [num_choices]
  int4* ind = nullptr;           // [count]
  int32_t* fac = nullptr;        // [count] factor index in the flat wiring
};

// Variable sums: binary variables (both states from one compressed slot per edge) and the
// states of all other variables (one slot per edge), each with its slots in edge order. The slot
// list of unit u is either explicit (slots[off[u] .. off[u + 1])) or, when the graph is regular
// enough that lists compress 4:1 or better, affine runs runs[run_off[u] .. run_off[u + 1]) of
// (first slot, stride, length): a run needs no index load in front of its message loads.
struct VarsumSet {
  int64_t count = 0;
  int32_t* vs = nullptr;         // [count] variable state (binary: state 0)
  bool use_runs = false;
  int32_t* off = nullptr;        // [count + 1]
  int32_t* slots = nullptr;
  int32_t* run_off = nullptr;    // [count + 1]
  int4* runs = nullptr;          // (first slot, stride, length, 0)
  // By variable (non-binary variables, whose K states see the same edges, K slots each): the
  // multi-kernel path reads per variable its first state and its edges' first slots, so a state
  // costs no index load. Units are grouped by K: group g = units grp[g].y .. grp[g + 1].y - 1,
  // state count grp[g].x, first variable grp[g].z (unit u -> variable z + (u - y) / x, state
  // (u - y) % x); grp has a sentinel entry.
  int byvar_groups = 0;
  int64_t byvar_units = 0;
  int4* byvar_grp = nullptr;
  int32_t* byvar_vs0 = nullptr;   // [variables] first variable state
  int32_t* byvar_eoff = nullptr;  // [variables + 1]
  int32_t* byvar_eslot = nullptr; // first slot of each edge, edge order
};

// Energy of a decoding (pgbp_energy): the launch walks work segments of items, each chunk of
// kEnergyChunk items one CTA. Kinds: variables (the evidence term), one dense pairwise bucket
// (param = bucket index), the generic Enum factors, OR (param 0) / AND (param 1) factors, Pool
// factors.
enum EnergyKind { kEnergyVars = 0, kEnergyPairwise, kEnergyGeneric, kEnergyLogical, kEnergyPool };
struct EnergySeg {
  int kind = 0, param = 0;
  int64_t items = 0, chunk_begin = 0;
};

struct Plan {
  int device = 0;
  int sm_count = 0;
  int64_t num_edge_states = 0, num_var_states = 0, num_edges = 0, num_variables = 0;
  int64_t num_potentials = 0;
  int64_t num_slots = 0;
  int64_t msgs_range[4][2] = {};
  int64_t potentials_range[4][2] = {};
  // var-state CSR over edge states, increasing edge-state order (pgbp_beliefs)
  int32_t* vs_off = nullptr;        // [num_var_states + 1]
  int32_t* vs_edges = nullptr;      // [num_edge_states]
  int32_t* vs_of_es = nullptr;      // [num_edge_states] var_states_for_edge_states (adjoint)
  int32_t* edge_start = nullptr;    // [num_edges + 1] first edge state of each edge
  int32_t* edge_slot = nullptr;     // [num_edges + 1] first slot of each edge
  int64_t num_factors = 0;
  int32_t* fac_edge_off = nullptr;  // [num_factors + 1] first edge of each factor (SDLP)
  // every edge binary and no variable with more than kInlineMaxDegree edges: the cluster path may
  // compute a factor's variable sums inline (vb_unit_of_vs[first state] = its binary varsum unit)
  bool inline_vsum = false;
  int32_t* vb_unit_of_vs = nullptr;  // [num_var_states], -1 where no unit starts
  int32_t* var_off = nullptr;       // [num_variables + 1] (decode / marginals), may be null
  int32_t* var_of_vs = nullptr;     // [num_var_states] evidence_to_vars (energy), may be null
  std::vector<EnergySeg> energy_segs;
  int64_t energy_chunks = 0;
  VarsumSet varsum_binary, varsum_other;
  std::vector<PairwiseBucket> pairwise;
  EnumGeneric enum_generic;
  // The multi-kernel iteration runs the generic Enum factors that are unary on a binary variable
  // with configs (0), (1) in that order (unary evidence factors, e.g. an RBM's biases) with a
  // kernel of their own: rec (first edge state, slot, first variable state, first potential);
  // enum_generic_rest holds the other generic factors (every other path takes enum_generic).
  struct Unary2Set {
    int64_t count = 0;
    int4* rec = nullptr;
  } unary2;
  EnumGeneric enum_generic_rest;
  LogicalSet logical[2];
  PoolSet pool;
  int64_t flags = 0;
  bool shared_potentials = false;  // Enum factors read tables through enum_factor_potential_offsets
  int64_t small_graph_smem = 0;  // bytes per CTA of the small-graph path; 0 = not eligible
  int cluster_size = 0;          // CTAs per instance of the cluster path; 0 = not eligible
  // execution path chosen per (batch, temperature == 0) by timing the eligible paths once
  mutable std::mutex tune_mu;
  mutable std::map<std::pair<int64_t, bool>, int> tuned_path;
  // kernel variant per launch site of the multi-kernel path (tune_sites in pgbp_kernels.cu), per
  // (batch, temperature == 0): site 0 the binary variable sums, 1 the other variable sums,
  // 2 .. pairwise.size() + 1 the dense pairwise buckets, then OR and AND; -1 = the built-in rule
  mutable std::map<std::pair<int64_t, bool>, std::vector<int>> tuned_sites;
  int64_t device_bytes = 0;
  std::vector<void*> allocations;
  // Fault word of the plan's launches, in mapped pinned host memory: a kernel whose bounded wait
  // gave up sets it (fault_dev is its device alias); the entry points and pgbp_plan_check read
  // it on the host without synchronising and report PGBP_ERR_TIMEOUT.
  unsigned* fault_host = nullptr;
  unsigned* fault_dev = nullptr;
  int64_t num_enum_factors = 0, num_enum_pairwise = 0;
};

// Records `message` as the calling thread's pgbp_last_error() and returns `code`.
int set_last_error(int code, const char* message);

// Makes `device` current for the guard's lifetime and gives the calling thread its previous
// current device back on destruction, so no entry point leaves the caller on another device.
class DeviceGuard {
 public:
  explicit DeviceGuard(int device) {
    err_ = cudaGetDevice(&prev_);
    if (err_ == cudaSuccess && prev_ != device) {
      err_ = cudaSetDevice(device);
      switched_ = err_ == cudaSuccess;
    }
  }
  ~DeviceGuard() {
    if (switched_) cudaSetDevice(prev_);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;
  cudaError_t status() const { return err_; }

 private:
  int prev_ = 0;
  bool switched_ = false;
  cudaError_t err_ = cudaSuccess;
};

// PGBP_ERR_TIMEOUT (and clears the plan's fault word) when a launch on this plan recorded a
// bounded device wait that gave up, else PGBP_OK. Reads host memory only: it sees the launches
// that have completed.
int take_plan_fault(const Plan& p);

// Debug settings (pgbp_debug_set): the bounded waits' limit in ns (0 = the built-in 2 s),
// whether the exp-domain kernels arm their table barrier without issuing the copy, so their wait
// runs out with nothing in flight, and whether K = 64 at B = 1 runs the mma.sync kernel.
// Launch sites the autotuner decides per (batch, temperature == 0), in the order of
// pgbp_tuning_entry::site: binary sums, other sums, the pairwise buckets, OR, AND, generic Enum.
inline int num_tune_sites(const Plan& p) { return 5 + (int)p.pairwise.size(); }

struct DebugKnobs {
  unsigned long long wait_limit_ns = 0;
  int skip_table_copy = 0;
  int legacy_mma = 0;  // K = 64 at B = 1 on the mma.sync kernel instead of the tcgen05 one
  int enum_kernel = 0;  // generic Enum factors: 0 = tuned / rule, 1 = per-thread, 2 = staged
};
DebugKnobs debug_knobs();

size_t workspace_bytes(const Plan& p, int64_t batch, int64_t iters, bool ev_batched, bool lp_batched);

// Decides whether the plan can run on the one-CTA-per-instance shared-memory path and prepares
// the kernels for it (pgbp_kernels.cu). Sets p.small_graph_smem.
cudaError_t prepare_small_graph(Plan& p);

// Kernel-class timing (pgbp_profile_*): RAII bracket around one launch when profiling is on.
enum ProfileClass { kProfVarsum = 0, kProfPairwise, kProfEnumGeneric, kProfOr, kProfAnd, kProfPool,
                    kProfLayout, kProfReadout, kProfSmallGraph, kProfAdjoint, kProfPairwiseExp };
bool profiling_enabled();
void profile_record(int cls, cudaStream_t s, bool start);
struct ProfileScope {
  int cls;
  cudaStream_t s;
  bool on;
  ProfileScope(int c, cudaStream_t st) : cls(c), s(st), on(profiling_enabled()) {
    if (on) profile_record(cls, s, true);
  }
  ~ProfileScope() {
    if (on) profile_record(cls, s, false);
  }
};

// pgbp_run_to_tolerance: stop once every instance's residual fell below tol.
struct ToleranceRun {
  double tol;
  int64_t max_iters;
  int32_t* first_below;  // device [B]
  int64_t* iters_run;    // host
};

// pgbp_run_perturbed: evidence = base + scale * the Gumbel stream of `seed` (pgbp_gumbel.h),
// generated in the run's evidence transpose; evidence_out (optional) receives it [B][N_vs].
struct Perturbation {
  uint64_t seed;
  float scale;
  float* evidence_out;
};

// Kernel launchers (pgbp_kernels.cu). They return cudaGetLastError() of their launches.
cudaError_t run_bp(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                   const float* ev, int64_t ev_stride, const float* msgs_in, int64_t msgs_stride,
                   float* msgs_out, float* deltas, int64_t iters, double damping, double temperature,
                   void* ws, size_t ws_bytes, int64_t checkpoint_every = 0,
                   float* checkpoints = nullptr, const ToleranceRun* tol_run = nullptr,
                   const Perturbation* pert = nullptr);
// out[c] = draw c of the Gumbel stream of `seed`, c < count (pgbp_gumbel)
cudaError_t gumbel(cudaStream_t s, uint64_t seed, int64_t count, float* out, int sm_count);
cudaError_t factor_update(const Plan& p, cudaStream_t s, int type, int64_t B, const float* vtof,
                          int64_t vtof_stride, const float* lp, int64_t lp_stride, double temperature,
                          int normalize, float* out, int64_t out_stride);
cudaError_t beliefs(const Plan& p, cudaStream_t s, int64_t B, const float* ev, int64_t ev_stride,
                    const float* msgs, int64_t msgs_stride, float* out);
cudaError_t decode(const Plan& p, cudaStream_t s, int64_t B, const float* beliefs, int64_t stride,
                   int32_t* map);
cudaError_t marginals(const Plan& p, cudaStream_t s, int64_t B, const float* beliefs, int64_t stride,
                      float* out);
// decode / marginals of a dense [rows, k] array (pgbp_argmax_rows / pgbp_softmax_rows)
cudaError_t rows_argmax(cudaStream_t s, int64_t rows, int64_t k, const float* in, int32_t* out,
                        int sm_count);
cudaError_t rows_softmax(cudaStream_t s, int64_t rows, int64_t k, const float* in, float* out,
                         int sm_count);

// Shared-table exp-domain pairwise update (pgbp_expgemm.cu), multi-kernel path, T > 0, potentials
// shared by the batch. expgemm_prepare fills the bucket's run-time tables from the clipped
// potentials once per run; expgemm_iterate runs one iteration of the bucket (fused damping,
// normalisation, clipping, residual), the counterpart of the dense pairwise kernel.
bool expgemm_eligible(const PairwiseBucket& q);
// Reads and resets the count of bounded device waits that gave up (pgbp_wait_timeouts).
cudaError_t read_wait_timeouts(unsigned long long* count);
cudaError_t expgemm_prepare(const Plan& p, const PairwiseBucket& q, cudaStream_t s,
                            const float* lpc, float t, float* tables);
cudaError_t expgemm_iterate(const Plan& p, const PairwiseBucket& q, cudaStream_t s, int64_t B,
                            const float* cur, float* nxt, const float* vsum, const float* lpc,
                            const float* tables, float d, float omd, float t, unsigned* dacc);

// Adjoint (pgbp_adjoint.cu). An empty string when the plan can be differentiated, else why not.
const char* adjoint_unsupported(const Plan& p);
size_t vjp_workspace_bytes(const Plan& p, int64_t B, int64_t iters, int64_t checkpoint_every,
                           bool ev_shared, bool lp_shared);
cudaError_t run_vjp(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                    const float* ev, int64_t ev_stride, const float* checkpoints, int64_t iters,
                    int64_t checkpoint_every, double damping, double temperature,
                    const float* g_msgs, float* g_lp, float* g_ev, float* g_msgs_in, void* ws,
                    size_t ws_bytes);
cudaError_t beliefs_vjp(const Plan& p, cudaStream_t s, int64_t B, const float* g_beliefs,
                        int64_t gb_stride, float* g_msgs);

// Smooth dual LP-MAP (SDLP, pgbp_kernels.cu). One objective evaluation (objval [B]; optional
// gradient, raw factor updates [B][E_s] and per-edge logsumexp [B][num_edges]) or num_iters
// accelerated (sub)gradient steps. Messages are [B][E_s] rows, ms floats apart.
size_t sdlp_workspace_bytes(const Plan& p, int64_t B);
cudaError_t sdlp_objective(const Plan& p, cudaStream_t s, int64_t B, const float* lp,
                           int64_t lp_stride, const float* ev, int64_t ev_stride,
                           const float* msgs, int64_t ms, double temperature, float* objval,
                           float* grad, float* updates, float* edge_lse, void* ws);
cudaError_t sdlp_run(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                     const float* ev, int64_t ev_stride, const float* msgs_in, int64_t ms,
                     float* msgs_out, float* objvals, int64_t iters, double temperature, double lr,
                     void* ws);

// Energy of decodings (pgbp_energy.cu). energy_plan fills p.energy_segs / p.energy_chunks.
void energy_plan(Plan& p);
size_t energy_workspace_bytes(const Plan& p, int64_t B);
cudaError_t energy_terms(const Plan& p, cudaStream_t s, int64_t B, const float* ev,
                         int64_t ev_stride, const int32_t* map, int64_t map_stride, float* var_e,
                         int32_t* fac_cfg);
cudaError_t energy(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                   const float* ev, int64_t ev_stride, const int32_t* map, int64_t map_stride,
                   float* out, void* ws, size_t ws_bytes);

#ifdef __CUDACC__
// Programmatic dependent launch. A kernel launched with launch_pdl may be scheduled while the
// kernel before it in the stream is still finishing; pdl_begin(), its first statement, waits
// until that kernel has completed and its writes are visible (for a normal launch it returns at
// once) and then lets the kernel after it be scheduled the same way. Only the launch latency
// between dependent kernels is hidden; their work never overlaps.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launches `kernel` (which must begin with pdl_begin()) as a programmatic dependent of the
// previous kernel in stream s, with `smem` bytes of dynamic shared memory.
template <class... KArgs, class... Args>
void launch_pdl_smem(cudaStream_t s, dim3 grid, dim3 block, size_t smem,
                     void (*kernel)(KArgs...), Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// launch_pdl_smem without dynamic shared memory.
template <class... KArgs, class... Args>
void launch_pdl(cudaStream_t s, dim3 grid, dim3 block, void (*kernel)(KArgs...), Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
#endif

}  // namespace pgbp

// The opaque handle of include/pgbp.h.
struct pgbp_plan {
  pgbp::Plan p;
};
