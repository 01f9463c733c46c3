// Plan compiler and C-ABI entry points of pgbp (see include/pgbp.h).
//
// pgbp_plan_create turns the flat wiring PGMax's InfererContext compiles
// (pgmax/infer/inferer.py:76-118; per-type arguments enum.py:54-72, logical.py:76-104,
// pool.py:62-83) into device-resident schedules:
//   * a CSR of edge states per variable state (the scatter-add of bp.py:217, kept in increasing
//     edge-state order so the per-variable sums are the reference's serial sums);
//   * the edge boundaries (normalize_and_clip_msgs, bp.py:249-259);
//   * Enum factors split into dense pairwise buckets (n1 x n2 tables in the row-major config order
//     of PairwiseFactorGroup, fgroup/enum.py:303-310) and a generic list with per-factor config
//     rows (enum.py:364-394);
//   * OR / AND parents and Pool choices grouped per factor (logical.py:458-488, pool.py:151-180).
// Every index is validated on the host first; a wiring the kernels could read out of bounds is
// rejected with PGBP_ERR_INVALID_WIRING, one whose layout they cannot schedule with
// PGBP_ERR_UNSUPPORTED.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "pgbp_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(PGBP_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

pgbp::DebugKnobs g_debug;

struct Builder {
  pgbp::Plan& p;
  int err = PGBP_OK;

  template <class T>
  T* upload(const std::vector<T>& v) {
    if (err) return nullptr;
    size_t bytes = sizeof(T) * std::max<size_t>(v.size(), 1);
    void* d = nullptr;
    cudaError_t e = cudaMalloc(&d, bytes);
    if (e != cudaSuccess) {
      err = cuda_fail(e, "cudaMalloc(plan)");
      return nullptr;
    }
    p.allocations.push_back(d);
    p.device_bytes += (int64_t)bytes;
    if (!v.empty()) {
      e = cudaMemcpy(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        err = cuda_fail(e, "cudaMemcpy(plan)");
        return nullptr;
      }
    }
    return static_cast<T*>(d);
  }
};

void free_plan(pgbp::Plan& p) {
  for (void* a : p.allocations) cudaFree(a);
  p.allocations.clear();
  if (p.fault_host) cudaFreeHost(p.fault_host);
  p.fault_host = p.fault_dev = nullptr;
}

bool in_range(int64_t x, int64_t lo, int64_t hi) { return x >= lo && x < hi; }

// ----------------------------------------------------------------------------- profiling
struct ProfEvent {
  int cls;
  cudaEvent_t start, stop;
};
bool g_prof_on = false;
std::vector<ProfEvent> g_prof_events;  // recorded, not yet read
std::vector<cudaEvent_t> g_prof_pool;   // created, free for reuse
std::vector<std::pair<int, cudaEvent_t>> g_prof_open;

cudaEvent_t prof_event() {
  if (!g_prof_pool.empty()) {
    cudaEvent_t e = g_prof_pool.back();
    g_prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

}  // namespace

namespace pgbp {
int set_last_error(int code, const char* message) { return fail(code, "%s", message); }

int take_plan_fault(const Plan& p) {
  if (!p.fault_host) return PGBP_OK;
  volatile unsigned* w = p.fault_host;
  if (*w == 0u) return PGBP_OK;
  *w = 0u;
  return fail(PGBP_ERR_TIMEOUT,
              "a bounded device wait of an earlier launch on this plan gave up; that launch's "
              "results are invalid");
}

DebugKnobs debug_knobs() { return g_debug; }
bool profiling_enabled() { return g_prof_on; }
void profile_record(int cls, cudaStream_t s, bool start) {
  cudaEvent_t e = prof_event();
  if (!e) return;
  cudaEventRecord(e, s);
  if (start) {
    g_prof_open.push_back({cls, e});
  } else if (!g_prof_open.empty()) {
    ProfEvent pe{g_prof_open.back().first, g_prof_open.back().second, e};
    g_prof_open.pop_back();
    g_prof_events.push_back(pe);
  }
}
}  // namespace pgbp

extern "C" {

int pgbp_profile_enable(int enable) {
  g_prof_on = enable != 0;
  return PGBP_OK;
}

int pgbp_profile_read(pgbp_profile* out) {
  if (!out) return fail(PGBP_ERR_INVALID_ARGUMENT, "null argument");
  memset(out, 0, sizeof(*out));
  int rc = PGBP_OK;
  for (const ProfEvent& pe : g_prof_events) {
    float ms = 0.0f;
    cudaError_t e = cudaEventSynchronize(pe.stop);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, pe.start, pe.stop);
    if (e != cudaSuccess) rc = cuda_fail(e, "pgbp_profile_read");
    if (pe.cls >= 0 && pe.cls < PGBP_PROFILE_CLASSES) {
      out->launches[pe.cls] += 1;
      out->milliseconds[pe.cls] += ms;
    }
    g_prof_pool.push_back(pe.start);
    g_prof_pool.push_back(pe.stop);
  }
  g_prof_events.clear();
  return rc;
}

int pgbp_wait_timeouts(int64_t* count) {
  if (!count) return fail(PGBP_ERR_INVALID_ARGUMENT, "null argument");
  unsigned long long n = 0;
  const cudaError_t e = pgbp::read_wait_timeouts(&n);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_wait_timeouts");
  *count = (int64_t)n;
  if (n != 0) return fail(PGBP_ERR_TIMEOUT, "%lld bounded device waits gave up", (long long)n);
  return PGBP_OK;
}

int pgbp_plan_check(const pgbp_plan* plan) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  return pgbp::take_plan_fault(plan->p);
}

int pgbp_debug_set(int knob, int64_t value) {
  switch (knob) {
    case PGBP_DEBUG_WAIT_LIMIT_NS:
      if (value < 0 || value > 10000000000LL)
        return fail(PGBP_ERR_INVALID_ARGUMENT, "wait limit %lld ns outside [0, 1e10]",
                    (long long)value);
      g_debug.wait_limit_ns = (unsigned long long)value;
      return PGBP_OK;
    case PGBP_DEBUG_SKIP_TABLE_COPY:
      if (value != 0 && value != 1) return fail(PGBP_ERR_INVALID_ARGUMENT, "expected 0 or 1");
      g_debug.skip_table_copy = (int)value;
      return PGBP_OK;
    case PGBP_DEBUG_LEGACY_MMA:
      if (value != 0 && value != 1) return fail(PGBP_ERR_INVALID_ARGUMENT, "expected 0 or 1");
      g_debug.legacy_mma = (int)value;
      return PGBP_OK;
    case PGBP_DEBUG_ENUM_KERNEL:
      if (value < 0 || value > 2) return fail(PGBP_ERR_INVALID_ARGUMENT, "expected 0, 1 or 2");
      g_debug.enum_kernel = (int)value;
      return PGBP_OK;
    default:
      return fail(PGBP_ERR_INVALID_ARGUMENT, "unknown debug knob %d", knob);
  }
}

const char* pgbp_last_error(void) { return g_last_error.c_str(); }

int pgbp_version(void) { return 200; }

int pgbp_plan_create(const pgbp_wiring_desc* d, int device, pgbp_plan** out) {
  if (!d || !out) return fail(PGBP_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  const int64_t ns = d->num_edge_states, nvs = d->num_var_states, ne = d->num_edges;
  if (ns < 0 || nvs < 0 || ne < 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "negative size");
  if (ns > INT32_MAX - 1 || nvs > INT32_MAX - 1)
    return fail(PGBP_ERR_UNSUPPORTED, "more than 2^31 edge or variable states");
  if (ns > 0 && (!d->var_states_for_edge_states || !d->edge_indices_for_edge_states ||
                 !d->factor_indices_for_edge_states))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "missing edge-state arrays");

  // --- message / potential ranges (registry order Enum, OR, AND, Pool; contiguous, fgraph.py:186-232)
  int64_t np_total = 0;
  {
    int64_t prev = 0;
    for (int t = 0; t < 4; ++t) {
      if (d->msgs_range[t][0] != prev || d->msgs_range[t][1] < d->msgs_range[t][0])
        return fail(PGBP_ERR_INVALID_WIRING, "message ranges must tile [0, num_edge_states)");
      prev = d->msgs_range[t][1];
      if (d->potentials_range[t][1] < d->potentials_range[t][0] || d->potentials_range[t][0] < 0)
        return fail(PGBP_ERR_INVALID_WIRING, "bad potentials range for type %d", t);
      np_total = std::max<int64_t>(np_total, d->potentials_range[t][1]);
    }
    if (prev != ns) return fail(PGBP_ERR_INVALID_WIRING, "message ranges end at %lld, expected %lld",
                                (long long)prev, (long long)ns);
  }

  auto* handle = new (std::nothrow) pgbp_plan();
  if (!handle) return fail(PGBP_ERR_INVALID_ARGUMENT, "out of host memory");
  pgbp::Plan& p = handle->p;
  p.device = device;
  p.num_edge_states = ns;
  p.num_var_states = nvs;
  p.num_edges = ne;
  p.num_potentials = np_total;
  memcpy(p.msgs_range, d->msgs_range, sizeof(p.msgs_range));
  memcpy(p.potentials_range, d->potentials_range, sizeof(p.potentials_range));

  auto bail = [&](int code) {
    free_plan(p);
    delete handle;
    return code;
  };

  pgbp::DeviceGuard guard(device);
  if (guard.status() != cudaSuccess) return bail(cuda_fail(guard.status(), "cudaSetDevice"));
  cudaError_t ce = cudaDeviceGetAttribute(&p.sm_count, cudaDevAttrMultiProcessorCount, device);
  if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaDeviceGetAttribute"));
  {
    void* h = nullptr;
    ce = cudaHostAlloc(&h, sizeof(unsigned), cudaHostAllocMapped | cudaHostAllocPortable);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaHostAlloc(fault word)"));
    p.fault_host = static_cast<unsigned*>(h);
    *p.fault_host = 0u;
    void* dptr = nullptr;
    ce = cudaHostGetDevicePointer(&dptr, h, 0);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaHostGetDevicePointer(fault word)"));
    p.fault_dev = static_cast<unsigned*>(dptr);
  }

  const int32_t* vs = d->var_states_for_edge_states;
  const int32_t* ei = d->edge_indices_for_edge_states;
  const int32_t* fi = d->factor_indices_for_edge_states;

  // --- edges: states of an edge are contiguous and edges are numbered in order
  std::vector<int32_t> edge_start(ne + 1, 0);
  {
    int64_t expect = 0;
    for (int64_t i = 0; i < ns; ++i) {
      if (!in_range(vs[i], 0, nvs))
        return bail(fail(PGBP_ERR_INVALID_WIRING, "var state %d of edge state %lld out of range",
                         vs[i], (long long)i));
      if (i == 0 || ei[i] != ei[i - 1]) {
        if (ei[i] != expect)
          return bail(fail(PGBP_ERR_UNSUPPORTED, "edge indices must enumerate edges in order"));
        edge_start[expect] = (int32_t)i;
        ++expect;
      }
    }
    if (expect != ne)
      return bail(fail(PGBP_ERR_INVALID_WIRING, "found %lld edges, num_edges is %lld",
                       (long long)expect, (long long)ne));
    edge_start[ne] = (int32_t)ns;
  }

  // --- CSR over variable states (stable: increasing edge state inside each var state)
  std::vector<int32_t> vs_off(nvs + 1, 0), vs_edges(ns);
  for (int64_t i = 0; i < ns; ++i) vs_off[vs[i] + 1]++;
  for (int64_t v = 0; v < nvs; ++v) vs_off[v + 1] += vs_off[v];
  {
    std::vector<int32_t> fill(vs_off.begin(), vs_off.end() - 1);
    for (int64_t i = 0; i < ns; ++i) vs_edges[fill[vs[i]]++] = (int32_t)i;
  }

  // factor ranges from factor indices (each factor owns a contiguous run of edge states)
  std::vector<int64_t> fac_es_begin, fac_es_end;
  {
    int64_t expect = 0;
    for (int64_t i = 0; i < ns; ++i) {
      if (i == 0 || fi[i] != fi[i - 1]) {
        if (fi[i] != expect)
          return bail(fail(PGBP_ERR_UNSUPPORTED, "factor indices must enumerate factors in order"));
        fac_es_begin.push_back(i);
        if (i > 0) fac_es_end.push_back(i);
        ++expect;
      }
      // a factor's edge states lie inside one edge sequence: edges do not straddle factors
      if (i > 0 && ei[i] == ei[i - 1] && fi[i] != fi[i - 1])
        return bail(fail(PGBP_ERR_INVALID_WIRING, "edge %d spans two factors", ei[i]));
    }
    if (ns > 0) fac_es_end.push_back(ns);
  }
  auto factor_of = [&](int64_t es) { return (int64_t)fi[es]; };

  // --- slots: one per binary edge (compressed pair), one per state otherwise; edge order. A
  // factor whose edges all have a multiple of 4 states starts at a multiple of 4 slots, so that
  // at B = 1 each of its messages is a 16-byte aligned row (the slots skipped are never read).
  std::vector<int32_t> edge_slot(ne + 1, 0);
  {
    std::vector<char> align4(ne, 0);
    for (size_t f = 0; f < fac_es_begin.size(); ++f) {
      bool all4 = true;
      for (int64_t i = fac_es_begin[f]; i < fac_es_end[f] && all4;
           i = edge_start[ei[i] + 1]) {
        const int32_t k = edge_start[ei[i] + 1] - edge_start[ei[i]];
        all4 = k >= 4 && k % 4 == 0;
      }
      if (all4) align4[ei[fac_es_begin[f]]] = 1;
    }
    int64_t next = 0;
    for (int64_t e = 0; e < ne; ++e) {
      const int32_t k = edge_start[e + 1] - edge_start[e];
      if (align4[e]) next = (next + 3) & ~(int64_t)3;
      edge_slot[e] = (int32_t)next;
      next += (k == 2 ? 1 : k);
    }
    if (next > INT32_MAX)
      return bail(fail(PGBP_ERR_UNSUPPORTED, "more than 2^31 message slots"));
    edge_slot[ne] = (int32_t)next;
  }
  p.num_slots = edge_slot[ne];
  auto slot_of_es = [&](int64_t es) {  // slot holding edge state es (binary: the edge's slot)
    const int32_t e = ei[es];
    const int32_t k = edge_start[e + 1] - edge_start[e];
    return k == 2 ? edge_slot[e] : edge_slot[e] + (int32_t)(es - edge_start[e]);
  };

  // --- variable sums: binary variables (per variable, both states) and other variable states,
  // each listing the slots of its edges in increasing edge order (= increasing edge state)
  std::vector<int32_t> vb_vs, vb_off{0}, vb_slots, vo_vs, vo_off{0}, vo_slots;
  {
    std::vector<char> binary_vs(nvs, 0);  // 1: state 0 of a binary variable, 2: its state 1
    for (int64_t e = 0; e < ne; ++e) {
      if (edge_start[e + 1] - edge_start[e] == 2) {
        const int32_t v0 = vs[edge_start[e]];
        if (vs[edge_start[e] + 1] != v0 + 1)
          return bail(fail(PGBP_ERR_INVALID_WIRING, "states of an edge must be consecutive"));
        binary_vs[v0] = 1;
        binary_vs[v0 + 1] = 2;
      }
    }
    for (int64_t v = 0; v < nvs; ++v) {
      if (vs_off[v + 1] == vs_off[v]) continue;  // no edge: its sum is never read
      if (binary_vs[v] == 1) {
        // both states of a binary variable see the same edges (one state each)
        if (vs_off[v + 2] - vs_off[v + 1] != vs_off[v + 1] - vs_off[v])
          return bail(fail(PGBP_ERR_INVALID_WIRING, "binary variable states with different edges"));
        vb_vs.push_back((int32_t)v);
        for (int32_t k = vs_off[v]; k < vs_off[v + 1]; ++k) {
          const int64_t es = vs_edges[k];
          if (vs_edges[vs_off[v + 1] + (k - vs_off[v])] != es + 1)
            return bail(fail(PGBP_ERR_INVALID_WIRING, "binary variable edges are not paired"));
          vb_slots.push_back(slot_of_es(es));
        }
        vb_off.push_back((int32_t)vb_slots.size());
      } else if (binary_vs[v] == 0) {
        vo_vs.push_back((int32_t)v);
        for (int32_t k = vs_off[v]; k < vs_off[v + 1]; ++k) vo_slots.push_back(slot_of_es(vs_edges[k]));
        vo_off.push_back((int32_t)vo_slots.size());
      }
    }
  }

  Builder bd{p};
  p.vs_off = bd.upload(vs_off);
  p.vs_edges = bd.upload(vs_edges);
  p.vs_of_es = bd.upload(std::vector<int32_t>(vs, vs + ns));
  p.edge_start = bd.upload(edge_start);
  p.edge_slot = bd.upload(edge_slot);
  {
    // edges of factor f: fac_edge_off[f] .. fac_edge_off[f + 1] - 1 (edges follow factor order)
    std::vector<int32_t> feo(fac_es_begin.size() + 1, (int32_t)ne);
    for (size_t f = 0; f < fac_es_begin.size(); ++f) feo[f] = ei[fac_es_begin[f]];
    p.num_factors = (int64_t)fac_es_begin.size();
    p.fac_edge_off = bd.upload(feo);
  }
  // slot lists as affine runs (first, stride, length); used when they compress 4:1 or better
  auto fill_varsum = [&](pgbp::VarsumSet& v, const std::vector<int32_t>& units,
                         const std::vector<int32_t>& off, const std::vector<int32_t>& slots) {
    v.count = (int64_t)units.size();
    v.vs = bd.upload(units);
    std::vector<int32_t> run_off{0};
    std::vector<int4> runs;
    for (size_t u = 0; u + 1 < off.size(); ++u) {
      int32_t k = off[u];
      while (k < off[u + 1]) {
        const int32_t first = slots[k];
        int32_t len = 1, stride = 1;
        if (k + 1 < off[u + 1]) {
          stride = slots[k + 1] - first;
          len = 2;
          while (k + len < off[u + 1] && slots[k + len] == first + len * stride) ++len;
        }
        runs.push_back(make_int4(first, stride, len, 0));
        k += len;
      }
      run_off.push_back((int32_t)runs.size());
    }
    v.use_runs = !slots.empty() && runs.size() * 4 <= slots.size();
    if (v.use_runs) {
      v.run_off = bd.upload(run_off);
      v.runs = bd.upload(runs);
    } else {
      v.off = bd.upload(off);
      v.slots = bd.upload(slots);
    }
  };
  fill_varsum(p.varsum_binary, vb_vs, vb_off, vb_slots);
  fill_varsum(p.varsum_other, vo_vs, vo_off, vo_slots);
  {
    // inline variable sums (cluster path): all-binary graphs of low degree
    bool ok = vo_vs.empty() && 2 * p.num_slots == ns && !vb_vs.empty();
    for (size_t u = 0; ok && u < vb_vs.size(); ++u) ok = vb_off[u + 1] - vb_off[u] <= 16;
    if (ok) {
      std::vector<int32_t> unit_of(nvs, -1);
      for (size_t u = 0; u < vb_vs.size(); ++u) unit_of[vb_vs[u]] = (int32_t)u;
      p.vb_unit_of_vs = bd.upload(unit_of);
      p.inline_vsum = true;
    }
  }
  if (bd.err) return bail(bd.err);
  // the non-binary variables by variable, when every one of their edges has all K states
  if (!vo_vs.empty()) {
    std::map<int32_t, std::pair<int32_t, std::vector<int32_t>>> vars;  // vs0 -> (K, edge slots)
    bool ok = true;
    for (int64_t e = 0; e < ne && ok; ++e) {
      const int32_t k = edge_start[e + 1] - edge_start[e];
      if (k <= 2) continue;
      const int32_t v0 = vs[edge_start[e]];
      for (int32_t j = 1; j < k && ok; ++j) ok = vs[edge_start[e] + j] == v0 + j;
      auto& var = vars[v0];
      if (var.first == 0) var.first = k;
      ok = ok && var.first == k;
      var.second.push_back(edge_slot[e]);
    }
    int64_t units = 0;
    for (auto& kv : vars) units += kv.second.first;
    std::map<int32_t, std::vector<int32_t>> by_k;  // K -> variables (vs0)
    for (auto& kv : vars) by_k[kv.second.first].push_back(kv.first);
    ok = ok && units == (int64_t)vo_vs.size() && by_k.size() <= 16;
    if (ok) {
      std::vector<int4> grp;
      std::vector<int32_t> vs0, eoff{0}, eslot;
      int64_t first_unit = 0;
      for (auto& kv : by_k) {
        grp.push_back(make_int4(kv.first, (int32_t)first_unit, (int32_t)vs0.size(), 0));
        for (int32_t v : kv.second) {
          vs0.push_back(v);
          const auto& slots = vars[v].second;
          eslot.insert(eslot.end(), slots.begin(), slots.end());
          eoff.push_back((int32_t)eslot.size());
          first_unit += kv.first;
        }
      }
      grp.push_back(make_int4(0, (int32_t)first_unit, (int32_t)vs0.size(), 0));
      pgbp::VarsumSet& vo = p.varsum_other;
      vo.byvar_groups = (int)by_k.size();
      vo.byvar_units = first_unit;
      vo.byvar_grp = bd.upload(grp);
      vo.byvar_vs0 = bd.upload(vs0);
      vo.byvar_eoff = bd.upload(eoff);
      vo.byvar_eslot = bd.upload(eslot);
      if (bd.err) return bail(bd.err);
    }
  }
  auto edge_rec = [&](int64_t es0) {  // (first edge state, first slot, first var state, 0)
    const int32_t e = ei[es0];
    return make_int4((int32_t)es0, edge_slot[e], vs[es0], 0);
  };

  // --- Enum factors
  {
    const int64_t e0 = d->msgs_range[0][0], e1 = d->msgs_range[0][1];
    const int64_t pot0 = d->potentials_range[0][0];
    const int64_t nrows = d->enum_num_rows, ncfg = d->enum_num_val_configs;
    const int32_t* ci = d->enum_factor_configs_indices;
    const int32_t* cf = d->enum_factor_configs_edge_states;
    // Implicit rows: every Enum factor is unary (configs = its states) or pairwise (all K1 x K2
    // configs in row-major order, the PairwiseFactorGroup layout), with its configs following the
    // previous factor's; the rows PGMax would list are not passed.
    const bool implicit = (d->flags & PGBP_FLAG_ENUM_IMPLICIT_ROWS) != 0;
    if (implicit && nrows != 0)
      return bail(fail(PGBP_ERR_INVALID_ARGUMENT, "implicit enum rows: enum_num_rows must be 0"));
    if (nrows > 0 && (!ci || !cf)) return bail(fail(PGBP_ERR_INVALID_ARGUMENT, "missing enum rows"));
    const int32_t* alias = d->enum_factor_potential_offsets;
    const int64_t npot_enum = d->potentials_range[0][1] - pot0;
    if (!alias && npot_enum < ncfg)
      return bail(fail(PGBP_ERR_INVALID_WIRING, "enum potentials range shorter than num_val_configs"));
    // Enum factors are the first factors; enumerate them by edge-state range
    std::vector<int64_t> facs;
    if (e1 > e0) {
      for (int64_t f = factor_of(e0); f <= factor_of(e1 - 1); ++f) facs.push_back(f);
    }
    // rows grouped per factor
    std::vector<int64_t> row_begin(facs.size() + 1, nrows);
    if (!implicit) {
      int64_t r = 0;
      for (size_t k = 0; k < facs.size(); ++k) {
        row_begin[k] = r;
        while (r < nrows) {
          if (!in_range(cf[r], 0, e1 - e0) || !in_range(ci[r], 0, ncfg))
            return bail(fail(PGBP_ERR_INVALID_WIRING, "enum row %lld out of range", (long long)r));
          if (factor_of(e0 + cf[r]) != facs[k]) break;
          ++r;
        }
      }
      row_begin[facs.size()] = r;
      if (r != nrows)
        return bail(fail(PGBP_ERR_UNSUPPORTED, "enum config rows are not grouped by factor"));
    }
    if (alias && d->enum_num_factors != (int64_t)facs.size())
      return bail(fail(PGBP_ERR_INVALID_WIRING, "enum_num_factors is %lld, the wiring has %lld",
                       (long long)d->enum_num_factors, (long long)facs.size()));
    p.shared_potentials = alias != nullptr;
    int64_t implicit_cfg = 0;
    std::map<std::pair<int, int>, std::pair<std::vector<int4>, std::vector<int32_t>>> buckets;
    std::map<std::pair<int, int>, std::vector<int32_t>> bucket_fac;  // factor index per record
    std::vector<int32_t> g_fac;
    std::vector<int32_t> g_es, g_nes, g_eoff{0}, g_esz, g_eslot, g_evs, g_rb, g_ncfg, g_nv, g_cfg,
        g_les;
    std::vector<char> g_u2;     // per generic factor: unary on a binary variable, configs (0), (1)
    std::vector<int4> u2_rec;
    int max_es = 0;
    std::vector<int32_t> esz, estart;  // per factor, reused
    for (size_t k = 0; k < facs.size(); ++k) {
      const int64_t f = facs[k];
      const int64_t fb = fac_es_begin[f], fe = fac_es_end[f];
      // edges of the factor: a factor starts at an edge boundary and holds whole edges
      esz.clear();
      for (int64_t i = fb; i < fe; i = edge_start[ei[i] + 1])
        esz.push_back(edge_start[ei[i] + 1] - (int32_t)i);
      const int nv = (int)esz.size();
      estart.assign(nv + 1, 0);
      for (int j = 0; j < nv; ++j) estart[j + 1] = estart[j] + esz[j];
      int64_t nc = 0, cfg0 = 0;
      std::vector<int32_t> les;
      // implied rows of a pairwise factor of at most 64 x 64 states are the dense row-major
      // table: such a factor goes to its bucket without its rows being spelled out
      const bool implicit_dense = implicit && nv == 2 && esz[0] <= 64 && esz[1] <= 64;
      if (implicit) {
        if (nv > 2)
          return bail(fail(PGBP_ERR_UNSUPPORTED, "implicit enum rows need unary or pairwise factors"));
        nc = nv == 1 ? esz[0] : (int64_t)esz[0] * esz[1];
        cfg0 = implicit_cfg;
        implicit_cfg += nc;
        if (!implicit_dense) {
          les.resize((size_t)(nc * nv));
          for (int64_t c = 0; c < nc; ++c) {
            if (nv == 1) {
              les[(size_t)c] = (int32_t)c;
            } else {
              les[(size_t)(2 * c)] = (int32_t)(c / esz[1]);
              les[(size_t)(2 * c + 1)] = (int32_t)(esz[0] + c % esz[1]);
            }
          }
        }
      }
      const int64_t r0 = implicit ? 0 : row_begin[k], r1 = implicit ? 0 : row_begin[k + 1];
      if (!implicit && (r1 - r0) % nv != 0)
        return bail(fail(PGBP_ERR_UNSUPPORTED, "enum factor rows not a multiple of its arity"));
      if (!implicit) {
        nc = (r1 - r0) / nv;
        cfg0 = nc > 0 ? ci[r0] : 0;
        les.resize((size_t)(r1 - r0));
      }
      // rows of config c are (var 0 .. var nv-1) with the state's edge state inside var i's edge
      for (int64_t c = 0; !implicit && c < nc; ++c) {
        for (int i = 0; i < nv; ++i) {
          const int64_t r = r0 + c * nv + i;
          const int64_t le = (e0 + cf[r]) - fb;
          if (ci[r] != cfg0 + c)
            return bail(fail(PGBP_ERR_UNSUPPORTED, "enum config indices not contiguous per factor"));
          if (le < estart[i] || le >= estart[i + 1])
            return bail(fail(PGBP_ERR_UNSUPPORTED, "enum row does not follow variable order"));
          les[(size_t)(c * nv + i)] = (int32_t)le;
        }
      }
      // first potential of the factor's table: its own configs', or the shared table's
      int64_t pot_first = pot0 + cfg0;
      if (alias) {
        if (alias[k] < 0 || alias[k] + nc > npot_enum)
          return bail(fail(PGBP_ERR_INVALID_WIRING, "potential offset of enum factor %lld out of range",
                           (long long)k));
        pot_first = pot0 + alias[k];
      }
      bool dense = nv == 2 && nc == (int64_t)esz[0] * esz[1] && esz[0] <= 64 && esz[1] <= 64;
      for (int64_t c = 0; dense && !implicit_dense && c < nc; ++c) {
        if (les[(size_t)(2 * c)] != c / esz[1] || les[(size_t)(2 * c + 1)] != esz[0] + c % esz[1])
          dense = false;
      }
      if (dense) {
        auto& bk = buckets[{esz[0], esz[1]}];
        const int4 r0 = edge_rec(fb);
        bk.first.push_back(make_int4(r0.x, r0.y, r0.z, vs[fb + esz[0]]));
        bk.second.push_back((int32_t)pot_first);
        bucket_fac[{esz[0], esz[1]}].push_back((int32_t)factor_of(fb));
      } else {
        g_fac.push_back((int32_t)factor_of(fb));
        g_es.push_back((int32_t)fb);
        g_nes.push_back((int32_t)(fe - fb));
        max_es = std::max<int>(max_es, (int)(fe - fb));
        for (int j = 0; j < nv; ++j) {
          const int4 r = edge_rec(fb + estart[j]);
          g_esz.push_back(esz[j]);
          g_eslot.push_back(r.y);
          g_evs.push_back(r.z);
        }
        g_eoff.push_back((int32_t)g_esz.size());
        g_rb.push_back((int32_t)g_les.size());
        g_les.insert(g_les.end(), les.begin(), les.end());
        g_ncfg.push_back((int32_t)nc);
        g_nv.push_back(nv);
        g_cfg.push_back((int32_t)pot_first);
        const bool u2 = nv == 1 && esz[0] == 2 && nc == 2 && les.size() == 2 && les[0] == 0 &&
                        les[1] == 1;
        g_u2.push_back(u2 ? 1 : 0);
        if (u2) {
          const int4 r = edge_rec(fb);
          u2_rec.push_back(make_int4(r.x, r.y, r.z, (int32_t)pot_first));
        }
      }
    }
    if (max_es > 512)
      return bail(fail(PGBP_ERR_UNSUPPORTED, "an EnumFactor has %d edge states (max 512)", max_es));
    if (implicit && implicit_cfg != ncfg)
      return bail(fail(PGBP_ERR_INVALID_WIRING, "implicit enum rows give %lld configs, num_val_configs is %lld",
                       (long long)implicit_cfg, (long long)ncfg));
    p.num_enum_factors = (int64_t)facs.size();
    for (auto& kv : buckets) {
      pgbp::PairwiseBucket q;
      q.n1 = kv.first.first;
      q.n2 = kv.first.second;
      q.count = (int64_t)kv.second.first.size();
      if (alias && q.n1 == q.n2 && (q.n1 == 16 || q.n1 == 32 || q.n1 == 64)) {
        // group the factors by table (stable: factor order inside a group)
        auto& recs = kv.second.first;
        auto& cfg = kv.second.second;
        std::vector<size_t> order(recs.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(),
                         [&](size_t a, size_t b) { return cfg[a] < cfg[b]; });
        auto& fac = bucket_fac[kv.first];
        std::vector<int4> r2(recs.size());
        std::vector<int32_t> c2(cfg.size()), f2(fac.size());
        for (size_t i = 0; i < order.size(); ++i) {
          r2[i] = recs[order[i]];
          c2[i] = cfg[order[i]];
          f2[i] = fac[order[i]];
        }
        recs.swap(r2);
        cfg.swap(c2);
        fac.swap(f2);
        std::vector<int32_t> gf, gc, gt;
        for (size_t i = 0; i < cfg.size(); ++i) {
          if (i == 0 || cfg[i] != cfg[i - 1]) {
            gf.push_back((int32_t)i);
            gc.push_back(0);
            gt.push_back(cfg[i]);
          }
          gc.back()++;
        }
        q.n_groups = (int)gf.size();
        q.grp_first = bd.upload(gf);
        q.grp_count = bd.upload(gc);
        q.grp_table = bd.upload(gt);
        q.grp_count_host.assign(gc.begin(), gc.end());
        q.rows16 = true;
        for (const int4& r : recs) q.rows16 = q.rows16 && (r.y & 3) == 0;
        q.gemm_floats = (int64_t)q.n_groups * (pgbp::expgemm_table_floats(q.n1) +
                                                pgbp::expgemm_tc_table_floats(q.n1));
      }
      q.rec = bd.upload(kv.second.first);
      q.cfg_begin = bd.upload(kv.second.second);
      q.fac = bd.upload(bucket_fac[kv.first]);
      p.num_enum_pairwise += q.count;
      p.pairwise.push_back(q);
    }
    // A generic set from the generic factors that `keep` selects, in their order, with each
    // factor's configs listed by edge state for the staged kernel: local edge state e of factor
    // f is held by configs inv_cfg[inv_off[inv_begin[f] + e]] .. inv_cfg[inv_off[inv_begin[f] +
    // e + 1] - 1], local config indices in increasing order (the order of the reference's scatter
    // of config sums onto edge states, enum.py:451-475).
    auto build_generic = [&](pgbp::EnumGeneric& out, auto&& keep) {
      std::vector<int32_t> o_es, o_nes, o_eoff{0}, o_esz, o_eslot, o_evs, o_rb, o_ncfg, o_nv,
          o_cfg, o_les, o_fac, o_ib, o_io, o_ic;
      std::vector<int32_t> cnt;
      for (size_t i = 0; i < g_es.size(); ++i) {
        if (!keep(i)) continue;
        const int nes = g_nes[i], nv = g_nv[i];
        const int64_t nc = g_ncfg[i];
        o_es.push_back(g_es[i]);
        o_nes.push_back(nes);
        out.max_es = std::max(out.max_es, nes);
        out.max_nv = std::max(out.max_nv, nv);
        out.max_cfg = std::max<int64_t>(out.max_cfg, nc);
        for (int32_t j = g_eoff[i]; j < g_eoff[i + 1]; ++j) {
          o_esz.push_back(g_esz[j]);
          o_eslot.push_back(g_eslot[j]);
          o_evs.push_back(g_evs[j]);
        }
        o_eoff.push_back((int32_t)o_esz.size());
        o_rb.push_back((int32_t)o_les.size());
        const int32_t* les = g_les.data() + g_rb[i];
        o_les.insert(o_les.end(), les, les + nc * nv);
        o_ncfg.push_back((int32_t)nc);
        o_nv.push_back(nv);
        o_cfg.push_back(g_cfg[i]);
        o_fac.push_back(g_fac[i]);
        // inverse lists: counting sort of the (config, edge state) pairs by edge state
        cnt.assign((size_t)nes + 1, 0);
        for (int64_t r = 0; r < nc * nv; ++r) cnt[(size_t)les[r] + 1]++;
        for (int e = 0; e < nes; ++e) cnt[(size_t)e + 1] += cnt[(size_t)e];
        const int32_t base = (int32_t)o_ic.size();
        o_ib.push_back((int32_t)o_io.size());
        for (int e = 0; e <= nes; ++e) o_io.push_back(base + cnt[(size_t)e]);
        o_ic.resize((size_t)base + (size_t)(nc * nv));
        for (int64_t c = 0; c < nc; ++c)
          for (int v = 0; v < nv; ++v) o_ic[(size_t)base + (size_t)cnt[(size_t)les[c * nv + v]]++] = (int32_t)c;
      }
      out.count = (int64_t)o_es.size();
      if (out.count == 0) return;
      out.es_begin = bd.upload(o_es);
      out.n_es = bd.upload(o_nes);
      out.edge_off = bd.upload(o_eoff);
      out.edge_size = bd.upload(o_esz);
      out.edge_slot = bd.upload(o_eslot);
      out.edge_vs = bd.upload(o_evs);
      out.row_begin = bd.upload(o_rb);
      out.n_cfg = bd.upload(o_ncfg);
      out.n_vars = bd.upload(o_nv);
      out.cfg_begin = bd.upload(o_cfg);
      out.row_les = bd.upload(o_les);
      out.fac = bd.upload(o_fac);
      out.inv_begin = bd.upload(o_ib);
      out.inv_off = bd.upload(o_io);
      out.inv_cfg = bd.upload(o_ic);
    };
    build_generic(p.enum_generic, [](size_t) { return true; });
    if (!u2_rec.empty()) {
      p.unary2.count = (int64_t)u2_rec.size();
      p.unary2.rec = bd.upload(u2_rec);
      // the other generic factors, in their order
      build_generic(p.enum_generic_rest, [&](size_t i) { return !g_u2[i]; });
    }
    if (bd.err) return bail(bd.err);
  }

  // --- OR / AND factors
  for (int w = 0; w < 2; ++w) {
    const int t = 1 + w;
    const int off = w == 0 ? 1 : -1;
    const int64_t m0 = d->msgs_range[t][0], m1 = d->msgs_range[t][1];
    const int64_t P = d->logical_num_parents[w], F = d->logical_num_factors[w];
    const int32_t* pfi = d->logical_parents_factor_indices[w];
    const int32_t* pmi = d->logical_parents_msg_indices[w];
    const int32_t* ch = d->logical_children_edge_states[w];
    if (F == 0 && P == 0) continue;
    if (F <= 0 || P <= 0 || !pfi || !pmi || !ch)
      return bail(fail(PGBP_ERR_INVALID_WIRING, "logical factors without parents or children"));
    std::vector<int32_t> pb(F + 1, 0);
    std::vector<int4> pes(P), ces(F);
    int64_t cur = -1;
    for (int64_t i = 0; i < P; ++i) {
      if (!in_range(pfi[i], 0, F))
        return bail(fail(PGBP_ERR_INVALID_WIRING, "parent factor index out of range"));
      if (pfi[i] < cur || (pfi[i] > cur + 1 && i > 0) || (i == 0 && pfi[0] != 0))
        return bail(fail(PGBP_ERR_UNSUPPORTED, "parents must be grouped by factor in order"));
      if (pfi[i] != cur) {
        cur = pfi[i];
        pb[cur] = (int32_t)i;
      }
      const int64_t e = m0 + pmi[i];
      if (!in_range(e, m0, m1) || !in_range(e + off, m0, m1) || ei[e] != ei[e + off] ||
          edge_start[ei[e] + 1] - edge_start[ei[e]] != 2)
        return bail(fail(PGBP_ERR_INVALID_WIRING, "logical parent message index out of range"));
      pes[i] = edge_rec(std::min<int64_t>(e, e + off));
    }
    if (cur != F - 1) return bail(fail(PGBP_ERR_INVALID_WIRING, "a logical factor has no parent"));
    pb[F] = (int32_t)P;
    for (int64_t f = 0; f < F; ++f) {
      const int64_t e = m0 + ch[f];
      if (!in_range(e, m0, m1) || !in_range(e + off, m0, m1) || ei[e] != ei[e + off] ||
          edge_start[ei[e] + 1] - edge_start[ei[e]] != 2)
        return bail(fail(PGBP_ERR_INVALID_WIRING, "logical child edge state out of range"));
      ces[f] = edge_rec(std::min<int64_t>(e, e + off));
    }
    pgbp::LogicalSet& g = p.logical[w];
    g.count = F;
    g.num_parents = P;
    g.off = off;
    g.par_begin = bd.upload(pb);
    g.par = bd.upload(pes);
    g.child = bd.upload(ces);
    {
      std::vector<int32_t> fac(F);
      for (int64_t f = 0; f < F; ++f) fac[f] = (int32_t)factor_of(m0 + ch[f]);
      g.fac = bd.upload(fac);
    }
    if (bd.err) return bail(bd.err);
  }

  // --- Pool factors
  {
    const int64_t m0 = d->msgs_range[3][0], m1 = d->msgs_range[3][1];
    const int64_t P = d->pool_num_choices, F = d->pool_num_factors;
    const int32_t* cfi = d->pool_choices_factor_indices;
    const int32_t* cmi = d->pool_choices_msg_indices;
    const int32_t* ind = d->pool_indicators_edge_states;
    if (F > 0 || P > 0) {
      if (F <= 0 || P <= 0 || !cfi || !cmi || !ind)
        return bail(fail(PGBP_ERR_INVALID_WIRING, "pool factors without choices or indicators"));
      std::vector<int32_t> cb(F + 1, 0);
      std::vector<int4> ces(P), ies(F);
      int64_t cur = -1;
      for (int64_t i = 0; i < P; ++i) {
        if (!in_range(cfi[i], 0, F))
          return bail(fail(PGBP_ERR_INVALID_WIRING, "pool factor index out of range"));
        if (cfi[i] < cur || (cfi[i] > cur + 1 && i > 0) || (i == 0 && cfi[0] != 0))
          return bail(fail(PGBP_ERR_UNSUPPORTED, "pool choices must be grouped by factor in order"));
        if (cfi[i] != cur) {
          cur = cfi[i];
          cb[cur] = (int32_t)i;
        }
        const int64_t e = m0 + cmi[i];
        if (!in_range(e, m0, m1) || !in_range(e + 1, m0, m1) || ei[e] != ei[e + 1] ||
            edge_start[ei[e] + 1] - edge_start[ei[e]] != 2)
          return bail(fail(PGBP_ERR_INVALID_WIRING, "pool choice message index out of range"));
        ces[i] = edge_rec(e);
      }
      if (cur != F - 1) return bail(fail(PGBP_ERR_INVALID_WIRING, "a pool factor has no choice"));
      cb[F] = (int32_t)P;
      for (int64_t f = 0; f < F; ++f) {
        const int64_t e = m0 + ind[f];
        if (!in_range(e, m0, m1) || !in_range(e + 1, m0, m1) || ei[e] != ei[e + 1] ||
            edge_start[ei[e] + 1] - edge_start[ei[e]] != 2)
          return bail(fail(PGBP_ERR_INVALID_WIRING, "pool indicator edge state out of range"));
        ies[f] = edge_rec(e);
      }
      pgbp::PoolSet& g = p.pool;
      g.count = F;
      g.num_choices = P;
      g.ch_begin = bd.upload(cb);
      g.ch = bd.upload(ces);
      g.ind = bd.upload(ies);
      std::vector<int32_t> fac(F);
      for (int64_t f = 0; f < F; ++f) fac[f] = (int32_t)factor_of(m0 + ind[f]);
      g.fac = bd.upload(fac);
      if (bd.err) return bail(bd.err);
    }
  }

  // --- variables (decode / marginals)
  if (d->evidence_to_vars && d->num_variables > 0) {
    const int64_t nv = d->num_variables;
    std::vector<int32_t> voff(nv + 1, 0);
    int64_t expect = 0;
    for (int64_t i = 0; i < nvs; ++i) {
      const int32_t v = d->evidence_to_vars[i];
      if (i == 0 || v != d->evidence_to_vars[i - 1]) {
        if (v != expect)
          return bail(fail(PGBP_ERR_INVALID_WIRING, "evidence_to_vars must enumerate variables"));
        voff[v] = (int32_t)i;
        ++expect;
      }
    }
    if (expect != nv) return bail(fail(PGBP_ERR_INVALID_WIRING, "num_variables mismatch"));
    voff[nv] = (int32_t)nvs;
    p.num_variables = nv;
    p.var_off = bd.upload(voff);
    p.var_of_vs = bd.upload(std::vector<int32_t>(d->evidence_to_vars, d->evidence_to_vars + nvs));
    if (bd.err) return bail(bd.err);
  }
  // inline variable sums only for graphs of Enum factors: the OR / AND / Pool units load each
  // parent's messages several times, which would repeat the sums
  p.inline_vsum = p.inline_vsum && p.logical[0].count == 0 && p.logical[1].count == 0 &&
                  p.pool.count == 0;
  pgbp::energy_plan(p);

  p.flags = d->flags;
  ce = pgbp::prepare_small_graph(p);
  if (ce != cudaSuccess) return bail(cuda_fail(ce, "small-graph path set-up"));
  ce = cudaDeviceSynchronize();
  if (ce != cudaSuccess) return bail(cuda_fail(ce, "plan upload"));
  *out = handle;
  return PGBP_OK;
}

int pgbp_plan_destroy(pgbp_plan* plan) {
  if (!plan) return PGBP_OK;
  pgbp::DeviceGuard guard(plan->p.device);
  free_plan(plan->p);
  delete plan;
  return PGBP_OK;
}

int pgbp_plan_get_info(const pgbp_plan* plan, pgbp_plan_info* info) {
  if (!plan || !info) return fail(PGBP_ERR_INVALID_ARGUMENT, "null argument");
  const pgbp::Plan& p = plan->p;
  info->num_edge_states = p.num_edge_states;
  info->num_var_states = p.num_var_states;
  info->num_edges = p.num_edges;
  info->num_variables = p.num_variables;
  info->num_potentials = p.num_potentials;
  info->num_enum_factors = p.num_enum_factors;
  info->num_enum_pairwise_factors = p.num_enum_pairwise;
  info->num_or_factors = p.logical[0].count;
  info->num_and_factors = p.logical[1].count;
  info->num_pool_factors = p.pool.count;
  info->num_pairwise_buckets = (int64_t)p.pairwise.size();
  info->device_bytes = p.device_bytes;
  info->num_slots = p.num_slots;
  info->small_graph_smem_bytes = p.small_graph_smem;
  return PGBP_OK;
}

size_t pgbp_workspace_size(const pgbp_plan* plan, int64_t batch, int64_t num_iters) {
  if (!plan) return 0;
  // sized for batched evidence and potentials, which covers every stride choice
  return pgbp::workspace_bytes(plan->p, batch, num_iters, true, true);
}

}  // extern "C"

namespace {

// pgbp_run and pgbp_run_checkpointed: argument checks, then the engine.
int run_checked(const pgbp_plan* plan, void* stream, int64_t batch, const float* log_potentials,
                int64_t lp_stride, const float* evidence, int64_t ev_stride, const float* msgs_in,
                int64_t msgs_stride, float* msgs_out, float* deltas, int64_t num_iters,
                double damping, double temperature, void* workspace, size_t workspace_bytes,
                int64_t checkpoint_every, float* checkpoints,
                const pgbp::ToleranceRun* tol_run = nullptr,
                const pgbp::Perturbation* pert = nullptr) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  if (batch <= 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "batch must be positive");
  if (lp_stride < 0 || ev_stride < 0 || msgs_stride < 0)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "negative stride");
  if (lp_stride != 0 && lp_stride < p.num_potentials)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "log_potentials stride %lld < %lld", (long long)lp_stride,
                (long long)p.num_potentials);
  if (ev_stride != 0 && ev_stride < p.num_var_states)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "evidence stride too small");
  if (msgs_stride != 0 && msgs_stride < p.num_edge_states)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "messages stride too small");
  if ((p.num_potentials > 0 && !log_potentials) ||
      (p.num_var_states > 0 && !evidence && pert == nullptr) ||
      (p.num_edge_states > 0 && (!msgs_in || !msgs_out)))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "null data pointer");
  if (!(damping == damping) || !(temperature == temperature) || temperature < 0.0)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "damping and temperature must be numbers, temperature >= 0");
  const size_t need = pgbp::workspace_bytes(p, batch, num_iters, ev_stride != 0 || pert != nullptr,
                                            lp_stride != 0);
  if (!workspace || workspace_bytes < need)
    return fail(PGBP_ERR_WORKSPACE, "workspace of %zu bytes needed, got %zu", need, workspace_bytes);
  if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
    return fail(PGBP_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  e = pgbp::run_bp(p, static_cast<cudaStream_t>(stream), batch, log_potentials, lp_stride, evidence,
                   ev_stride, msgs_in, msgs_stride, msgs_out, deltas, num_iters, damping, temperature,
                   workspace, workspace_bytes, checkpoint_every, checkpoints, tol_run, pert);
  if (e == cudaErrorStreamCaptureUnsupported && tol_run)
    return fail(PGBP_ERR_UNSUPPORTED, "pgbp_run_to_tolerance reads a count on the host: "
                "it cannot run inside a stream capture");
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_run launch");
  return PGBP_OK;
}

}  // namespace

extern "C" {

int pgbp_run(const pgbp_plan* plan, void* stream, int64_t batch, const float* log_potentials,
             int64_t lp_stride, const float* evidence, int64_t ev_stride, const float* msgs_in,
             int64_t msgs_stride, float* msgs_out, float* deltas, int64_t num_iters, double damping,
             double temperature, void* workspace, size_t workspace_bytes) {
  return run_checked(plan, stream, batch, log_potentials, lp_stride, evidence, ev_stride, msgs_in,
                     msgs_stride, msgs_out, deltas, num_iters, damping, temperature, workspace,
                     workspace_bytes, 0, nullptr);
}

int pgbp_run_perturbed(const pgbp_plan* plan, void* stream, int64_t batch,
                       const float* log_potentials, int64_t lp_stride, const float* evidence_base,
                       int64_t ev_stride, uint64_t seed, double noise_scale, const float* msgs_in,
                       int64_t msgs_stride, float* msgs_out, float* deltas, float* evidence_out,
                       int64_t num_iters, double damping, double temperature, void* workspace,
                       size_t workspace_bytes) {
  if (!(noise_scale == noise_scale) || noise_scale - noise_scale != 0.0)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "noise_scale must be finite");
  if (!evidence_base && ev_stride != 0)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "a null evidence base takes ev_stride 0");
  const pgbp::Perturbation pert{seed, (float)noise_scale, evidence_out};
  return run_checked(plan, stream, batch, log_potentials, lp_stride, evidence_base, ev_stride,
                     msgs_in, msgs_stride, msgs_out, deltas, num_iters, damping, temperature,
                     workspace, workspace_bytes, 0, nullptr, nullptr, &pert);
}

int pgbp_gumbel(void* stream, uint64_t seed, int64_t count, float* out) {
  if (count < 0 || (count > 0 && !out)) return fail(PGBP_ERR_INVALID_ARGUMENT, "bad count or null");
  int dev = 0, sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = pgbp::gumbel(static_cast<cudaStream_t>(stream), seed, count, out, sm);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_gumbel");
  return PGBP_OK;
}

int pgbp_run_checkpointed(const pgbp_plan* plan, void* stream, int64_t batch,
                          const float* log_potentials, int64_t lp_stride, const float* evidence,
                          int64_t ev_stride, const float* msgs_in, int64_t msgs_stride,
                          float* msgs_out, float* deltas, int64_t num_iters,
                          int64_t checkpoint_every, double damping, double temperature,
                          float* checkpoints, void* workspace, size_t workspace_bytes) {
  if (checkpoint_every <= 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "checkpoint_every must be >= 1");
  if (plan && plan->p.num_edge_states > 0 && !checkpoints)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "null checkpoints");
  return run_checked(plan, stream, batch, log_potentials, lp_stride, evidence, ev_stride, msgs_in,
                     msgs_stride, msgs_out, deltas, num_iters, damping, temperature, workspace,
                     workspace_bytes, checkpoint_every, checkpoints);
}

int pgbp_run_to_tolerance(const pgbp_plan* plan, void* stream, int64_t batch,
                          const float* log_potentials, int64_t lp_stride, const float* evidence,
                          int64_t ev_stride, const float* msgs_in, int64_t msgs_stride,
                          float* msgs_out, double tolerance, int64_t max_iters,
                          int64_t check_every, double damping, double temperature,
                          int32_t* first_below, int64_t* iters_run, void* workspace,
                          size_t workspace_bytes) {
  if (!(tolerance > 0.0) || max_iters < 1 || check_every < 1)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "tolerance > 0, max_iters >= 1, check_every >= 1");
  if (!first_below || !iters_run) return fail(PGBP_ERR_INVALID_ARGUMENT, "null output pointer");
  const pgbp::ToleranceRun tr{tolerance, max_iters, first_below, iters_run};
  return run_checked(plan, stream, batch, log_potentials, lp_stride, evidence, ev_stride, msgs_in,
                     msgs_stride, msgs_out, nullptr, check_every, damping, temperature, workspace,
                     workspace_bytes, 0, nullptr, &tr);
}

size_t pgbp_vjp_workspace_size(const pgbp_plan* plan, int64_t batch, int64_t num_iters,
                               int64_t checkpoint_every) {
  if (!plan || batch <= 0 || checkpoint_every <= 0) return 0;
  size_t n = 0;
  for (int ev_shared = 0; ev_shared < 2; ++ev_shared)
    for (int lp_shared = 0; lp_shared < 2; ++lp_shared)
      n = std::max(n, pgbp::vjp_workspace_bytes(plan->p, batch, num_iters, checkpoint_every,
                                                ev_shared != 0, lp_shared != 0));
  return n;
}

int pgbp_run_vjp(const pgbp_plan* plan, void* stream, int64_t batch, const float* log_potentials,
                 int64_t lp_stride, const float* evidence, int64_t ev_stride,
                 const float* checkpoints, int64_t num_iters, int64_t checkpoint_every,
                 double damping, double temperature, const float* g_msgs_out,
                 float* g_log_potentials, float* g_evidence, float* g_msgs_in, void* workspace,
                 size_t workspace_bytes) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  const char* why = pgbp::adjoint_unsupported(p);
  if (why[0]) return fail(PGBP_ERR_UNSUPPORTED, "%s", why);
  if (batch <= 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "batch must be positive");
  if (checkpoint_every <= 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "checkpoint_every must be >= 1");
  if (lp_stride < 0 || ev_stride < 0 || (lp_stride != 0 && lp_stride < p.num_potentials) ||
      (ev_stride != 0 && ev_stride < p.num_var_states))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad stride");
  if ((p.num_potentials > 0 && (!log_potentials || !g_log_potentials)) ||
      (p.num_var_states > 0 && (!evidence || !g_evidence)) ||
      (p.num_edge_states > 0 && (!checkpoints || !g_msgs_out)))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "null data pointer");
  if (!(damping == damping) || !(temperature > 0.0))
    return fail(PGBP_ERR_UNSUPPORTED,
                "the adjoint needs temperature > 0 (max-product messages are piecewise linear)");
  const size_t need = pgbp::vjp_workspace_bytes(p, batch, num_iters, checkpoint_every,
                                                ev_stride == 0, lp_stride == 0);
  if (!workspace || workspace_bytes < need)
    return fail(PGBP_ERR_WORKSPACE, "workspace of %zu bytes needed, got %zu", need, workspace_bytes);
  if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
    return fail(PGBP_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  e = pgbp::run_vjp(p, static_cast<cudaStream_t>(stream), batch, log_potentials, lp_stride,
                    evidence, ev_stride, checkpoints, num_iters, checkpoint_every, damping,
                    temperature, g_msgs_out, g_log_potentials, g_evidence, g_msgs_in, workspace,
                    workspace_bytes);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_run_vjp launch");
  return PGBP_OK;
}

int pgbp_beliefs_vjp(const pgbp_plan* plan, void* stream, int64_t batch, const float* g_beliefs,
                     int64_t gb_stride, float* g_msgs) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  if (batch <= 0 || gb_stride < 0 || (batch > 1 && gb_stride != 0 && gb_stride < p.num_var_states))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad batch or stride");
  if (p.num_edge_states > 0 && (!g_beliefs || !g_msgs))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "null data pointer");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  e = pgbp::beliefs_vjp(p, static_cast<cudaStream_t>(stream), batch, g_beliefs, gb_stride, g_msgs);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_beliefs_vjp launch");
  return PGBP_OK;
}

int pgbp_factor_update(const pgbp_plan* plan, void* stream, int type, int64_t batch,
                       const float* vtof, int64_t vtof_stride, const float* log_potentials,
                       int64_t lp_stride, double temperature, int normalize, float* out,
                       int64_t out_stride) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  if (type < 0 || type > 3) return fail(PGBP_ERR_INVALID_ARGUMENT, "factor type %d", type);
  if (batch <= 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "batch must be positive");
  const int64_t n = p.msgs_range[type][1] - p.msgs_range[type][0];
  const int64_t np = p.potentials_range[type][1] - p.potentials_range[type][0];
  if (n == 0) return PGBP_OK;
  if (!vtof || !out) return fail(PGBP_ERR_INVALID_ARGUMENT, "null data pointer");
  if (type == PGBP_ENUM && np > 0 && !log_potentials)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "null log_potentials");
  if ((batch > 1 && (vtof_stride < n || out_stride < n)) || (lp_stride != 0 && lp_stride < np) ||
      lp_stride < 0)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad stride");
  if (!(temperature == temperature) || temperature < 0.0)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "temperature must be >= 0");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // every output slot not written by a factor (the "other" states when normalizing) must be zero
  for (int64_t b = 0; b < batch; ++b) {
    e = cudaMemsetAsync(out + b * out_stride, 0, sizeof(float) * (size_t)n, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  }
  e = pgbp::factor_update(p, s, type, batch, vtof, vtof_stride, log_potentials, lp_stride,
                          temperature, normalize, out, out_stride);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_factor_update launch");
  return PGBP_OK;
}

int pgbp_beliefs(const pgbp_plan* plan, void* stream, int64_t batch, const float* evidence,
                 int64_t ev_stride, const float* msgs, int64_t msgs_stride, float* beliefs) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  if (batch <= 0 || ev_stride < 0 || msgs_stride < 0)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad batch or stride");
  if (p.num_var_states > 0 && (!evidence || !beliefs)) return fail(PGBP_ERR_INVALID_ARGUMENT, "null");
  if (p.num_edge_states > 0 && !msgs) return fail(PGBP_ERR_INVALID_ARGUMENT, "null msgs");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  e = pgbp::beliefs(p, static_cast<cudaStream_t>(stream), batch, evidence, ev_stride, msgs,
                    msgs_stride, beliefs);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_beliefs launch");
  return PGBP_OK;
}

int pgbp_decode(const pgbp_plan* plan, void* stream, int64_t batch, const float* beliefs,
                int64_t beliefs_stride, int32_t* map) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  if (!p.var_off) return fail(PGBP_ERR_INVALID_ARGUMENT, "plan has no evidence_to_vars");
  if (batch <= 0 || beliefs_stride < 0 || !beliefs || !map)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad argument");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  e = pgbp::decode(p, static_cast<cudaStream_t>(stream), batch, beliefs, beliefs_stride, map);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_decode launch");
  return PGBP_OK;
}

namespace {

// Every (batch, temperature == 0) key the plan has a path or site decision for.
std::vector<std::pair<int64_t, bool>> tuning_keys(const pgbp::Plan& p) {
  std::vector<std::pair<int64_t, bool>> keys;
  for (const auto& kv : p.tuned_path) keys.push_back(kv.first);
  for (const auto& kv : p.tuned_sites)
    if (!p.tuned_path.count(kv.first)) keys.push_back(kv.first);
  std::sort(keys.begin(), keys.end());
  return keys;
}

}  // namespace

int64_t pgbp_plan_tuning_count(const pgbp_plan* plan) {
  if (!plan) return 0;
  std::lock_guard<std::mutex> lock(plan->p.tune_mu);
  return (int64_t)tuning_keys(plan->p).size();
}

int pgbp_plan_tuning_get(const pgbp_plan* plan, pgbp_tuning_entry* entries, int64_t max_entries) {
  if (!plan || (max_entries > 0 && !entries)) return fail(PGBP_ERR_INVALID_ARGUMENT, "null argument");
  const pgbp::Plan& p = plan->p;
  std::lock_guard<std::mutex> lock(p.tune_mu);
  const auto keys = tuning_keys(p);
  for (int64_t i = 0; i < (int64_t)keys.size() && i < max_entries; ++i) {
    pgbp_tuning_entry& e = entries[i];
    memset(&e, 0, sizeof(e));
    e.batch = keys[(size_t)i].first;
    e.temperature0 = keys[(size_t)i].second ? 1 : 0;
    auto pt = p.tuned_path.find(keys[(size_t)i]);
    e.path = pt != p.tuned_path.end() ? pt->second : -1;
    auto st = p.tuned_sites.find(keys[(size_t)i]);
    if (st != p.tuned_sites.end() && st->second.size() <= PGBP_TUNE_MAX_SITES) {
      e.num_sites = (int32_t)st->second.size();
      for (size_t k = 0; k < st->second.size(); ++k) e.site[k] = st->second[k];
    }
  }
  return PGBP_OK;
}

int pgbp_plan_tuning_set(const pgbp_plan* plan, const pgbp_tuning_entry* entries,
                         int64_t num_entries) {
  if (!plan || (num_entries > 0 && !entries)) return fail(PGBP_ERR_INVALID_ARGUMENT, "null argument");
  const pgbp::Plan& p = plan->p;
  const int sites = pgbp::num_tune_sites(p);
  for (int64_t i = 0; i < num_entries; ++i) {
    const pgbp_tuning_entry& e = entries[i];
    if (e.batch <= 0 || e.path < -1 || e.path > 2 || (e.num_sites != 0 && e.num_sites != sites))
      return fail(PGBP_ERR_INVALID_ARGUMENT, "tuning entry %lld does not fit this plan", (long long)i);
    for (int k = 0; k < e.num_sites; ++k)
      if (e.site[k] < -1 || e.site[k] > (k == 0 ? 2 : 1))
        return fail(PGBP_ERR_INVALID_ARGUMENT, "tuning entry %lld: variant out of range", (long long)i);
    if ((e.path == 1 && p.small_graph_smem == 0) || (e.path == 2 && p.cluster_size == 0))
      return fail(PGBP_ERR_INVALID_ARGUMENT, "tuning entry %lld: path not available", (long long)i);
  }
  std::lock_guard<std::mutex> lock(p.tune_mu);
  for (int64_t i = 0; i < num_entries; ++i) {
    const pgbp_tuning_entry& e = entries[i];
    const std::pair<int64_t, bool> key{e.batch, e.temperature0 != 0};
    if (e.path >= 0) p.tuned_path[key] = e.path;
    if (e.num_sites > 0) p.tuned_sites[key] = std::vector<int>(e.site, e.site + e.num_sites);
  }
  return PGBP_OK;
}

int pgbp_plan_signature(const pgbp_plan* plan, char* buf, size_t len) {
  if (!plan || !buf || len == 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "null argument");
  const pgbp::Plan& p = plan->p;
  // "sites<n>": the layout of the decision table, so that tables of another layout are not found
  std::string sig = "pgbp200|sites" + std::to_string(pgbp::num_tune_sites(p)) + "|sm=" +
                    std::to_string(p.sm_count) + "|es=" +
                    std::to_string(p.num_edge_states) + "|vs=" + std::to_string(p.num_var_states) +
                    "|slots=" + std::to_string(p.num_slots) + "|vb=" +
                    std::to_string(p.varsum_binary.count) + "|vo=" +
                    std::to_string(p.varsum_other.count) + "|pw=";
  for (const pgbp::PairwiseBucket& q : p.pairwise)
    sig += std::to_string(q.n1) + "x" + std::to_string(q.n2) + ":" + std::to_string(q.count) + ":" +
           std::to_string(q.n_groups) + ",";
  sig += "|gen=" + std::to_string(p.enum_generic.count) + "|or=" +
         std::to_string(p.logical[0].count) + ":" + std::to_string(p.logical[0].num_parents) +
         "|and=" + std::to_string(p.logical[1].count) + ":" +
         std::to_string(p.logical[1].num_parents) + "|pool=" + std::to_string(p.pool.count) +
         "|flags=" + std::to_string(p.flags);
  if (sig.size() + 1 > len) return fail(PGBP_ERR_INVALID_ARGUMENT, "buffer of %zu bytes, need %zu", len,
                                        sig.size() + 1);
  memcpy(buf, sig.c_str(), sig.size() + 1);
  return PGBP_OK;
}

size_t pgbp_sdlp_workspace_size(const pgbp_plan* plan, int64_t batch) {
  if (!plan || batch <= 0) return 0;
  return pgbp::sdlp_workspace_bytes(plan->p, batch);
}

// Argument checks shared by the SDLP entry points; the temperature message is the reference's
// (dual_lp.py:270-274).
static int sdlp_check(const pgbp::Plan& p, int64_t batch, const float* lp, int64_t lp_stride,
               const float* ev, int64_t ev_stride, const float* msgs, int64_t ms,
               double temperature, void* workspace, size_t workspace_bytes) {
  if (!p.var_off) return fail(PGBP_ERR_INVALID_ARGUMENT, "plan has no evidence_to_vars");
  if (batch <= 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "batch must be positive");
  if (!(temperature >= 0.0 && temperature <= 1.0))
    return fail(PGBP_ERR_INVALID_ARGUMENT,
                "The log sum-exp temperature of the Dual LP-MAP solver has to be between 0.0 "
                "and 1.0");
  if (lp_stride < 0 || ev_stride < 0 || (lp_stride != 0 && lp_stride < p.num_potentials) ||
      (ev_stride != 0 && ev_stride < p.num_var_states) ||
      ms < (batch > 1 ? p.num_edge_states : 0))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad stride");
  if ((p.num_potentials > 0 && !lp) || (p.num_var_states > 0 && !ev) ||
      (p.num_edge_states > 0 && !msgs))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "null data pointer");
  const size_t need = pgbp::sdlp_workspace_bytes(p, batch);
  if (!workspace || workspace_bytes < need)
    return fail(PGBP_ERR_WORKSPACE, "workspace of %zu bytes needed, got %zu", need, workspace_bytes);
  if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
    return fail(PGBP_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  return PGBP_OK;
}

int pgbp_sdlp_objective(const pgbp_plan* plan, void* stream, int64_t batch,
                        const float* log_potentials, int64_t lp_stride, const float* evidence,
                        int64_t ev_stride, const float* msgs, int64_t msgs_stride,
                        double logsumexp_temp, float* objval, float* grad, float* bp_updates,
                        float* edge_lse, void* workspace, size_t workspace_bytes) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  int rc = sdlp_check(p, batch, log_potentials, lp_stride, evidence, ev_stride, msgs, msgs_stride,
                      logsumexp_temp, workspace, workspace_bytes);
  if (rc) return rc;
  if (!objval) return fail(PGBP_ERR_INVALID_ARGUMENT, "null objval");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  e = pgbp::sdlp_objective(p, static_cast<cudaStream_t>(stream), batch, log_potentials, lp_stride,
                           evidence, ev_stride, msgs, msgs_stride, logsumexp_temp, objval, grad,
                           bp_updates, edge_lse, workspace);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_sdlp_objective launch");
  return PGBP_OK;
}

int pgbp_sdlp_run(const pgbp_plan* plan, void* stream, int64_t batch, const float* log_potentials,
                  int64_t lp_stride, const float* evidence, int64_t ev_stride,
                  const float* msgs_in, int64_t msgs_stride, float* msgs_out, float* objvals,
                  int64_t num_iters, double logsumexp_temp, double lr, void* workspace,
                  size_t workspace_bytes) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  int rc = sdlp_check(p, batch, log_potentials, lp_stride, evidence, ev_stride, msgs_in,
                      msgs_stride, logsumexp_temp, workspace, workspace_bytes);
  if (rc) return rc;
  if (num_iters < 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "num_iters must be >= 0");
  if (p.num_edge_states > 0 && !msgs_out) return fail(PGBP_ERR_INVALID_ARGUMENT, "null msgs_out");
  if (!(lr > 0.0)) lr = logsumexp_temp != 0.0 ? logsumexp_temp : 0.01;  // dual_lp.py:282-286
  else if (logsumexp_temp != 0.0 && lr > logsumexp_temp)
    return fail(PGBP_ERR_INVALID_ARGUMENT,
                "For gradient descent, the learning rate must be smaller than the log sum-exp "
                "temperature.");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  e = pgbp::sdlp_run(p, static_cast<cudaStream_t>(stream), batch, log_potentials, lp_stride,
                     evidence, ev_stride, msgs_in, msgs_stride, msgs_out, objvals, num_iters,
                     logsumexp_temp, lr, workspace);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_sdlp_run launch");
  return PGBP_OK;
}

size_t pgbp_energy_workspace_size(const pgbp_plan* plan, int64_t batch) {
  if (!plan || batch <= 0) return 0;
  return pgbp::energy_workspace_bytes(plan->p, batch);
}

int pgbp_energy(const pgbp_plan* plan, void* stream, int64_t batch, const float* log_potentials,
                int64_t lp_stride, const float* evidence, int64_t ev_stride, const int32_t* map,
                int64_t map_stride, float* energy, void* workspace, size_t workspace_bytes) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  if (!p.var_of_vs) return fail(PGBP_ERR_INVALID_ARGUMENT, "plan has no evidence_to_vars");
  if (batch <= 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "batch must be positive");
  if (lp_stride < 0 || ev_stride < 0 || map_stride < 0 ||
      (lp_stride != 0 && lp_stride < p.num_potentials) ||
      (ev_stride != 0 && ev_stride < p.num_var_states) ||
      (map_stride != 0 && map_stride < p.num_variables))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad stride");
  if (!map || !energy || (p.num_var_states > 0 && !evidence) ||
      (p.num_enum_factors > 0 && !log_potentials))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "null data pointer");
  const size_t need = pgbp::energy_workspace_bytes(p, batch);
  if (!workspace || workspace_bytes < need)
    return fail(PGBP_ERR_WORKSPACE, "workspace of %zu bytes needed, got %zu", need, workspace_bytes);
  if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
    return fail(PGBP_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  e = pgbp::energy(p, static_cast<cudaStream_t>(stream), batch, log_potentials, lp_stride, evidence,
                   ev_stride, map, map_stride, energy, workspace, workspace_bytes);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_energy launch");
  return PGBP_OK;
}

int pgbp_energy_terms(const pgbp_plan* plan, void* stream, int64_t batch, const float* evidence,
                      int64_t ev_stride, const int32_t* map, int64_t map_stride,
                      float* var_energy, int32_t* factor_config) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  if (!p.var_of_vs) return fail(PGBP_ERR_INVALID_ARGUMENT, "plan has no evidence_to_vars");
  if (batch <= 0) return fail(PGBP_ERR_INVALID_ARGUMENT, "batch must be positive");
  if (ev_stride < 0 || map_stride < 0 ||
      (ev_stride != 0 && ev_stride < p.num_var_states) ||
      (map_stride != 0 && map_stride < p.num_variables))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad stride");
  if (!map || (p.num_variables > 0 && !var_energy) || (p.num_factors > 0 && !factor_config) ||
      (p.num_var_states > 0 && !evidence))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "null data pointer");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  const cudaError_t e = pgbp::energy_terms(p, static_cast<cudaStream_t>(stream), batch, evidence,
                                           ev_stride, map, map_stride, var_energy, factor_config);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_energy_terms launch");
  return PGBP_OK;
}

namespace {

// Arguments of pgbp_softmax_rows / pgbp_argmax_rows; the current device's SM count in *sm.
int rows_check(int64_t rows, int64_t k, const void* in, const void* out, int* sm) {
  if (rows < 0 || k < 0 || (rows > 0 && k == 0) || (rows > 0 && (!in || !out)))
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad rows, k or null pointer");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(sm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  return PGBP_OK;
}

}  // namespace

int pgbp_softmax_rows(void* stream, int64_t rows, int64_t k, const float* in, float* out) {
  int sm = 0;
  if (const int rc = rows_check(rows, k, in, out, &sm)) return rc;
  const cudaError_t e = pgbp::rows_softmax(static_cast<cudaStream_t>(stream), rows, k, in, out, sm);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_softmax_rows launch");
  return PGBP_OK;
}

int pgbp_argmax_rows(void* stream, int64_t rows, int64_t k, const float* in, int32_t* out) {
  int sm = 0;
  if (const int rc = rows_check(rows, k, in, out, &sm)) return rc;
  const cudaError_t e = pgbp::rows_argmax(static_cast<cudaStream_t>(stream), rows, k, in, out, sm);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_argmax_rows launch");
  return PGBP_OK;
}

int pgbp_marginals(const pgbp_plan* plan, void* stream, int64_t batch, const float* beliefs,
                   int64_t beliefs_stride, float* marginals) {
  if (!plan) return fail(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  const pgbp::Plan& p = plan->p;
  if (!p.var_off) return fail(PGBP_ERR_INVALID_ARGUMENT, "plan has no evidence_to_vars");
  if (batch <= 0 || beliefs_stride < 0 || !beliefs || !marginals)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "bad argument");
  pgbp::DeviceGuard guard(p.device);
  if (guard.status() != cudaSuccess) return cuda_fail(guard.status(), "cudaSetDevice");
  if (const int rc = pgbp::take_plan_fault(p)) return rc;
  cudaError_t e;
  e = pgbp::marginals(p, static_cast<cudaStream_t>(stream), batch, beliefs, beliefs_stride, marginals);
  if (e != cudaSuccess) return cuda_fail(e, "pgbp_marginals launch");
  return PGBP_OK;
}

}  // extern "C"
