"""ctypes front-end of the C oracle (bp_oracle.c). TEST INFRASTRUCTURE ONLY.

Imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline and reference arms,
where it is the checker (and the timed CPU stand-in for the reference's JAX-CPU path, which cannot
run without jax). The product package never imports it.

`Wiring` takes the flat arrays of PGMax's InfererContext (pgmax/infer/inferer.py:76-118) as a dict
with keys `var_states_for_edge_states`, `edge_indices_for_edge_states`, `num_edges`,
`num_var_states`, `msgs_ranges` [4,2], `potentials_ranges` [4,2] and the per-type inference
arguments `enum.factor_configs_indices`, `enum.factor_configs_edge_states`,
`enum.num_val_configs`, `or.parents_factor_indices`, `or.parents_msg_indices`,
`or.children_edge_states` (same for `and.`), `pool.pool_choices_factor_indices`,
`pool.pool_choices_msg_indices`, `pool.pool_indicators_edge_states` - the layout the golden
fixtures store and `pgmax_gb300.infer.InfererContext.flat_wiring()` returns.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bp_oracle.c")
LIB = os.path.join(HERE, "_build", "libbp_oracle.so")

_i64 = ctypes.c_int64
_p32 = ctypes.POINTER(ctypes.c_int32)
_pf = ctypes.POINTER(ctypes.c_float)


class _CWiring(ctypes.Structure):
  _fields_ = [
      ("num_edge_states", _i64), ("num_var_states", _i64), ("num_edges", _i64),
      ("var_states_for_edge_states", _p32), ("edge_indices_for_edge_states", _p32),
      ("msgs_range", (_i64 * 2) * 4), ("potentials_range", (_i64 * 2) * 4),
      ("enum_num_rows", _i64), ("enum_factor_configs_indices", _p32),
      ("enum_factor_configs_edge_states", _p32), ("enum_num_val_configs", _i64),
      ("logical_num_parents", _i64 * 2), ("logical_parents_factor_indices", _p32 * 2),
      ("logical_parents_msg_indices", _p32 * 2), ("logical_num_factors", _i64 * 2),
      ("logical_children_edge_states", _p32 * 2),
      ("pool_num_choices", _i64), ("pool_choices_factor_indices", _p32),
      ("pool_choices_msg_indices", _p32), ("pool_num_factors", _i64),
      ("pool_indicators_edge_states", _p32),
  ]


def build(force=False):
  """Compiles the oracle with gcc (-ffp-contract=off keeps every float op separately rounded)."""
  if os.path.exists(LIB) and not force and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
    return LIB
  os.makedirs(os.path.dirname(LIB), exist_ok=True)
  cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
         "-std=c11", SRC, "-o", LIB + ".tmp", "-lm"]
  subprocess.check_call(cmd)
  os.replace(LIB + ".tmp", LIB)
  return LIB


_lib = None


def lib():
  global _lib
  if _lib is None:
    build()
    L = ctypes.CDLL(LIB)
    W = ctypes.POINTER(_CWiring)
    L.bpo_factor_update.argtypes = [W, ctypes.c_int, _pf, _pf, ctypes.c_double, ctypes.c_int, _pf]
    L.bpo_run.argtypes = [W, _pf, _pf, _pf, _i64, ctypes.c_double, ctypes.c_double, _pf, _pf]
    L.bpo_run_batch.argtypes = [W, _i64, _pf, _i64, _pf, _i64, _pf, _i64, _i64, ctypes.c_double,
                                ctypes.c_double, _pf, _pf, ctypes.c_int]
    L.bpo_beliefs.argtypes = [W, _pf, _pf, _pf]
    for f in (L.bpo_factor_update, L.bpo_run, L.bpo_run_batch, L.bpo_beliefs):
      f.restype = ctypes.c_int
    L.bpo_gumbel.argtypes = [ctypes.c_uint64, _i64, _i64, _pf]
    L.bpo_gumbel.restype = None
    _lib = L
  return _lib


def _f32(a):
  return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _fp(a):
  return a.ctypes.data_as(_pf)


class Wiring:
  """Holds the index arrays (int32, contiguous) and the C struct pointing at them."""

  def __init__(self, arrays):
    g = lambda k, default=None: arrays.get(k, default)
    self._keep = []

    def i32(k):
      v = g(k)
      if v is None:
        v = np.zeros((0,), np.int32)
      v = np.ascontiguousarray(np.asarray(v, dtype=np.int32).reshape(-1))
      self._keep.append(v)
      return v

    c = _CWiring()
    vs = i32("var_states_for_edge_states")
    ei = i32("edge_indices_for_edge_states")
    c.num_edge_states = vs.shape[0]
    c.num_var_states = int(g("num_var_states"))
    c.num_edges = int(g("num_edges"))
    c.var_states_for_edge_states = vs.ctypes.data_as(_p32)
    c.edge_indices_for_edge_states = ei.ctypes.data_as(_p32)
    mr = np.asarray(g("msgs_ranges"), dtype=np.int64).reshape(4, 2)
    pr = np.asarray(g("potentials_ranges"), dtype=np.int64).reshape(4, 2)
    for t in range(4):
      for j in range(2):
        c.msgs_range[t][j] = int(mr[t, j])
        c.potentials_range[t][j] = int(pr[t, j])
    ci = i32("enum.factor_configs_indices")
    ce = i32("enum.factor_configs_edge_states")
    c.enum_num_rows = ci.shape[0]
    c.enum_factor_configs_indices = ci.ctypes.data_as(_p32)
    c.enum_factor_configs_edge_states = ce.ctypes.data_as(_p32)
    c.enum_num_val_configs = int(g("enum.num_val_configs", 0))
    for j, name in enumerate(("or", "and")):
      pfi = i32(f"{name}.parents_factor_indices")
      pmi = i32(f"{name}.parents_msg_indices")
      ch = i32(f"{name}.children_edge_states")
      c.logical_num_parents[j] = pfi.shape[0]
      c.logical_parents_factor_indices[j] = pfi.ctypes.data_as(_p32)
      c.logical_parents_msg_indices[j] = pmi.ctypes.data_as(_p32)
      c.logical_num_factors[j] = ch.shape[0]
      c.logical_children_edge_states[j] = ch.ctypes.data_as(_p32)
    cfi = i32("pool.pool_choices_factor_indices")
    cmi = i32("pool.pool_choices_msg_indices")
    ind = i32("pool.pool_indicators_edge_states")
    c.pool_num_choices = cfi.shape[0]
    c.pool_choices_factor_indices = cfi.ctypes.data_as(_p32)
    c.pool_choices_msg_indices = cmi.ctypes.data_as(_p32)
    c.pool_num_factors = ind.shape[0]
    c.pool_indicators_edge_states = ind.ctypes.data_as(_p32)
    self.c = c
    self.num_edge_states = int(c.num_edge_states)
    self.num_var_states = int(c.num_var_states)
    self.msgs_ranges = mr
    self.potentials_ranges = pr

  @property
  def ptr(self):
    return ctypes.byref(self.c)


def run(wiring, log_potentials, evidence, msgs_in, num_iters, damping=0.5, temperature=0.0):
  """Returns (msgs_out [E_s], deltas [max(num_iters, 1)]) for one instance."""
  lp, ev, m = _f32(log_potentials), _f32(evidence), _f32(msgs_in)
  out = np.empty(wiring.num_edge_states, np.float32)
  deltas = np.empty(max(int(num_iters), 1), np.float32)
  rc = lib().bpo_run(wiring.ptr, _fp(lp), _fp(ev), _fp(m), int(num_iters), float(damping),
                     float(temperature), _fp(out), _fp(deltas))
  if rc:
    raise RuntimeError(f"oracle bpo_run failed ({rc})")
  return out, deltas


def run_batch(wiring, log_potentials, evidence, msgs_in, num_iters, damping=0.5,
              temperature=0.0, num_threads=None):
  """Batched run; each input is [B, n] or [n] (broadcast). One OpenMP thread per instance."""
  lp, ev, m = _f32(log_potentials), _f32(evidence), _f32(msgs_in)
  B = max(a.shape[0] for a in (lp, ev, m) if a.ndim == 2) if any(
      a.ndim == 2 for a in (lp, ev, m)) else 1
  stride = lambda a: a.shape[1] if a.ndim == 2 else 0
  out = np.empty((B, wiring.num_edge_states), np.float32)
  nd = max(int(num_iters), 1)
  deltas = np.empty((B, nd), np.float32)
  nt = num_threads or len(os.sched_getaffinity(0))
  rc = lib().bpo_run_batch(wiring.ptr, B, _fp(lp), stride(lp), _fp(ev), stride(ev), _fp(m),
                           stride(m), int(num_iters), float(damping), float(temperature),
                           _fp(out), _fp(deltas), int(nt))
  if rc:
    raise RuntimeError(f"oracle bpo_run_batch failed ({rc})")
  return out, deltas


def factor_update(wiring, ftype, vtof_slice, lp_slice, temperature, normalize=True):
  """FAC_TO_VAR_UPDATES[type] on one type's message slice (ftype 0 Enum, 1 OR, 2 AND, 3 Pool)."""
  v, lp = _f32(vtof_slice), _f32(lp_slice)
  if lp.size == 0:
    lp = np.zeros(1, np.float32)
  out = np.empty(v.shape[0], np.float32)
  rc = lib().bpo_factor_update(wiring.ptr, int(ftype), _fp(v), _fp(lp), float(temperature),
                               int(bool(normalize)), _fp(out))
  if rc:
    raise RuntimeError(f"oracle bpo_factor_update failed ({rc})")
  return out


def beliefs(wiring, evidence, msgs):
  ev, m = _f32(evidence), _f32(msgs)
  out = np.empty(wiring.num_var_states, np.float32)
  lib().bpo_beliefs(wiring.ptr, _fp(ev), _fp(m), _fp(out))
  return out


def gumbel(seed, count, first=0):
  """Draws first .. first + count - 1 of the engine's Gumbel(0, 1) noise stream of `seed`
  (pgbp_gumbel), restated on the CPU."""
  out = np.empty(int(count), np.float32)
  lib().bpo_gumbel(int(seed) & (2**64 - 1), int(first), int(count), _fp(out))
  return out
