"""Host wrapper of the pgbp C ABI: one compiled plan per factor graph, device buffers from torch.

PyTorch supplies device memory, the current stream and the caching allocator; every computation
is a libpgbp kernel. There is no CPU path: without a CUDA device (or without libpgbp.so) every call
raises.
"""

import atexit
import ctypes
import json
import os
import weakref
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import native

TYPE_KEYS = ("enum", "or", "and", "pool")

# A JSON file caching the autotuner's decision tables across processes, keyed by plan signature
# ({signature: [entries]}): read when a plan is created, merged and written back at exit.
TUNE_CACHE_ENV = "PGBP_TUNE_CACHE"
_LIVE_PLANS = weakref.WeakSet()


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


def _require_cuda():
  torch = _torch()
  if not torch.cuda.is_available():
    raise RuntimeError("pgmax_gb300 runs belief propagation on a CUDA GPU (sm_103a); no CUDA "
                       "device is available and there is no CPU fallback")
  return torch


class Plan:
  """A device plan compiled from the flat wiring (see include/pgbp.h, pgbp_plan_create).

  `wiring` holds the flat arrays of the reference's InfererContext: keys
  var_states_for_edge_states, edge_indices_for_edge_states, factor_indices_for_edge_states,
  num_edges, num_var_states, msgs_ranges [4, 2], potentials_ranges [4, 2], the per-type inference
  arguments (enum.factor_configs_indices, ..., pool.pool_indicators_edge_states) and optionally
  evidence_to_vars / num_variables.
  """

  def __init__(self, wiring: Dict[str, np.ndarray], device: Optional[int] = None, flags: int = 0):
    torch = _require_cuda()
    self.lib = native.load()
    self.device = torch.cuda.current_device() if device is None else int(device)
    keep = []

    def i32(key):
      v = wiring.get(key)
      if v is None:
        return None, 0
      a = np.ascontiguousarray(np.asarray(v, dtype=np.int32).reshape(-1))
      keep.append(a)
      return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), a.shape[0]

    d = native.WiringDesc()
    p, n = i32("var_states_for_edge_states")
    d.var_states_for_edge_states, d.num_edge_states = p, n
    d.edge_indices_for_edge_states, _ = i32("edge_indices_for_edge_states")
    d.factor_indices_for_edge_states, _ = i32("factor_indices_for_edge_states")
    d.num_var_states = int(wiring["num_var_states"])
    d.num_edges = int(wiring["num_edges"])
    mr = np.asarray(wiring["msgs_ranges"], dtype=np.int64).reshape(4, 2)
    pr = np.asarray(wiring["potentials_ranges"], dtype=np.int64).reshape(4, 2)
    for t in range(4):
      for j in range(2):
        d.msgs_range[t][j] = int(mr[t, j])
        d.potentials_range[t][j] = int(pr[t, j])
    d.enum_factor_configs_indices, d.enum_num_rows = i32("enum.factor_configs_indices")
    d.enum_factor_configs_edge_states, _ = i32("enum.factor_configs_edge_states")
    d.enum_num_val_configs = int(wiring.get("enum.num_val_configs", 0))
    for w, key in enumerate(("or", "and")):
      d.logical_parents_factor_indices[w], d.logical_num_parents[w] = i32(
          f"{key}.parents_factor_indices")
      d.logical_parents_msg_indices[w], _ = i32(f"{key}.parents_msg_indices")
      d.logical_children_edge_states[w], d.logical_num_factors[w] = i32(
          f"{key}.children_edge_states")
    d.pool_choices_factor_indices, d.pool_num_choices = i32("pool.pool_choices_factor_indices")
    d.pool_choices_msg_indices, _ = i32("pool.pool_choices_msg_indices")
    d.pool_indicators_edge_states, d.pool_num_factors = i32("pool.pool_indicators_edge_states")
    if wiring.get("evidence_to_vars") is not None:
      d.evidence_to_vars, _ = i32("evidence_to_vars")
      d.num_variables = int(wiring.get("num_variables",
                                       int(np.max(wiring["evidence_to_vars"], initial=-1)) + 1))
    d.flags = int(flags) | (native.FLAG_ENUM_IMPLICIT_ROWS if wiring.get("enum.implicit_rows")
                            else 0)
    # shared potential tables (optional): first potential of every Enum factor's table
    d.enum_factor_potential_offsets, d.enum_num_factors = i32("enum.factor_potential_offsets")
    handle = ctypes.c_void_p()
    with torch.cuda.device(self.device):
      native.check(self.lib.pgbp_plan_create(ctypes.byref(d), self.device, ctypes.byref(handle)),
                   "pgbp_plan_create")
    self.handle = handle
    self.num_edge_states = int(d.num_edge_states)
    self.num_var_states = int(d.num_var_states)
    self.msgs_ranges = mr
    self.potentials_ranges = pr
    self.num_potentials = int(pr[:, 1].max()) if pr.size else 0
    info = native.PlanInfo()
    native.check(self.lib.pgbp_plan_get_info(handle, ctypes.byref(info)), "pgbp_plan_get_info")
    self.info = {k: int(getattr(info, k)) for k, _ in native.PlanInfo._fields_}
    del keep
    cache = os.environ.get(TUNE_CACHE_ENV)
    if cache:
      table = _read_cache(cache)
      if self.signature() in table:
        self.load_tuning(table[self.signature()])
    _LIVE_PLANS.add(self)

  def __del__(self):
    h = getattr(self, "handle", None)
    if h is not None and h.value:
      try:
        self.lib.pgbp_plan_destroy(h)
      except Exception:  # pylint: disable=broad-except
        pass
      self.handle = None

  def check(self, synchronize=True):
    """Raises PgbpError (a RuntimeError, status PGBP_ERR_TIMEOUT) when a launch on this plan gave
    up a bounded device wait since the last check (pgbp_plan_check): that launch's results are
    invalid. Synchronises the plan's device first unless `synchronize` is False, in which case
    only launches that have already completed are seen."""
    if synchronize:
      _torch().cuda.synchronize(self.device)
    native.check(self.lib.pgbp_plan_check(self.handle), "pgbp_plan_check")

  # ------------------------------------------------------------------------- autotuner
  def signature(self) -> str:
    buf = ctypes.create_string_buffer(1024)
    native.check(self.lib.pgbp_plan_signature(self.handle, buf, len(buf)), "pgbp_plan_signature")
    return buf.value.decode()

  def tuning(self) -> List[Dict]:
    """The autotuner's decisions so far: one dict per (batch, temperature == 0) with the
    execution path (-1: not tuned) and the kernel variant of every multi-kernel launch site."""
    n = int(self.lib.pgbp_plan_tuning_count(self.handle))
    arr = (native.TuningEntry * max(n, 1))()
    native.check(self.lib.pgbp_plan_tuning_get(self.handle, arr, n), "pgbp_plan_tuning_get")
    return [{"batch": int(e.batch), "temperature0": bool(e.temperature0), "path": int(e.path),
             "sites": [int(e.site[k]) for k in range(e.num_sites)]} for e in arr[:n]]

  def load_tuning(self, entries: List[Dict]):
    """Installs decisions (as tuning() returns them); later runs with those keys skip timing."""
    arr = (native.TuningEntry * max(len(entries), 1))()
    for i, d in enumerate(entries):
      sites = list(d.get("sites", []))
      if len(sites) > native.TUNE_MAX_SITES:
        raise ValueError("too many launch sites in a tuning entry")
      arr[i].batch = int(d["batch"])
      arr[i].temperature0 = int(bool(d["temperature0"]))
      arr[i].path = int(d.get("path", -1))
      arr[i].num_sites = len(sites)
      for k, v in enumerate(sites):
        arr[i].site[k] = int(v)
    native.check(self.lib.pgbp_plan_tuning_set(self.handle, arr, len(entries)),
                 "pgbp_plan_tuning_set")

  def save_tuning(self, path: str):
    """Merges this plan's decisions into the JSON decision table at `path`."""
    table = _read_cache(path)
    mine = {(e["batch"], e["temperature0"]): e for e in table.get(self.signature(), [])}
    for e in self.tuning():
      mine[(e["batch"], e["temperature0"])] = e
    table[self.signature()] = list(mine.values())
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "w") as f:
      json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)

  # ------------------------------------------------------------------------- helpers
  def _dev(self, x, dtype=None):
    torch = _torch()
    dtype = dtype or torch.float32
    if isinstance(x, torch.Tensor):
      t = x.to(device=f"cuda:{self.device}", dtype=dtype)
    else:
      t = torch.as_tensor(np.asarray(x), device=f"cuda:{self.device}").to(dtype)
    return t.contiguous()

  @staticmethod
  def _rows(t, n):
    """(pointer-able tensor, batch, stride) of a [n] or [B, n] array."""
    if t.ndim == 1:
      if t.shape[0] != n:
        raise ValueError(f"expected length {n}, got {tuple(t.shape)}")
      return t, 1, 0
    if t.ndim == 2 and t.shape[1] == n:
      return t, t.shape[0], t.stride(0)
    raise ValueError(f"expected shape ({n},) or (B, {n}), got {tuple(t.shape)}")

  def _stream(self):
    return ctypes.c_void_p(_torch().cuda.current_stream(self.device).cuda_stream)

  # ------------------------------------------------------------------------- entry points
  def _inputs(self, log_potentials, evidence, ftov_msgs):
    """Device copies of the three BPArrays fields with their strides and the batch size."""
    torch = _torch()
    lp = self._dev(log_potentials) if self.num_potentials > 0 else torch.zeros(
        1, device=f"cuda:{self.device}")
    ev = self._dev(evidence)
    m = self._dev(ftov_msgs)
    lp_t, b1, lps = self._rows(lp, self.num_potentials) if self.num_potentials > 0 else (lp, 1, 0)
    ev_t, b2, evs = self._rows(ev, self.num_var_states)
    m_t, b3, ms = self._rows(m, self.num_edge_states)
    bs = {b for b, nd in ((b1, lp.ndim), (b2, ev.ndim), (b3, m.ndim)) if nd == 2}
    if len(bs) > 1:
      raise ValueError(f"inconsistent batch sizes {sorted(bs)}")
    B = bs.pop() if bs else 1
    batched = any(t.ndim == 2 for t in (lp, ev, m))
    return (lp_t, lps), (ev_t, evs), (m_t, ms), B, batched

  def _run(self, lp, ev, m, B, out, deltas, num_iters, damping, temperature):
    ws_bytes = int(self.lib.pgbp_workspace_size(self.handle, B, max(int(num_iters), 1)))
    ws = _torch().empty(ws_bytes, dtype=_torch().uint8, device=out.device)
    native.check(self.lib.pgbp_run(
        self.handle, self._stream(), B, lp[0].data_ptr(), lp[1], ev[0].data_ptr(), ev[1],
        m[0].data_ptr(), m[1], out.data_ptr(), deltas.data_ptr() if deltas is not None else None,
        int(num_iters), float(damping), float(temperature), ws.data_ptr(), ws_bytes), "pgbp_run")

  def run(self, log_potentials, evidence, ftov_msgs, num_iters, damping=0.5, temperature=0.0,
          with_deltas=True):
    """run_with_diffs on the GPU. Inputs [n] or [B, n]; returns (msgs [B?, E_s], deltas)."""
    torch = _torch()
    lp, ev, m, B, batched = self._inputs(log_potentials, evidence, ftov_msgs)
    iters = max(int(num_iters), 1)
    dev = m[0].device
    out = torch.empty((B, self.num_edge_states), dtype=torch.float32, device=dev)
    deltas = torch.empty((B, iters), dtype=torch.float32, device=dev) if with_deltas else None
    self._run(lp, ev, m, B, out, deltas, num_iters, damping, temperature)
    if not batched:
      out = out[0]
      deltas = deltas[0] if deltas is not None else None
    return out, deltas

  def run_perturbed(self, log_potentials, evidence, ftov_msgs, num_iters, seed, batch,
                    noise_scale=1.0, damping=0.5, temperature=0.0, with_deltas=True):
    """Perturb-and-MAP in one call (pgbp_run_perturbed): run() on `batch` instances whose evidence
    is `evidence` (the base: [N_vs] shared, [batch, N_vs], or None for zeros) plus noise_scale times
    the Gumbel(0, 1) stream of `seed`, generated inside the run. Returns (msgs [batch, E_s],
    deltas [batch, iters] or None, the perturbed evidence [batch, N_vs])."""
    torch = _torch()
    B = int(batch)
    if B < 1:
      raise ValueError(f"batch must be >= 1, got {B}")
    dev = f"cuda:{self.device}"
    lp = self._dev(log_potentials) if self.num_potentials > 0 else torch.zeros(1, device=dev)
    lp_t, b1, lps = self._rows(lp, self.num_potentials) if self.num_potentials > 0 else (lp, 1, 0)
    m_t, b3, ms = self._rows(self._dev(ftov_msgs), self.num_edge_states)
    if evidence is None:
      b2, evs, ev_ptr = B, 0, None
    else:
      ev_t, b2, evs = self._rows(self._dev(evidence), self.num_var_states)
      ev_ptr = ev_t.data_ptr()
    for name, b, stride in (("log_potentials", b1, lps), ("evidence", b2, evs), ("ftov_msgs", b3, ms)):
      if stride != 0 and b != B:
        raise ValueError(f"{name} holds {b} instances, batch is {B}")
    iters = max(int(num_iters), 1)
    out = torch.empty((B, self.num_edge_states), dtype=torch.float32, device=dev)
    deltas = torch.empty((B, iters), dtype=torch.float32, device=dev) if with_deltas else None
    ev_out = torch.empty((B, self.num_var_states), dtype=torch.float32, device=dev)
    ws_bytes = int(self.lib.pgbp_workspace_size(self.handle, B, iters))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    native.check(self.lib.pgbp_run_perturbed(
        self.handle, self._stream(), B, lp_t.data_ptr(), lps, ev_ptr, evs,
        int(seed) & (2**64 - 1), float(noise_scale), m_t.data_ptr(), ms, out.data_ptr(),
        deltas.data_ptr() if deltas is not None else None, ev_out.data_ptr(), int(num_iters),
        float(damping), float(temperature), ws.data_ptr(), ws_bytes), "pgbp_run_perturbed")
    return out, deltas, ev_out

  def run_checkpointed(self, log_potentials, evidence, ftov_msgs, num_iters, damping=0.5,
                       temperature=0.0, checkpoint_every=10):
    """run() that also keeps the messages every `checkpoint_every` iterations
    (pgbp_run_checkpointed): returns (msgs, deltas, checkpoints [ceil(iters / k), B, E_s]) for
    run_vjp; msgs and deltas are bit for bit those of run()."""
    torch = _torch()
    k = int(checkpoint_every)
    if k < 1:
      raise ValueError(f"checkpoint_every must be >= 1, got {k}")
    lp, ev, m, B, batched = self._inputs(log_potentials, evidence, ftov_msgs)
    iters = max(int(num_iters), 1)
    k = min(k, iters)
    n_ck = -(-iters // k)
    dev = m[0].device
    ck = torch.empty((n_ck, B, self.num_edge_states), dtype=torch.float32, device=dev)
    out = torch.empty((B, self.num_edge_states), dtype=torch.float32, device=dev)
    deltas = torch.empty((B, iters), dtype=torch.float32, device=dev)
    ws_bytes = int(self.lib.pgbp_workspace_size(self.handle, B, iters))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    native.check(self.lib.pgbp_run_checkpointed(
        self.handle, self._stream(), B, lp[0].data_ptr(), lp[1], ev[0].data_ptr(), ev[1],
        m[0].data_ptr(), m[1], out.data_ptr(), deltas.data_ptr(), int(num_iters), k,
        float(damping), float(temperature), ck.data_ptr(), ws.data_ptr(), ws_bytes),
                 "pgbp_run_checkpointed")
    if not batched:
      return out[0], deltas[0], ck
    return out, deltas, ck

  def run_to_tolerance(self, log_potentials, evidence, ftov_msgs, tolerance, max_iters,
                       damping=0.5, temperature=0.0, check_every=1):
    """BP until every instance's residual is below `tolerance` (pgbp_run_to_tolerance): returns
    (msgs, first iteration below the tolerance per instance (-1 if none, host int32),
    iterations run)."""
    torch = _torch()
    lp, ev, m, B, batched = self._inputs(log_potentials, evidence, ftov_msgs)
    dev = m[0].device
    out = torch.empty((B, self.num_edge_states), dtype=torch.float32, device=dev)
    first = torch.empty(B, dtype=torch.int32, device=dev)
    ran = ctypes.c_int64(0)
    ws_bytes = int(self.lib.pgbp_workspace_size(self.handle, B, int(check_every)))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    native.check(self.lib.pgbp_run_to_tolerance(
        self.handle, self._stream(), B, lp[0].data_ptr(), lp[1], ev[0].data_ptr(), ev[1],
        m[0].data_ptr(), m[1], out.data_ptr(), float(tolerance), int(max_iters),
        int(check_every), float(damping), float(temperature), first.data_ptr(),
        ctypes.byref(ran), ws.data_ptr(), ws_bytes), "pgbp_run_to_tolerance")
    first = first.cpu()
    if not batched:
      return out[0], first[0], int(ran.value)
    return out, first, int(ran.value)

  def run_vjp(self, log_potentials, evidence, checkpoints, num_iters, g_msgs, damping=0.5,
              temperature=1.0, checkpoint_every=10, want_msgs_in=False):
    """Gradients (g_log_potentials, g_evidence, g_msgs_in or None) of a loss with gradient g_msgs
    on run()'s output messages, by the hand-written adjoint (pgbp_run_vjp). Shared (1-D)
    potentials / evidence get gradients summed over the batch."""
    torch = _torch()
    ck = checkpoints
    n_ck, B, n_es = ck.shape
    lp, ev, _, b, _ = self._inputs(log_potentials, evidence, ck[0])
    if b != B:
      raise ValueError(f"checkpoints hold {B} instances, inputs {b}")
    g = self._dev(g_msgs)
    g = g.expand(B, n_es).contiguous() if g.ndim == 1 else g
    if tuple(g.shape) != (B, n_es):
      raise ValueError(f"g_msgs shape {tuple(g.shape)}, expected {(B, n_es)}")
    dev = ck.device
    P = max(self.num_potentials, 1)
    g_lp = torch.empty((B, P) if lp[1] else (P,), dtype=torch.float32, device=dev)
    g_ev = torch.empty((B, self.num_var_states) if ev[1] else (self.num_var_states,),
                       dtype=torch.float32, device=dev)
    g_m = torch.empty((B, n_es), dtype=torch.float32, device=dev) if want_msgs_in else None
    ws_bytes = int(self.lib.pgbp_vjp_workspace_size(self.handle, B, int(num_iters),
                                                    int(checkpoint_every)))
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
    native.check(self.lib.pgbp_run_vjp(
        self.handle, self._stream(), B, lp[0].data_ptr(), lp[1], ev[0].data_ptr(), ev[1],
        ck.data_ptr(), int(num_iters), int(checkpoint_every), float(damping), float(temperature),
        g.data_ptr(), g_lp.data_ptr(), g_ev.data_ptr(), g_m.data_ptr() if g_m is not None else None,
        ws.data_ptr(), ws_bytes), "pgbp_run_vjp")
    if self.num_potentials == 0:
      g_lp = g_lp[..., :0]
    return g_lp, g_ev, g_m

  def beliefs_vjp(self, g_beliefs):
    """dL/d(messages) [B?, E_s] from dL/d(flat beliefs) (pgbp_beliefs_vjp)."""
    torch = _torch()
    g = self._dev(g_beliefs)
    g_t, B, gs = self._rows(g, self.num_var_states)
    out = torch.empty((B, self.num_edge_states), dtype=torch.float32, device=g.device)
    native.check(self.lib.pgbp_beliefs_vjp(self.handle, self._stream(), B, g_t.data_ptr(), gs,
                                           out.data_ptr()), "pgbp_beliefs_vjp")
    return out if g.ndim == 2 else out[0]

  def factor_update(self, ftype, vtof_msgs, log_potentials, temperature, normalize=True):
    """FAC_TO_VAR_UPDATES[type] on one type's message slice ([n] or [B, n])."""
    torch = _torch()
    n = int(self.msgs_ranges[ftype, 1] - self.msgs_ranges[ftype, 0])
    npot = int(self.potentials_ranges[ftype, 1] - self.potentials_ranges[ftype, 0])
    v = self._dev(vtof_msgs)
    v_t, B, vs = self._rows(v, n)
    if log_potentials is not None and npot > 0:
      lp = self._dev(log_potentials)
      lp_t, _, lps = self._rows(lp, npot)
      lp_ptr = lp_t.data_ptr()
    else:
      lp_ptr, lps = None, 0
    out = torch.empty((B, n), dtype=torch.float32, device=v.device)
    native.check(self.lib.pgbp_factor_update(
        self.handle, self._stream(), int(ftype), B, v_t.data_ptr(), vs, lp_ptr, lps,
        float(temperature), int(bool(normalize)), out.data_ptr(), n), "pgbp_factor_update")
    return out if v.ndim == 2 else out[0]

  def beliefs(self, evidence, ftov_msgs):
    torch = _torch()
    ev = self._dev(evidence)
    m = self._dev(ftov_msgs)
    ev_t, b1, evs = self._rows(ev, self.num_var_states)
    m_t, b2, ms = self._rows(m, self.num_edge_states)
    B = max(b1 if ev.ndim == 2 else 1, b2 if m.ndim == 2 else 1)
    out = torch.empty((B, self.num_var_states), dtype=torch.float32, device=m.device)
    native.check(self.lib.pgbp_beliefs(self.handle, self._stream(), B, ev_t.data_ptr(), evs,
                                       m_t.data_ptr(), ms, out.data_ptr()), "pgbp_beliefs")
    return out if (ev.ndim == 2 or m.ndim == 2) else out[0]

  def decode(self, flat_beliefs, num_variables):
    torch = _torch()
    b = self._dev(flat_beliefs)
    b_t, B, bs = self._rows(b, self.num_var_states)
    out = torch.empty((B, num_variables), dtype=torch.int32, device=b.device)
    native.check(self.lib.pgbp_decode(self.handle, self._stream(), B, b_t.data_ptr(), bs,
                                      out.data_ptr()), "pgbp_decode")
    return out if b.ndim == 2 else out[0]

  # ------------------------------------------------------------------------- SDLP
  def _sdlp_ws(self, B, dev):
    nb = int(self.lib.pgbp_sdlp_workspace_size(self.handle, B))
    return _torch().empty(max(nb, 1), dtype=_torch().uint8, device=dev), nb

  def sdlp_run(self, log_potentials, evidence, ftov_msgs, num_iters, temperature, lr=None):
    """run_with_objvals of the smooth dual LP-MAP solver (pgbp_sdlp_run): returns
    (messages [B?, E_s], objective values [B?, num_iters])."""
    torch = _torch()
    lp, ev, m, B, batched = self._inputs(log_potentials, evidence, ftov_msgs)
    dev = m[0].device
    iters = int(num_iters)
    out = torch.empty((B, self.num_edge_states), dtype=torch.float32, device=dev)
    objvals = torch.empty((B, max(iters, 0)), dtype=torch.float32, device=dev)
    ws, nb = self._sdlp_ws(B, dev)
    native.check(self.lib.pgbp_sdlp_run(
        self.handle, self._stream(), B, lp[0].data_ptr(), lp[1], ev[0].data_ptr(), ev[1],
        m[0].data_ptr(), m[1], out.data_ptr(), objvals.data_ptr() if iters > 0 else None, iters,
        float(temperature), -1.0 if lr is None else float(lr), ws.data_ptr(), nb),
                 "pgbp_sdlp_run")
    return (out, objvals) if batched else (out[0], objvals[0])

  def sdlp_objective(self, log_potentials, evidence, ftov_msgs, temperature, grad=False,
                     updates=False, edge_lse=False):
    """smooth_dual_objval_and_grad (pgbp_sdlp_objective): a dict with "objval" [B?] and, when
    asked for, "grad" and "updates" [B?, E_s] and "edge_lse" [B?, num_edges]."""
    torch = _torch()
    lp, ev, m, B, batched = self._inputs(log_potentials, evidence, ftov_msgs)
    dev = m[0].device
    n_es, ne = self.num_edge_states, int(self.info["num_edges"])
    out = {"objval": torch.empty(B, dtype=torch.float32, device=dev)}
    if grad:
      out["grad"] = torch.empty((B, n_es), dtype=torch.float32, device=dev)
    if updates:
      out["updates"] = torch.empty((B, n_es), dtype=torch.float32, device=dev)
    if edge_lse:
      out["edge_lse"] = torch.empty((B, ne), dtype=torch.float32, device=dev)
    ptr = lambda k: out[k].data_ptr() if k in out else None
    ws, nb = self._sdlp_ws(B, dev)
    native.check(self.lib.pgbp_sdlp_objective(
        self.handle, self._stream(), B, lp[0].data_ptr(), lp[1], ev[0].data_ptr(), ev[1],
        m[0].data_ptr(), m[1], float(temperature), ptr("objval"), ptr("grad"), ptr("updates"),
        ptr("edge_lse"), ws.data_ptr(), nb), "pgbp_sdlp_objective")
    return out if batched else {k: v[0] for k, v in out.items()}

  def energy(self, log_potentials, evidence, map_states):
    """Energies of decodings (pgbp_energy): map_states [num_variables] or [B, num_variables]
    (int), log_potentials / evidence [n] or [B, n] as BPArrays hold them. Returns float32 [B]
    (or a 0-d tensor when nothing is batched)."""
    torch = _torch()
    m = self._dev(map_states, torch.int32)
    lp = self._dev(log_potentials) if log_potentials is not None else None
    ev = self._dev(evidence)
    nvars = int(self.info["num_variables"])
    m_t, b1, mst = self._rows(m, nvars)
    ev_t, b2, evs = self._rows(ev, self.num_var_states)
    if lp is not None:
      lp_t, b3, lps = self._rows(lp, self.num_potentials)
    else:
      lp_t, b3, lps = None, 1, 0
    batched = [t.ndim == 2 for t in (m, ev) + ((lp,) if lp is not None else ())]
    sizes = {b for b, bt in zip((b1, b2, b3), batched) if bt}
    if len(sizes) > 1:
      raise ValueError(f"batch sizes differ: {sorted(sizes)}")
    B = sizes.pop() if sizes else 1
    out = torch.empty(B, dtype=torch.float32, device=ev.device)
    nb = int(self.lib.pgbp_energy_workspace_size(self.handle, B))
    ws = torch.empty(max(nb, 1), dtype=torch.uint8, device=ev.device)
    native.check(self.lib.pgbp_energy(
        self.handle, self._stream(), B, lp_t.data_ptr() if lp_t is not None else None, lps,
        ev_t.data_ptr(), evs, m_t.data_ptr(), mst, out.data_ptr(), ws.data_ptr(), nb),
        "pgbp_energy")
    return out if any(batched) else out[0]

  def energy_terms(self, evidence, map_states):
    """Per-variable energies and per-factor decoded configs of decodings (pgbp_energy_terms,
    compute_energy's debug mode): map_states [num_variables] or [B, num_variables] (int),
    evidence [n] or [B, n]. Returns (var_energy float32 [.., num_variables], factor_config int32
    [.., num_factors]), with the batch axis when an input carries one."""
    torch = _torch()
    m = self._dev(map_states, torch.int32)
    ev = self._dev(evidence)
    nvars = int(self.info["num_variables"])
    nf = sum(int(self.info[k]) for k in ("num_enum_factors", "num_or_factors", "num_and_factors",
                                          "num_pool_factors"))
    m_t, b1, mst = self._rows(m, nvars)
    ev_t, b2, evs = self._rows(ev, self.num_var_states)
    batched = [t.ndim == 2 for t in (m, ev)]
    sizes = {b for b, bt in zip((b1, b2), batched) if bt}
    if len(sizes) > 1:
      raise ValueError(f"batch sizes differ: {sorted(sizes)}")
    B = sizes.pop() if sizes else 1
    var_e = torch.empty((B, nvars), dtype=torch.float32, device=ev.device)
    fac_c = torch.empty((B, nf), dtype=torch.int32, device=ev.device)
    native.check(self.lib.pgbp_energy_terms(
        self.handle, self._stream(), B, ev_t.data_ptr(), evs, m_t.data_ptr(), mst,
        var_e.data_ptr(), fac_c.data_ptr()), "pgbp_energy_terms")
    if any(batched):
      return var_e, fac_c
    return var_e[0], fac_c[0]

  def marginals(self, flat_beliefs):
    torch = _torch()
    b = self._dev(flat_beliefs)
    b_t, B, bs = self._rows(b, self.num_var_states)
    out = torch.empty((B, self.num_var_states), dtype=torch.float32, device=b.device)
    native.check(self.lib.pgbp_marginals(self.handle, self._stream(), B, b_t.data_ptr(), bs,
                                         out.data_ptr()), "pgbp_marginals")
    return out if b.ndim == 2 else out[0]


def gumbel(seed, count, device=None):
  """Draws 0 .. count - 1 of the Gumbel(0, 1) stream of `seed` that run_perturbed adds to the
  evidence (pgbp_gumbel), as a float32 CUDA tensor."""
  torch = _require_cuda()
  dev = torch.device("cuda", torch.cuda.current_device() if device is None else int(device))
  out = torch.empty(int(count), dtype=torch.float32, device=dev)
  with torch.cuda.device(dev):
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    native.check(native.load().pgbp_gumbel(stream, int(seed) & (2**64 - 1), int(count),
                                           out.data_ptr()), "pgbp_gumbel")
  return out


def _dense_rows(x):
  """x (torch or NumPy, shape (..., k)) as a contiguous float32 CUDA tensor, detached."""
  torch = _require_cuda()
  t = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x, dtype=np.float32))
  dev = t.device if t.is_cuda else torch.device("cuda", torch.cuda.current_device())
  return t.detach().to(device=dev, dtype=torch.float32).contiguous()


def softmax_last(x):
  """get_marginals of one belief array of any shape (..., k) that did not come from a plan:
  exp(x - logsumexp(x)) over the last axis by the pgbp_softmax_rows kernel (padded -inf states
  get 0). Returns a CUDA tensor."""
  torch = _torch()
  t = _dense_rows(x)
  if t.numel() == 0:
    return t.clone()
  k = int(t.shape[-1])
  out = torch.empty_like(t)
  with torch.cuda.device(t.device):
    stream = ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)
    native.check(native.load().pgbp_softmax_rows(stream, t.numel() // k, k, t.data_ptr(),
                                                 out.data_ptr()), "pgbp_softmax_rows")
  return out


def argmax_last(x):
  """decode_map_states of one belief array of any shape (..., k) that did not come from a plan:
  the first maximum (or first NaN) over the last axis by the pgbp_argmax_rows kernel, int32; an
  empty array decodes to zeros of shape (...) as in the reference. Returns a CUDA tensor."""
  torch = _torch()
  t = _dense_rows(x)
  if t.numel() == 0:
    return torch.zeros(t.shape[:-1], dtype=torch.float32, device=t.device)
  k = int(t.shape[-1])
  out = torch.empty(t.shape[:-1], dtype=torch.int32, device=t.device)
  with torch.cuda.device(t.device):
    stream = ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)
    native.check(native.load().pgbp_argmax_rows(stream, t.numel() // k, k, t.data_ptr(),
                                                out.data_ptr()), "pgbp_argmax_rows")
  return out


def _read_cache(path: str) -> Dict:
  try:
    with open(path) as f:
      table = json.load(f)
    return table if isinstance(table, dict) else {}
  except (OSError, ValueError):
    return {}


@atexit.register
def _save_live_tunings():
  path = os.environ.get(TUNE_CACHE_ENV)
  if not path:
    return
  for plan in list(_LIVE_PLANS):
    try:
      if plan.handle is not None and plan.tuning():
        plan.save_tuning(path)
    except Exception:  # pylint: disable=broad-except
      pass
