"""InfererContext and read-out: PGMax's pgmax/infer/inferer.py on the GPU engine.

`InfererContext` flattens the wiring exactly as the reference does (inferer.py:65-118) and owns the
compiled device plan (created on first use, on the current CUDA device). `get_beliefs` returns a
dict of per-group beliefs; `decode_map_states` and `get_marginals` accept it.
"""

import dataclasses
from typing import Any, Dict, Hashable, Optional, Sequence

import numpy as np

from .. import factor as factor_mod
from .. import vgroup as vgroup_mod
from ..factor import FAC_TO_VAR_UPDATES
from . import bp_state as bpstate
from .bp_state import BPArrays, BPState, Evidence, FToVMessages, LogPotentials

TYPE_KEYS = ("enum", "or", "and", "pool")



def registered_context(fg_state):
  """The first context of `fg_state` that compiled a plan (kept on the FactorGraphState), or
  None: functions that take only a BPState (compute_energy) reuse its plan."""
  return getattr(fg_state, "_pgbp_context", None)


def register_context(ctx):
  if registered_context(ctx.bp_state.fg_state) is None:
    object.__setattr__(ctx.bp_state.fg_state, "_pgbp_context", ctx)


def _is_torch(x):
  return type(x).__module__.startswith("torch")


class Beliefs(dict):
  """Per-group beliefs; remembers the flat device array so decode / marginals run as kernels."""

  flat = None
  context = None


@dataclasses.dataclass(frozen=True, eq=False)
class Inferer:
  init: Any
  update: Any
  to_bp_state: Any
  get_beliefs: Any
  run: Any


@dataclasses.dataclass(frozen=True, eq=False)
class InfererContext:
  """Shared inference context (pgmax/infer/inferer.py:55-225)."""

  bp_state: BPState
  # execution flags of the compiled plan (pgmax_gb300.native.FLAG_*; 0 = automatic path choice)
  exec_flags: int = 0

  def __post_init__(self):
    fg_state = self.bp_state.fg_state
    object.__setattr__(self, "wiring", fg_state.wiring)
    object.__setattr__(self, "evidence_to_vars", fg_state.evidence_to_vars)
    vse = factor_mod.concatenate_var_states_for_edges(
        [self.wiring[t].var_states_for_edges for t in FAC_TO_VAR_UPDATES])
    object.__setattr__(self, "var_states_for_edge_states", vse[..., 0])
    object.__setattr__(self, "edge_indices_for_edge_states", vse[..., 1])
    object.__setattr__(self, "factor_indices_for_edge_states", vse[..., 2])
    num_variables = int(fg_state.evidence_to_vars[-1]) + 1 if fg_state.evidence_to_vars.size else 0
    object.__setattr__(self, "num_variables", num_variables)
    object.__setattr__(self, "num_edges", int(vse[-1, 1]) + 1 if vse.shape[0] else 0)
    object.__setattr__(self, "num_factors", int(vse[-1, 2]) + 1 if vse.shape[0] else 0)
    args = {}
    for t in FAC_TO_VAR_UPDATES:
      a = dict(self.wiring[t].get_inference_arguments())
      args[t] = a
    object.__setattr__(self, "inference_arguments", args)
    object.__setattr__(self, "factor_type_to_msgs_range", fg_state.factor_type_to_msgs_range)
    object.__setattr__(self, "factor_type_to_potentials_range",
                       fg_state.factor_type_to_potentials_range)
    object.__setattr__(self, "_plan", None)

  # ------------------------------------------------------------------------- plan
  def flat_wiring(self) -> Dict[str, Any]:
    """The flat arrays the C ABI consumes (pgbp_wiring_desc), keyed as the golden fixtures are."""
    fg_state = self.bp_state.fg_state
    d = {
        "var_states_for_edge_states": self.var_states_for_edge_states,
        "edge_indices_for_edge_states": self.edge_indices_for_edge_states,
        "factor_indices_for_edge_states": self.factor_indices_for_edge_states,
        "num_edges": self.num_edges,
        "num_factors": self.num_factors,
        "num_var_states": fg_state.num_var_states,
        "evidence_to_vars": fg_state.evidence_to_vars,
        "num_variables": self.num_variables,
        "msgs_ranges": np.array([self.factor_type_to_msgs_range[t] for t in FAC_TO_VAR_UPDATES],
                                dtype=np.int64),
        "potentials_ranges": np.array(
            [self.factor_type_to_potentials_range[t] for t in FAC_TO_VAR_UPDATES], dtype=np.int64),
    }
    for t, key in zip(FAC_TO_VAR_UPDATES, TYPE_KEYS):
      for k, v in self.inference_arguments[t].items():
        if k != "plan":
          d[f"{key}.{k}"] = v
    return d

  @property
  def plan(self):
    if self._plan is None:
      from .. import engine  # pylint: disable=g-import-not-at-top
      object.__setattr__(self, "_plan", engine.Plan(self.flat_wiring(), flags=self.exec_flags))
      for t in FAC_TO_VAR_UPDATES:
        self.inference_arguments[t]["plan"] = self._plan
      register_context(self)
    return self._plan

  # ------------------------------------------------------------------------- state
  def _device(self, x):
    return self.plan._dev(x)  # pylint: disable=protected-access

  def _defaults(self):
    """Device copies of the BPState's arrays, uploaded once (the updates below never write into
    them: they copy first). Keeps init() free of host-to-device copies, so a step that calls it
    can be captured in a CUDA graph."""
    cached = getattr(self, "_default_arrays", None)
    if cached is None:
      cached = tuple(self._device(x.value) for x in (
          self.bp_state.log_potentials, self.bp_state.ftov_msgs, self.bp_state.evidence))
      object.__setattr__(self, "_default_arrays", cached)
    return cached

  def update(self, bp_arrays: Optional[BPArrays] = None, log_potentials_updates=None,
             ftov_msgs_updates=None, evidence_updates=None) -> BPArrays:
    fg_state = self.bp_state.fg_state
    if bp_arrays is not None:
      lp, msgs, ev = bp_arrays.log_potentials, bp_arrays.ftov_msgs, bp_arrays.evidence
    else:
      lp, msgs, ev = self._defaults()
    if log_potentials_updates is not None:
      lp = bpstate.update_log_potentials(lp, log_potentials_updates, fg_state)
    if ftov_msgs_updates is not None:
      msgs = bpstate.update_ftov_msgs(msgs, ftov_msgs_updates, fg_state)
    if evidence_updates is not None:
      ev = bpstate.update_evidence(ev, evidence_updates, fg_state)
    return BPArrays(log_potentials=lp, ftov_msgs=msgs, evidence=ev)

  def init(self, log_potentials_updates=None, ftov_msgs_updates=None,
           evidence_updates=None) -> BPArrays:
    return self.update(None, log_potentials_updates, ftov_msgs_updates, evidence_updates)

  def to_bp_state(self, bp_arrays: BPArrays) -> BPState:
    fg_state = self.bp_state.fg_state
    host = lambda x: np.asarray(x.detach().cpu().numpy() if _is_torch(x) else x)
    return BPState(
        log_potentials=LogPotentials(fg_state=fg_state, value=host(bp_arrays.log_potentials)),
        ftov_msgs=FToVMessages(fg_state=fg_state, value=host(bp_arrays.ftov_msgs)),
        evidence=Evidence(fg_state=fg_state, value=host(bp_arrays.evidence)),
    )

  def get_beliefs(self, bp_arrays: BPArrays) -> Dict[Hashable, Any]:
    """evidence.at[var_states_for_edge_states].add(ftov_msgs), unflattened per group."""
    from .. import autodiff  # pylint: disable=g-import-not-at-top
    if autodiff.wants_grad(bp_arrays.evidence, bp_arrays.ftov_msgs):
      flat = autodiff.beliefs(self.plan, bp_arrays.evidence, bp_arrays.ftov_msgs)
    else:
      flat = self.plan.beliefs(bp_arrays.evidence, bp_arrays.ftov_msgs)
    out = Beliefs(unflatten_beliefs(flat, self.bp_state.fg_state.variable_groups))
    out.flat = flat
    out.context = self
    return out


def unflatten_beliefs(flat_beliefs, variable_groups: Sequence[vgroup_mod.VarGroup],
                      per_state: bool = True) -> Dict[Hashable, Any]:
  """Splits flat (optionally batched) per-state data by variable group (inferer.py:228-248)."""
  beliefs = {}
  start = 0
  batched = flat_beliefs.ndim == 2
  for vg in variable_groups:
    length = int(np.asarray(vg.num_states).sum()) if per_state else vg.num_variables
    part = flat_beliefs[..., start:start + length]
    if batched and isinstance(vg, vgroup_mod.VarDict):
      offs = vg.state_offsets() if per_state else np.arange(vg.num_variables + 1)
      beliefs[vg] = {n: part[:, offs[i]:offs[i + 1]] if per_state else part[:, i]
                     for i, n in enumerate(vg.variable_names)}
    else:
      beliefs[vg] = vg.unflatten(part, per_state)
    start += length
  return beliefs


def _tree_map(fn, tree):
  if isinstance(tree, dict):
    return {k: _tree_map(fn, v) for k, v in tree.items()}
  return fn(tree)


def _argmax_last(x):
  from .. import engine  # pylint: disable=g-import-not-at-top
  return engine.argmax_last(x)


def decode_map_states(beliefs: Dict[Hashable, Any]) -> Dict[Hashable, Any]:
  """MAP states: argmax over each variable's states, first maximum wins (inferer.py:251-264).
  Beliefs from get_beliefs are decoded by the pgbp_decode kernel over the flat array, any other
  belief arrays by pgbp_argmax_rows."""
  ctx = getattr(beliefs, "context", None)
  if ctx is not None and getattr(beliefs, "flat", None) is not None and ctx.num_variables > 0:
    flat_map = ctx.plan.decode(beliefs.flat, ctx.num_variables)
    return unflatten_beliefs(flat_map, ctx.bp_state.fg_state.variable_groups, per_state=False)
  return _tree_map(_argmax_last, beliefs)
