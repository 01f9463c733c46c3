"""FactorGraph and FactorGraphState: PGMax's pgmax/fgraph/fgraph.py over NumPy.

Layout (identical to the reference, so BPArrays are interchangeable):
  * evidence: variable groups in order, each group's variables in their flat order, each variable's
    states contiguous (fgraph.py:94-124);
  * messages and potentials: factor types in registry order (Enum, OR, AND, Pool), then factor
    groups in insertion order (compute_offsets, fgraph.py:185-232);
  * wiring: each type's groups compiled and concatenated with edge / factor / config offsets
    (fgraph.py:234-256).
"""

import collections
import copy
import dataclasses
import types
from typing import Any, Dict, List, Mapping, Sequence, Tuple, Union

import numpy as np

from . import factor as factor_mod
from . import fgroup as fgroup_mod
from . import vgroup as vgroup_mod
from .factor import FAC_TO_VAR_UPDATES


class VarsToStarts(Mapping):
  """variable (hash, num_states) -> index of its first state in the flat evidence.

  Behaves like the reference's `vars_to_starts` dict; `starts_of` resolves whole arrays of variable
  hashes at once (each group's hashes are one contiguous range)."""

  def __init__(self, variable_groups):
    self._groups = list(variable_groups)
    hashes, counts, starts, offs = [], [], [], []
    total = 0
    for g in self._groups:
      so = g.state_offsets()
      hashes.append(hash(g))
      counts.append(g.num_variables)
      starts.append(total)
      offs.append(so)
      total += int(so[-1])
    order = np.argsort(np.asarray(hashes, dtype=np.int64), kind="stable")
    self._h = np.asarray(hashes, dtype=np.int64)[order]
    self._n = np.asarray(counts, dtype=np.int64)[order]
    self._base = np.asarray(starts, dtype=np.int64)[order]
    self._offs = [offs[i] for i in order]
    self._ns = [np.asarray(self._groups[i].num_states).reshape(-1).astype(np.int64) for i in order]
    self.num_var_states = total
    self._len = int(np.sum(counts))

  def _locate(self, hashes):
    hashes = np.asarray(hashes, dtype=np.int64)
    gi = np.searchsorted(self._h, hashes, side="right") - 1
    ok = gi >= 0
    gi_c = np.where(ok, gi, 0)
    idx = hashes - self._h[gi_c]
    ok &= (idx >= 0) & (idx < self._n[gi_c])
    return gi_c, idx, ok

  def starts_of(self, hashes, num_states=None) -> np.ndarray:
    gi, idx, ok = self._locate(hashes)
    out = np.empty(gi.shape[0], dtype=np.int64)
    for g in np.unique(gi):
      sel = gi == g
      ii = np.where(ok[sel], idx[sel], 0)
      out[sel] = self._base[g] + self._offs[g][ii]
      if num_states is not None:
        ok[sel] &= self._ns[g][ii] == np.asarray(num_states)[sel]
    if not ok.all():
      bad = int(np.nonzero(~ok)[0][0])
      raise ValueError(f"Variable {(int(np.asarray(hashes)[bad]),)} is not in the FactorGraph")
    return out

  def __getitem__(self, var):
    h, n = var
    gi, idx, ok = self._locate(np.array([h]))
    if not ok[0] or self._ns[gi[0]][idx[0]] != n:
      raise KeyError(var)
    return int(self._base[gi[0]] + self._offs[gi[0]][idx[0]])

  def __contains__(self, var):
    try:
      if not isinstance(var, tuple) or len(var) != 2:
        return False
      self[var]
      return True
    except (KeyError, TypeError, ValueError):
      return False

  def __iter__(self):
    for g in self._groups:
      yield from g.variables

  def __len__(self):
    return self._len


@dataclasses.dataclass(frozen=True, eq=False)
class FactorGraphState:
  """Static description of a compiled factor graph (fgraph.py:34-78)."""

  variable_groups: Sequence[vgroup_mod.VarGroup]
  vars_to_starts: Mapping[Tuple[int, int], int]
  num_var_states: int
  total_factor_num_states: int
  factor_type_to_msgs_range: Mapping[type, Tuple[int, int]]
  factor_type_to_potentials_range: Mapping[type, Tuple[int, int]]
  factor_group_to_potentials_starts: Mapping[Any, int]
  log_potentials: np.ndarray
  evidence_to_vars: np.ndarray
  wiring: Mapping[type, factor_mod.Wiring]

  def __post_init__(self):
    for f in dataclasses.fields(self):
      v = getattr(self, f.name)
      if isinstance(v, np.ndarray):
        v.flags.writeable = False
      if isinstance(v, dict):
        object.__setattr__(self, f.name, types.MappingProxyType(v))


@dataclasses.dataclass
class FactorGraph:
  """A factor graph: variable groups plus factor groups clustered by type (fgraph.py:81-371)."""

  variable_groups: Union[vgroup_mod.VarGroup, Sequence[vgroup_mod.VarGroup]]

  def __post_init__(self):
    if isinstance(self.variable_groups, vgroup_mod.VarGroup):
      self.variable_groups = [self.variable_groups]
    self.variable_groups = list(self.variable_groups)
    self._factor_types_to_groups = collections.OrderedDict(
        [(t, []) for t in FAC_TO_VAR_UPDATES])
    self._factor_types_to_variables_for_factors = collections.OrderedDict(
        [(t, set()) for t in FAC_TO_VAR_UPDATES])
    self._vars_to_starts = VarsToStarts(self.variable_groups)
    self._num_var_states = self._vars_to_starts.num_var_states
    self._cache = {}

  def __hash__(self) -> int:
    return hash(tuple(g for gs in self._factor_types_to_groups.values() for g in gs))

  def add_factors(self, factors) -> None:
    """Adds a Factor, a FactorGroup or a list of them (fgraph.py:137-183)."""
    if isinstance(factors, list):
      for f in factors:
        self.add_factors(f)
      return None
    if isinstance(factors, fgroup_mod.FactorGroup):
      group = factors
    elif isinstance(factors, factor_mod.Factor):
      group = fgroup_mod.SingleFactorGroup(variables_for_factors=[factors.variables],
                                           single_factor=factors)
    else:
      raise ValueError(f"Cannot add {type(factors)} to a FactorGraph")
    ftype = group.factor_type
    seen = self._factor_types_to_variables_for_factors[ftype]
    for vs in group.variables_for_factors:
      key = frozenset(vs)
      if len(vs) != len(key):
        raise ValueError(f"A Factor of type {ftype} involving variables {vs} contains variables"
                         " duplicates.")
      if key in seen:
        raise ValueError(f"A Factor of type {ftype} involving variables {key} already exists."
                         " Please merge the corresponding factors.")
      seen.add(key)
    self._factor_types_to_groups[ftype].append(group)
    self._cache.clear()

  def compute_offsets(self) -> None:
    if "offsets" in self._cache:
      return
    msgs_range, group_msgs, pot_range, group_pot = (collections.OrderedDict() for _ in range(4))
    ns_cum, cfg_cum = 0, 0
    for ftype, groups in self._factor_types_to_groups.items():
      ns0, cfg0 = ns_cum, cfg_cum
      for g in groups:
        group_msgs[g] = ns_cum
        group_pot[g] = cfg_cum
        ns_cum += int(g.factor_edges_num_states.sum())
        cfg_cum += int(g.factor_group_log_potentials.shape[0])
      msgs_range[ftype] = (ns0, ns_cum)
      pot_range[ftype] = (cfg0, cfg_cum)
    self._factor_type_to_msgs_range = msgs_range
    self._factor_group_to_msgs_starts = group_msgs
    self._factor_type_to_potentials_range = pot_range
    self._factor_group_to_potentials_starts = group_pot
    self._total_factor_num_states = ns_cum
    self._total_factor_num_configs = cfg_cum
    self._cache["offsets"] = True

  @property
  def wiring(self):
    if "wiring" not in self._cache:
      w = collections.OrderedDict()
      for ftype, groups in self._factor_types_to_groups.items():
        w[ftype] = ftype.concatenate_wirings(
            [g.compile_wiring(self._vars_to_starts) for g in groups])
      self._cache["wiring"] = w
    return self._cache["wiring"]

  @property
  def log_potentials(self):
    if "log_potentials" not in self._cache:
      lp = collections.OrderedDict()
      for ftype, groups in self._factor_types_to_groups.items():
        lp[ftype] = (np.concatenate([g.factor_group_log_potentials for g in groups])
                     if groups else np.empty((0,)))
      self._cache["log_potentials"] = lp
    return self._cache["log_potentials"]

  @property
  def factors(self):
    out = collections.OrderedDict()
    for ftype, groups in self._factor_types_to_groups.items():
      out[ftype] = tuple(f for g in groups for f in g.factors)
    return out

  @property
  def factor_groups(self):
    return self._factor_types_to_groups

  @property
  def evidence_to_vars(self) -> np.ndarray:
    counts = np.concatenate([np.asarray(g.num_states).reshape(-1) for g in self.variable_groups]
                            ) if self.variable_groups else np.zeros(0, np.int64)
    return np.repeat(np.arange(counts.shape[0], dtype=np.int64), counts.astype(np.int64))

  @property
  def fg_state(self) -> FactorGraphState:
    if "fg_state" not in self._cache:
      self.compute_offsets()
      lp = np.concatenate([self.log_potentials[t] for t in self.log_potentials]).astype(
          np.float64, copy=False) if self.log_potentials else np.empty((0,))
      self._cache["fg_state"] = FactorGraphState(
          variable_groups=self.variable_groups,
          vars_to_starts=self._vars_to_starts,
          num_var_states=self._num_var_states,
          total_factor_num_states=self._total_factor_num_states,
          factor_type_to_msgs_range=copy.copy(self._factor_type_to_msgs_range),
          factor_type_to_potentials_range=copy.copy(self._factor_type_to_potentials_range),
          factor_group_to_potentials_starts=copy.copy(self._factor_group_to_potentials_starts),
          log_potentials=lp,
          evidence_to_vars=self.evidence_to_vars,
          wiring=self.wiring,
      )
    return self._cache["fg_state"]

  @property
  def bp_state(self):
    self.compute_offsets()
    from .infer import bp_state  # pylint: disable=g-import-not-at-top
    return bp_state.BPState(
        log_potentials=bp_state.LogPotentials(fg_state=self.fg_state),
        ftov_msgs=bp_state.FToVMessages(fg_state=self.fg_state),
        evidence=bp_state.Evidence(fg_state=self.fg_state),
    )
