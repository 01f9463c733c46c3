"""Factors and their wirings: PGMax's pgmax/factor/ package, re-implemented over NumPy.

The wiring arrays are the flat layout the engine consumes, identical to PGMax's:
  * `var_states_for_edges` [E_s, 3]: per edge state its (variable state, edge, factor) indices
    (pgmax/factor/factor.py:27-57, 197-225);
  * EnumWiring.factor_configs_edge_states [C, 2]: per (config, variable) row its global config
    index and edge state (enum.py:33-72, 364-394);
  * LogicalWiring.parents_edge_states [P, 2] / children_edge_states [F] with the relevant state
    offset (+1 OR, -1 AND) (logical.py:37-104, 458-488);
  * PoolWiring: the logical layout with offset +1 (pool.py:32-83, 151-180).
Compilation here is vectorised NumPy instead of numba loops; `concatenate_wirings` applies the same
edge / factor / config offsets as the reference.

`FAC_TO_VAR_UPDATES` maps each factor type to its factor-to-variable update, run on the GPU by
libpgbp (`pgbp_factor_update`); the registry order Enum, OR, AND, Pool fixes the message layout
(pgmax/factor/__init__.py:37-44).
"""

import collections
import dataclasses
from typing import Any, Dict, List, Mapping, Optional, Sequence, Tuple, Union

import numpy as np


# ----------------------------------------------------------------------------- wirings


@dataclasses.dataclass(frozen=True, eq=False)
class Wiring:
  var_states_for_edges: np.ndarray

  def __post_init__(self):
    for f in dataclasses.fields(self):
      v = getattr(self, f.name)
      if isinstance(v, np.ndarray):
        v.flags.writeable = False

  def get_inference_arguments(self):
    raise NotImplementedError("Please subclass the Wiring class and override this method.")


@dataclasses.dataclass(frozen=True, eq=False)
class EnumWiring(Wiring):
  factor_configs_edge_states: np.ndarray

  def get_inference_arguments(self) -> Dict[str, Any]:
    fces = self.factor_configs_edge_states
    num_val_configs = 0 if fces.shape[0] == 0 else int(fces[-1, 0]) + 1
    vse = self.var_states_for_edges
    num_factors = 0 if vse.shape[0] == 0 else int(vse[-1, 2]) + 1
    object.__setattr__(self, "num_val_configs", num_val_configs)
    object.__setattr__(self, "num_factors", num_factors)
    return {
        "factor_configs_indices": fces[..., 0],
        "factor_configs_edge_states": fces[..., 1],
        "num_val_configs": num_val_configs,
        "num_factors": num_factors,
    }


@dataclasses.dataclass(frozen=True, eq=False)
class LogicalWiring(Wiring):
  parents_edge_states: np.ndarray
  children_edge_states: np.ndarray
  edge_states_offset: int

  def get_inference_arguments(self) -> Dict[str, Any]:
    if self.children_edge_states.shape[0] > 0:
      idx = self.parents_edge_states[:, 0]
      n = self.children_edge_states.shape[0]
      if np.unique(idx).shape[0] != n:
        raise ValueError(f"The LogicalWiring must have {n} different LogicalFactor indices")
      if idx.max() >= n:
        raise ValueError(f"The highest LogicalFactor index must be {n - 1}")
      if self.edge_states_offset not in (1, -1):
        raise ValueError("The LogicalWiring's edge_states_offset must be 1 (for OR) and -1"
                         f" (for AND), but is {self.edge_states_offset}")
    return {
        "parents_factor_indices": self.parents_edge_states[..., 0],
        "parents_msg_indices": self.parents_edge_states[..., 1],
        "children_edge_states": self.children_edge_states,
        "edge_states_offset": self.edge_states_offset,
    }


@dataclasses.dataclass(frozen=True, eq=False)
class PoolWiring(Wiring):
  pool_choices_edge_states: np.ndarray
  pool_indicators_edge_states: np.ndarray

  def get_inference_arguments(self) -> Dict[str, Any]:
    if self.pool_choices_edge_states.shape[0] > 0:
      idx = self.pool_choices_edge_states[:, 0]
      n = self.pool_indicators_edge_states.shape[0]
      if np.unique(idx).shape[0] != n:
        raise ValueError(f"The PoolWiring must have {n} different PoolFactor indices")
      if idx.max() >= n:
        raise ValueError(f"The highest PoolFactor index must be {n - 1}")
    return {
        "pool_choices_factor_indices": self.pool_choices_edge_states[..., 0],
        "pool_choices_msg_indices": self.pool_choices_edge_states[..., 1],
        "pool_indicators_edge_states": self.pool_indicators_edge_states,
    }


def _offsets(counts):
  return np.concatenate([[0], np.cumsum(counts)])[:-1].astype(np.int64)


def concatenate_var_states_for_edges(list_var_states_for_edges: Sequence[np.ndarray]) -> np.ndarray:
  """Stacks wirings, shifting edge and factor indices (pgmax/factor/factor.py:132-192)."""
  if list_var_states_for_edges is None:
    raise ValueError("list_var_states_for_edges cannot be None")
  parts = []
  for v in list_var_states_for_edges:
    if v is None:
      raise ValueError("var_states_for_edges cannot be None")
    if v.shape[0] > 0:
      parts.append(v)
  if not parts:
    return np.empty((0, 3), dtype=np.int64)
  edge_off = _offsets([p[-1, 1] + 1 for p in parts])
  fac_off = _offsets([p[-1, 2] + 1 for p in parts])
  return np.concatenate(
      [p + np.array([[0, edge_off[i], fac_off[i]]], dtype=np.int64) for i, p in enumerate(parts)],
      axis=0)


def compile_var_states_for_edges(factor_edges_num_states: np.ndarray,
                                 first_var_state_by_edges: np.ndarray,
                                 factor_indices: np.ndarray) -> np.ndarray:
  """[E_s, 3] rows (var state, edge, factor) for edges with the given state counts."""
  ns = np.asarray(factor_edges_num_states, dtype=np.int64)
  n_es = int(ns.sum())
  edge_of = np.repeat(np.arange(ns.shape[0], dtype=np.int64), ns)
  starts = np.concatenate([[0], np.cumsum(ns)])[:-1]
  within = np.arange(n_es, dtype=np.int64) - starts[edge_of]
  out = np.empty((n_es, 3), dtype=np.int64)
  out[:, 0] = np.asarray(first_var_state_by_edges, dtype=np.int64)[edge_of] + within
  out[:, 1] = edge_of
  out[:, 2] = np.asarray(factor_indices, dtype=np.int64)[edge_of]
  return out


# ----------------------------------------------------------------------------- factors


@dataclasses.dataclass(frozen=True, eq=False)
class Factor:
  """Base factor: variables are (hash, num_states) tuples (pgmax/factor/factor.py:60-129)."""

  variables: List[Tuple[int, int]]
  log_potentials: np.ndarray

  def __post_init__(self):
    if not hasattr(self, "compile_wiring"):
      raise NotImplementedError("Please implement compile_wiring in for your factor")

  @staticmethod
  def concatenate_wirings(wirings):
    raise NotImplementedError("Please subclass the Wiring class and override this method.")


@dataclasses.dataclass(frozen=True, eq=False)
class EnumFactor(Factor):
  """Explicit table of valid configurations (pgmax/factor/enum.py:75-135)."""

  factor_configs: np.ndarray
  log_potentials: np.ndarray

  def __post_init__(self):
    self.factor_configs.flags.writeable = False
    if not np.issubdtype(self.factor_configs.dtype, np.integer):
      raise ValueError(f"Configurations should be integers. Got {self.factor_configs.dtype}.")
    if not np.issubdtype(self.log_potentials.dtype, np.floating):
      raise ValueError(f"Potential should be floats. Got {self.log_potentials.dtype}.")
    if self.factor_configs.ndim != 2:
      raise ValueError("factor_configs should be a 2D array containing a list of valid"
                       " configurations for EnumFactor. Got a factor_configs array of shape"
                       f" {self.factor_configs.shape}.")
    if len(self.variables) != self.factor_configs.shape[1]:
      raise ValueError(f"Number of variables {len(self.variables)} doesn't match given"
                       f" configurations {self.factor_configs.shape}")
    if self.log_potentials.shape != (self.factor_configs.shape[0],):
      raise ValueError("Expected log potentials of shape"
                       f" {(self.factor_configs.shape[0],)} for"
                       f" ({self.factor_configs.shape[0]}) valid configurations. Got log"
                       f" potentials of shape {self.log_potentials.shape}.")
    ns = np.array([v[1] for v in self.variables])
    if not np.logical_and(self.factor_configs >= 0, self.factor_configs < ns[None]).all():
      raise ValueError("Invalid configurations for given variables")

  @staticmethod
  def concatenate_wirings(wirings: Sequence[EnumWiring]) -> EnumWiring:
    if not wirings:
      return EnumWiring(var_states_for_edges=np.empty((0, 3), dtype=np.int64),
                        factor_configs_edge_states=np.empty((0, 2), dtype=np.int64))
    vse = concatenate_var_states_for_edges([w.var_states_for_edges for w in wirings])
    cfg_off = _offsets([w.factor_configs_edge_states[-1, 0] + 1 if w.factor_configs_edge_states.shape[0]
                        else 0 for w in wirings])
    es_off = _offsets([w.var_states_for_edges.shape[0] for w in wirings])
    fces = np.concatenate(
        [w.factor_configs_edge_states + np.array([[cfg_off[i], es_off[i]]], dtype=np.int64)
         for i, w in enumerate(wirings)], axis=0)
    return EnumWiring(var_states_for_edges=vse, factor_configs_edge_states=fces)

  @staticmethod
  def compile_wiring(factor_edges_num_states: np.ndarray, first_var_states: np.ndarray,
                     factor_configs: np.ndarray, num_factors: int) -> EnumWiring:
    """All factors share `factor_configs` [n_cfg, n_vars]; edges are listed factor by factor."""
    n_cfg, n_vars = factor_configs.shape
    if factor_edges_num_states.shape != (num_factors * n_vars,):
      raise ValueError(f"Expected factor_edges_num_states shape is {(num_factors * n_vars,)}."
                       f" Got {factor_edges_num_states.shape}.")
    fidx = np.repeat(np.arange(num_factors, dtype=np.int64), n_vars)
    vse = compile_var_states_for_edges(factor_edges_num_states, first_var_states, fidx)
    edge_starts = np.concatenate([[0], np.cumsum(factor_edges_num_states)])[:-1].astype(np.int64)
    edge_starts = edge_starts.reshape(num_factors, n_vars)
    col1 = edge_starts[:, None, :] + np.asarray(factor_configs, dtype=np.int64)[None, :, :]
    fces = np.empty((num_factors * n_cfg * n_vars, 2), dtype=np.int64)
    fces[:, 0] = np.repeat(np.arange(num_factors * n_cfg, dtype=np.int64), n_vars)
    fces[:, 1] = col1.reshape(-1)
    return EnumWiring(var_states_for_edges=vse, factor_configs_edge_states=fces)


@dataclasses.dataclass(frozen=True, eq=False)
class LogicalFactor(Factor):
  """OR / AND factor (p1, ..., pn, c) with binary variables (pgmax/factor/logical.py:107-206)."""

  log_potentials: np.ndarray = dataclasses.field(init=False,
                                                 default_factory=lambda: np.empty((0,)))
  edge_states_offset: int = dataclasses.field(init=False)

  def __post_init__(self):
    if len(self.variables) < 2:
      raise ValueError("A LogicalFactor requires at least one parent variable and one child"
                       " variable")
    if not np.all([v[1] == 2 for v in self.variables]):
      raise ValueError("All the variables in a LogicalFactor should be binary")

  @staticmethod
  def concatenate_wirings(wirings: Sequence[LogicalWiring]) -> LogicalWiring:
    if not wirings:
      return LogicalWiring(var_states_for_edges=np.empty((0, 3), dtype=np.int64),
                           parents_edge_states=np.empty((0, 2), dtype=np.int64),
                           children_edge_states=np.empty((0,), dtype=np.int64),
                           edge_states_offset=1)
    vse = concatenate_var_states_for_edges([w.var_states_for_edges for w in wirings])
    fac_off = _offsets([w.parents_edge_states[-1, 0] + 1 for w in wirings])
    es_off = _offsets([w.var_states_for_edges.shape[0] for w in wirings])
    parents = [w.parents_edge_states + np.array([[fac_off[i], es_off[i]]], dtype=np.int64)
               for i, w in enumerate(wirings)]
    children = [w.children_edge_states + es_off[i] for i, w in enumerate(wirings)]
    return LogicalWiring(var_states_for_edges=vse,
                         parents_edge_states=np.concatenate(parents, axis=0),
                         children_edge_states=np.concatenate(children, axis=0),
                         edge_states_offset=wirings[0].edge_states_offset)

  @staticmethod
  def compile_wiring(factor_edges_num_states: np.ndarray, first_var_states: np.ndarray,
                     factor_sizes: np.ndarray, edge_states_offset: int) -> LogicalWiring:
    """Parents then child per factor; every variable binary. The relevant state is 1 for OR and
    0 for AND; parents_edge_states[:, 1] points at the other state (logical.py:262-279)."""
    sizes = np.asarray(factor_sizes, dtype=np.int64)
    fidx = np.repeat(np.arange(sizes.shape[0], dtype=np.int64), sizes)
    vse = compile_var_states_for_edges(np.full(fidx.shape[0], 2, dtype=np.int64), first_var_states,
                                       fidx)
    num_parents = sizes - 1
    relevant_state = (-edge_states_offset + 1) // 2
    fstart = np.concatenate([[0], np.cumsum(2 * sizes)])[:-1]
    pf = np.repeat(np.arange(sizes.shape[0], dtype=np.int64), num_parents)
    pstart = np.concatenate([[0], np.cumsum(num_parents)])[:-1]
    within = np.arange(pf.shape[0], dtype=np.int64) - pstart[pf]
    parents = np.empty((pf.shape[0], 2), dtype=np.int64)
    parents[:, 0] = pf
    parents[:, 1] = fstart[pf] + relevant_state + 2 * within
    children = fstart + 2 * num_parents + relevant_state
    return LogicalWiring(var_states_for_edges=vse, parents_edge_states=parents,
                         children_edge_states=children, edge_states_offset=edge_states_offset)


@dataclasses.dataclass(frozen=True, eq=False)
class ORFactor(LogicalFactor):
  edge_states_offset: int = dataclasses.field(init=False, default=1)


@dataclasses.dataclass(frozen=True, eq=False)
class ANDFactor(LogicalFactor):
  edge_states_offset: int = dataclasses.field(init=False, default=-1)


@dataclasses.dataclass(frozen=True, eq=False)
class PoolFactor(Factor):
  """Pool factor (pc1, ..., pcn, pi): all zero, or pi = 1 and exactly one choice on
  (pgmax/factor/pool.py:86-272)."""

  log_potentials: np.ndarray = dataclasses.field(init=False,
                                                 default_factory=lambda: np.empty((0,)))

  def __post_init__(self):
    if len(self.variables) < 2:
      raise ValueError("A PoolFactor requires at least one pool choice and one pool indicator.")
    if not np.all([v[1] == 2 for v in self.variables]):
      raise ValueError("All the variables in a PoolFactor should all be binary")

  @staticmethod
  def concatenate_wirings(wirings: Sequence[PoolWiring]) -> PoolWiring:
    if not wirings:
      return PoolWiring(var_states_for_edges=np.empty((0, 3), dtype=np.int64),
                        pool_choices_edge_states=np.empty((0, 2), dtype=np.int64),
                        pool_indicators_edge_states=np.empty((0,), dtype=np.int64))
    lw = LogicalFactor.concatenate_wirings([
        LogicalWiring(var_states_for_edges=w.var_states_for_edges,
                      parents_edge_states=w.pool_choices_edge_states,
                      children_edge_states=w.pool_indicators_edge_states, edge_states_offset=1)
        for w in wirings])
    return PoolWiring(var_states_for_edges=lw.var_states_for_edges,
                      pool_choices_edge_states=lw.parents_edge_states,
                      pool_indicators_edge_states=lw.children_edge_states)

  @staticmethod
  def compile_wiring(factor_edges_num_states: np.ndarray, first_var_states: np.ndarray,
                     factor_sizes: np.ndarray) -> PoolWiring:
    lw = LogicalFactor.compile_wiring(factor_edges_num_states, first_var_states, factor_sizes, 1)
    return PoolWiring(var_states_for_edges=lw.var_states_for_edges,
                      pool_choices_edge_states=lw.parents_edge_states,
                      pool_indicators_edge_states=lw.children_edge_states)


# ----------------------------------------------------------------------------- device updates


def _factor_update(ftype_index, vtof_msgs, log_potentials, temperature, normalize, plan):
  if plan is None:
    raise ValueError("pgmax_gb300 factor updates run on a compiled plan: pass the `plan` entry of "
                     "InfererContext.inference_arguments[factor_type]")
  return plan.factor_update(ftype_index, vtof_msgs, log_potentials, temperature, normalize)


def pass_enum_fac_to_var_messages(vtof_msgs, factor_configs_indices=None,
                                  factor_configs_edge_states=None, log_potentials=None,
                                  num_val_configs=None, num_factors=None, temperature=0.0,
                                  normalize=True, plan=None):
  """EnumFactor update (pgmax/factor/enum.py:398-475) on the GPU. `normalize` is unused."""
  del factor_configs_indices, factor_configs_edge_states, num_val_configs, num_factors
  return _factor_update(0, vtof_msgs, log_potentials, temperature, normalize, plan)


def pass_logical_fac_to_var_messages(vtof_msgs, parents_factor_indices=None,
                                     parents_msg_indices=None, children_edge_states=None,
                                     edge_states_offset=1, temperature=0.0, normalize=True,
                                     log_potentials=None, plan=None):
  """OR / AND update (pgmax/factor/logical.py:492-779) on the GPU."""
  del parents_factor_indices, parents_msg_indices, children_edge_states, log_potentials
  return _factor_update(1 if edge_states_offset == 1 else 2, vtof_msgs, None, temperature,
                        normalize, plan)


def pass_pool_fac_to_var_messages(vtof_msgs, pool_choices_factor_indices=None,
                                  pool_choices_msg_indices=None, pool_indicators_edge_states=None,
                                  temperature=0.0, normalize=True, log_potentials=None, plan=None):
  """Pool update (pgmax/factor/pool.py:276-474) on the GPU."""
  del pool_choices_factor_indices, pool_choices_msg_indices, pool_indicators_edge_states
  del log_potentials
  return _factor_update(3, vtof_msgs, None, temperature, normalize, plan)


FAC_TO_VAR_UPDATES = collections.OrderedDict([
    (EnumFactor, pass_enum_fac_to_var_messages),
    (ORFactor, pass_logical_fac_to_var_messages),
    (ANDFactor, pass_logical_fac_to_var_messages),
    (PoolFactor, pass_pool_fac_to_var_messages),
])
