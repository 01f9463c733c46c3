"""Belief-propagation state containers: PGMax's pgmax/infer/bp_state.py.

`BPArrays` is the flat state the engine consumes and returns (log_potentials [P], ftov_msgs
[E_s], evidence [N_vs], each optionally with a leading batch axis, as `jax.vmap` would produce).
Fields are torch tensors on the GPU after `init` / `run`, or NumPy arrays when built on the host.
The structured views (LogPotentials, FToVMessages, Evidence, BPState) keep host NumPy values.
"""

import dataclasses
from typing import Any, Dict, Optional, Tuple, Union

import numpy as np

from .. import fgroup as fgroup_mod
from .. import vgroup as vgroup_mod


def _is_torch(x):
  return type(x).__module__.startswith("torch")


def _f32(x):
  """float32 copy (device tensors stay on their device)."""
  if _is_torch(x):
    return x.float().clone()
  return np.array(x, dtype=np.float32)


def _set_slice(arr, start, stop, data):
  """arr[..., start:stop] = data, broadcasting a batched update over a shared array."""
  lead = tuple(data.shape[:-1])
  if _is_torch(arr):
    import torch  # pylint: disable=g-import-not-at-top
    data = data.to(device=arr.device, dtype=arr.dtype) if _is_torch(data) else torch.as_tensor(
        np.asarray(data, dtype=np.float32), device=arr.device)
    if lead and arr.ndim == 1:
      arr = arr.expand(lead + tuple(arr.shape)).clone()
    arr[..., start:stop] = data
    return arr
  data = np.asarray(data.detach().cpu().numpy() if _is_torch(data) else data, dtype=np.float32)
  if lead and arr.ndim == 1:
    arr = np.broadcast_to(arr, lead + arr.shape).copy()
  arr[..., start:stop] = data
  return arr


@dataclasses.dataclass(frozen=True, eq=False)
class BPArrays:
  """Flat arrays of belief propagation (pgmax/infer/bp_state.py:30-55)."""

  log_potentials: Any
  ftov_msgs: Any
  evidence: Any

  def __post_init__(self):
    for f in dataclasses.fields(self):
      v = getattr(self, f.name)
      if isinstance(v, np.ndarray):
        v.flags.writeable = False

  @property
  def batch_shape(self) -> Tuple[int, ...]:
    for v, n in ((self.ftov_msgs, 1), (self.evidence, 1), (self.log_potentials, 1)):
      if v is not None and v.ndim == 2:
        return (int(v.shape[0]),)
    return ()


def update_log_potentials(log_potentials, updates: Dict[Any, Any], fg_state):
  """Writes factor-group log potentials into the flat array (bp_state.py:58-101)."""
  out = _f32(log_potentials)
  for group, data in updates.items():
    if group in fg_state.factor_group_to_potentials_starts:
      batched = _batched_group_data(group, data)
      flat = (group.flatten(data) if not batched else
              _stack([group.flatten(data[i]) for i in range(data.shape[0])]))
      expected = group.factor_group_log_potentials.shape
      if tuple(flat.shape[-1:]) != tuple(expected):
        raise ValueError(f"Expected log potentials shape {expected} for factor group. Got"
                         f" incompatible data shape {tuple(data.shape)}.")
      start = fg_state.factor_group_to_potentials_starts[group]
      out = _set_slice(out, start, start + flat.shape[-1], flat)
    else:
      raise ValueError("Invalid FactorGroup for log potentials updates.")
  return out


def _batched_group_data(group, data):
  try:
    group.flatten(data)
    return False
  except (ValueError, NotImplementedError):
    if getattr(data, "ndim", 0) >= 2:
      try:
        group.flatten(data[0])
        return True
      except (ValueError, NotImplementedError):
        pass
    raise


def _stack(parts):
  if parts and _is_torch(parts[0]):
    import torch  # pylint: disable=g-import-not-at-top
    return torch.stack(parts)
  return np.stack([np.asarray(p) for p in parts])


def update_ftov_msgs(ftov_msgs, updates: Dict[Any, Any], fg_state):
  """Sets messages of a factor type, or spreads a variable's message over its edges
  (bp_state.py:172-234)."""
  out = _f32(ftov_msgs)
  for name, data in updates.items():
    if name in fg_state.factor_type_to_msgs_range:
      s, e = fg_state.factor_type_to_msgs_range[name]
      if tuple(data.shape[-1:]) != (e - s,) or data.ndim > 2:
        raise ValueError(f"Expected ftov_msgs shape {(e - s,)} for factor type {name}. Got"
                         f" incompatible shape {tuple(data.shape)}.")
      out = _set_slice(out, s, e, data)
    elif name in fg_state.vars_to_starts:
      n = int(name[1])
      if tuple(data.shape[-1:]) != (n,) or data.ndim > 2:
        raise ValueError(f"Expected ftov_msgs shape {(n,)} for variable {name}. Got"
                         f" incompatible shape {tuple(data.shape)}.")
      vs = np.concatenate([w.var_states_for_edges[..., 0] for w in fg_state.wiring.values()])
      starts = np.nonzero(vs == fg_state.vars_to_starts[name])[0]
      if starts.shape[0] == 0:
        continue
      if _is_torch(data):
        spread = data.float() / starts.shape[0]
      else:
        spread = np.asarray(data, dtype=np.float32) / np.float32(starts.shape[0])
      for st in starts:
        out = _set_slice(out, int(st), int(st) + n, spread)
    else:
      raise ValueError("Provided variable or factor type is not in the FactorGraph")
  return out


def update_evidence(evidence, updates: Dict[Any, Any], fg_state):
  """Writes evidence of variable groups or single variables (bp_state.py:292-342)."""
  out = _f32(evidence)
  for name, data in updates.items():
    if isinstance(name, vgroup_mod.VarGroup) and name in fg_state.variable_groups:
      flat = name.flatten(data)
      start = fg_state.vars_to_starts[name.variables[0]]
      out = _set_slice(out, start, start + flat.shape[-1], flat)
    elif name in fg_state.vars_to_starts:
      start = fg_state.vars_to_starts[name]
      n = int(name[1])
      if tuple(data.shape[-1:]) != (n,) or data.ndim > 2:
        raise ValueError(f"Expected evidence shape {(n,)} for variable {name}. Got incompatible"
                         f" shape {tuple(data.shape)}.")
      out = _set_slice(out, start, start + n, data)
    else:
      raise ValueError("Got evidence for a variable or a VarGroup not in the FactorGraph!")
  return out


def _host(x):
  return np.asarray(x.detach().cpu().numpy() if _is_torch(x) else x)


@dataclasses.dataclass(frozen=True, eq=False)
class LogPotentials:
  """Flat log potentials with per-group access (bp_state.py:104-169)."""

  fg_state: Any
  value: Optional[np.ndarray] = None

  def __post_init__(self):
    if self.value is None:
      object.__setattr__(self, "value", self.fg_state.log_potentials)
    elif tuple(self.value.shape) != tuple(self.fg_state.log_potentials.shape):
      raise ValueError(f"Expected log potentials shape {self.fg_state.log_potentials.shape}. "
                       f"Got {tuple(self.value.shape)}.")

  def __getitem__(self, group):
    if group in self.fg_state.factor_group_to_potentials_starts:
      start = self.fg_state.factor_group_to_potentials_starts[group]
      return self.value[start:start + group.factor_group_log_potentials.shape[0]]
    raise ValueError("Invalid FactorGroup queried to access log potentials.")

  def __setitem__(self, group, data):
    object.__setattr__(self, "value", _host(update_log_potentials(self.value, {group: data},
                                                                  self.fg_state)))


@dataclasses.dataclass(frozen=True, eq=False)
class FToVMessages:
  """Flat factor-to-variable messages (bp_state.py:237-289)."""

  fg_state: Any
  value: Optional[np.ndarray] = None

  def __post_init__(self):
    n = self.fg_state.total_factor_num_states
    if self.value is None:
      object.__setattr__(self, "value", np.zeros(n))
    elif tuple(self.value.shape) != (n,):
      raise ValueError(f"Expected messages shape {(n,)}. Got {tuple(self.value.shape)}.")

  def __setitem__(self, variable, data):
    object.__setattr__(self, "value", _host(update_ftov_msgs(self.value, {variable: data},
                                                             self.fg_state)))


@dataclasses.dataclass(frozen=True, eq=False)
class Evidence:
  """Flat evidence (bp_state.py:345-405)."""

  fg_state: Any
  value: Optional[np.ndarray] = None

  def __post_init__(self):
    n = self.fg_state.num_var_states
    if self.value is None:
      object.__setattr__(self, "value", np.zeros((n,)))
    elif tuple(self.value.shape) != (n,):
      raise ValueError(f"Expected evidence shape {(n,)}. Got {tuple(self.value.shape)}.")

  def __getitem__(self, variable):
    start = self.fg_state.vars_to_starts[variable]
    return self.value[start:start + variable[1]]

  def __setitem__(self, name, data):
    object.__setattr__(self, "value", _host(update_evidence(self.value, {name: data},
                                                            self.fg_state)))


@dataclasses.dataclass(frozen=True, eq=False)
class BPState:
  """log potentials + messages + evidence of one factor graph (bp_state.py:408-436)."""

  log_potentials: LogPotentials
  ftov_msgs: FToVMessages
  evidence: Evidence

  def __post_init__(self):
    if (self.log_potentials.fg_state != self.ftov_msgs.fg_state) or (
        self.ftov_msgs.fg_state != self.evidence.fg_state):
      raise ValueError("log_potentials, ftov_msgs and evidence should be derived from the"
                       " same fg_state.")

  @property
  def fg_state(self):
    return self.log_potentials.fg_state
