"""Variable groups: the same classes and flat layouts as PGMax's pgmax/vgroup/ package.

A variable is the tuple (hash, num_states). A group's hashes are `group_hash + index` with
`group_hash = (id(group) mod 2^32) * 1e9`, so variables of different groups never collide
(pgmax/vgroup/vgroup.py:46-51). Flat per-state data (evidence, beliefs) lists each variable's
states in the group's variable order (varray.py:129-207, vdict.py:87-189).

Host data is NumPy; `unflatten` of a torch tensor (device beliefs) stays in torch.
"""

import dataclasses
from typing import Any, Dict, Hashable, List, Tuple, Union

import numpy as np

MAX_SIZE = 1e9


def _is_torch(x):
  return type(x).__module__.startswith("torch")


@dataclasses.dataclass(frozen=True, eq=False)
class VarGroup:
  """Base class of variable groups (pgmax/vgroup/vgroup.py:29-137)."""

  num_states: Union[int, np.ndarray]
  _hash: int = dataclasses.field(init=False)

  def __post_init__(self):
    this_hash = (id(self) % 2**32) * int(MAX_SIZE)
    assert this_hash < 2**63
    object.__setattr__(self, "_hash", this_hash)

  def __hash__(self):
    return self._hash

  def __eq__(self, other):
    return hash(self) == hash(other)

  def __lt__(self, other):
    return hash(self) < hash(other)

  def __getitem__(self, val):
    raise NotImplementedError("Please subclass the VarGroup class and override this method")

  @property
  def variable_hashes(self) -> np.ndarray:
    raise NotImplementedError("Please subclass the VarGroup class and override this method")

  @property
  def variables(self) -> List[Tuple[int, int]]:
    cached = self.__dict__.get("_variables")
    if cached is None:
      cached = list(zip(self.variable_hashes.flatten(), self.num_states.flatten()))
      object.__setattr__(self, "_variables", cached)
    return cached

  @property
  def num_variables(self) -> int:
    return int(np.asarray(self.num_states).size)

  def state_offsets(self) -> np.ndarray:
    """Start of each variable's states within the group's flat per-state data, plus the end."""
    ns = np.asarray(self.num_states).reshape(-1).astype(np.int64)
    return np.concatenate([[0], np.cumsum(ns)])

  def flatten(self, data: Any):
    raise NotImplementedError("Please subclass the VarGroup class and override this method")

  def unflatten(self, flat_data, per_state: bool):
    raise NotImplementedError("Please subclass the VarGroup class and override this method")


def _check_num_states(num_states, shape):
  if np.isscalar(num_states):
    return np.full(shape, fill_value=num_states, dtype=np.int64)
  if isinstance(num_states, np.ndarray) and np.issubdtype(num_states.dtype, np.integer):
    if num_states.shape != tuple(shape):
      raise ValueError(f"Expected num_states shape {tuple(shape)}. Got {num_states.shape}.")
    return num_states
  raise ValueError("num_states should be an integer or a NumPy array of dtype int")


@dataclasses.dataclass(frozen=True, eq=False)
class NDVarArray(VarGroup):
  """An n-dimensional grid of variables (pgmax/vgroup/varray.py:27-207)."""

  shape: Tuple[int, ...]
  _hash: int = dataclasses.field(init=False)

  def __post_init__(self):
    super().__post_init__()
    if np.prod(self.shape) > int(MAX_SIZE):
      raise ValueError(f"Currently only support NDVarArray of size smaller than {int(MAX_SIZE)}."
                       f" Got {np.prod(self.shape)}")
    object.__setattr__(self, "num_states", _check_num_states(self.num_states, tuple(self.shape)))

  def __repr__(self) -> str:
    ns = self.num_states
    if ns.size == 0:
      s = f"num_states={ns}"
    elif ns.min() == ns.max():
      s = f"num_states={ns.min()}"
    else:
      s = f"min_num_states={ns.min()}, max_num_states={ns.max()}"
    return f"NDVarArray(shape={self.shape}, {s}, _hash={self._hash})"

  def __getitem__(self, val):
    names = self.variable_hashes[val]
    ns = self.num_states[val]
    if isinstance(names, np.ndarray):
      return list(zip(names.flatten(), ns.flatten()))
    return (names, ns)

  @property
  def variable_hashes(self) -> np.ndarray:
    cached = self.__dict__.get("_variable_hashes")
    if cached is None:
      cached = self.__hash__() + np.arange(int(np.prod(self.shape)), dtype=np.int64).reshape(self.shape)
      object.__setattr__(self, "_variable_hashes", cached)
    return cached

  def _uniform_states(self) -> bool:
    """Every variable has the maximum number of states: per-state data needs no mask."""
    return bool(np.all(self.num_states == self.num_states.max(initial=0)))

  def _state_mask(self) -> np.ndarray:
    """[n * max_states] mask of the real states in shape + (max_states,) data."""
    kmax = int(self.num_states.max(initial=0))
    return (np.arange(kmax) < self.num_states[..., None]).reshape(-1)

  def _torch_index(self, like):
    """Device index tensor of the real states, built once per device: indexing with it copies no
    host data, so flatten / unflatten can run inside a CUDA graph capture."""
    import torch  # pylint: disable=g-import-not-at-top
    cache = self.__dict__.setdefault("_index_cache", {})
    key = str(like.device)
    if key not in cache:
      cache[key] = torch.as_tensor(np.flatnonzero(self._state_mask()), device=like.device)
    return cache[key]

  def flatten(self, data):
    """shape -> per-variable flat data; shape + (max_states,) -> per-state flat data.
    A leading batch axis is kept: (B,) + shape [+ (max_states,)] -> [B, n]."""
    data = data if _is_torch(data) else np.asarray(data)
    kmax = int(self.num_states.max(initial=0))
    tshape = tuple(data.shape)
    nd = len(self.shape)
    if tshape == tuple(self.shape):
      return data.reshape(-1)
    if tshape == tuple(self.shape) + (kmax,):
      flat = data.reshape(-1)
      if self._uniform_states():
        return flat
      mask = self._state_mask()
      return flat[mask] if not _is_torch(data) else flat[self._torch_index(data)]
    if len(tshape) == nd + 2 and tshape[1:] == tuple(self.shape) + (kmax,):
      flat = data.reshape(tshape[0], -1)
      if self._uniform_states():
        return flat
      mask = self._state_mask()
      return flat[:, mask] if not _is_torch(data) else flat[:, self._torch_index(data)]
    if len(tshape) == nd + 1 and tshape[1:] == tuple(self.shape):
      return data.reshape(tshape[0], -1)
    raise ValueError(f"data should be of shape {tuple(self.shape)} or "
                     f"{tuple(self.shape) + (kmax,)}. Got {tshape}.")

  def unflatten(self, flat_data, per_state: bool):
    """Inverse of flatten; per-state data is padded with -inf. Accepts a leading batch axis."""
    if flat_data.ndim not in (1, 2):
      raise ValueError(f"Can only unflatten 1D array. Got a {flat_data.ndim}D array.")
    batched = flat_data.ndim == 2
    n = flat_data.shape[-1]
    lead = (flat_data.shape[0],) if batched else ()
    if per_state:
      if n != self.num_states.sum():
        raise ValueError(f"flat_data size should be equal to {self.num_states.sum()}. "
                         f"Got size {n}.")
      kmax = int(self.num_states.max(initial=0))
      if self._uniform_states():
        return flat_data.reshape(lead + tuple(self.shape) + (kmax,))
      mask = self._state_mask()
      if _is_torch(flat_data):
        import torch  # pylint: disable=g-import-not-at-top
        out = torch.full(lead + (int(np.prod(self.shape)) * kmax,), -float("inf"),
                         dtype=flat_data.dtype, device=flat_data.device)
        out[..., self._torch_index(flat_data)] = flat_data
      else:
        out = np.full(lead + (int(np.prod(self.shape)) * kmax,), -np.inf, dtype=flat_data.dtype)
        out[..., mask] = flat_data
      return out.reshape(lead + tuple(self.shape) + (kmax,))
    if n != np.prod(self.shape):
      raise ValueError(f"flat_data size should be equal to {np.prod(self.shape)}. "
                       f"Got size {n}.")
    return flat_data.reshape(lead + tuple(self.shape))




@dataclasses.dataclass(frozen=True, eq=False)
class VarDict(VarGroup):
  """Named variables (pgmax/vgroup/vdict.py:26-189)."""

  variable_names: Tuple[Any, ...]
  _hash: int = dataclasses.field(init=False)

  def __post_init__(self):
    super().__post_init__()
    object.__setattr__(self, "num_states",
                       _check_num_states(self.num_states, (len(self.variable_names),)))
    object.__setattr__(self, "_index", {n: i for i, n in enumerate(self.variable_names)})

  @property
  def variable_hashes(self) -> np.ndarray:
    return self.__hash__() + np.arange(len(self.variable_names), dtype=np.int64)

  def __getitem__(self, var_name) -> Tuple[int, int]:
    idx = self._index.get(var_name) if _hashable(var_name) else None
    if idx is None:
      raise ValueError(f"Variable {var_name} is not in VarDict")
    return (self.variable_hashes[idx], self.num_states[idx])

  def flatten(self, data: Dict[Any, Any]):
    for name in data:
      if name not in self._index:
        raise ValueError(f"data is referring to a non-existent variable {name}.")
      idx = self._index[name]
      shp = tuple(np.shape(data[name]))
      if shp != (self.num_states[idx],) and shp != (1,):
        raise ValueError(f"Variable {name} expects a data array of shape "
                         f"{(self.num_states[idx],)} or (1,). Got {shp}.")
    parts = [data[name] for name in self.variable_names]
    if parts and _is_torch(parts[0]):
      import torch  # pylint: disable=g-import-not-at-top
      return torch.cat([p.reshape(-1) for p in parts])
    return np.concatenate([np.asarray(p).reshape(-1) for p in parts]) if parts else np.zeros(0)

  def unflatten(self, flat_data, per_state: bool) -> Dict[Hashable, Any]:
    if flat_data.ndim != 1:
      raise ValueError(f"Can only unflatten 1D array. Got a {flat_data.ndim}D array.")
    if per_state:
      total = int(self.num_states.sum())
      if flat_data.shape[0] != total:
        raise ValueError(f"flat_data should be shape (num_variable_states(={total}),). Got "
                         f"{tuple(flat_data.shape)}")
      offs = self.state_offsets()
      return {n: flat_data[offs[i]:offs[i + 1]] for i, n in enumerate(self.variable_names)}
    if flat_data.shape[0] != len(self.variable_names):
      raise ValueError(f"flat_data should be shape (num_variables(={len(self.variables)}),). Got "
                       f"{tuple(flat_data.shape)}")
    return dict(zip(self.variable_names, flat_data))


def _hashable(x):
  try:
    hash(x)
    return True
  except TypeError:
    return False
