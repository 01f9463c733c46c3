"""Factor groups: PGMax's pgmax/fgroup/ classes (FactorGroup, SingleFactorGroup, EnumFactorGroup,
PairwiseFactorGroup, LogicalFactorGroup, ORFactorGroup, ANDFactorGroup, PoolFactorGroup).

A group holds many factors of one type; its flat log potentials are the per-factor tables
concatenated in factor order (fgroup.py:137-140, enum.py:62-95, 303-325). `compile_wiring` builds the
group's wiring from the global start of every variable's states.
"""

import collections
import dataclasses
import itertools
from typing import Any, List, Optional, Sequence, Tuple, Type

import numpy as np

from . import factor


def _is_torch(x):
  return type(x).__module__.startswith("torch")


def _size(x):
  return int(x.numel()) if _is_torch(x) else int(np.size(x))


def flat_variables(variables_for_factors) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
  """(hash per edge, num_states per edge, factor sizes) of a list of factors' variable lists."""
  sizes = np.fromiter((len(v) for v in variables_for_factors), dtype=np.int64,
                      count=len(variables_for_factors))
  flat = list(itertools.chain.from_iterable(variables_for_factors))
  if not flat:
    return np.zeros(0, np.int64), np.zeros(0, np.int64), sizes
  arr = np.array(flat, dtype=np.int64).reshape(-1, 2)
  return arr[:, 0], arr[:, 1], sizes


@dataclasses.dataclass(frozen=True, eq=False)
class FactorGroup:
  """Base class (pgmax/fgroup/fgroup.py:28-219)."""

  variables_for_factors: Sequence[List[Tuple[int, int]]]
  factor_configs: np.ndarray = dataclasses.field(init=False)
  log_potentials: np.ndarray = dataclasses.field(init=False,
                                                 default_factory=lambda: np.empty((0,)))
  factor_type: Type[Any] = dataclasses.field(init=False)

  def __post_init__(self):
    if not self.variables_for_factors:
      raise ValueError("Cannot create a FactorGroup with no Factor.")

  def __hash__(self):
    return id(self)

  def __eq__(self, other):
    return hash(self) == hash(other)

  def __lt__(self, other):
    return hash(self) < hash(other)

  def _cached(self, name, fn):
    v = self.__dict__.get(name)
    if v is None:
      v = fn()
      object.__setattr__(self, name, v)
    return v

  def _flat(self):
    return self._cached("_flat_vars", lambda: flat_variables(self.variables_for_factors))

  @property
  def factor_sizes(self) -> np.ndarray:
    return self._flat()[2]

  @property
  def factor_edges_num_states(self) -> np.ndarray:
    return self._flat()[1]

  @property
  def edge_variable_hashes(self) -> np.ndarray:
    return self._flat()[0]

  @property
  def num_factors(self) -> int:
    return len(self.variables_for_factors)

  @property
  def factor_group_log_potentials(self) -> np.ndarray:
    return self._cached("_flat_lp", lambda: np.asarray(self.log_potentials).reshape(-1))

  @property
  def _variables_to_factors(self):
    return self._cached("_v2f", self._get_variables_to_factors)

  @property
  def factors(self):
    return tuple(self._variables_to_factors.values())

  def __getitem__(self, variables):
    key = frozenset(variables)
    if key not in self._variables_to_factors:
      raise ValueError(f"The queried factor connected to the set of variables {key} is"
                       " not present in the factor group.")
    return self._variables_to_factors[key]

  def _get_variables_to_factors(self):
    raise NotImplementedError("Please subclass the FactorGroup class and override this method")

  def flatten(self, data):
    raise NotImplementedError("Please subclass the FactorGroup class and override this method")

  def unflatten(self, flat_data):
    raise NotImplementedError("Please subclass the FactorGroup class and override this method")

  def compile_wiring(self, vars_to_starts) -> factor.Wiring:
    """Wiring of the group given a vectorised variable -> first-state lookup."""
    first = vars_to_starts.starts_of(self.edge_variable_hashes, self.factor_edges_num_states)
    ft = self.factor_type
    if issubclass(ft, factor.EnumFactor):
      return factor.EnumFactor.compile_wiring(self.factor_edges_num_states, first,
                                              np.asarray(self.factor_configs), self.num_factors)
    if issubclass(ft, factor.PoolFactor):
      return factor.PoolFactor.compile_wiring(self.factor_edges_num_states, first,
                                              self.factor_sizes)
    if issubclass(ft, factor.LogicalFactor):
      return factor.LogicalFactor.compile_wiring(self.factor_edges_num_states, first,
                                                 self.factor_sizes, ft.edge_states_offset)
    raise NotImplementedError(f"No wiring compiler for {ft}")


@dataclasses.dataclass(frozen=True, eq=False)
class SingleFactorGroup(FactorGroup):
  """A group wrapping one Factor added on its own (fgroup.py:223-295)."""

  single_factor: factor.Factor

  def __post_init__(self):
    super().__post_init__()
    if len(self.variables_for_factors) != 1:
      raise ValueError("SingleFactorGroup should only contain one factor. Got"
                       f" {len(self.variables_for_factors)}")
    object.__setattr__(self, "factor_type", type(self.single_factor))
    if isinstance(self.single_factor, factor.EnumFactor):
      object.__setattr__(self, "factor_configs", self.single_factor.factor_configs)
    else:
      object.__setattr__(self, "factor_configs", None)
    lp = self.single_factor.log_potentials
    if lp.shape[0] > 0:
      lp = lp[None]
    object.__setattr__(self, "log_potentials", lp)

  def _get_variables_to_factors(self):
    return collections.OrderedDict(
        [(frozenset(self.variables_for_factors[0]), self.single_factor)])

  def flatten(self, data):
    raise NotImplementedError("SingleFactorGroup does not support vectorized factor operations.")

  def unflatten(self, flat_data):
    raise NotImplementedError("SingleFactorGroup does not support vectorized factor operations.")


@dataclasses.dataclass(frozen=True, eq=False)
class EnumFactorGroup(FactorGroup):
  """EnumFactors sharing one config table (pgmax/fgroup/enum.py:29-206)."""

  factor_configs: np.ndarray
  log_potentials: Optional[np.ndarray] = None
  factor_type: Type[Any] = dataclasses.field(init=False, default=factor.EnumFactor)

  def __post_init__(self):
    super().__post_init__()
    n_cfg = self.factor_configs.shape[0]
    if self.log_potentials is None:
      lp = np.zeros((self.num_factors, n_cfg), dtype=float)
    else:
      lp = self.log_potentials
      if _is_torch(lp):
        lp = lp.detach().cpu().numpy()
      if lp.shape != (n_cfg,) and lp.shape != (self.num_factors, n_cfg):
        raise ValueError(f"Expected log potentials shape: {(n_cfg,)} or"
                         f" {(self.num_factors, n_cfg)}. Got {lp.shape}.")
      lp = np.broadcast_to(lp, (self.num_factors, n_cfg))
    if not np.issubdtype(lp.dtype, np.floating):
      raise ValueError(f"Potentials should be floats. Got {lp.dtype}.")
    object.__setattr__(self, "log_potentials", lp)

  def _get_variables_to_factors(self):
    lp = np.array(self.log_potentials)
    return collections.OrderedDict([
        (frozenset(v), factor.EnumFactor(variables=v, factor_configs=self.factor_configs,
                                         log_potentials=lp[i]))
        for i, v in enumerate(self.variables_for_factors)])

  def _edge_states_per_factor(self):
    return int(sum(v[1] for v in self.variables_for_factors[0]))

  def flatten(self, data):
    n = self.num_factors
    n_cfg = self.factor_configs.shape[0]
    nes = self._edge_states_per_factor()
    shp = tuple(data.shape)
    if shp not in ((n, n_cfg), (n, nes), (n_cfg,)):
      raise ValueError(f"data should be of shape {(n, n_cfg)} or {(n, nes)} or {(n_cfg,)}."
                       f" Got {shp}.")
    if shp == (n_cfg,):
      return np.tile(np.asarray(data), n) if not _is_torch(data) else data.repeat(n)
    return data.reshape(-1)

  def unflatten(self, flat_data):
    if flat_data.ndim != 1:
      raise ValueError(f"Can only unflatten 1D array. Got a {flat_data.ndim}D array.")
    n = self.num_factors
    n_cfg = self.factor_configs.shape[0]
    nes = self._edge_states_per_factor()
    size = _size(flat_data)
    if size == n * n_cfg:
      return flat_data.reshape((n, n_cfg))
    if size == n * nes:
      return flat_data.reshape((n, nes))
    raise ValueError(f"flat_data should be compatible with shape {(n, n_cfg)} or {(n, nes)}. Got"
                     f" {tuple(flat_data.shape)}.")


@dataclasses.dataclass(frozen=True, eq=False)
class PairwiseFactorGroup(FactorGroup):
  """EnumFactors over two variables with every config valid (pgmax/fgroup/enum.py:209-435).
  Configs are ordered row-major: config i * n2 + j is (state i, state j)."""

  log_potential_matrix: Optional[np.ndarray] = None
  factor_type: Type[Any] = dataclasses.field(init=False, default=factor.EnumFactor)

  def __post_init__(self):
    super().__post_init__()
    vff = self.variables_for_factors
    if self.log_potential_matrix is None:
      m = np.zeros((vff[0][0][1], vff[0][1][1]))
    else:
      m = self.log_potential_matrix
      if _is_torch(m):
        m = m.detach().cpu().numpy()
    if not (m.ndim == 2 or m.ndim == 3):
      raise ValueError("log_potential_matrix should be either a 2D array, specifying shared"
                       " parameters for all pairwise factors, or 3D array, specifying"
                       " parameters for individual pairwise factors. Got a"
                       f" {m.ndim}D log_potential_matrix array.")
    if not np.issubdtype(m.dtype, np.floating):
      raise ValueError(f"Potential matrix should be floats. Got {m.dtype}.")
    if m.ndim == 3 and m.shape[0] != len(vff):
      raise ValueError(f"Expected log_potential_matrix for {len(vff)} factors. Got"
                       f" log_potential_matrix for {m.shape[0]} factors.")
    hashes, ns, sizes = self._flat()
    if np.any(sizes != 2):
      bad = int(np.nonzero(sizes != 2)[0][0])
      raise ValueError("All pairwise factors should connect to exactly 2 variables. Got a"
                       f" factor connecting to {len(vff[bad])} variables ({vff[bad]}).")
    ns2 = ns.reshape(-1, 2)
    mismatch = np.nonzero((ns2[:, 0] != m.shape[-2]) | (ns2[:, 1] != m.shape[-1]))[0]
    if mismatch.size:
      v = vff[int(mismatch[0])]
      raise ValueError(f"The specified pairwise factor {v} (with {(v[0][1], v[1][1])}"
                       "configurations) does not match the specified log_potential_matrix (with"
                       f" {m.shape[-2:]} configurations).")
    object.__setattr__(self, "log_potential_matrix", m)
    configs = np.mgrid[:m.shape[-2], :m.shape[-1]].transpose((1, 2, 0)).reshape((-1, 2))
    object.__setattr__(self, "factor_configs", configs)
    lp = np.broadcast_to(m, (len(vff),) + m.shape[-2:]).reshape(len(vff), -1)
    object.__setattr__(self, "log_potentials", lp)

  def _get_variables_to_factors(self):
    return collections.OrderedDict([
        (frozenset(v), factor.EnumFactor(variables=v, factor_configs=self.factor_configs,
                                         log_potentials=np.asarray(self.log_potentials[i])))
        for i, v in enumerate(self.variables_for_factors)])

  def flatten(self, data):
    n = self.num_factors
    k = self.log_potential_matrix.shape[-2:]
    shp = tuple(data.shape)
    if shp not in ((n,) + k, (n, int(np.sum(k))), k):
      raise ValueError(f"data should be of shape {(n,) + k} or {(n, int(np.sum(k)))} or {k}."
                       f" Got {shp}.")
    if shp == k:
      flat = data.reshape(-1)
      return np.tile(np.asarray(flat), n) if not _is_torch(data) else flat.repeat(n)
    return data.reshape(-1)

  def unflatten(self, flat_data):
    if flat_data.ndim != 1:
      raise ValueError(f"Can only unflatten 1D array. Got a {flat_data.ndim}D array.")
    n = self.num_factors
    k = self.log_potential_matrix.shape[-2:]
    size = _size(flat_data)
    if size == n * int(np.prod(k)):
      return flat_data.reshape((n,) + k)
    if size == n * int(np.sum(k)):
      return flat_data.reshape((n, int(np.sum(k))))
    raise ValueError(f"flat_data should be compatible with shape {(n,) + k} or"
                     f" {(n, int(np.sum(k)))}. Got {tuple(flat_data.shape)}.")


@dataclasses.dataclass(frozen=True, eq=False)
class LogicalFactorGroup(FactorGroup):
  """OR / AND factors; each factor lists its parents then its child (fgroup/logical.py:28-63)."""

  factor_configs: Optional[np.ndarray] = dataclasses.field(init=False, default=None)
  edge_states_offset: int = dataclasses.field(init=False)

  def _get_variables_to_factors(self):
    return collections.OrderedDict([(frozenset(v), self.factor_type(variables=v))
                                    for v in self.variables_for_factors])


@dataclasses.dataclass(frozen=True, eq=False)
class ORFactorGroup(LogicalFactorGroup):
  edge_states_offset: int = dataclasses.field(init=False, default=1)
  factor_type: Type[Any] = dataclasses.field(init=False, default=factor.ORFactor)


@dataclasses.dataclass(frozen=True, eq=False)
class ANDFactorGroup(LogicalFactorGroup):
  edge_states_offset: int = dataclasses.field(init=False, default=-1)
  factor_type: Type[Any] = dataclasses.field(init=False, default=factor.ANDFactor)


@dataclasses.dataclass(frozen=True, eq=False)
class PoolFactorGroup(FactorGroup):
  """Pool factors; each factor lists its choices then its indicator (fgroup/pool.py:27-61)."""

  factor_configs: Optional[np.ndarray] = dataclasses.field(init=False, default=None)
  factor_type: Type[Any] = dataclasses.field(init=False, default=factor.PoolFactor)

  def _get_variables_to_factors(self):
    return collections.OrderedDict([(frozenset(v), factor.PoolFactor(variables=v))
                                    for v in self.variables_for_factors])
