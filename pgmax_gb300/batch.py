"""Uneven multi-graph batches: many factor graphs of different sizes and factor types run as one.

PGMax batches only instances of one graph (`jax.vmap` over BPArrays). A batch of *different*
graphs is their disjoint union: one flat wiring whose per-type message ranges hold every graph's
segment of that type, with every index shifted by the graph's offsets. One `pgbp_run` then updates
all graphs with one launch per kernel class per iteration, each kernel spanning the factors of that
class in every graph. Per graph the arithmetic is unchanged (a variable's edge states keep their
order, every factor update is local), so each graph's messages equal those of its own run; the
residuals returned are the maximum over all graphs.

Union layout (`union_wiring`):
  * messages: for each factor type in registry order (Enum, OR, AND, Pool), the segments of graph
    0, 1, ... of that type; `Layout.perm` maps union positions to positions in the graph-major
    concatenation of per-graph message arrays;
  * evidence / beliefs / MAP states: graph-major (graph 0's variable states first);
  * potentials: graph-major concatenation of each graph's Enum potentials. Graphs whose wiring
    carries `enum.factor_potential_offsets` share tables (compact potentials); when any graph does,
    the union carries offsets for every Enum factor.
"""

import dataclasses
from typing import Dict, List, Sequence

import numpy as np

TYPE_KEYS = ("enum", "or", "and", "pool")


@dataclasses.dataclass
class Layout:
  """Where each graph's arrays sit in the union."""
  num_graphs: int
  msgs_offsets: np.ndarray       # [G + 1] graph-major message offsets
  var_state_offsets: np.ndarray  # [G + 1]
  variable_offsets: np.ndarray   # [G + 1]
  potential_offsets: np.ndarray  # [G + 1]
  perm: np.ndarray               # [E_union] union position -> graph-major position

  def graph_major_to_union(self, msgs):
    """[..., E] graph-major messages -> union order (numpy or torch)."""
    return msgs[..., self._perm_like(msgs)]

  def union_to_graph_major(self, msgs):
    return msgs[..., self._inv_like(msgs)]

  def _perm_like(self, x):
    return self._index(x, "perm")

  def _inv_like(self, x):
    return self._index(x, "inv")

  def _index(self, x, which):
    if not hasattr(self, "_cache"):
      inv = np.empty_like(self.perm)
      inv[self.perm] = np.arange(self.perm.shape[0], dtype=self.perm.dtype)
      object.__setattr__(self, "_cache", {"perm": {"np": self.perm}, "inv": {"np": inv}})
    c = self._cache[which]
    if type(x).__module__.startswith("torch"):
      import torch  # pylint: disable=g-import-not-at-top
      key = str(x.device)
      if key not in c:
        c[key] = torch.as_tensor(c["np"], device=x.device)
      return c[key]
    return c["np"]

  def split(self, flat, kind: str) -> List:
    """Per-graph slices of a graph-major [..., n] array; kind: 'msgs', 'var_states',
    'variables' or 'potentials'."""
    off = {"msgs": self.msgs_offsets, "var_states": self.var_state_offsets,
           "variables": self.variable_offsets, "potentials": self.potential_offsets}[kind]
    return [flat[..., int(off[g]):int(off[g + 1])] for g in range(self.num_graphs)]


def _arr(w, key, dtype=np.int64):
  v = w.get(key)
  return np.zeros(0, dtype) if v is None else np.asarray(v, dtype=dtype).reshape(-1)


def _enum_factor_first_configs(w):
  """First config index of every Enum factor (factor order), from the config rows."""
  ci = _arr(w, "enum.factor_configs_indices")
  if ci.size == 0:
    return np.zeros(0, np.int64)
  cf = _arr(w, "enum.factor_configs_edge_states")
  e0 = int(np.asarray(w["msgs_ranges"]).reshape(4, 2)[0, 0])
  fac = _arr(w, "factor_indices_for_edge_states")[e0 + cf]
  starts = np.concatenate([[0], np.nonzero(np.diff(fac))[0] + 1])
  return ci[starts]


def union_wiring(wirings: Sequence[Dict]) -> (Dict, Layout):
  """The flat wiring of the disjoint union of `wirings` (keys of InfererContext.flat_wiring())."""
  G = len(wirings)
  mr = [np.asarray(w["msgs_ranges"], np.int64).reshape(4, 2) for w in wirings]
  pr = [np.asarray(w["potentials_ranges"], np.int64).reshape(4, 2) for w in wirings]
  n_es = [int(_arr(w, "var_states_for_edge_states").shape[0]) for w in wirings]
  n_vs = [int(w["num_var_states"]) for w in wirings]
  n_var = [int(w.get("num_variables", int(np.max(_arr(w, "evidence_to_vars"), initial=-1)) + 1))
           for w in wirings]
  n_pot = [int(p[0, 1] - p[0, 0]) for p in pr]
  msgs_off = np.concatenate([[0], np.cumsum(n_es)]).astype(np.int64)
  vs_off = np.concatenate([[0], np.cumsum(n_vs)]).astype(np.int64)
  var_off = np.concatenate([[0], np.cumsum(n_var)]).astype(np.int64)
  pot_off = np.concatenate([[0], np.cumsum(n_pot)]).astype(np.int64)
  shared = any(w.get("enum.factor_potential_offsets") is not None for w in wirings)
  with_enum = [w for g, w in enumerate(wirings) if mr[g][0, 1] > mr[g][0, 0]]
  implicit = bool(with_enum) and all(w.get("enum.implicit_rows") for w in with_enum)
  if not implicit and any(w.get("enum.implicit_rows") for w in with_enum):
    raise ValueError("a union mixes graphs with implicit and explicit Enum config rows")

  vs_l, ed_l, fa_l, perm_l = [], [], [], []
  rows_ci, rows_cf, alias_l = [], [], []
  logical = {1: ([], [], []), 2: ([], [], [])}
  pool = ([], [], [])
  out_mr = np.zeros((4, 2), np.int64)
  edge_count = fac_count = pos = 0
  cfg_count = 0
  for t in range(4):
    out_mr[t, 0] = pos
    es_t = 0       # edge states of type t placed so far (relative indices of the type)
    fac_t = 0      # factors of type t placed so far
    for g, w in enumerate(wirings):
      r0, r1 = int(mr[g][t, 0]), int(mr[g][t, 1])
      n = r1 - r0
      if n == 0:
        continue
      vs_l.append(_arr(w, "var_states_for_edge_states")[r0:r1] + vs_off[g])
      ed = _arr(w, "edge_indices_for_edge_states")[r0:r1]
      ed_l.append(ed - ed[0] + edge_count)
      edge_count += int(ed[-1] - ed[0]) + 1
      fa = _arr(w, "factor_indices_for_edge_states")[r0:r1]
      fa_l.append(fa - fa[0] + fac_count)
      n_fac = int(fa[-1] - fa[0]) + 1
      fac_count += n_fac
      perm_l.append(np.arange(msgs_off[g] + r0, msgs_off[g] + r1, dtype=np.int64))
      key = TYPE_KEYS[t]
      if t == 0:
        rows_ci.append(_arr(w, "enum.factor_configs_indices") + cfg_count)
        rows_cf.append(_arr(w, "enum.factor_configs_edge_states") + es_t)
        cfg_count += int(w.get("enum.num_val_configs", 0))
        if shared:
          own = w.get("enum.factor_potential_offsets")
          if own is None and implicit:
            raise ValueError("implicit-row graphs of a shared-table union need potential offsets")
          first = (np.asarray(own, np.int64).reshape(-1) if own is not None
                   else _enum_factor_first_configs(w))
          alias_l.append(first + pot_off[g])
      elif t in (1, 2):
        pfi, pmi, ch = logical[t]
        pfi.append(_arr(w, f"{key}.parents_factor_indices") + fac_t)
        pmi.append(_arr(w, f"{key}.parents_msg_indices") + es_t)
        ch.append(_arr(w, f"{key}.children_edge_states") + es_t)
      else:
        cfi, cmi, ind = pool
        cfi.append(_arr(w, "pool.pool_choices_factor_indices") + fac_t)
        cmi.append(_arr(w, "pool.pool_choices_msg_indices") + es_t)
        ind.append(_arr(w, "pool.pool_indicators_edge_states") + es_t)
      es_t += n
      fac_t += n_fac
      pos += n
    out_mr[t, 1] = pos

  cat = lambda parts: (np.concatenate(parts) if parts else np.zeros(0, np.int64)).astype(np.int32)
  total_pot = int(pot_off[-1])
  out_pr = np.array([[0, total_pot], [total_pot] * 2, [total_pot] * 2, [total_pot] * 2], np.int64)
  e2v = [(_arr(w, "evidence_to_vars") + var_off[g]) for g, w in enumerate(wirings)]
  u = {
      "var_states_for_edge_states": cat(vs_l),
      "edge_indices_for_edge_states": cat(ed_l),
      "factor_indices_for_edge_states": cat(fa_l),
      "num_edges": edge_count,
      "num_factors": fac_count,
      "num_var_states": int(vs_off[-1]),
      "evidence_to_vars": cat(e2v),
      "num_variables": int(var_off[-1]),
      "msgs_ranges": out_mr,
      "potentials_ranges": out_pr,
      "enum.factor_configs_indices": cat(rows_ci),
      "enum.factor_configs_edge_states": cat(rows_cf),
      "enum.num_val_configs": cfg_count,
  }
  for t in (1, 2):
    pfi, pmi, ch = logical[t]
    u[f"{TYPE_KEYS[t]}.parents_factor_indices"] = cat(pfi)
    u[f"{TYPE_KEYS[t]}.parents_msg_indices"] = cat(pmi)
    u[f"{TYPE_KEYS[t]}.children_edge_states"] = cat(ch)
  u["pool.pool_choices_factor_indices"] = cat(pool[0])
  u["pool.pool_choices_msg_indices"] = cat(pool[1])
  u["pool.pool_indicators_edge_states"] = cat(pool[2])
  if shared:
    u["enum.factor_potential_offsets"] = cat(alias_l)
  if implicit:
    del u["enum.factor_configs_indices"], u["enum.factor_configs_edge_states"]
    u["enum.implicit_rows"] = True
  layout = Layout(G, msgs_off, vs_off, var_off, pot_off, np.concatenate(perm_l) if perm_l else
                  np.zeros(0, np.int64))
  return u, layout


class GraphBatch:
  """A compiled batch of different factor graphs (one union plan on the GPU).

  `wirings`: flat wirings (InfererContext(bp_state).flat_wiring(), or generated with the same
  keys; graphs of identical structure may repeat the same dict). Arrays passed to `run` are in
  union layout: potentials and evidence graph-major (`concat`), messages in union order
  (`Layout.graph_major_to_union`). A leading batch axis runs instances of the whole batch.
  """

  def __init__(self, wirings: Sequence[Dict], device=None, flags: int = 0):
    from . import engine  # pylint: disable=g-import-not-at-top
    self.wiring, self.layout = union_wiring(wirings)
    self.plan = engine.Plan(self.wiring, device=device, flags=flags)

  @staticmethod
  def concat(parts):
    """Graph-major concatenation of per-graph [..., n_g] arrays (numpy or torch)."""
    if parts and type(parts[0]).__module__.startswith("torch"):
      import torch  # pylint: disable=g-import-not-at-top
      return torch.cat(list(parts), dim=-1)
    return np.concatenate([np.asarray(p) for p in parts], axis=-1)

  def run(self, log_potentials, evidence, ftov_msgs, num_iters, damping=0.5, temperature=0.0):
    """run_with_diffs over every graph; returns (union-order messages, residuals)."""
    return self.plan.run(log_potentials, evidence, ftov_msgs, num_iters, damping, temperature)

  def beliefs(self, evidence, ftov_msgs):
    return self.plan.beliefs(evidence, ftov_msgs)

  def decode(self, flat_beliefs):
    return self.plan.decode(flat_beliefs, int(self.wiring["num_variables"]))


def grid_wiring(L: int, K: int, shared_table: bool = False, implicit_rows: bool = False) -> Dict:
  """The flat wiring FactorGraph compiles for an open L x L NDVarArray of K-state variables with a
  top-down PairwiseFactorGroup (factors ((i, j), (i + 1, j)), row-major) followed by a left-right
  one (((i, j), (i, j + 1))), generated directly with vectorised NumPy: for batches of large grids,
  whose per-factor Python construction would dominate. `shared_table`: every factor reads one
  K x K table (compact potentials of K * K floats). `implicit_rows`: the config rows are left out
  (PGBP_FLAG_ENUM_IMPLICIT_ROWS; 2 * K * K int32 rows per factor otherwise)."""
  i, j = np.meshgrid(np.arange(L - 1), np.arange(L), indexing="ij")
  td = np.stack([i * L + j, (i + 1) * L + j], -1).reshape(-1, 2)
  i, j = np.meshgrid(np.arange(L), np.arange(L - 1), indexing="ij")
  lr = np.stack([i * L + j, i * L + j + 1], -1).reshape(-1, 2)
  pairs = np.concatenate([td, lr]).astype(np.int64)        # [F, 2] variable indices
  F = pairs.shape[0]
  s = np.arange(K, dtype=np.int64)
  vs = (pairs[:, :, None] * K + s).reshape(-1)             # [F * 2K], edge-state order
  es = np.arange(2 * K * F, dtype=np.int64)
  edge = es // K
  fac = es // (2 * K)
  E = 2 * K * F
  P = K * K if shared_table else F * K * K
  w = {
      "var_states_for_edge_states": vs.astype(np.int32),
      "edge_indices_for_edge_states": edge.astype(np.int32),
      "factor_indices_for_edge_states": fac.astype(np.int32),
      "num_edges": 2 * F, "num_factors": F, "num_var_states": L * L * K,
      "evidence_to_vars": np.repeat(np.arange(L * L), K).astype(np.int32),
      "num_variables": L * L,
      "msgs_ranges": np.array([[0, E], [E, E], [E, E], [E, E]], np.int64),
      "potentials_ranges": np.array([[0, P], [P, P], [P, P], [P, P]], np.int64),
      "enum.num_val_configs": F * K * K,
  }
  if shared_table:
    w["enum.factor_potential_offsets"] = np.zeros(F, np.int32)
  if implicit_rows:
    w["enum.implicit_rows"] = True
  else:
    a, b = np.meshgrid(s, s, indexing="ij")                # config c = a * K + b
    base = (2 * K * np.arange(F))[:, None, None]
    w["enum.factor_configs_edge_states"] = np.stack([base + a, base + K + b], -1).reshape(-1).astype(
        np.int32)
    w["enum.factor_configs_indices"] = np.repeat(np.arange(F * K * K, dtype=np.int32), 2)
  return w
