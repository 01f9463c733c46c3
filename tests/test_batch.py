"""Multi-graph batches (pgmax_gb300/batch.py) on CPU: the union wiring, checked with the oracle.

The oracle run on the union of several graphs must give, for every graph, bit for bit the
messages of that graph's own run (a union changes no per-graph arithmetic), at temperature 0 and
above. Shared potential tables are checked by expanding the compact potentials back to one table
per factor.
"""

import numpy as np
import pytest

import fixtures
from oracle import oracle
from pgmax_gb300 import batch

MIX = ["case_mixed_T1", "case_ising12_T1", "case_potts_K4", "case_deconv_T1", "case_mixed_T0",
       "case_rbm_s0"]


def _load(name):
  return fixtures.load(f"{fixtures.FIXTURES}/{name}.npz")


def _wiring(d):
  w = dict(d["wiring"])
  w["num_variables"] = int(np.max(w["evidence_to_vars"], initial=-1)) + 1
  return w


def expand_potentials(w, lp_compact):
  """One table per factor (the PGMax layout) from shared tables."""
  first = batch._enum_factor_first_configs(w)  # pylint: disable=protected-access
  off = np.asarray(w["enum.factor_potential_offsets"], np.int64)
  n_cfg = np.diff(np.concatenate([first, [int(w["enum.num_val_configs"])]]))
  full = np.zeros(int(w["enum.num_val_configs"]), np.float32)
  for f0, o, n in zip(first, off, n_cfg):
    full[f0:f0 + n] = lp_compact[o:o + n]
  return full


@pytest.mark.parametrize("temperature", [0.0, 1.0])
def test_union_runs_every_graph_as_its_own_run(temperature):
  ds = [_load(n) for n in MIX]
  ws = [_wiring(d) for d in ds]
  u, lay = batch.union_wiring(ws)
  assert lay.num_graphs == len(ds)
  lp = np.concatenate([d["log_potentials"] for d in ds]).astype(np.float32)
  ev = np.concatenate([d["evidence"] for d in ds]).astype(np.float32)
  rng = np.random.default_rng(0)
  m_parts = [(0.2 * rng.normal(size=d["ftov_msgs_in"].shape)).astype(np.float32) for d in ds]
  m = lay.graph_major_to_union(np.concatenate(m_parts))
  uw = oracle.Wiring(u)
  out, _ = oracle.run(uw, lp, ev, m, 9, 0.5, temperature)
  per_graph = lay.split(lay.union_to_graph_major(out), "msgs")
  for d, w, mi, got in zip(ds, ws, m_parts, per_graph):
    want, _ = oracle.run(oracle.Wiring(w), d["log_potentials"], d["evidence"], mi, 9, 0.5,
                         temperature)
    np.testing.assert_array_equal(got, want)
  bel = oracle.beliefs(uw, ev, out)
  for g, (d, w) in enumerate(zip(ds, ws)):
    own, _ = oracle.run(oracle.Wiring(w), d["log_potentials"], d["evidence"], m_parts[g], 9, 0.5,
                        temperature)
    np.testing.assert_array_equal(lay.split(bel, "var_states")[g],
                                  oracle.beliefs(oracle.Wiring(w), d["evidence"], own))


def test_union_index_ranges():
  ds = [_load(n) for n in MIX]
  u, lay = batch.union_wiring([_wiring(d) for d in ds])
  n_es = u["var_states_for_edge_states"].shape[0]
  assert n_es == sum(d["ftov_msgs_in"].shape[0] for d in ds)
  assert sorted(lay.perm.tolist()) == list(range(n_es))
  assert np.all(np.diff(u["edge_indices_for_edge_states"]) >= 0)
  assert np.all(np.diff(u["factor_indices_for_edge_states"]) >= 0)
  mr = u["msgs_ranges"]
  assert mr[0, 0] == 0 and mr[3, 1] == n_es and np.all(mr[1:, 0] == mr[:-1, 1])
  assert u["num_var_states"] == sum(d["evidence"].shape[0] for d in ds)


def _potts_wiring_shared(d):
  """A Potts fixture's wiring with every factor reading one shared K x K table."""
  w = _wiring(d)
  n_fac = batch._enum_factor_first_configs(w).shape[0]  # pylint: disable=protected-access
  w["enum.factor_potential_offsets"] = np.zeros(n_fac, np.int32)
  k2 = int(np.asarray(w["enum.num_val_configs"])) // n_fac
  w["potentials_ranges"] = np.array([[0, k2]] + [[k2, k2]] * 3, np.int64)  # compact: one table
  return w


def test_shared_tables_in_a_union_expand_to_per_factor_tables():
  dk, dm = _load("case_potts_K4"), _load("case_mixed_T1")
  ws = _potts_wiring_shared(dk)
  wm = _wiring(dm)
  u, lay = batch.union_wiring([ws, wm, ws])
  rng = np.random.default_rng(1)
  tables = [rng.normal(size=16).astype(np.float32), dm["log_potentials"].astype(np.float32),
            rng.normal(size=16).astype(np.float32)]
  lp_c = np.concatenate(tables)
  # graph 0 and 2: every factor gets its graph's table; graph 1 keeps its own potentials
  u_plain = {k: v for k, v in u.items() if k != "enum.factor_potential_offsets"}
  full = expand_potentials(u, lp_c)
  ev = np.concatenate([dk["evidence"], dm["evidence"], dk["evidence"]]).astype(np.float32)
  m = np.zeros(u["var_states_for_edge_states"].shape[0], np.float32)
  out_u, _ = oracle.run(oracle.Wiring(dict(u_plain, **{"potentials_ranges": np.array(
      [[0, full.shape[0]]] + [[full.shape[0]] * 2] * 3)})), full, ev, m, 6, 0.5, 1.0)
  parts = lay.split(lay.union_to_graph_major(out_u), "msgs")
  n_fac_k = batch._enum_factor_first_configs(ws).shape[0]  # pylint: disable=protected-access
  for g, (w_plain, table) in enumerate([(_wiring(dk), np.tile(tables[0], n_fac_k)),
                                         (wm, tables[1]), (_wiring(dk), np.tile(tables[2], n_fac_k))]):
    d = [dk, dm, dk][g]
    want, _ = oracle.run(oracle.Wiring(w_plain), table, d["evidence"],
                         np.zeros(d["ftov_msgs_in"].shape, np.float32), 6, 0.5, 1.0)
    np.testing.assert_array_equal(parts[g], want)


@pytest.mark.parametrize("L,K", [(4, 3), (5, 2), (3, 4), (6, 1)])
def test_grid_wiring_is_the_factor_graph_wiring(L, K):
  import pgmax_gb300 as pg  # pylint: disable=g-import-not-at-top
  from golden import cases  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer  # pylint: disable=g-import-not-at-top
  fg, _, _ = cases.potts(pg, L=L, K=K, seed=0)
  fw = infer.InfererContext(fg.bp_state).flat_wiring()
  gw = batch.grid_wiring(L, K)
  for k, v in gw.items():
    np.testing.assert_array_equal(np.asarray(fw[k]), np.asarray(v), err_msg=k)
  imp = batch.grid_wiring(L, K, shared_table=True, implicit_rows=True)
  assert imp["enum.implicit_rows"] and "enum.factor_configs_indices" not in imp
  assert imp["potentials_ranges"][0, 1] == K * K


def test_union_of_implicit_row_graphs_and_mixing_rules():
  a = batch.grid_wiring(4, 3, shared_table=True, implicit_rows=True)
  b = batch.grid_wiring(5, 2, shared_table=True, implicit_rows=True)
  d = _wiring(_load("case_deconv_T1"))          # no Enum factors: may join an implicit union
  u, lay = batch.union_wiring([a, d, b, a])
  assert u["enum.implicit_rows"] and "enum.factor_configs_indices" not in u
  assert u["enum.num_val_configs"] == 2 * a["enum.num_val_configs"] + b["enum.num_val_configs"]
  np.testing.assert_array_equal(lay.potential_offsets, [0, 9, 9, 13, 22])
  off = u["enum.factor_potential_offsets"]
  n_a, n_b = a["num_factors"], b["num_factors"]
  np.testing.assert_array_equal(off, np.concatenate([np.zeros(n_a), np.full(n_b, 9),
                                                     np.full(n_a, 13)]))
  with pytest.raises(ValueError, match="implicit and explicit"):
    batch.union_wiring([a, batch.grid_wiring(3, 2)])
