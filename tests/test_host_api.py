"""Host side of the drop-in: graph construction, flat wiring, state updates (no GPU).

The flat wiring that pgmax_gb300 compiles must be identical to what the reference compiles for the
same graph (the layout BPArrays are defined against), mirroring the reference's layout-invariance
tests (tests/fgroup/test_wiring.py) and API tests (tests/fgraph/test_fgraph.py,
tests/vgroup/test_vgroup.py, tests/fgroup/test_fgroup.py).
"""

import glob
import types

import numpy as np
import pytest

import cases
import fixtures
from pgmax_gb300 import factor, fgraph, fgroup, infer, vgroup
from pgmax_gb300.infer import bp_state as bs

API = types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer,
                            vgroup=vgroup)
CASES = sorted(glob.glob(f"{fixtures.FIXTURES}/case_*.npz"))


@pytest.mark.parametrize("path", CASES, ids=fixtures.fixture_id)
def test_wiring_and_inputs_identical_to_reference(path):
  f = fixtures.load(path)
  meta = f["meta"]
  fg, groups, ev = cases.BUILDERS[meta["builder"]](API, **meta["builder_kwargs"])
  ctx = infer.InfererContext(fg.bp_state)
  w = ctx.flat_wiring()
  for k, ref in f["wiring"].items():
    got = np.asarray(w[k])
    assert got.shape == ref.shape, k
    np.testing.assert_array_equal(got.astype(np.int64), ref.astype(np.int64), err_msg=k)
  np.testing.assert_array_equal(np.asarray(fg.bp_state.log_potentials.value, np.float32),
                                f["log_potentials"])
  evidence = bs.update_evidence(np.zeros(fg.fg_state.num_var_states), ev, fg.fg_state)
  np.testing.assert_array_equal(evidence, f["evidence"])
  msgs = np.zeros(fg.fg_state.total_factor_num_states, np.float32)
  if meta["builder"] == "mixed":
    msgs = bs.update_ftov_msgs(msgs, cases.mixed_ftov_updates(API, groups, meta["builder_kwargs"]["seed"]),
                               fg.fg_state)
  np.testing.assert_array_equal(msgs, f["ftov_msgs_in"])


def _wiring(fg):
  ctx = infer.InfererContext(fg.bp_state)
  return ctx.flat_wiring()


def test_wiring_invariant_to_grouping():
  """One group vs many groups vs single factors give the same wiring (test_wiring.py:29-269)."""
  v = vgroup.NDVarArray(num_states=3, shape=(6,))
  configs = np.array([[0, 0], [1, 1], [2, 2], [0, 2]])
  vff = [[v[i], v[i + 1]] for i in range(5)]

  fg1 = fgraph.FactorGraph(v)
  fg1.add_factors(fgroup.EnumFactorGroup(variables_for_factors=vff, factor_configs=configs))
  fg2 = fgraph.FactorGraph(v)
  fg2.add_factors([fgroup.EnumFactorGroup(variables_for_factors=vff[:2], factor_configs=configs),
                   fgroup.EnumFactorGroup(variables_for_factors=vff[2:], factor_configs=configs)])
  fg3 = fgraph.FactorGraph(v)
  for x in vff:
    fg3.add_factors(factor.EnumFactor(variables=x, factor_configs=configs,
                                      log_potentials=np.zeros(4)))
  w1, w2, w3 = _wiring(fg1), _wiring(fg2), _wiring(fg3)
  for k in ("var_states_for_edge_states", "edge_indices_for_edge_states",
            "enum.factor_configs_edge_states", "enum.factor_configs_indices"):
    np.testing.assert_array_equal(w1[k], w2[k])
    np.testing.assert_array_equal(w1[k], w3[k])

  b = vgroup.NDVarArray(num_states=2, shape=(7,))
  lists = [[b[0], b[1], b[2]], [b[3], b[4]], [b[5], b[6]]]
  for group_cls, fac_cls, key in ((fgroup.ORFactorGroup, factor.ORFactor, "or"),
                                  (fgroup.ANDFactorGroup, factor.ANDFactor, "and"),
                                  (fgroup.PoolFactorGroup, factor.PoolFactor, "pool")):
    ga = fgraph.FactorGraph(b)
    ga.add_factors(group_cls(lists))
    gb = fgraph.FactorGraph(b)
    for x in lists:
      gb.add_factors(fac_cls(variables=x))
    wa, wb = _wiring(ga), _wiring(gb)
    for k in wa:
      if k.startswith(key + "."):
        np.testing.assert_array_equal(np.asarray(wa[k]), np.asarray(wb[k]), err_msg=k)


def test_logical_wiring_relevant_states():
  """OR: relevant state 1, AND: relevant state 0; parents index the other state
  (pgmax/factor/logical.py:262-279)."""
  b = vgroup.NDVarArray(num_states=2, shape=(3,))
  fg = fgraph.FactorGraph(b)
  fg.add_factors(factor.ORFactor(variables=[b[0], b[1], b[2]]))
  w = _wiring(fg)
  np.testing.assert_array_equal(w["or.parents_msg_indices"], [0, 2])
  np.testing.assert_array_equal(w["or.children_edge_states"], [4])
  fg = fgraph.FactorGraph(b)
  fg.add_factors(factor.ANDFactor(variables=[b[0], b[1], b[2]]))
  w = _wiring(fg)
  np.testing.assert_array_equal(w["and.parents_msg_indices"], [1, 3])
  np.testing.assert_array_equal(w["and.children_edge_states"], [5])


def test_factor_graph_errors():
  vg = vgroup.VarDict(variable_names=(0,), num_states=15)
  fg = fgraph.FactorGraph(vg)
  dup = factor.EnumFactor(variables=[vg[0], vg[0]],
                          factor_configs=np.array([[i, i] for i in range(15)]),
                          log_potentials=np.zeros(15))
  with pytest.raises(ValueError, match="contains variables duplicates"):
    fg.add_factors(dup)
  f1 = factor.EnumFactor(variables=[vg[0]], factor_configs=np.arange(15)[:, None],
                         log_potentials=np.zeros(15))
  fg.add_factors(f1)
  with pytest.raises(ValueError, match="already exists"):
    fg.add_factors(factor.EnumFactor(variables=[vg[0]], factor_configs=np.arange(15)[:, None],
                                     log_potentials=np.zeros(15)))


def test_factor_validation():
  v = vgroup.NDVarArray(num_states=2, shape=(3,))
  with pytest.raises(ValueError, match="Configurations should be integers"):
    factor.EnumFactor(variables=[v[0]], factor_configs=np.zeros((1, 1), float),
                      log_potentials=np.zeros(1))
  with pytest.raises(ValueError, match="Invalid configurations"):
    factor.EnumFactor(variables=[v[0]], factor_configs=np.array([[2]]), log_potentials=np.zeros(1))
  with pytest.raises(ValueError, match="at least one parent"):
    factor.ORFactor(variables=[v[0]])
  with pytest.raises(ValueError, match="should be binary"):
    w = vgroup.NDVarArray(num_states=3, shape=(2,))
    factor.ANDFactor(variables=[w[0], w[1]])
  with pytest.raises(ValueError, match="at least one pool choice"):
    factor.PoolFactor(variables=[v[0]])
  with pytest.raises(ValueError, match="exactly 2 variables"):
    fgroup.PairwiseFactorGroup(variables_for_factors=[[v[0], v[1], v[2]]],
                               log_potential_matrix=np.zeros((2, 2)))
  with pytest.raises(ValueError, match="Cannot create a FactorGroup with no Factor"):
    fgroup.ORFactorGroup([])


def test_vgroups_flatten_unflatten():
  ns = np.array([2, 3, 4])
  a = vgroup.NDVarArray(num_states=ns, shape=(3,))
  data = np.arange(12, dtype=float).reshape(3, 4)
  flat = a.flatten(data)
  np.testing.assert_array_equal(flat, [0, 1, 4, 5, 6, 8, 9, 10, 11])
  back = a.unflatten(flat, True)
  assert np.isneginf(back[0, 2:]).all() and np.isneginf(back[1, 3])
  np.testing.assert_array_equal(a.unflatten(np.array([1, 0, 2]), False), [1, 0, 2])
  with pytest.raises(ValueError, match="data should be of shape"):
    a.flatten(np.zeros((2, 2)))
  d = vgroup.VarDict(variable_names=("x", "y"), num_states=np.array([2, 3]))
  flat = d.flatten({"x": np.array([1.0, 2.0]), "y": np.array([3.0, 4.0, 5.0])})
  np.testing.assert_array_equal(flat, [1, 2, 3, 4, 5])
  un = d.unflatten(flat, True)
  np.testing.assert_array_equal(un["y"], [3, 4, 5])
  with pytest.raises(ValueError, match="non-existent variable"):
    d.flatten({"z": np.zeros(2)})
  with pytest.raises(ValueError, match="is not in VarDict"):
    _ = d["z"]
  assert a[1] == (a.variable_hashes[1], 3)


def test_bp_state_errors_and_updates():
  v = vgroup.VarDict(variable_names=(0, 1), num_states=15)
  fg = fgraph.FactorGraph(v)
  g = fgroup.EnumFactorGroup(variables_for_factors=[[v[0], v[1]]],
                             factor_configs=np.arange(10)[:, None] + np.zeros((1, 2), int))
  fg.add_factors(g)
  with pytest.raises(ValueError, match="Expected evidence shape"):
    infer.Evidence(fg_state=fg.fg_state, value=np.zeros((20,)))
  with pytest.raises(ValueError, match="Expected messages shape"):
    infer.FToVMessages(fg_state=fg.fg_state, value=np.zeros((5,)))
  with pytest.raises(ValueError, match="Expected log potentials shape"):
    infer.LogPotentials(fg_state=fg.fg_state, value=np.zeros((3,)))
  state = fg.bp_state
  state.evidence[v[0]] = np.arange(15.0)
  np.testing.assert_array_equal(state.evidence[v[0]], np.arange(15.0))
  with pytest.raises(ValueError, match="not in the FactorGraph"):
    state.evidence[(123, 2)] = np.zeros(2)
  state.ftov_msgs[v[1]] = np.ones(15)
  np.testing.assert_array_equal(state.ftov_msgs.value[15:30], np.ones(15, np.float32))
  with pytest.raises(ValueError, match="Provided variable or factor type is not in the FactorGraph"):
    state.ftov_msgs[(0, 1)] = np.zeros(1)
  state.log_potentials[g] = np.ones((1, 10))
  np.testing.assert_array_equal(state.log_potentials[g], np.ones(10))
  with pytest.raises(ValueError, match="Invalid FactorGroup"):
    _ = state.log_potentials[fgroup.EnumFactorGroup(variables_for_factors=[[v[0]]],
                                                    factor_configs=np.arange(2)[:, None])]


def test_ndvararray_flatten_torch_matches_numpy_with_ragged_states():
  import torch  # pylint: disable=g-import-not-at-top
  import pgmax_gb300 as pg  # pylint: disable=g-import-not-at-top
  g = pg.vgroup.NDVarArray(num_states=np.array([[2, 3], [3, 1]]), shape=(2, 2))
  rng = np.random.default_rng(0)
  for shape in ((2, 2, 3), (4, 2, 2, 3)):
    x = rng.normal(size=shape).astype(np.float32)
    np.testing.assert_array_equal(g.flatten(torch.as_tensor(x)).numpy(), g.flatten(x))
