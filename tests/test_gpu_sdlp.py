"""GPU parity of the SDLP kernels (pgbp_sdlp_run / pgbp_sdlp_objective) through the C ABI and
the drop-in host API (pgmax_gb300.infer.SDLP).

Against the reference: every recorded SDLP call (tests/golden/fixtures/sdlp_*.npz). Bars, as for
the oracle (tests/test_sdlp_oracle.py): temperature 0 messages, factor updates and per-edge
maxima bit for bit, objective values within 1e-6 relative; temperature > 0 single evaluations
within 1e-5 absolute, runs within 1e-4 + 10 x the case's sensitivity (the oracle's change under
a random relative 2^-20 change of the evidence) and the first objective within 1e-5 relative. Batched runs equal the single-instance runs bit for bit.
"""

import types

import numpy as np
import pytest

import cases
import fixtures
from oracle import sdlp as oracle_sdlp
from test_sdlp_oracle import lr_of, sensitivity

pytestmark = pytest.mark.gpu

SDLP = fixtures.sdlp_fixture_paths()


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


def _plan(wiring):
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  w = dict(wiring)
  w["num_variables"] = int(np.max(w["evidence_to_vars"], initial=-1)) + 1
  return engine.Plan(w)


def _api():
  from pgmax_gb300 import factor, fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  return types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer,
                               vgroup=vgroup)


def _np(t):
  return t.detach().cpu().numpy()


@pytest.mark.parametrize("path", SDLP, ids=fixtures.fixture_id)
def test_sdlp_matches_reference(path):
  fx = fixtures.load(path)
  plan = _plan(fx["wiring"])
  call = fx["meta"]["call"]
  T = float(fx["logsumexp_temp"])
  lp, ev, m = fx["log_potentials"], fx["evidence"], fx["ftov_msgs_in"]
  if call == "run_with_objvals":
    lr = lr_of(fx)
    out, obj = plan.sdlp_run(lp, ev, m, int(fx["num_iters"]), T, lr)
    out, obj = _np(out), _np(obj).astype(np.float64)
    want_obj = fx["objvals"].astype(np.float64)
    if T == 0.0:
      assert np.array_equal(out, fx["ftov_msgs_out"])
      np.testing.assert_allclose(obj, want_obj, rtol=1e-6, atol=1e-6)
    else:
      if obj.size:
        assert abs(obj[0] - want_obj[0]) <= 1e-5 * max(1.0, abs(want_obj[0]))
      sens, _ = sensitivity(oracle_sdlp.Problem(fx["wiring"]), fx)
      assert np.max(np.abs(out - fx["ftov_msgs_out"]), initial=0.0) <= 1e-4 + 10 * sens
  elif call == "get_bp_updates":
    got = plan.sdlp_objective(lp, ev, m, T, updates=True, edge_lse=True)
    upd, lse = _np(got["updates"]), _np(got["edge_lse"])
    if T == 0.0:
      assert np.array_equal(upd, fx["bp_updates"])
      assert np.array_equal(lse, fx["edge_lse"])
    else:
      np.testing.assert_allclose(upd, fx["bp_updates"], atol=1e-5, rtol=0)
      np.testing.assert_allclose(lse, fx["edge_lse"], atol=1e-5, rtol=0)
  else:
    obj = float(plan.sdlp_objective(lp, ev, m, 0.0)["objval"])
    assert abs(obj - float(fx["objval"])) <= 1e-6 * max(1.0, abs(float(fx["objval"])))


def _case(builder, **kw):
  api = _api()
  fg, groups, ev = cases.BUILDERS[builder](api, **kw)
  ctx = api.infer.InfererContext(fg.bp_state)
  return fg, groups, ev, ctx


@pytest.mark.parametrize("builder,kw", [
    ("mixed", dict(seed=2)), ("deconv", dict(seed=3)), ("potts", dict(L=5, K=4, seed=1)),
    ("rbm", dict(nh=9, nv=11, seed=4, sample=0)),
])
@pytest.mark.parametrize("T", [0.0, 1e-3, 0.2, 1.0])
def test_gradient_and_objective_match_oracle(builder, kw, T):
  _, _, _, ctx = _case(builder, **kw)
  w = ctx.flat_wiring()
  plan = ctx.plan
  rng = np.random.default_rng(11)
  n_es, nvs = plan.num_edge_states, plan.num_var_states
  lp = rng.normal(size=(plan.num_potentials,)).astype(np.float32)
  ev = rng.gumbel(size=(nvs,)).astype(np.float32)
  m = rng.normal(size=(n_es,)).astype(np.float32)
  got = plan.sdlp_objective(lp, ev, m, T, grad=True, updates=True, edge_lse=True)
  obj, grad, upd, lse = oracle_sdlp.Problem(w).objective(lp, ev, m, T)
  if T == 0.0:
    assert np.array_equal(_np(got["grad"]), grad)
    assert np.array_equal(_np(got["updates"]), upd)
    assert np.array_equal(_np(got["edge_lse"]), lse)
  else:
    np.testing.assert_allclose(_np(got["grad"]), grad, atol=1e-5, rtol=0)
    np.testing.assert_allclose(_np(got["updates"]), upd, atol=1e-5, rtol=0)
    np.testing.assert_allclose(_np(got["edge_lse"]), lse, atol=1e-5, rtol=0)
  assert abs(float(got["objval"]) - obj) <= 1e-5 * max(1.0, abs(obj))


@pytest.mark.parametrize("T,lr", [(0.0, None), (0.05, 0.01), (1.0, None)])
def test_batched_run_equals_single_runs(T, lr):
  torch = _torch()
  _, _, _, ctx = _case("mixed", seed=1)
  plan = ctx.plan
  rng = np.random.default_rng(5)
  B = 6
  lp = rng.normal(size=(plan.num_potentials,)).astype(np.float32)
  ev = rng.gumbel(size=(B, plan.num_var_states)).astype(np.float32)
  m = rng.normal(size=(B, plan.num_edge_states)).astype(np.float32)
  out, obj = plan.sdlp_run(torch.as_tensor(lp), torch.as_tensor(ev), torch.as_tensor(m), 17, T, lr)
  assert tuple(out.shape) == (B, plan.num_edge_states) and tuple(obj.shape) == (B, 17)
  for b in range(B):
    o1, ob1 = plan.sdlp_run(lp, ev[b], m[b], 17, T, lr)
    assert torch.equal(out[b], o1) and torch.equal(obj[b], ob1)


def test_zero_iterations_copy_the_messages():
  _, _, _, ctx = _case("deconv", seed=2)
  plan = ctx.plan
  rng = np.random.default_rng(1)
  m = rng.normal(size=(plan.num_edge_states,)).astype(np.float32)
  ev = rng.normal(size=(plan.num_var_states,)).astype(np.float32)
  out, obj = plan.sdlp_run(np.zeros(0, np.float32), ev, m, 0, 0.5)
  assert np.array_equal(_np(out), m) and obj.numel() == 0


# ------------------------------------------------------------------ drop-in host API
def test_host_api_validates_like_the_reference():
  api = _api()
  fg, _, ev, _ = _case("potts", L=3, K=3, seed=0)
  sdlp = api.infer.build_inferer(fg.bp_state, backend="sdlp")
  arrays = sdlp.init(evidence_updates=ev)
  with pytest.raises(ValueError, match="has to be between 0.0 and 1.0"):
    sdlp.run(arrays, logsumexp_temp=1.01, num_iters=1)
  with pytest.raises(ValueError, match="learning rate must be smaller"):
    sdlp.run(arrays, logsumexp_temp=0.01, num_iters=1, lr=0.1)


@pytest.mark.parametrize("logsumexp_temp", [1e-3, 0.0])
def test_host_api_bounds_meet_on_a_tight_relaxation(logsumexp_temp):
  """The scenario of the reference's tests/lp/test_dual_lp.py::test_lp_primal_vs_dual_ising
  (fully connected 4 x 4 grid of 3-state variables, potentials 0.01 N(0, 1), Gumbel evidence),
  without the cvxpy primal: after 5,000 steps the primal upper bound and the MAP lower bound
  (minus the energy of the decoded unaries) agree within the reference's 5e-3, and the lower
  bound never exceeds the upper one."""
  api = _api()
  rng = np.random.default_rng(7)
  n, k = 4, 3
  variables = api.vgroup.NDVarArray(num_states=k, shape=(n, n))
  fg = api.fgraph.FactorGraph(variable_groups=variables)
  vff = [[variables[i, j], variables[a, b]] for i in range(n) for j in range(n)
         for a in range(i + 1, n) for b in range(j + 1, n)]
  fg.add_factors(api.fgroup.PairwiseFactorGroup(
      variables_for_factors=vff, log_potential_matrix=0.01 * rng.normal(size=(len(vff), k, k))))
  sdlp = api.infer.build_inferer(fg.bp_state, backend="sdlp")
  arrays = sdlp.init(evidence_updates={variables: rng.gumbel(size=(n, n, k))})
  arrays, objvals = sdlp.run_with_objvals(arrays, logsumexp_temp=logsumexp_temp, num_iters=5000)
  decoded, _ = sdlp.decode_primal_unaries(arrays)
  upper = float(sdlp.get_primal_upper_bound(arrays))
  lower = float(sdlp.get_map_lower_bound(arrays, decoded))
  assert lower <= upper + 1e-4
  assert np.isclose(lower, upper, rtol=5e-3)
  assert objvals.shape == (5000,)
  assert float(objvals[-1]) <= float(objvals[0])


def test_host_api_mixed_graph_runs_decodes_and_bounds():
  api = _api()
  fg, groups, ev, _ = _case("mixed", seed=4, vardict=False)
  sdlp = api.infer.SDLP(fg.bp_state)
  arrays = sdlp.run(sdlp.init(evidence_updates=ev), logsumexp_temp=0.1, num_iters=300)
  decoded, beliefs = sdlp.decode_primal_unaries(arrays)
  assert set(decoded) == set(groups) and set(beliefs) == set(groups)
  upper = float(sdlp.get_primal_upper_bound(arrays))
  lower = float(sdlp.get_map_lower_bound(arrays, decoded))
  assert lower <= upper + 1e-4
  upd, lse = sdlp.get_bp_updates(arrays, logsumexp_temp=0.1)
  assert tuple(upd.shape) == tuple(arrays.ftov_msgs.shape)
  assert tuple(lse.shape) == (api.infer.InfererContext(fg.bp_state).num_edges,)
