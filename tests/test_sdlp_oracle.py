"""The SDLP oracle (oracle/sdlp.py) against the reference's own solver outputs.

Fixtures: every SDLP call of the reference's tests/lp/test_bp_for_lp.py and of the seeded cases of
tests/golden/cases.py (tests/golden/make_golden.py --sdlp-only). Bars:
  * temperature 0 (max-product updates, subgradient steps): messages bit for bit, factor updates
    and per-edge maxima bit for bit, objective values within 1e-6 relative (float64 vs float32
    sums);
  * temperature > 0, one evaluation (get_bp_updates): within 1e-5 absolute;
  * temperature > 0, runs: the first objective within 1e-5 relative; final messages within
    1e-4 + 10 x the case's sensitivity, measured by rerunning the oracle with the evidence moved
    by a random relative 2^-20 (accelerated gradient descent at lr = T is chaotic on some graphs:
    such a change there moves the messages by up to 5e-2, elsewhere by 1e-5 at most).
"""

import numpy as np
import pytest

import fixtures
from oracle import sdlp as oracle_sdlp

SDLP = fixtures.sdlp_fixture_paths()


def lr_of(fx):
  lr = float(fx["lr"])
  return None if lr < 0 else lr


def sensitivity(problem, fx):
  """Largest output change of the oracle's run when every evidence value moves by a random
  relative 2^-20 (about eight ulps, the size of the differences between two float32 exp / log
  implementations compounded over a few calls)."""
  T, n = float(fx["logsumexp_temp"]), int(fx["num_iters"])
  a, oa = problem.run_with_objvals(fx["log_potentials"], fx["evidence"], fx["ftov_msgs_in"], T, n,
                                   lr_of(fx))
  rng = np.random.default_rng(0)
  ev = fx["evidence"]
  ev = (ev * (1 + rng.uniform(-1, 1, ev.shape) * 2.0**-20)).astype(np.float32)
  b, ob = problem.run_with_objvals(fx["log_potentials"], ev, fx["ftov_msgs_in"], T, n, lr_of(fx))
  return float(np.max(np.abs(a - b), initial=0.0)), float(np.max(np.abs(oa - ob), initial=0.0))


def test_fixture_set_covers_calls_and_temperatures():
  calls = set()
  temps = set()
  for p in SDLP:
    fx = fixtures.load(p)
    calls.add(fx["meta"]["call"])
    temps.add(float(fx["logsumexp_temp"]))
  assert {"run_with_objvals", "get_bp_updates", "get_primal_upper_bound"} <= calls
  assert {0.0, 1e-3, 0.05, 1.0} <= temps
  assert len(SDLP) >= 150


@pytest.mark.parametrize("path", SDLP, ids=fixtures.fixture_id)
def test_oracle_matches_reference_sdlp(path):
  fx = fixtures.load(path)
  problem = oracle_sdlp.Problem(fx["wiring"])
  call = fx["meta"]["call"]
  T = float(fx["logsumexp_temp"])
  if call == "run_with_objvals":
    out, obj = problem.run_with_objvals(fx["log_potentials"], fx["evidence"], fx["ftov_msgs_in"],
                                        T, int(fx["num_iters"]), lr_of(fx))
    want_obj = fx["objvals"].astype(np.float64)
    if T == 0.0:
      assert np.array_equal(out, fx["ftov_msgs_out"])
      np.testing.assert_allclose(obj, want_obj, rtol=1e-6, atol=1e-6)
    else:
      if obj.size:
        assert abs(obj[0] - want_obj[0]) <= 1e-5 * max(1.0, abs(want_obj[0]))
      sens, _ = sensitivity(problem, fx)
      assert np.max(np.abs(out - fx["ftov_msgs_out"]), initial=0.0) <= 1e-4 + 10 * sens
  elif call == "get_bp_updates":
    _, _, upd, lse = problem.objective(fx["log_potentials"], fx["evidence"], fx["ftov_msgs_in"], T)
    if T == 0.0:
      assert np.array_equal(upd, fx["bp_updates"])
      assert np.array_equal(lse, fx["edge_lse"])
    else:
      np.testing.assert_allclose(upd, fx["bp_updates"], atol=1e-5, rtol=0)
      np.testing.assert_allclose(lse, fx["edge_lse"], atol=1e-5, rtol=0)
  else:
    obj, _, _, _ = problem.objective(fx["log_potentials"], fx["evidence"], fx["ftov_msgs_in"], 0.0)
    assert abs(obj - float(fx["objval"])) <= 1e-6 * max(1.0, abs(float(fx["objval"])))
