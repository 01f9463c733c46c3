"""The C oracle (oracle/bp_oracle.c) against the reference's own outputs.

Pins the checker before it is trusted: every BP run captured from the reference (its own tests and
the seeded cases, run through PGMax 0.6.1 itself, see tests/golden/make_golden.py) must be
reproduced bit for bit at temperature 0 and within 1e-5 at temperature > 0 (exp/log differ from
XLA's by ulps). Includes the 84-message golden vector of the reference's tests/test_pgmax.py:63-152
(atol 1e-6) and its MAP states.
"""

import numpy as np
import pytest

import fixtures
from oracle import oracle

RUNS = fixtures.run_fixture_paths()
T_POS_ATOL = 1e-5


@pytest.mark.parametrize("path", RUNS, ids=fixtures.fixture_id)
def test_oracle_matches_reference_run(path):
  f = fixtures.load(path)
  w = oracle.Wiring(f["wiring"])
  out, deltas = oracle.run(w, f["log_potentials"], f["evidence"], f["ftov_msgs_in"],
                           int(f["num_iters"]), float(f["damping"]), float(f["temperature"]))
  ref = f["ftov_msgs_out"]
  if float(f["temperature"]) == 0.0:
    np.testing.assert_array_equal(out, ref)
    np.testing.assert_array_equal(deltas, f["deltas"])
  else:
    np.testing.assert_allclose(out, ref, atol=T_POS_ATOL, rtol=0)
    np.testing.assert_allclose(deltas, f["deltas"], atol=T_POS_ATOL, rtol=0)
  bel = oracle.beliefs(w, f["evidence"], out)
  np.testing.assert_allclose(bel, f["flat_beliefs"], atol=T_POS_ATOL, rtol=0)


def test_golden_vector_of_reference_test_suite():
  path = [p for p in RUNS if "test_e2e_sanity_check" in p][0]
  f = fixtures.load(path)
  w = oracle.Wiring(f["wiring"])
  out, _ = oracle.run(w, f["log_potentials"], f["evidence"], f["ftov_msgs_in"],
                      int(f["num_iters"]), float(f["damping"]), float(f["temperature"]))
  assert out.shape == (84,)
  # the reference test's own assertion: jnp.allclose(msgs, golden, atol=1e-6)
  assert np.allclose(out, f["golden_expected"], atol=1e-6)
  # MAP states (tests/test_pgmax.py:252-265, 419-421) from the oracle's beliefs
  bel = oracle.beliefs(w, f["evidence"], out)
  e2v = f["wiring"]["evidence_to_vars"]
  starts = np.concatenate([[0], np.nonzero(np.diff(e2v))[0] + 1])
  ends = np.concatenate([starts[1:], [e2v.shape[0]]])
  decoded = np.array([int(np.argmax(bel[s:e])) for s, e in zip(starts, ends)])
  np.testing.assert_array_equal(decoded, f["map_flat"])


def test_factor_updates_match_reference():
  z = np.load(f"{fixtures.FIXTURES}/factor_updates_mixed.npz")
  w = oracle.Wiring({k[2:]: z[k] for k in z.files if k.startswith("w.")})
  lp = z["log_potentials"]
  checked = 0
  for u in range(int(z["num_updates"])):
    vt = z[f"upd{u}.vtof"]
    t = float(z[f"upd{u}.temperature"])
    nz = bool(z[f"upd{u}.normalize"])
    for ti, name in enumerate(("enum", "or", "and", "pool")):
      key = f"upd{u}.{name}"
      if key not in z.files:
        continue
      ms, me = w.msgs_ranges[ti]
      ps, pe = w.potentials_ranges[ti]
      out = oracle.factor_update(w, ti, vt[ms:me], lp[ps:pe], t, nz)
      np.testing.assert_allclose(out, z[key], atol=T_POS_ATOL, rtol=0)
      if t == 0.0:
        np.testing.assert_array_equal(out, z[key])
      checked += 1
  assert checked >= 40


def test_num_iters_zero_runs_one_iteration():
  """bp.py:142-146: num_iters <= 1 performs exactly one update."""
  path = [p for p in RUNS if "mixed_iters0" in p][0]
  f = fixtures.load(path)
  w = oracle.Wiring(f["wiring"])
  a, da = oracle.run(w, f["log_potentials"], f["evidence"], f["ftov_msgs_in"], 0, 0.5, 1.0)
  b, db = oracle.run(w, f["log_potentials"], f["evidence"], f["ftov_msgs_in"], 1, 0.5, 1.0)
  np.testing.assert_array_equal(a, b)
  assert da.shape == (1,) and db.shape == (1,)


def test_oracle_batch_equals_single_runs():
  path = [p for p in RUNS if "rbm_s0" in p][0]
  f = fixtures.load(path)
  w = oracle.Wiring(f["wiring"])
  rng = np.random.default_rng(0)
  ev = f["evidence"][None] + rng.gumbel(size=(3,) + f["evidence"].shape).astype(np.float32)
  outs, ds = oracle.run_batch(w, f["log_potentials"], ev, f["ftov_msgs_in"], 20, 0.5, 0.0,
                              num_threads=3)
  for b in range(3):
    o, d = oracle.run(w, f["log_potentials"], ev[b], f["ftov_msgs_in"], 20, 0.5, 0.0)
    np.testing.assert_array_equal(outs[b], o)
    np.testing.assert_array_equal(ds[b], d)
