"""The reference's get_marginals fixtures (tests/golden/make_golden.py), checked on the CPU.

Each fixture holds a seeded run's output messages, the reference's flat beliefs, its unflattened
beliefs (padded with -inf where a group mixes state counts) and its marginals, leaf by leaf. The
flat beliefs must be the oracle's beliefs of the same evidence and messages, and the marginals a
softmax of the unflattened beliefs (float64 here, so within float32 rounding).
"""

import numpy as np
import pytest

import fixtures
from oracle import oracle

PATHS = fixtures.marginals_fixture_paths()


def test_fixtures_exist():
  names = {fixtures.fixture_id(p) for p in PATHS}
  assert {"marginals_mixed_T0", "marginals_deconv_T1", "marginals_rbm_T0"} <= names
  assert any(fixtures.fixture_id(p).startswith("marginals_potts") for p in PATHS)


@pytest.mark.parametrize("path", PATHS, ids=fixtures.fixture_id)
def test_reference_marginals_are_the_softmax_of_the_oracle_beliefs(path):
  d = fixtures.load(path)
  w = oracle.Wiring(d["wiring"])
  np.testing.assert_array_equal(oracle.beliefs(w, d["evidence"], d["ftov_msgs"]),
                                d["flat_beliefs"])
  padded = 0
  for k in range(int(d["num_leaves"])):
    b = d[f"leaf{k}.beliefs"].astype(np.float64)
    m = d[f"leaf{k}.marginals"]
    padded += int(np.isneginf(b).sum())
    mx = np.max(b, axis=-1, keepdims=True)
    want = np.exp(b - (np.log(np.sum(np.exp(b - mx), axis=-1, keepdims=True)) + mx))
    np.testing.assert_allclose(m, want, atol=2e-6, rtol=1e-5)
    assert np.all(m[np.isneginf(b)] == 0.0)
  if "mixed" in d["name"]:
    assert padded > 0  # the 2 / 3 / 4-state group is padded with -inf


def test_direct_fixture_edge_cases():
  z = np.load(f"{fixtures.FIXTURES}/marginals_direct.npz")
  a, out = z["in0"], z["out0"]
  assert out[0, 1] == 0.0 and np.all(out[1, :3] == 0.0)
  assert np.all(np.isnan(out[2]))          # every state -inf
  np.testing.assert_allclose(out[3], 0.2, rtol=1e-6)
  assert z["out2"].shape == (0, 4)
  assert np.isfinite(z["out1"]).all()
  assert a.shape == out.shape
