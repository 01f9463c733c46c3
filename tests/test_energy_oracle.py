"""The energy oracle (oracle/energy.py) against the reference's own compute_energy outputs.

The fixtures are every non-debug `infer.compute_energy` call of the reference's tests
(tests/test_energy.py, tests/factor/test_{or,and,pool}.py) and of the seeded cases of
tests/golden/cases.py (BP decodings, random, repaired, out-of-range and negative states, infinite
evidence), recorded by tests/golden/make_golden.py. Infinite and nan energies must match exactly;
finite ones within 2e-6 of the sum of |evidence| and |log potentials| (the reference sums in
float32, the oracle in float64).
"""

import numpy as np
import pytest

import fixtures
from oracle import energy as oracle_energy

ENERGIES = fixtures.energy_fixture_paths()
REL = 2e-6


def scale_of(fx):
  ev = fx["evidence"].astype(np.float64)
  lp = fx["log_potentials"].astype(np.float64)
  return np.abs(ev[np.isfinite(ev)]).sum() + np.abs(lp[np.isfinite(lp)]).sum()


def assert_energy_close(got, want, scale, rel=REL):
  if np.isnan(want):
    assert np.isnan(got), (got, want)
  elif np.isinf(want):
    assert got == want, (got, want)
  else:
    assert np.isfinite(got) and abs(got - want) <= rel * scale + 1e-6, (got, want, scale)


def test_fixture_set_covers_every_outcome():
  kinds = {"finite": 0, "inf": 0, "nan": 0}
  sources = set()
  for p in ENERGIES:
    fx = fixtures.load(p)
    e = float(fx["energy"])
    kinds["nan" if np.isnan(e) else "inf" if np.isinf(e) else "finite"] += 1
    sources.add(fx["meta"]["source"].split("::")[0])
  assert len(ENERGIES) >= 100
  assert min(kinds.values()) > 0, kinds
  assert {"test_energy", "factor.test_or", "factor.test_and", "factor.test_pool",
          "energy_case"} <= sources, sources


@pytest.mark.parametrize("path", ENERGIES, ids=fixtures.fixture_id)
def test_oracle_matches_reference_energy(path):
  fx = fixtures.load(path)
  got = oracle_energy.compute_energy(fx["wiring"], fx["log_potentials"], fx["evidence"],
                                     fx["map_flat"])
  assert_energy_close(got, float(fx["energy"]), scale_of(fx))


def test_oracle_one_hot_wraps_negative_states_once():
  e2v = np.array([0, 0, 0, 1, 1], np.int32)
  oh = oracle_energy.var_state_onehot(e2v, np.array([-1, 2]))
  assert oh.tolist() == [0, 0, 1, 0, 0]
  oh = oracle_energy.var_state_onehot(e2v, np.array([-4, -2]))
  assert oh.tolist() == [0, 0, 0, 1, 0]


DEBUG = [p for p in ENERGIES if "debug_energy" in np.load(p).files]


def _same_terms(got, want):
  """Bit-equal float32 values in float64, nan matching nan."""
  got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
  return got.shape == want.shape and np.array_equal(got, want, equal_nan=True)


def test_debug_fixtures_exist():
  # the reference's debug mode fails on graphs with single factors; the rest are recorded
  assert len(DEBUG) >= 100


@pytest.mark.parametrize("path", DEBUG, ids=fixtures.fixture_id)
def test_debug_terms_match_reference(path):
  """compute_energy_terms against the reference's debug mode (energy.py:151-204): every variable
  and factor term bit for bit, and the total summed as the reference sums it (variables, then
  factors, in Python floats)."""
  fx = fixtures.load(path)
  var_t, fac_t = oracle_energy.compute_energy_terms(fx["wiring"], fx["debug_factor_potentials"],
                                                    fx["evidence"], fx["map_flat"])
  assert _same_terms(var_t, fx["debug_var_terms"])
  assert _same_terms(fac_t, fx["debug_fac_terms"])
  total = 0.0
  for x in list(var_t) + list(fac_t):
    total += float(x)
  want = float(fx["debug_energy"])
  assert (np.isnan(total) and np.isnan(want)) or total == want
