"""The Gumbel(0, 1) noise stream of perturb-and-MAP runs, as the oracle restates it (CPU).

The engine adds this stream to the evidence inside pgbp_run_perturbed; its specification (SplitMix64
counters, 23-bit uniforms, -ln(-ln(u)) with a float32 logarithm by range reduction and the atanh
series) is restated in C in oracle/bp_oracle.c and, here, a third time in NumPy float32, which must
agree with the C restatement bit for bit. The draws must follow the Gumbel(0, 1) law: a
Kolmogorov-Smirnov test against its CDF and its first two moments (Euler's constant, pi^2 / 6).
"""

import numpy as np
import pytest

from oracle import oracle

F = np.float32


def _ln(x):
  x = np.asarray(x, np.float32)
  b = x.view(np.uint32)
  e = ((b >> np.uint32(23)) & np.uint32(0xFF)).astype(np.int64) - 127
  m = ((b & np.uint32(0x7FFFFF)) | np.uint32(0x3F800000)).astype(np.uint32).view(np.float32).copy()
  big = m > F(float.fromhex("0x1.6a09e6p+0"))
  m[big] = m[big] * F(0.5)
  e[big] += 1
  s = (m - F(1)) / (m + F(1))
  z = s * s
  p = np.full_like(z, F(float.fromhex("0x1.c71c72p-4")))
  for c in ("0x1.24924ap-3", "0x1.99999ap-3", "0x1.555556p-2"):
    p = p * z + F(float.fromhex(c))
  p = p * z + F(1)
  return e.astype(np.float32) * F(float.fromhex("0x1.62e430p-1")) + (s * p) * F(2)


def _mix64(z):
  z = np.asarray(z, np.uint64)
  with np.errstate(over="ignore"):
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
  return z ^ (z >> np.uint64(31))


def numpy_gumbel(seed, count, first=0):
  key = _mix64(np.uint64(seed))
  c = np.arange(first, first + count, dtype=np.uint64)
  with np.errstate(over="ignore"):
    r = _mix64(key + (c + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15))
  k = (r >> np.uint64(41)).astype(np.uint32)
  u = (np.uint32(2) * k + np.uint32(1)).astype(np.float32) * F(2.0 ** -24)
  return -_ln(-_ln(u))


@pytest.mark.parametrize("seed", [0, 1, 1000, 2**63 + 5, 2**64 - 1])
def test_numpy_restatement_equals_the_c_oracle(seed):
  np.testing.assert_array_equal(numpy_gumbel(seed, 100_000), oracle.gumbel(seed, 100_000))


def test_stream_positions_and_seeds():
  a = oracle.gumbel(3, 5000)
  np.testing.assert_array_equal(oracle.gumbel(3, 1000, first=4000), a[4000:])
  assert not np.array_equal(a, oracle.gumbel(4, 5000))
  np.testing.assert_array_equal(a, oracle.gumbel(3, 5000))


def test_draws_follow_the_gumbel_law():
  stats = pytest.importorskip("scipy.stats")
  g = oracle.gumbel(11, 1_000_000).astype(np.float64)
  assert abs(g.mean() - np.euler_gamma) < 5 * np.sqrt(np.pi ** 2 / 6 / g.size)
  assert abs(g.var() - np.pi ** 2 / 6) < 0.02
  assert stats.kstest(g[:200_000], "gumbel_r").pvalue > 1e-3
  assert g.min() > -3.0 and g.max() < 17.0


def test_logarithm_is_accurate():
  x = np.exp(np.random.default_rng(0).uniform(np.log(5e-8), np.log(17.0), 200_000)).astype(np.float32)
  err = np.abs(_ln(x).astype(np.float64) - np.log(x.astype(np.float64)))
  assert np.all(err <= 4 * np.spacing(np.abs(np.log(x)).astype(np.float32)))
