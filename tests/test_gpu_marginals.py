"""get_marginals and decode_map_states on the GPU against the reference's own outputs.

The fixtures (tests/golden/make_golden.py) hold, for seeded runs of the reference, its output
messages, its unflattened beliefs and the marginals its get_marginals (pgmax/infer/bp.py:263-288)
returned for them, leaf by leaf, including the mixed graph whose 2 / 3 / 4-state group is padded
with -inf. Here the same graph is rebuilt with pgmax_gb300, the reference's messages go through
bp.get_beliefs (the pgbp_beliefs kernel) and infer.get_marginals (the pgbp_marginals kernel), and
every leaf is compared element-wise: beliefs bit for bit (the same serial sums), marginals within
1e-5 absolute (CUDA's expf / logf against NumPy's float32 ones), padded states exactly 0. The
hand-made arrays of marginals_direct.npz (-inf states, a row of -inf that gives nan, magnitudes of
1e4, an empty array) go through the plan-free kernels pgbp_softmax_rows / pgbp_argmax_rows.
"""

import types

import numpy as np
import pytest

import cases
import fixtures

pytestmark = pytest.mark.gpu

ATOL = 1e-5
PATHS = fixtures.marginals_fixture_paths()


def _api():
  from pgmax_gb300 import factor, fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  return types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer,
                               vgroup=vgroup)


def _leaves(tree, prefix=()):
  out = []
  for k, v in tree.items():
    if isinstance(v, dict):
      out += _leaves(v, prefix + (k,))
    else:
      out.append((prefix + (k,), v))
  return out


def _sorted_leaves(tree, groups):
  keyed = {groups.index(g): v for g, v in tree.items()}
  return sorted(_leaves(keyed), key=lambda x: str(x[0]))


def _np(x):
  return x.detach().cpu().numpy() if hasattr(x, "detach") else np.asarray(x)


@pytest.mark.parametrize("path", PATHS, ids=fixtures.fixture_id)
def test_marginals_match_reference_get_marginals(path):
  import torch  # pylint: disable=g-import-not-at-top
  d = fixtures.load(path)
  meta = d["meta"]
  api = _api()
  fg, groups, _ = cases.BUILDERS[meta["builder"]](api, **meta["builder_kwargs"])
  bp = api.infer.BP(fg.bp_state, temperature=meta["run_kwargs"]["temperature"])
  arrays = api.infer.BPArrays(
      log_potentials=torch.as_tensor(d["log_potentials"], device="cuda"),
      ftov_msgs=torch.as_tensor(d["ftov_msgs"], device="cuda"),
      evidence=torch.as_tensor(d["evidence"], device="cuda"))
  beliefs = bp.get_beliefs(arrays)
  marg = api.infer.get_marginals(beliefs)
  bl = _sorted_leaves(beliefs, groups)
  ml = dict(_sorted_leaves(marg, groups))
  assert len(bl) == int(d["num_leaves"])
  for k, (path_k, b) in enumerate(bl):
    want_b = d[f"leaf{k}.beliefs"]
    want_m = d[f"leaf{k}.marginals"]
    np.testing.assert_array_equal(_np(b), want_b, err_msg=f"beliefs leaf {path_k}")
    got_m = _np(ml[path_k])
    np.testing.assert_allclose(got_m, want_m, atol=ATOL, rtol=0, err_msg=f"marginals {path_k}")
    assert np.all(got_m[np.isneginf(want_b)] == 0.0)
  # batched: two instances of the same beliefs through pgbp_marginals give the same rows
  flat = torch.as_tensor(d["flat_beliefs"], device="cuda")
  two = bp.context.plan.marginals(torch.stack([flat, flat]))
  one = bp.context.plan.marginals(flat)
  assert torch.equal(two[0], one) and torch.equal(two[1], one)


def test_direct_arrays_match_reference_get_marginals():
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer  # pylint: disable=g-import-not-at-top
  z = np.load(f"{fixtures.FIXTURES}/marginals_direct.npz")
  ins = {k: z[k] for k in ("in0", "in1", "in2", "in3")}
  for src in (ins, {k: torch.as_tensor(v, device="cuda") for k, v in ins.items()}):
    got = infer.get_marginals(src)
    for k in ins:
      want = z["out" + k[2:]]
      g = _np(got[k])
      assert g.shape == want.shape
      np.testing.assert_array_equal(np.isnan(g), np.isnan(want))
      ok = ~np.isnan(want)
      np.testing.assert_allclose(g[ok], want[ok], atol=ATOL, rtol=0)
      assert np.all(g[ok & (want == 0.0)] == 0.0)


def test_direct_arrays_decode_like_jnp_argmax():
  from pgmax_gb300 import infer  # pylint: disable=g-import-not-at-top
  rng = np.random.default_rng(2)
  a = rng.integers(0, 3, size=(50, 6)).astype(np.float32)   # many ties: first maximum wins
  a[3, 2] = np.nan                                           # first NaN wins
  a[4, :] = -np.inf
  b = rng.normal(size=(3, 4, 7)).astype(np.float32)
  got = infer.decode_map_states({"a": a, "b": b, "e": np.zeros((0, 3), np.float32)})
  np.testing.assert_array_equal(_np(got["a"]), np.argmax(a, axis=-1))
  np.testing.assert_array_equal(_np(got["b"]), np.argmax(b, axis=-1))
  assert _np(got["a"]).dtype == np.int32
  assert _np(got["e"]).shape == (0,)
