"""The autotuner of the multi-kernel path (include/pgbp.h, pgbp_plan_tuning_*): decisions are
taken on the first run, exported, imported and cached as JSON; every tuned variant gives
bit-identical results, so a decision never changes what a run computes."""

import json
import types

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


def _api():
  from pgmax_gb300 import factor, fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  return types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer,
                               vgroup=vgroup)


def _plan(wiring, flags=None):
  from pgmax_gb300 import engine, native  # pylint: disable=g-import-not-at-top
  w = dict(wiring)
  w["num_variables"] = int(np.max(w["evidence_to_vars"], initial=-1)) + 1
  return engine.Plan(w, flags=native.FLAG_PATH_MULTI if flags is None else flags)


def _inputs(plan, B, seed):
  torch = _torch()
  rng = np.random.default_rng(seed)
  lp = torch.as_tensor(rng.normal(size=(plan.num_potentials,)).astype(np.float32), device="cuda")
  ev = torch.as_tensor(rng.gumbel(size=(B, plan.num_var_states)).astype(np.float32), device="cuda")
  m = torch.as_tensor(rng.normal(size=(B, plan.num_edge_states)).astype(np.float32), device="cuda")
  return lp, ev, m


def _wiring(builder, **kw):
  api = _api()
  fg, _, _ = cases.BUILDERS[builder](api, **kw)
  return api.infer.InfererContext(fg.bp_state).flat_wiring()


def test_first_run_tunes_and_exports_the_sites():
  w = _wiring("rbm", nh=40, nv=60, seed=1, sample=0)
  plan = _plan(w)
  lp, ev, m = _inputs(plan, 128, 0)
  plan.run(lp, ev, m, 5, 0.5, 0.0)
  entries = plan.tuning()
  e = [x for x in entries if x["batch"] == 128 and x["temperature0"]]
  assert len(e) == 1
  sites = e[0]["sites"]
  assert len(sites) == 5 + plan.info["num_pairwise_buckets"]
  assert sites[0] in (0, 1, 2) and sites[2] in (0, 1)  # binary sums and the 2 x 2 bucket timed
  assert sites[1] == -1                             # no other variables
  # no other bucket, no OR / AND factors, no generic Enum factors beyond the unary biases (which
  # run on their own kernel)
  assert all(v == -1 for v in sites[3:])


@pytest.mark.parametrize("temperature", [0.0, 1.0])
@pytest.mark.parametrize("builder,kw", [("rbm", dict(nh=40, nv=60, seed=2, sample=0)),
                                        ("deconv", dict(seed=4)),
                                        ("mixed", dict(seed=5))])
def test_every_variant_gives_identical_results(builder, kw, temperature):
  torch = _torch()
  w = _wiring(builder, **kw)
  outs = []
  # every site on variant 0, every site on variant 1, and the binary sums on variant 2 (two
  # instances per thread) with the rest on 0
  for forced in ((0, 0), (1, 1), (2, 0)):
    plan = _plan(w)
    n = 5 + plan.info["num_pairwise_buckets"]
    plan.load_tuning([{"batch": 8, "temperature0": temperature == 0.0, "path": 0,
                       "sites": [forced[0]] + [forced[1]] * (n - 1)}])
    lp, ev, m = _inputs(plan, 8, 3)
    out, deltas = plan.run(lp, ev, m, 12, 0.5, temperature)
    outs.append((out, deltas))
  # bit patterns, so that NaN compares equal to NaN (random messages drive one deconvolution
  # instance to NaN at T = 1, in the float32 oracle as well)
  same = lambda a, b: torch.equal(a.contiguous().view(torch.int32), b.contiguous().view(torch.int32))
  for o in outs[1:]:
    assert same(outs[0][0], o[0]) and same(outs[0][1], o[1])


def test_decisions_round_trip_and_json_cache(tmp_path, monkeypatch):
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  w = _wiring("deconv", seed=6)
  plan = _plan(w)
  lp, ev, m = _inputs(plan, 8, 1)
  plan.run(lp, ev, m, 3, 0.5, 0.0)
  first = plan.tuning()
  assert first and all(len(e["sites"]) == 5 + plan.info["num_pairwise_buckets"] for e in first)
  path = str(tmp_path / "tune.json")
  plan.save_tuning(path)
  table = json.load(open(path))
  assert plan.signature() in table
  monkeypatch.setenv(engine.TUNE_CACHE_ENV, path)
  again = _plan(w)
  assert again.tuning() == first
  # a plan of another graph ignores the table
  other = _plan(_wiring("deconv", seed=6, n_feat=3))
  assert other.tuning() == []


def test_entries_that_do_not_fit_the_plan_are_rejected():
  w = _wiring("mixed", seed=1)
  plan = _plan(w)
  with pytest.raises(Exception, match="does not fit"):
    plan.load_tuning([{"batch": 4, "temperature0": True, "path": 0, "sites": [0, 1]}])
  with pytest.raises(Exception, match="out of range"):
    n = 5 + plan.info["num_pairwise_buckets"]
    plan.load_tuning([{"batch": 4, "temperature0": True, "path": 0, "sites": [2] * n}])
