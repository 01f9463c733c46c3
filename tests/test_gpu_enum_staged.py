"""Generic EnumFactors (config tables that are not dense pairwise) on the two generic kernels.

The staged kernel runs a CTA per (factor, group of up to 32 instances) with the factor's
variable-to-factor messages, the running max / exp-sum per edge state, a tile of its config rows
and the tile's config sums in shared memory; the per-thread kernel runs a thread per
(factor, instance). Both perform pass_enum_fac_to_var_messages (pgmax/factor/enum.py:451-475)
with the same float32 operations in the same order, so their messages must be bit-identical.
Both are also checked against the C oracle: bit-exact at temperature 0; at temperature > 0
within 1e-5 for one factor update and 1e-4 after four iterations on these random inputs, whose
messages reach magnitudes of 15: each iteration's sums of up to hundreds of exponentials carry
CUDA's and glibc's expf / logf ulp differences into the next (the same bound as the other
perturbed-input tests). The graphs cover tables spanning several tiles, edges of
2 states (stored as one compressed slot), states that no config holds, and batches that leave
a group of instances partly empty.
"""

import itertools
import types

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

ATOL = 1e-5
RUN_T_POS_ATOL = 1e-4


def _api():
  from pgmax_gb300 import factor, fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  return types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer,
                               vgroup=vgroup)


# name: (variable states, arity, factors, fraction of configs kept)
SHAPES = {
    "ternary_dense_k10": ((10,), 3, 12, 1.0),         # 1,000 configs: several tiles
    "quaternary_mixed": ((2, 3, 4, 6), 4, 40, 0.3),    # binary edges, sparse tables
    "wide_binary": ((2,), 9, 16, 0.5),                 # 9 binary edges, 256 configs
    "pairwise_sparse_big": ((150, 120), 2, 6, 0.3),    # 270 edge states, 5,400 configs
}


def _graph(name, seed=0):
  states, arity, n_fac, keep = SHAPES[name]
  api = _api()
  rng = np.random.RandomState(seed)
  n_vars = max(3 * arity, 8)
  ns = np.array([states[i % len(states)] for i in range(n_vars)], dtype=np.int64)
  var = api.vgroup.NDVarArray(num_states=ns, shape=(n_vars,))
  fg = api.fgraph.FactorGraph(variable_groups=[var])
  seen = set()
  while len(seen) < n_fac:
    vs = sorted(rng.choice(n_vars, size=arity, replace=False).tolist())
    if tuple(vs) in seen:  # one factor per variable set
      continue
    seen.add(tuple(vs))
    allc = np.array(list(itertools.product(*[range(int(ns[v])) for v in vs])), dtype=np.int64)
    if keep < 1.0:
      sel = rng.rand(allc.shape[0]) < keep
      sel[rng.randint(allc.shape[0])] = True
      allc = allc[sel]
    fg.add_factors(api.factor.EnumFactor(variables=[var[v] for v in vs], factor_configs=allc,
                                         log_potentials=rng.normal(size=(allc.shape[0],))))
  w = api.infer.InfererContext(fg.bp_state).flat_wiring()
  lp = np.asarray(fg.bp_state.log_potentials.value, np.float32)
  return w, lp


def _plan(w):
  from pgmax_gb300 import engine, native  # pylint: disable=g-import-not-at-top
  w = dict(w)
  w["num_variables"] = int(np.max(w["evidence_to_vars"], initial=-1)) + 1
  return engine.Plan(w, flags=native.FLAG_NO_SMALL_GRAPH)


def _with_kernel(knob, fn):
  from pgmax_gb300 import native  # pylint: disable=g-import-not-at-top
  native.debug_set(native.DEBUG_ENUM_KERNEL, knob)
  try:
    return fn()
  finally:
    native.debug_set(native.DEBUG_ENUM_KERNEL, 0)


def _inputs(w, lp, B, seed):
  rng = np.random.RandomState(seed + 7)
  nvs = int(np.asarray(w["var_states_for_edge_states"]).max()) + 1
  nes = np.asarray(w["var_states_for_edge_states"]).shape[0]
  ev = rng.gumbel(size=(B, nvs)).astype(np.float32)
  msgs = rng.normal(size=(B, nes)).astype(np.float32)
  lpb = np.broadcast_to(lp, (B, lp.shape[0])).copy()
  lpb += rng.normal(scale=0.1, size=lpb.shape).astype(np.float32)  # per-instance potentials
  return lpb, ev, msgs


@pytest.mark.parametrize("T", [0.0, 0.7])
@pytest.mark.parametrize("B", [1, 5, 40])
@pytest.mark.parametrize("name", sorted(SHAPES))
def test_staged_kernel_equals_per_thread_kernel_and_oracle(name, B, T):
  w, lp = _graph(name)
  plan = _plan(w)
  lpb, ev, msgs = _inputs(w, lp, B, 0)
  iters = 4
  outs = {}
  for knob in (1, 2):
    out, deltas = _with_kernel(knob, lambda: plan.run(lpb, ev, msgs, iters, 0.5, T))
    outs[knob] = (out.cpu().numpy(), deltas.cpu().numpy())
  np.testing.assert_array_equal(outs[2][0], outs[1][0])
  np.testing.assert_array_equal(outs[2][1], outs[1][1])
  ow = oracle.Wiring(w)
  for b in sorted({0, B - 1}):
    o_out, o_d = oracle.run(ow, lpb[b], ev[b], msgs[b], iters, 0.5, T)
    if T == 0.0:
      np.testing.assert_array_equal(outs[2][0][b], o_out)
      np.testing.assert_array_equal(outs[2][1][b], o_d)
    else:
      np.testing.assert_allclose(outs[2][0][b], o_out, atol=RUN_T_POS_ATOL, rtol=0)


@pytest.mark.parametrize("T", [0.0, 0.7])
@pytest.mark.parametrize("name", ["quaternary_mixed", "ternary_dense_k10"])
def test_staged_kernel_factor_update_equals_per_thread_kernel_and_oracle(name, T):
  """FAC_TO_VAR_UPDATES[EnumFactor] on caller arrays through both kernels."""
  w, lp = _graph(name, seed=3)
  plan = _plan(w)
  B = 6
  rng = np.random.RandomState(11)
  n = int(plan.msgs_ranges[0, 1] - plan.msgs_ranges[0, 0])
  vt = rng.normal(size=(B, n)).astype(np.float32)
  got = {k: _with_kernel(k, lambda: plan.factor_update(0, vt, lp, T).cpu().numpy()) for k in (1, 2)}
  np.testing.assert_array_equal(got[2], got[1])
  ow = oracle.Wiring(w)
  for b in (0, B - 1):
    orc = oracle.factor_update(ow, 0, vt[b], lp, T, True)
    if T == 0.0:
      np.testing.assert_array_equal(got[2][b], orc)
    else:
      fin = np.isfinite(orc)
      np.testing.assert_array_equal(np.isfinite(got[2][b]), fin)
      np.testing.assert_allclose(got[2][b][fin], orc[fin], atol=ATOL, rtol=0)


def test_tuner_times_the_generic_site():
  """The first run at a batch times both generic kernels and records the faster as the last site."""
  w, lp = _graph("quaternary_mixed", seed=5)
  plan = _plan(w)
  lpb, ev, msgs = _inputs(w, lp, 64, 5)
  out_tuned, _ = plan.run(lpb, ev, msgs, 3, 0.5, 0.0)
  e = [x for x in plan.tuning() if x["batch"] == 64 and x["temperature0"]]
  assert len(e) == 1
  sites = e[0]["sites"]
  assert len(sites) == 5 + plan.info["num_pairwise_buckets"]
  assert sites[-1] in (0, 1)
  out_ref, _ = _with_kernel(1, lambda: plan.run(lpb, ev, msgs, 3, 0.5, 0.0))
  np.testing.assert_array_equal(out_tuned.cpu().numpy(), out_ref.cpu().numpy())
