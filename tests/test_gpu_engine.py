"""GPU parity: the CUDA engine (through the C ABI) against the C oracle and the reference's outputs.

Tolerances: temperature 0 is bit-exact (same float32 operations in the same order; the engine is
built with -fmad=false); temperature > 0 within 1e-5 absolute of both the oracle and the
reference, the bar the BP north star sets; MAP decodes identical except where the two best
beliefs of a variable are within 1e-4 (a tie at this tolerance), which the tests count.
"""

import types

import numpy as np
import pytest

import cases
import fixtures
from oracle import oracle

pytestmark = pytest.mark.gpu

ATOL = 1e-5
RUNS = fixtures.run_fixture_paths()


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


# Execution paths (include/pgbp.h): "multi" = one launch per kernel class per iteration; "small" =
# one CTA per instance with its state in shared memory; "cluster" = one thread-block cluster per
# instance; "auto" = the fastest of the eligible ones, timed on first use. Every path must give
# the same results.
PATHS = ("auto", "multi", "small", "cluster")


def _plan(wiring, path="auto"):
  from pgmax_gb300 import engine, native  # pylint: disable=g-import-not-at-top
  w = dict(wiring)
  if "evidence_to_vars" in w:
    w["num_variables"] = int(np.max(w["evidence_to_vars"], initial=-1)) + 1
  flags = {"auto": 0, "multi": native.FLAG_NO_SMALL_GRAPH, "small": native.FLAG_PATH_SMALL,
           "cluster": native.FLAG_PATH_CLUSTER}[path]
  return engine.Plan(w, flags=flags)


def _np(t):
  return t.detach().cpu().numpy()


def _decode_host(bel, e2v):
  starts = np.concatenate([[0], np.nonzero(np.diff(e2v))[0] + 1])
  ends = np.concatenate([starts[1:], [e2v.shape[0]]])
  return np.array([int(np.argmax(bel[s:e])) for s, e in zip(starts, ends)]), starts, ends


def _near_tie(bel, starts, ends, tol=1e-4):
  out = []
  for s, e in zip(starts, ends):
    x = np.sort(bel[s:e])[::-1]
    out.append(x.shape[0] > 1 and x[0] - x[1] < tol)
  return np.array(out)


@pytest.mark.parametrize("exec_path", PATHS)
@pytest.mark.parametrize("path", RUNS, ids=fixtures.fixture_id)
def test_run_matches_oracle_and_reference(path, exec_path):
  f = fixtures.load(path)
  plan = _plan(f["wiring"], exec_path)
  T = float(f["temperature"])
  args = (int(f["num_iters"]), float(f["damping"]), T)
  out, deltas = plan.run(f["log_potentials"], f["evidence"], f["ftov_msgs_in"], *args)
  out, deltas = _np(out), _np(deltas)
  w = oracle.Wiring(f["wiring"])
  o_out, o_deltas = oracle.run(w, f["log_potentials"], f["evidence"], f["ftov_msgs_in"], *args)
  if T == 0.0:
    np.testing.assert_array_equal(out, o_out)
    np.testing.assert_array_equal(deltas, o_deltas)
    np.testing.assert_array_equal(out, f["ftov_msgs_out"])
  else:
    np.testing.assert_allclose(out, o_out, atol=ATOL, rtol=0)
    np.testing.assert_allclose(out, f["ftov_msgs_out"], atol=ATOL, rtol=0)
    np.testing.assert_allclose(deltas, o_deltas, atol=ATOL, rtol=0)
  bel = _np(plan.beliefs(f["evidence"], out))
  np.testing.assert_allclose(bel, oracle.beliefs(w, f["evidence"], out), atol=1e-6, rtol=1e-6)
  np.testing.assert_allclose(bel, f["flat_beliefs"], atol=ATOL, rtol=1e-6)
  e2v = f["wiring"]["evidence_to_vars"]
  got = _np(plan.decode(bel, int(e2v[-1]) + 1))
  host, starts, ends = _decode_host(bel, e2v)
  np.testing.assert_array_equal(got, host)
  mism = got != f["map_flat"]
  assert not (mism & ~_near_tie(f["flat_beliefs"], starts, ends)).any()


# On randomly perturbed inputs at temperature > 0 the OR/AND updates subtract nearly equal
# log-sums (logminusexp_with_temp, pgmax/factor/update_utils.py:169-190), which amplifies the ulp
# differences between CUDA's and glibc's expf/log1pf; 1e-4 bounds the engine-oracle gap there.
# Against the reference's own captured runs the engine stays within 1e-5 (test above).
PERTURBED_T_POS_ATOL = 1e-4


@pytest.mark.parametrize("exec_path", PATHS)
@pytest.mark.parametrize("name", ["case_rbm_s0", "case_mixed_T0", "case_mixed_T1", "case_deconv_T1",
                                  "case_potts_K8"])
def test_batched_run_equals_single_instances(name, exec_path):
  f = fixtures.load(f"{fixtures.FIXTURES}/{name}.npz")
  plan = _plan(f["wiring"], exec_path)
  w = oracle.Wiring(f["wiring"])
  rng = np.random.default_rng(1)
  B = 37
  ev = (f["evidence"][None] + rng.gumbel(size=(B,) + f["evidence"].shape)).astype(np.float32)
  msgs = (f["ftov_msgs_in"][None] + rng.normal(size=(B,) + f["ftov_msgs_in"].shape)).astype(np.float32)
  lp = (f["log_potentials"][None] + 0.1 * rng.normal(size=(B,) + f["log_potentials"].shape)).astype(np.float32)
  T = float(f["temperature"])
  for lp_in in (f["log_potentials"], lp):
    out, deltas = plan.run(lp_in, ev, msgs, 9, 0.5, T)
    out, deltas = _np(out), _np(deltas)
    assert out.shape == (B, f["ftov_msgs_in"].shape[0]) and deltas.shape == (B, 9)
    for b in (0, 5, B - 1):
      lpb = lp_in if lp_in.ndim == 1 else lp_in[b]
      single, single_d = plan.run(lpb, ev[b], msgs[b], 9, 0.5, T)
      np.testing.assert_array_equal(out[b], _np(single))
      np.testing.assert_array_equal(deltas[b], _np(single_d))
      o, d = oracle.run(w, lpb, ev[b], msgs[b], 9, 0.5, T)
      if T == 0.0:
        np.testing.assert_array_equal(out[b], o)
        np.testing.assert_array_equal(deltas[b], d)
      else:
        np.testing.assert_allclose(out[b], o, atol=PERTURBED_T_POS_ATOL, rtol=0)
        np.testing.assert_allclose(deltas[b], d, atol=PERTURBED_T_POS_ATOL, rtol=0)


@pytest.mark.parametrize("name,B", [("case_rbm_s0", 8), ("case_rbm_s1", 12), ("case_ising12_T1", 4),
                                    ("case_ising50_T0", 16), ("case_rbm_s0", "x4"),
                                    ("case_ising12_T1", "x4"), ("case_ising50_T0", "x4"),
                                    ("case_ising50_T1", "x4")])
def test_four_instances_per_thread_path(name, B):
  """Batches that are a multiple of 4 and large enough to leave >= 16 warps per SM (B = "x4":
  sized from the GPU's SM count) run the 4-instances-per-thread kernels (binary pairwise factors,
  binary variable sums) on the multi-kernel path; small ones run one instance per thread. Every
  instance must equal its own oracle run."""
  torch = _torch()
  f = fixtures.load(f"{fixtures.FIXTURES}/{name}.npz")
  plan = _plan(f["wiring"], "multi")
  w = oracle.Wiring(f["wiring"])
  if B == "x4":
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    n_pw = plan.info["num_enum_pairwise_factors"]
    n_vars = int(np.max(f["wiring"]["evidence_to_vars"])) + 1
    units = n_pw if name.startswith("case_rbm") else min(n_pw, n_vars)
    B = 4 * (-(-sms * 16 * 32 // units))
  rng = np.random.default_rng(3)
  ev = (f["evidence"][None] + rng.gumbel(size=(B,) + f["evidence"].shape)).astype(np.float32)
  T = float(f["temperature"])
  lp_b = (f["log_potentials"][None] + 0.05 * rng.normal(size=(B,) + f["log_potentials"].shape)
          ).astype(np.float32)
  for lp in (f["log_potentials"], lp_b):
    out, deltas = plan.run(lp, ev, f["ftov_msgs_in"], 15, 0.5, T)
    out, deltas = _np(out), _np(deltas)
    o, d = oracle.run_batch(w, lp, ev, f["ftov_msgs_in"], 15, 0.5, T)
    if T == 0.0:
      np.testing.assert_array_equal(out, o)
      np.testing.assert_array_equal(deltas, d)
    else:
      np.testing.assert_allclose(out, o, atol=ATOL, rtol=0)
      np.testing.assert_allclose(deltas, d, atol=ATOL, rtol=0)


@pytest.mark.parametrize("exec_path", PATHS)
def test_runs_are_bitwise_deterministic(exec_path):
  f = fixtures.load(f"{fixtures.FIXTURES}/case_deconv_T1.npz")
  plan = _plan(f["wiring"], exec_path)
  a = _np(plan.run(f["log_potentials"], f["evidence"], f["ftov_msgs_in"], 40, 0.5, 1.0)[0])
  b = _np(plan.run(f["log_potentials"], f["evidence"], f["ftov_msgs_in"], 40, 0.5, 1.0)[0])
  np.testing.assert_array_equal(a, b)


def test_factor_updates_match_reference_and_oracle():
  z = np.load(f"{fixtures.FIXTURES}/factor_updates_mixed.npz")
  wiring = {k[2:]: z[k] for k in z.files if k.startswith("w.")}
  plan = _plan(wiring)
  w = oracle.Wiring(wiring)
  lp = z["log_potentials"]
  n = 0
  for u in range(int(z["num_updates"])):
    vt = z[f"upd{u}.vtof"]
    T = float(z[f"upd{u}.temperature"])
    nz = bool(z[f"upd{u}.normalize"])
    for ti, key in enumerate(("enum", "or", "and", "pool")):
      if f"upd{u}.{key}" not in z.files:
        continue
      ms, me = w.msgs_ranges[ti]
      ps, pe = w.potentials_ranges[ti]
      got = _np(plan.factor_update(ti, vt[ms:me], lp[ps:pe] if pe > ps else None, T, nz))
      ref = z[f"upd{u}.{key}"]
      orc = oracle.factor_update(w, ti, vt[ms:me], lp[ps:pe], T, nz)
      fin = np.isfinite(ref)
      np.testing.assert_array_equal(np.isfinite(got), fin)
      np.testing.assert_allclose(got[fin], ref[fin], atol=ATOL, rtol=0)
      if T == 0.0:
        np.testing.assert_array_equal(got, orc)
      n += 1
  assert n >= 40


def test_drop_in_api_end_to_end():
  """pgmax_gb300.infer.BP used exactly like pgmax.infer.BP on the mixed graph."""
  from pgmax_gb300 import factor, fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  api = types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer, vgroup=vgroup)
  f = fixtures.load(f"{fixtures.FIXTURES}/case_mixed_T0.npz")
  fg, groups, ev = cases.mixed(api, seed=0)
  bp = infer.build_inferer(fg.bp_state, backend="bp")
  bp_arrays = bp.init(evidence_updates=ev,
                      ftov_msgs_updates=cases.mixed_ftov_updates(api, groups, seed=0))
  bp_arrays, deltas = bp.run_with_diffs(bp_arrays, num_iters=7, damping=0.5, temperature=0.0)
  np.testing.assert_array_equal(_np(bp_arrays.ftov_msgs), f["ftov_msgs_out"])
  np.testing.assert_array_equal(_np(deltas), f["deltas"])
  beliefs = bp.get_beliefs(bp_arrays)
  decoded = infer.decode_map_states(beliefs)
  flat = []
  for g in groups:
    m = decoded[g]
    flat += [int(m[n]) for n in g.variable_names] if isinstance(m, dict) else list(_np(m).reshape(-1))
  np.testing.assert_array_equal(flat, f["map_flat"])
  marg = infer.get_marginals(beliefs)
  for g in groups:
    m = marg[g]
    if isinstance(m, dict):
      for v in m.values():
        assert abs(float(v.sum()) - 1.0) < 1e-5
    else:
      np.testing.assert_allclose(_np(m).sum(-1), 1.0, atol=1e-5)
  state = bp.to_bp_state(bp_arrays)
  np.testing.assert_array_equal(state.ftov_msgs.value, f["ftov_msgs_out"])
  with pytest.warns(UserWarning, match="deprecated"):
    again = bp.run_bp(bp.init(evidence_updates=ev), num_iters=3)
  assert again.ftov_msgs.shape == bp_arrays.ftov_msgs.shape


def test_small_graph_path_is_taken_for_small_graphs():
  f = fixtures.load(f"{fixtures.FIXTURES}/case_ising50_T1.npz")
  assert _plan(f["wiring"]).info["small_graph_smem_bytes"] > 0
  assert _plan(f["wiring"], "multi").info["small_graph_smem_bytes"] == 0


def test_all_paths_agree_bitwise_on_a_batch():
  f = fixtures.load(f"{fixtures.FIXTURES}/case_deconv_T1.npz")
  rng = np.random.default_rng(9)
  ev = (f["evidence"][None] + rng.gumbel(size=(6,) + f["evidence"].shape)).astype(np.float32)
  outs = []
  for path in PATHS:
    plan = _plan(f["wiring"], path)
    o, d = plan.run(f["log_potentials"], ev, f["ftov_msgs_in"], 17, 0.5, 1.0)
    outs.append((_np(o), _np(d)))
  for o, d in outs[1:]:
    np.testing.assert_array_equal(o, outs[0][0])
    np.testing.assert_array_equal(d, outs[0][1])


def test_full_size_rbm_batch_bit_exact_on_sampled_instances():
  """The bench workload (784 x 500 RBM, 128 perturb-and-MAP samples, T=0, damping 0.5) for a few
  iterations; instances 0, 64 and 127 re-run on the oracle must agree bit for bit."""
  from pgmax_gb300 import factor, fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  api = types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer, vgroup=vgroup)
  fg, groups, _ = cases.rbm(api, nh=500, nv=784, seed=0)
  ctx = infer.InfererContext(fg.bp_state)
  plan = ctx.plan
  info = plan.info
  assert info["num_enum_pairwise_factors"] == 392000
  B = 128
  rng = np.random.default_rng(5)
  ev = rng.gumbel(size=(B, fg.fg_state.num_var_states)).astype(np.float32)
  lp = np.asarray(fg.fg_state.log_potentials, np.float32)
  msgs = np.zeros(fg.fg_state.total_factor_num_states, np.float32)
  out, deltas = plan.run(lp, ev, msgs, 6, 0.5, 0.0)
  out, deltas = _np(out), _np(deltas)
  w = oracle.Wiring(ctx.flat_wiring())
  for b in (0, 64, 127):
    o, d = oracle.run(w, lp, ev[b], msgs, 6, 0.5, 0.0)
    np.testing.assert_array_equal(out[b], o)
    np.testing.assert_array_equal(deltas[b], d)


def test_invalid_wiring_is_rejected():
  f = fixtures.load(f"{fixtures.FIXTURES}/case_mixed_T0.npz")
  w = dict(f["wiring"])
  vs = w["var_states_for_edge_states"].copy()
  vs[3] = 10**6
  w["var_states_for_edge_states"] = vs
  with pytest.raises(ValueError, match="out of range"):
    _plan(w)
  w = dict(f["wiring"])
  cf = w["enum.factor_configs_edge_states"].copy()
  cf[0] = -5
  w["enum.factor_configs_edge_states"] = cf
  with pytest.raises(ValueError):
    _plan(w)


def test_bad_run_arguments_raise():
  f = fixtures.load(f"{fixtures.FIXTURES}/case_mixed_T0.npz")
  plan = _plan(f["wiring"])
  with pytest.raises(ValueError):
    plan.run(f["log_potentials"], f["evidence"][:-1], f["ftov_msgs_in"], 3)
  with pytest.raises(ValueError):
    plan.run(f["log_potentials"], f["evidence"], f["ftov_msgs_in"], 3, 0.5, -1.0)


@pytest.mark.parametrize("check_every", [1, 3, 7])
def test_run_to_tolerance_matches_one_run_of_the_same_length(check_every):
  """pgbp_run_to_tolerance stops once every instance's residual fell below the tolerance; its
  messages are those of one pgbp_run of the iterations it ran, and its first-below indices are
  read off that run's residuals."""
  torch = _torch()
  f = fixtures.load(f"{fixtures.FIXTURES}/case_ising12_T1.npz")
  plan = _plan(f["wiring"], "multi")
  rng = np.random.default_rng(check_every)
  B = 5
  ev = (f["evidence"][None] + rng.gumbel(size=(B,) + f["evidence"].shape)).astype(np.float32)
  tol = 1e-4
  out, first, ran = plan.run_to_tolerance(f["log_potentials"], ev, f["ftov_msgs_in"], tol, 500,
                                          0.5, 1.0, check_every=check_every)
  want, deltas = plan.run(f["log_potentials"], ev, f["ftov_msgs_in"], ran, 0.5, 1.0)
  torch.cuda.synchronize()
  assert torch.equal(out, want)
  d = deltas.cpu().numpy()
  for b in range(B):
    below = np.nonzero(d[b] < tol)[0]
    assert int(first[b]) == (int(below[0]) + 1 if below.size else -1)
  if int(first.min()) > 0:   # every instance converged: the run stopped at the first check after
    assert ran % check_every == 0 and ran - int(first.max()) < check_every
  else:                      # some instance oscillates: the run went to max_iters
    assert ran == 500


def test_entry_points_leave_the_callers_device_current():
  """Every C ABI call makes the plan's device current for its work and gives the caller's current
  device back (a caller inside a host framework must not find its device changed)."""
  import torch  # pylint: disable=g-import-not-at-top
  f = fixtures.load(f"{fixtures.FIXTURES}/case_mixed_T1.npz")
  torch.cuda.set_device(0)
  plan = _plan(f["wiring"])
  out, _ = plan.run(f["log_potentials"], f["evidence"], f["ftov_msgs_in"], 3, 0.5, 1.0)
  plan.beliefs(f["evidence"], out)
  torch.cuda.synchronize()
  assert torch.cuda.current_device() == 0
