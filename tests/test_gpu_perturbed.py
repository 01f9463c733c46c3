"""Perturb-and-MAP with the noise generated inside the run (pgbp_run_perturbed, pgbp_gumbel).

* The device's Gumbel stream equals the oracle's restatement of it bit for bit, and so follows the
  Gumbel(0, 1) law (tests/test_gumbel_oracle.py checks the law on the oracle's draws; a KS test
  runs here on the device's too).
* A fused run equals pgbp_run on the evidence base + noise made on the host from the oracle's copy
  of the stream, bit for bit: messages, every residual and the perturbed evidence it hands back,
  on every execution path, for shared, batched and absent (zero) bases, at T = 0 and T > 0.
* Through the drop-in API, BP.run_perturbed on the RBM bench workload (784 x 500, 128 samples,
  200 iterations, T = 0) gives the messages, beliefs and MAP states of BP.run on host-made
  evidence, bit for bit.
"""

import numpy as np
import pytest

import bench
import fixtures
from oracle import oracle

pytestmark = pytest.mark.gpu

PATHS = {"auto": 0, "multi": 1, "small": 2, "cluster": 4}


def _plan(wiring, flags=0):
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  w = dict(wiring)
  w["num_variables"] = int(np.max(w["evidence_to_vars"], initial=-1)) + 1
  return engine.Plan(w, flags=flags)


@pytest.mark.parametrize("seed", [0, 12345, 2**64 - 1])
def test_device_stream_equals_the_oracle(seed):
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  n = 3_000_001
  np.testing.assert_array_equal(engine.gumbel(seed, n).cpu().numpy(), oracle.gumbel(seed, n))


def test_device_draws_follow_the_gumbel_law():
  stats = pytest.importorskip("scipy.stats")
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  g = engine.gumbel(99, 400_000).cpu().numpy().astype(np.float64)
  assert stats.kstest(g, "gumbel_r").pvalue > 1e-3
  assert abs(g.mean() - np.euler_gamma) < 0.01


@pytest.mark.parametrize("path", list(PATHS))
@pytest.mark.parametrize("base", ["shared", "batched", "none"])
@pytest.mark.parametrize("name", ["case_mixed_T0", "case_mixed_T1", "case_deconv_T0"])
def test_fused_run_equals_run_on_host_made_evidence(name, base, path):
  import torch  # pylint: disable=g-import-not-at-top
  f = fixtures.load(f"{fixtures.FIXTURES}/{name}.npz")
  plan = _plan(f["wiring"], PATHS[path])
  T = float(f["temperature"])
  B, iters, seed, scale = 5, 9, 77, 0.75
  nvs = plan.num_var_states
  rng = np.random.default_rng(3)
  ev0 = np.asarray(f["evidence"], np.float32)
  if base == "shared":
    ev_base, ev_full = ev0, np.broadcast_to(ev0, (B, nvs))
  elif base == "batched":
    ev_base = (ev0[None] + rng.normal(size=(B, nvs))).astype(np.float32)
    ev_full = ev_base
  else:
    ev_base, ev_full = None, np.zeros((B, nvs), np.float32)
  noise = oracle.gumbel(seed, B * nvs).reshape(B, nvs)
  host_ev = (ev_full + np.float32(scale) * noise).astype(np.float32)
  msgs, deltas, ev_out = plan.run_perturbed(f["log_potentials"], ev_base, f["ftov_msgs_in"], iters,
                                            seed, B, scale, 0.5, T)
  want, want_d = plan.run(f["log_potentials"], host_ev, f["ftov_msgs_in"], iters, 0.5, T)
  torch.cuda.synchronize()
  np.testing.assert_array_equal(ev_out.cpu().numpy(), host_ev)
  np.testing.assert_array_equal(msgs.cpu().numpy(), want.cpu().numpy())
  np.testing.assert_array_equal(deltas.cpu().numpy(), want_d.cpu().numpy())


def test_rbm_bench_workload_through_the_drop_in_api():
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer  # pylint: disable=g-import-not-at-top
  fg, hidden, visible = bench.build_rbm(seed=0)
  bp = infer.BP(fg.bp_state, temperature=0.0)
  arrays = bp.init()
  seed = 4242
  out = bp.run_perturbed(arrays, bench.ITERS, seed, bench.BATCH, damping=bench.DAMPING)
  nvs = fg.fg_state.num_var_states
  host_ev = oracle.gumbel(seed, bench.BATCH * nvs).reshape(bench.BATCH, nvs)
  ref_in = infer.BPArrays(log_potentials=arrays.log_potentials, ftov_msgs=arrays.ftov_msgs,
                          evidence=torch.as_tensor(host_ev, device="cuda"))
  ref = bp.run(ref_in, bench.ITERS, bench.DAMPING)
  assert torch.equal(out.evidence, ref.evidence)
  assert torch.equal(out.ftov_msgs, ref.ftov_msgs)
  got_map = infer.decode_map_states(bp.get_beliefs(out))
  want_map = infer.decode_map_states(bp.get_beliefs(ref))
  for g in (hidden, visible):
    assert torch.equal(got_map[g], want_map[g])
  # the oracle agrees on a sampled instance (pins the whole chain, not just the two GPU paths)
  w = oracle.Wiring(bp.context.flat_wiring())
  lp = np.asarray(fg.fg_state.log_potentials, np.float32)
  o, _ = oracle.run(w, lp, host_ev[100], np.zeros(fg.fg_state.total_factor_num_states, np.float32),
                    bench.ITERS, bench.DAMPING, 0.0)
  np.testing.assert_array_equal(out.ftov_msgs[100].cpu().numpy(), o)
