"""The benchmarked workloads themselves, at their bench sizes and lengths, against the oracle.

* RBM perturb-and-MAP (784 x 500, 128 samples, 200 iterations, T = 0, damping 0.5), built by
  bench.build_rbm with bench.gumbel_evidence's seed for rank 0 and run through the drop-in API:
  the messages, every per-iteration residual, the flat beliefs and the MAP states of three sampled
  instances must equal the C oracle's bit for bit. The trajectory is rounding-sensitive (float32
  and float64 runs end in different oscillation phases), so this pins the exact operation order
  over the full 200 iterations, not just the first few.
* The uneven multi-graph batch: the first 24 graphs of bench.build_multigraph (the same seeded
  draws as the bench's 256) run as one union plan for 200 iterations. The largest Potts grid of
  family (a) and the smallest K = 64 grid of family (b) (the exp-domain tensor-core kernel) must
  match their own oracle runs within 1e-5 at T = 1, the bench's temperature. A deconvolution graph
  of family (c) must match bit for bit at T = 0. At T = 1 family (c) is ill-conditioned in float32:
  its messages reach magnitudes of 100 against the +-100 evidence clamps, and OR / AND updates
  subtract nearly equal log-sums, so moving the evidence by one unit in the last place moves the
  oracle's own messages by 1e-5 after one iteration, 2e-2 after ten and flips clipped messages
  (1e32) within 100. There the engine must stay within the oracle's own sensitivity: no larger
  maximum difference, and no more messages off by more than 1e-5, than a run of the oracle on
  evidence moved by a relative 2^-22; and within 1e-5 (plus 2^-22 relative) after one iteration.
"""

import numpy as np
import pytest

import bench
from oracle import oracle

pytestmark = pytest.mark.gpu


def _decode_binary(flat_beliefs):
  b = flat_beliefs.reshape(-1, 2)
  return (b[:, 1] > b[:, 0]).astype(np.int32)   # first maximum wins a tie


def test_rbm_bench_workload_full_length_bit_exact_on_sampled_instances():
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer  # pylint: disable=g-import-not-at-top
  fg, hidden, visible = bench.build_rbm(seed=0)
  bp = infer.BP(fg.bp_state, temperature=bench.TEMPERATURE)
  nvs = fg.fg_state.num_var_states
  n_es = fg.fg_state.total_factor_num_states
  ev = bench.gumbel_evidence(nvs, bench.BATCH, 1000)   # the bench's rank-0 host evidence
  lp = np.asarray(fg.fg_state.log_potentials, np.float32)
  msgs0 = np.zeros(n_es, np.float32)
  arrays = infer.BPArrays(log_potentials=torch.as_tensor(lp, device="cuda"),
                          ftov_msgs=torch.zeros(n_es, device="cuda"),
                          evidence=torch.as_tensor(ev, device="cuda"))
  out, deltas = bp.run_with_diffs(arrays, num_iters=bench.ITERS, damping=bench.DAMPING,
                                  temperature=bench.TEMPERATURE)
  beliefs = bp.get_beliefs(out)
  dec = infer.decode_map_states(beliefs)
  msgs = out.ftov_msgs.cpu().numpy()
  deltas = deltas.cpu().numpy()
  flat = beliefs.flat.cpu().numpy()
  map_h, map_v = dec[hidden].cpu().numpy(), dec[visible].cpu().numpy()
  assert msgs.shape == (bench.BATCH, n_es) and deltas.shape == (bench.BATCH, bench.ITERS)
  w = oracle.Wiring(bp.context.flat_wiring())
  sample = [0, 77, 127]
  want, want_d = oracle.run_batch(w, lp, ev[sample], msgs0, bench.ITERS, bench.DAMPING,
                                  bench.TEMPERATURE, num_threads=len(sample))
  for i, b in enumerate(sample):
    np.testing.assert_array_equal(msgs[b], want[i], err_msg=f"messages of instance {b}")
    np.testing.assert_array_equal(deltas[b], want_d[i], err_msg=f"residuals of instance {b}")
    want_bel = oracle.beliefs(w, ev[b], want[i])
    np.testing.assert_array_equal(flat[b], want_bel, err_msg=f"beliefs of instance {b}")
    want_map = _decode_binary(want_bel)
    np.testing.assert_array_equal(map_h[b], want_map[:bench.NH])
    np.testing.assert_array_equal(map_v[b], want_map[bench.NH:])


def test_multigraph_bench_families_through_the_union():
  from pgmax_gb300 import batch  # pylint: disable=g-import-not-at-top
  wirings, tables, evs, fam = bench.build_multigraph(seed=0, n_graphs=24)
  assert fam == {"a": 8, "b": 8, "c": 8}
  gb = batch.GraphBatch(wirings)
  m0 = np.zeros(gb.layout.perm.shape[0], np.float32)

  def union_run(iters, temperature):
    out, _ = gb.run(gb.concat(tables), gb.concat(evs), m0, iters, 0.5, temperature)
    return gb.layout.split(gb.layout.union_to_graph_major(out.cpu().numpy()), "msgs")

  side = lambda g: int(round(np.sqrt(wirings[g]["num_variables"])))
  ga = max((g for g in range(24) if g % 3 == 0), key=side)
  gbb = min((g for g in range(24) if g % 3 == 1), key=side)
  assert side(ga) >= 100
  parts = union_run(bench.MG_ITERS, 1.0)
  for kind, g in (("a", ga), ("b", gbb)):
    K = int(round(np.sqrt(tables[g].shape[0])))
    wp = batch.grid_wiring(side(g), K)
    want, _ = oracle.run(oracle.Wiring(wp), np.tile(tables[g], wp["num_factors"]), evs[g],
                         np.zeros(wp["var_states_for_edge_states"].shape[0], np.float32),
                         bench.MG_ITERS, 0.5, 1.0)
    np.testing.assert_allclose(parts[g], want, atol=1e-5, rtol=0,
                               err_msg=f"family {kind}, graph {g}")
  # family (c): bit for bit at T = 0, within the oracle's own sensitivity at T = 1
  gc = 2
  w = oracle.Wiring(wirings[gc])
  mc = np.zeros(wirings[gc]["var_states_for_edge_states"].shape[0], np.float32)
  want0, _ = oracle.run(w, tables[gc], evs[gc], mc, bench.MG_ITERS, 0.5, 0.0)
  np.testing.assert_array_equal(union_run(bench.MG_ITERS, 0.0)[gc], want0)
  # one iteration: 1e-5, plus 2^-22 relative for messages of magnitude up to about 60 (there 1e-5
  # is under three units in the last place)
  np.testing.assert_allclose(union_run(1, 1.0)[gc], oracle.run(w, tables[gc], evs[gc], mc, 1, 0.5,
                                                               1.0)[0], atol=1e-5, rtol=2.0**-22)
  want1, _ = oracle.run(w, tables[gc], evs[gc], mc, bench.MG_ITERS, 0.5, 1.0)
  rng = np.random.default_rng(1)
  ev_moved = (evs[gc] * (1 + rng.choice([-1.0, 1.0], evs[gc].shape) * 2.0**-22)).astype(np.float32)
  moved, _ = oracle.run(w, tables[gc], ev_moved, mc, bench.MG_ITERS, 0.5, 1.0)
  diff, sens = np.abs(parts[gc] - want1), np.abs(moved - want1)
  assert diff.max() <= sens.max(), (diff.max(), sens.max())
  assert (diff > 1e-5).mean() <= (sens > 1e-5).mean(), ((diff > 1e-5).mean(), (sens > 1e-5).mean())
