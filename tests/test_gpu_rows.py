"""Fused rows of a binary pairwise group.

When a dense 2 x 2 group's factors come in rows of one first variable, the factor pass forms
those variables' sums itself (pairwise22_rows_kernel). An RBM's hidden units are the case: the
unary factors come first, then each hidden unit's factors in a row. The pass adds each new
message to the next iteration's sum in edge order, and the variable-sum pass covers the
remaining variables only. Every message and residual must be bit-identical to the unfused
iteration (PGBP_DEBUG_NO_ROWS), at T = 0 and T > 0, for batches taking 64 or 32 instances per
CTA. At T = 0 they must also equal the C oracle. Graphs without such rows (an Ising grid) plan
none.
"""

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _rbm(nh, nv, seed):
  """bench.build_rbm's construction at a small size."""
  from pgmax_gb300 import fgraph, fgroup, vgroup  # pylint: disable=g-import-not-at-top
  rng = np.random.default_rng(seed)
  w = rng.normal(0.0, 0.1, size=(nh, nv)).astype(np.float32)
  bh = rng.normal(0.0, 0.5, size=nh).astype(np.float32)
  bv = rng.normal(0.0, 0.5, size=nv).astype(np.float32)
  hidden = vgroup.NDVarArray(num_states=2, shape=(nh,))
  visible = vgroup.NDVarArray(num_states=2, shape=(nv,))
  fg = fgraph.FactorGraph(variable_groups=[hidden, visible])
  hu = fgroup.EnumFactorGroup(variables_for_factors=[[hidden[i]] for i in range(nh)],
                              factor_configs=np.arange(2)[:, None],
                              log_potentials=np.stack([np.zeros_like(bh), bh], axis=1))
  vu = fgroup.EnumFactorGroup(variables_for_factors=[[visible[j]] for j in range(nv)],
                              factor_configs=np.arange(2)[:, None],
                              log_potentials=np.stack([np.zeros_like(bv), bv], axis=1))
  lpm = np.zeros((nh * nv, 2, 2), dtype=np.float32)
  lpm[:, 1, 1] = w.ravel()
  hv, vv = hidden.variables, visible.variables
  pw = fgroup.PairwiseFactorGroup(
      variables_for_factors=[[hv[i], vv[j]] for i in range(nh) for j in range(nv)],
      log_potential_matrix=lpm)
  fg.add_factors([hu, vu, pw])
  return fg


def _run(bp, arrays, iters, temperature):
  out, deltas = bp.run_with_diffs(arrays, num_iters=iters, damping=0.5, temperature=temperature)
  return out.ftov_msgs.cpu().numpy(), deltas.cpu().numpy()


@pytest.mark.parametrize("batch,temperature", [(64, 0.0), (96, 0.0), (32, 0.5), (128, 1.0)])
def test_fused_rows_bit_identical_to_the_variable_sum_pass(batch, temperature):
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer, native  # pylint: disable=g-import-not-at-top
  nh, nv, iters = 24, 40, 25
  fg = _rbm(nh, nv, seed=batch)
  bp = infer.BP(fg.bp_state, temperature=temperature, exec_flags=native.FLAG_NO_SMALL_GRAPH)
  assert bp.context.plan.info["num_fused_rows"] == nh
  nvs = fg.fg_state.num_var_states
  n_es = fg.fg_state.total_factor_num_states
  rng = np.random.default_rng(batch + 7)
  ev = rng.gumbel(size=(batch, nvs)).astype(np.float32)
  lp = np.asarray(fg.fg_state.log_potentials, np.float32)
  arrays = infer.BPArrays(log_potentials=torch.as_tensor(lp, device="cuda"),
                          ftov_msgs=torch.zeros(n_es, device="cuda"),
                          evidence=torch.as_tensor(ev, device="cuda"))
  fused = _run(bp, arrays, iters, temperature)
  native.debug_set(native.DEBUG_NO_ROWS, 1)
  try:
    plain = _run(bp, arrays, iters, temperature)
  finally:
    native.debug_set(native.DEBUG_NO_ROWS, 0)
  np.testing.assert_array_equal(fused[0].view(np.uint32), plain[0].view(np.uint32))
  np.testing.assert_array_equal(fused[1].view(np.uint32), plain[1].view(np.uint32))
  assert native.wait_timeouts() == 0
  if temperature == 0.0:
    w = oracle.Wiring(bp.context.flat_wiring())
    sample = [0, batch - 1]
    want, want_d = oracle.run_batch(w, lp, ev[sample], np.zeros(n_es, np.float32), iters, 0.5,
                                    0.0, num_threads=2)
    for i, b in enumerate(sample):
      np.testing.assert_array_equal(fused[0][b], want[i])
      np.testing.assert_array_equal(fused[1][b], want_d[i])


def test_graphs_without_rows_plan_none():
  import bench  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer, native  # pylint: disable=g-import-not-at-top
  fg, _ = bench.build_ising(8)
  bp = infer.BP(fg.bp_state, exec_flags=native.FLAG_NO_SMALL_GRAPH)
  assert bp.context.plan.info["num_fused_rows"] == 0
