"""The spin-glass Potts family of the warm start, on CPU: its wiring is the one FactorGraph
compiles, and the network's output channels map one to one onto the flat messages."""

import numpy as np

import pgmax_gb300 as pg
from pgmax_gb300 import infer
from pgmax_gb300.warmstart import potts


def test_torus_wiring_is_the_factor_graph_wiring():
  L, K = 5, 3
  g = pg.vgroup.NDVarArray(num_states=K, shape=(L, L))
  fg = pg.fgraph.FactorGraph(variable_groups=g)
  down = [[g[i, j], g[(i + 1) % L, j]] for i in range(L) for j in range(L)]
  right = [[g[i, j], g[i, (j + 1) % L]] for i in range(L) for j in range(L)]
  for vff in (down, right):
    fg.add_factors(pg.fgroup.PairwiseFactorGroup(variables_for_factors=vff,
                                                 log_potential_matrix=np.eye(K)))
  fw = infer.InfererContext(fg.bp_state).flat_wiring()
  for k, v in potts.torus_wiring(L, K).items():
    np.testing.assert_array_equal(np.asarray(fw[k]), np.asarray(v), err_msg=k)


def test_message_index_covers_every_edge_state_of_the_right_variable():
  L, K = 6, 8
  w = potts.torus_wiring(L, K)
  idx = potts.message_index(L, K)
  assert np.unique(idx).size == idx.size == w["var_states_for_edge_states"].size
  vs = w["var_states_for_edge_states"][idx].reshape(L, L, 4, K)
  want = np.arange(L * L).reshape(L, L, 1, 1) * K + np.arange(K)
  np.testing.assert_array_equal(vs, np.broadcast_to(want, vs.shape))


def test_features_one_step_messages_and_potentials():
  import torch  # pylint: disable=g-import-not-at-top
  from oracle import oracle  # pylint: disable=g-import-not-at-top
  L, K = 4, 8
  J, u = potts.sample(0, 2, L, K)
  lp = potts.potentials(J, K)
  np.testing.assert_array_equal(lp.reshape(2, 2 * L * L, K, K)[:, :, 3, 3], J)
  assert np.all(lp.reshape(2, 2 * L * L, K, K)[:, :, 2, 5] == 0)
  Jt, ut = torch.as_tensor(J), torch.as_tensor(u)
  x = potts.features(Jt, ut, L, K)
  assert tuple(x.shape) == (2, L, L, potts.FEATURES)
  jd = J[:, :L * L].reshape(2, L, L)
  jr = J[:, L * L:].reshape(2, L, L)
  np.testing.assert_array_equal(x[:, 2, 3, K + 2].numpy(), jd[:, 1, 3])      # up edge of (2, 3)
  np.testing.assert_array_equal(x[:, 2, 0, K + 3].numpy(), jr[:, 2, L - 1])  # left edge wraps
  # the one-step messages are those of one undamped BP iteration from zero messages
  w = potts.torus_wiring(L, K)
  one, _ = oracle.run_batch(oracle.Wiring(w), lp, u, np.zeros(w["var_states_for_edge_states"].size,
                                                               np.float32), 1, 0.0, 1.0)
  idx = potts.message_index(L, K)
  m1 = potts.one_step_messages(Jt, ut, L, K).numpy()
  np.testing.assert_allclose(m1, one[:, idx].reshape(2, L, L, 4 * K), atol=1e-5)
  np.testing.assert_allclose(x[..., K + 4:K + 4 + 4 * K].numpy(), m1, atol=0)
