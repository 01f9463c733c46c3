"""Multi-graph batches, shared potential tables and implicit config rows on the GPU.

Every graph of a union must get the messages of its own oracle run: bit for bit at temperature 0,
within 1e-5 above it (CUDA's expf / logf against glibc's). Shared tables are checked against the
oracle on the same graph with the tables copied to every factor; implicit config rows against the
same plan with explicit rows (bit for bit).
"""

import numpy as np
import pytest

import fixtures
from oracle import oracle
from pgmax_gb300 import batch

pytestmark = pytest.mark.gpu

ATOL = 1e-5
# Graphs with OR / AND factors on perturbed evidence at T > 0: logminusexp_with_temp subtracts
# nearly equal log-sums and amplifies the ulp differences of CUDA's and glibc's expf / log1pf
# (the same bound as the engine tests use for them).
ATOL_LOGICAL = 1e-4
MIX = ["case_mixed_T1", "case_ising12_T1", "case_potts_K4", "case_deconv_T1", "case_rbm_s0"]
PATHS = {"auto": 0, "multi": 1}   # native.FLAG_NO_SMALL_GRAPH = 1


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


def _load(name):
  return fixtures.load(f"{fixtures.FIXTURES}/{name}.npz")


def _wiring(d):
  w = dict(d["wiring"])
  w["num_variables"] = int(np.max(w["evidence_to_vars"], initial=-1)) + 1
  return w


def _has_logical(w):
  mr = np.asarray(w["msgs_ranges"]).reshape(4, 2)
  return bool(np.any(mr[1:3, 1] > mr[1:3, 0]))


def _check(got, want, temperature, logical=False):
  if temperature == 0.0:
    np.testing.assert_array_equal(got, want)
  else:
    np.testing.assert_allclose(got, want, atol=ATOL_LOGICAL if logical else ATOL, rtol=0)


@pytest.mark.parametrize("path", list(PATHS))
@pytest.mark.parametrize("temperature", [0.0, 1.0])
def test_union_of_fixture_graphs_matches_each_graph_alone(path, temperature):
  ds = [_load(n) for n in MIX]
  gb = batch.GraphBatch([_wiring(d) for d in ds], flags=PATHS[path])
  lay = gb.layout
  B = 2
  rng = np.random.default_rng(5)
  lp = gb.concat([d["log_potentials"].astype(np.float32) for d in ds])
  evs = [np.asarray(d["evidence"], np.float32)[None] + rng.gumbel(size=(B,) + d["evidence"].shape)
         .astype(np.float32) for d in ds]
  ev = gb.concat(evs)
  m = np.zeros(lay.perm.shape[0], np.float32)
  out, _ = gb.run(lp, ev, m, 12, 0.5, temperature)
  out = lay.union_to_graph_major(out.cpu().numpy())
  for b in range(B):
    parts = lay.split(out[b], "msgs")
    for d, w, e, got in zip(ds, [_wiring(d) for d in ds], evs, parts):
      want, _ = oracle.run(oracle.Wiring(w), d["log_potentials"], e[b],
                           np.zeros(d["ftov_msgs_in"].shape, np.float32), 12, 0.5, temperature)
      _check(got, want, temperature, _has_logical(w))


@pytest.mark.parametrize("L,K", [(6, 2), (5, 3), (4, 8), (3, 16), (9, 16), (3, 32), (3, 64),
                                 (7, 64)])
@pytest.mark.parametrize("temperature", [0.0, 1.0, 0.7])
@pytest.mark.parametrize("path", list(PATHS))
def test_shared_tables_and_implicit_rows(L, K, temperature, path):
  """On the multi-kernel path at T > 0, K = 16 / 32 / 64 run the exp-domain tensor-core kernel
  (float32 accuracy, within 1e-5 of the oracle); everything else runs the direct kernels."""
  torch = _torch()
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  rng = np.random.default_rng(L * 100 + K)
  table = rng.normal(0.0, 0.5, size=K * K).astype(np.float32)
  ev = rng.normal(size=(3, L * L * K)).astype(np.float32)
  m = np.zeros(2 * K * (2 * L * (L - 1)), np.float32)
  w_plain = batch.grid_wiring(L, K)
  n_fac = w_plain["num_factors"]
  want = oracle.run_batch(oracle.Wiring(w_plain), np.tile(table, n_fac), ev, m, 10, 0.5,
                          temperature)[0]
  outs = []
  for implicit in (False, True):
    w = batch.grid_wiring(L, K, shared_table=True, implicit_rows=implicit)
    plan = engine.Plan(w, flags=PATHS[path])
    out, _ = plan.run(table, ev, m, 10, 0.5, temperature)
    outs.append(out)
    _check(out.cpu().numpy(), want, temperature)
  assert torch.equal(outs[0], outs[1])


def test_union_of_shared_grids_and_deconvolution_graphs():
  d = _load("case_deconv_T1")
  wd = _wiring(d)
  specs = [(6, 2), (5, 4), (4, 8), (5, 3)]
  ws = []
  for i, (L, K) in enumerate(specs):
    ws.append(batch.grid_wiring(L, K, shared_table=True, implicit_rows=True))
    if i % 2 == 0:
      ws.append(wd)
  gb = batch.GraphBatch(ws)
  rng = np.random.default_rng(9)
  tables, evs, wants = [], [], []
  for w in ws:
    if w is wd:
      tables.append(np.zeros(0, np.float32))
      evs.append(np.asarray(d["evidence"], np.float32))
    else:
      K = int(np.sqrt(w["potentials_ranges"][0, 1]))
      tables.append(rng.normal(0.0, 0.5, size=K * K).astype(np.float32))
      evs.append(rng.normal(size=w["num_var_states"]).astype(np.float32))
  for w, t, e in zip(ws, tables, evs):
    if w is wd:
      want = oracle.run(oracle.Wiring(wd), d["log_potentials"], e,
                        np.zeros(d["ftov_msgs_in"].shape, np.float32), 15, 0.5, 1.0)[0]
    else:
      L = int(round(np.sqrt(w["num_variables"])))
      K = int(np.sqrt(w["potentials_ranges"][0, 1]))
      wp = batch.grid_wiring(L, K)
      want = oracle.run(oracle.Wiring(wp), np.tile(t, wp["num_factors"]), e,
                        np.zeros(wp["var_states_for_edge_states"].shape, np.float32), 15, 0.5,
                        1.0)[0]
    wants.append(want)
  out, _ = gb.run(gb.concat(tables), gb.concat(evs),
                  np.zeros(gb.layout.perm.shape[0], np.float32), 15, 0.5, 1.0)
  parts = gb.layout.split(gb.layout.union_to_graph_major(out.cpu().numpy()), "msgs")
  for w, got, want in zip(ws, parts, wants):
    np.testing.assert_allclose(got, want, atol=ATOL_LOGICAL if _has_logical(w) else ATOL, rtol=0)


def test_exp_domain_kernel_over_many_tables_and_instances():
  """Groups of different tables in one bucket, columns (factor, instance) crossing factor and
  group boundaries inside a tile, potentials shared by a batch of 3."""
  specs = [(5, 64), (3, 64), (6, 64), (4, 32), (7, 16), (4, 64)]
  ws = [batch.grid_wiring(L, K, shared_table=True, implicit_rows=True) for L, K in specs]
  gb = batch.GraphBatch(ws, flags=1)
  rng = np.random.default_rng(3)
  tables = [rng.normal(0.0, 0.5, size=K * K).astype(np.float32) for _, K in specs]
  evs = [rng.normal(size=(3, L * L * K)).astype(np.float32) for L, K in specs]
  out, _ = gb.run(gb.concat(tables), gb.concat(evs), np.zeros(gb.layout.perm.shape[0], np.float32),
                  20, 0.5, 1.0)
  got = gb.layout.union_to_graph_major(out.cpu().numpy())
  for b in range(3):
    parts = gb.layout.split(got[b], "msgs")
    for (L, K), t, e, part in zip(specs, tables, evs, parts):
      wp = batch.grid_wiring(L, K)
      want = oracle.run(oracle.Wiring(wp), np.tile(t, wp["num_factors"]), e[b],
                        np.zeros(wp["var_states_for_edge_states"].shape, np.float32), 20, 0.5,
                        1.0)[0]
      np.testing.assert_allclose(part, want, atol=ATOL, rtol=0)
  # every group's table reached shared memory by its bulk copy within the wait limit
  from pgmax_gb300 import native  # pylint: disable=g-import-not-at-top
  assert native.wait_timeouts() == 0


def test_exp_domain_underflow_falls_back_to_the_direct_formula():
  """A table whose rows span hundreds (E = exp((psi - rowmax) / T) underflows where the messages
  concentrate) must still give the reference's messages: those sums are recomputed directly."""
  L, K = 4, 16
  rng = np.random.default_rng(11)
  table = np.where(rng.random(K * K) < 0.5, -300.0, 0.0).astype(np.float32)
  table[::K + 1] = -300.0   # the diagonal (where the evidence peaks) is far below the row max
  ev = np.full((L * L, K), -200.0, np.float32)
  ev[np.arange(L * L), rng.integers(0, K, L * L)] = 0.0
  w = batch.grid_wiring(L, K, shared_table=True, implicit_rows=True)
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  plan = engine.Plan(w, flags=1)
  out, _ = plan.run(table, ev.reshape(-1), np.zeros(2 * K * w["num_factors"], np.float32), 10,
                    0.5, 1.0)
  wp = batch.grid_wiring(L, K)
  want = oracle.run(oracle.Wiring(wp), np.tile(table, wp["num_factors"]), ev.reshape(-1),
                    np.zeros(2 * K * w["num_factors"], np.float32), 10, 0.5, 1.0)[0]
  np.testing.assert_allclose(out.cpu().numpy(), want, atol=1e-4, rtol=1e-6)


def test_table_wait_that_runs_out_is_an_error_and_the_plan_recovers():
  """The exp-domain kernels' bounded table wait. With the debug settings that arm the table
  barrier without issuing the copy and cut the limit to 1 ms, every CTA's wait runs out with
  nothing in flight: the kernel stops, the device count and the plan's fault word are set, the
  plan reports PGBP_ERR_TIMEOUT (RuntimeError) and the next launch is refused until the fault has
  been reported once. With the settings cleared the same plan runs normally and matches the
  oracle."""
  from pgmax_gb300 import engine, native  # pylint: disable=g-import-not-at-top
  L, K = 5, 64
  rng = np.random.default_rng(21)
  table = rng.normal(0.0, 0.5, size=K * K).astype(np.float32)
  ev = rng.normal(size=L * L * K).astype(np.float32)
  w = batch.grid_wiring(L, K, shared_table=True, implicit_rows=True)
  m = np.zeros(2 * K * w["num_factors"], np.float32)
  plan = engine.Plan(w, flags=1)
  plan.check()
  native.wait_timeouts()
  native.debug_set(native.DEBUG_WAIT_LIMIT_NS, 1_000_000)
  native.debug_set(native.DEBUG_SKIP_TABLE_COPY, 1)
  try:
    plan.run(table, ev, m, 2, 0.5, 1.0)
    with pytest.raises(RuntimeError, match="status 6"):
      plan.check()
    plan.run(table, ev, m, 2, 0.5, 1.0)
    _torch().cuda.synchronize()
    with pytest.raises(RuntimeError, match="gave up"):   # refused at entry: nothing enqueued
      plan.run(table, ev, m, 2, 0.5, 1.0)
  finally:
    native.debug_set(native.DEBUG_SKIP_TABLE_COPY, 0)
    native.debug_set(native.DEBUG_WAIT_LIMIT_NS, 0)
  assert native.wait_timeouts() > 0
  plan.check()
  out, _ = plan.run(table, ev, m, 10, 0.5, 1.0)
  plan.check()
  assert native.wait_timeouts() == 0
  wp = batch.grid_wiring(L, K)
  want = oracle.run(oracle.Wiring(wp), np.tile(table, wp["num_factors"]), ev, m, 10, 0.5, 1.0)[0]
  np.testing.assert_allclose(out.cpu().numpy(), want, atol=ATOL, rtol=0)


@pytest.mark.parametrize("temperature", [1.0, 0.7, 0.3])
def test_tcgen05_path_for_shared_64x64_tables(temperature):
  """Shared 64 x 64 tables of a single instance run the tcgen05 kernel (products on the
  fifth-generation tensor cores, accumulators in tensor memory, warp-specialised pipeline). A
  union of grids whose groups end in partial 128-column tiles, with more tiles than SMs so that
  CTAs walk several tiles and change groups inside their range, must match every graph's oracle
  run within 1e-5 and the warp-level mma.sync kernel (the debug setting) within 1e-5."""
  from pgmax_gb300 import native  # pylint: disable=g-import-not-at-top
  specs = [(5, 64), (90, 64), (3, 64), (23, 64), (2, 64), (12, 64)]
  ws = [batch.grid_wiring(L, K, shared_table=True, implicit_rows=True) for L, K in specs]
  gb = batch.GraphBatch(ws, flags=1)
  rng = np.random.default_rng(int(temperature * 10) + 40)
  tables = [rng.normal(0.0, 0.5, size=K * K).astype(np.float32) for _, K in specs]
  evs = [rng.normal(size=L * L * K).astype(np.float32) for L, K in specs]
  m0 = np.zeros(gb.layout.perm.shape[0], np.float32)
  iters = 12
  out, d_tc = gb.run(gb.concat(tables), gb.concat(evs), m0, iters, 0.5, temperature)
  got = out.cpu().numpy()
  native.debug_set(native.DEBUG_LEGACY_MMA, 1)
  try:
    out_mma, d_mma = gb.run(gb.concat(tables), gb.concat(evs), m0, iters, 0.5, temperature)
  finally:
    native.debug_set(native.DEBUG_LEGACY_MMA, 0)
  np.testing.assert_allclose(got, out_mma.cpu().numpy(), atol=ATOL, rtol=0)
  np.testing.assert_allclose(d_tc.cpu().numpy(), d_mma.cpu().numpy(), atol=ATOL, rtol=0)
  parts = gb.layout.split(gb.layout.union_to_graph_major(got), "msgs")
  for (L, K), t, e, part in zip(specs, tables, evs, parts):
    wp = batch.grid_wiring(L, K)
    want = oracle.run(oracle.Wiring(wp), np.tile(t, wp["num_factors"]), e,
                      np.zeros(wp["var_states_for_edge_states"].shape, np.float32), iters, 0.5,
                      temperature)[0]
    np.testing.assert_allclose(part, want, atol=ATOL, rtol=0, err_msg=f"L={L}")
  assert native.wait_timeouts() == 0


def test_tcgen05_path_underflow_falls_back_to_the_direct_formula():
  """K = 64, one instance: where E u underflows the epilogue recomputes the message directly."""
  L, K = 4, 64
  rng = np.random.default_rng(12)
  table = np.where(rng.random(K * K) < 0.5, -300.0, 0.0).astype(np.float32)
  table[::K + 1] = -300.0
  ev = np.full((L * L, K), -200.0, np.float32)
  ev[np.arange(L * L), rng.integers(0, K, L * L)] = 0.0
  w = batch.grid_wiring(L, K, shared_table=True, implicit_rows=True)
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  plan = engine.Plan(w, flags=1)
  out, _ = plan.run(table, ev.reshape(-1), np.zeros(2 * K * w["num_factors"], np.float32), 10,
                    0.5, 1.0)
  wp = batch.grid_wiring(L, K)
  want = oracle.run(oracle.Wiring(wp), np.tile(table, wp["num_factors"]), ev.reshape(-1),
                    np.zeros(2 * K * w["num_factors"], np.float32), 10, 0.5, 1.0)[0]
  np.testing.assert_allclose(out.cpu().numpy(), want, atol=1e-4, rtol=1e-6)
