"""Error of the float32 engine against a float64 run of the same configuration, per configuration
of the measured workloads (the float64 run is oracle/bp_torch.py, the reference's algorithm in
float64, on the GPU through torch; it stands in for a jax_enable_x64 run of the reference, which
cannot run here).

Each case prints one line `FP64 error | <case> | msgs <max abs> | beliefs <max abs> | ...` (run
with -s to see them), with the float64 run's last residual (max |change| of its last iteration),
and checks: when both the float64 run and the float32 run have settled (last residual <= 1e-4),
1e-4 on messages and beliefs and, for max-product runs, identical MAP decodes except at ties
within 1e-4. A run that has not settled carries float32 rounding into its trajectory in the
reference as well; its error is reported, and only checked to be finite. Max-product on the full
RBM is such a run: whether the float64 run settles within 200 iterations depends on its own
summation order (torch's float64 scatter-adds on the GPU are not ordered), and when it does the
float32 run, which equals the float32 reference bit for bit (test_gpu_bench_workloads.py), may
still be oscillating or end at another fixed point of max-product.
Configurations (synthetic, seeded, the shapes of the benchmarks):
  ising50_T1 / ising50_T0  50 x 50 toroidal Ising, 0.8 [[1, -1], [-1, 1]], Gumbel evidence,
                           1000 iterations
  rbm784x500_T0            784 x 500 RBM (W ~ N(0, 0.1^2), biases N(0, 0.5^2)), one
                           Gumbel-perturbed sample, 200 iterations at T = 0
  potts_L48_K16            an open Potts grid of the multi-graph batch's family (a), J I_16,
                           J ~ U(0, 1.5), unaries N(0, 1), 200 iterations at T = 1
  potts_L32_K64            a grid of family (b), K = 64, table ~ N(0, 0.5^2), 200 iterations
  grid64_b4_T1             the adjoint configuration's 64 x 64 binary grid, 4 instances, 100
                           iterations at T = 1
  torus96_K8_T1            the warm start's 96 x 96 toroidal spin-glass Potts family, K = 8,
                           200 iterations at T = 1
The deconvolution family of the multi-graph batch (OR / AND factors) has no float64
restatement; its float32 parity against the oracle is in test_gpu_batch.py.
"""

import types

import numpy as np
import pytest

import cases
from oracle import bp_torch

pytestmark = pytest.mark.gpu

BOUND = 1e-4


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


def _api():
  from pgmax_gb300 import factor, fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  return types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer,
                               vgroup=vgroup)


def _plan(wiring):
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  w = dict(wiring)
  w["num_variables"] = int(np.max(w["evidence_to_vars"], initial=-1)) + 1
  return engine.Plan(w)


def _compare(name, wiring, lp, ev, msgs, iters, temperature, damping=0.5, plan=None):
  """Runs both, prints the error line, checks the bound."""
  torch = _torch()
  plan = plan or _plan(wiring)
  lp32 = torch.as_tensor(np.asarray(lp, np.float32), device="cuda")
  ev32 = torch.as_tensor(np.asarray(ev, np.float32), device="cuda")
  m32 = torch.as_tensor(np.asarray(msgs, np.float32), device="cuda")
  out32, deltas32 = plan.run(lp32, ev32, m32, iters, damping, temperature)
  bel32 = plan.beliefs(ev32, out32)
  g = bp_torch.EnumGraph(wiring, device="cuda")
  with torch.no_grad():
    out64, last = g.run(lp32.double(), ev32.double(), m32.double(), iters, damping, temperature,
                        with_last_delta=True)
    bel64 = g.beliefs(ev32.double(), out64)
  settled = float(last.max()) <= BOUND and float(deltas32[..., -1].max()) <= BOUND
  out64 = out64.reshape(out32.shape)
  bel64 = bel64.reshape(bel32.shape)
  dm = float((out32.double() - out64).abs().max())
  db = float((bel32.double() - bel64).abs().max())
  extra = ""
  if temperature == 0.0:
    nv = int(np.max(wiring["evidence_to_vars"])) + 1
    e2v = torch.as_tensor(np.asarray(wiring["evidence_to_vars"], np.int64), device="cuda")
    b32 = bel32.reshape(-1, bel32.shape[-1])
    b64 = bel64.reshape(-1, bel64.shape[-1])
    map32 = plan.decode(b32, nv)
    # float64 decode and the gap between the two best states of every variable
    k = int(np.bincount(np.asarray(wiring["evidence_to_vars"])).max())
    first = torch.zeros(nv + 1, dtype=torch.int64, device="cuda")
    first[1:] = torch.bincount(e2v, minlength=nv).cumsum(0)
    idx = (first[:-1, None] + torch.arange(k, device="cuda")[None]).clamp(max=b64.shape[1] - 1)
    vals = b64[:, idx]
    valid = torch.arange(k, device="cuda")[None] < (first[1:] - first[:-1])[:, None]
    vals = torch.where(valid[None], vals, torch.full_like(vals, -float("inf")))
    map64 = vals.argmax(-1)
    top2 = vals.topk(2, dim=-1).values if k > 1 else None
    tie = (top2[..., 0] - top2[..., 1] <= BOUND) if top2 is not None else torch.zeros_like(map64,
                                                                                             dtype=bool)
    diff = map32.long() != map64
    extra = (f" | MAP differs {int(diff.sum())} of {diff.numel()} (ties within {BOUND:g}: "
             f"{int((diff & tie).sum())})")
    map_ok = int((diff & ~tie).sum()) == 0
  else:
    map_ok = True
  print(f"FP64 error | {name} | msgs {dm:.3g} | beliefs {db:.3g}{extra} | float64 last residual "
        f"{float(last.max()):.3g} | float32 last residual {float(deltas32[..., -1].max()):.3g}",
        flush=True)
  assert np.isfinite(dm) and np.isfinite(db)
  if settled:
    assert dm <= BOUND and db <= BOUND, (dm, db)
    assert map_ok
  return dm, db


@pytest.mark.parametrize("temperature", [1.0, 0.0])
def test_ising50(temperature):
  api = _api()
  fg, _, ev = cases.ising(api, n=50, seed=0)
  bp = api.infer.BP(fg.bp_state)
  a = bp.init(evidence_updates=ev)
  _compare(f"ising50_T{temperature:g}", bp.context.flat_wiring(), a.log_potentials.cpu(),
           a.evidence.cpu(), a.ftov_msgs.cpu(), 1000, temperature, plan=bp.context.plan)


def test_rbm784x500_t0():
  api = _api()
  fg, _, ev = cases.rbm(api, nh=500, nv=784, seed=0, sample=0)
  bp = api.infer.BP(fg.bp_state)
  a = bp.init(evidence_updates=ev)
  _compare("rbm784x500_T0", bp.context.flat_wiring(), a.log_potentials.cpu(), a.evidence.cpu(),
           a.ftov_msgs.cpu(), 200, 0.0, plan=bp.context.plan)


@pytest.mark.parametrize("L,K", [(48, 16), (32, 64)])
def test_potts_families_of_the_multigraph_batch(L, K):
  from pgmax_gb300 import batch  # pylint: disable=g-import-not-at-top
  rng = np.random.default_rng(L * 100 + K)
  w = batch.grid_wiring(L, K)
  F = 2 * L * (L - 1)
  if K == 64:
    table = rng.normal(0.0, 0.5, size=(K, K))
  else:
    table = rng.uniform(0.0, 1.5) * np.eye(K)
  lp = np.tile(table.reshape(-1), F).astype(np.float32)
  ev = rng.normal(size=(L * L * K,)).astype(np.float32)
  m = np.zeros(w["var_states_for_edge_states"].shape[0], np.float32)
  _compare(f"potts_L{L}_K{K}_T1", w, lp, ev, m, 200, 1.0)


def test_grid64_adjoint_configuration():
  from pgmax_gb300 import batch  # pylint: disable=g-import-not-at-top
  rng = np.random.default_rng(3)
  n, B = 64, 4
  w = batch.grid_wiring(n, 2)
  F = 2 * n * (n - 1)
  lp = np.tile(np.array([0.6, -0.6, -0.6, 0.6], np.float32), F)
  ev = (rng.normal(size=(B, n * n * 2)) * 1.5).astype(np.float32)
  m = np.zeros((B, w["var_states_for_edge_states"].shape[0]), np.float32)
  _compare("grid64_b4_T1", w, lp, ev, m, 100, 1.0)


def test_torus96_warm_start_family():
  torch = _torch()
  from pgmax_gb300.warmstart import potts  # pylint: disable=g-import-not-at-top
  L, K = 96, 8
  w = potts.torus_wiring(L, K)
  w = dict(w)
  J, u = potts.sample(5, 1, L, K, 0.7)
  lp = potts.potentials(torch.as_tensor(J, device="cuda"), K)[0].cpu().numpy()
  ev = np.asarray(u, np.float32).reshape(-1)
  m = np.zeros(w["var_states_for_edge_states"].shape[0], np.float32)
  _compare("torus96_K8_T1", w, lp, ev, m, 200, 1.0)
