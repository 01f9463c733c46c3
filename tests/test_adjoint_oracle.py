"""The float64 torch restatement that the adjoint is checked against, pinned on CPU.

Two pins: its forward messages agree with the golden fixtures recorded from the reference's own
bp.run (Enum-only graphs at temperature > 0), and its autograd gradients agree with float64
central finite differences (step 1e-6) of the same loss.
"""

import numpy as np
import pytest
import torch

import fixtures
from oracle import bp_torch

ENUM_T_POS = ["case_ising12_T1", "case_potts_K4", "case_potts_K8", "case_potts_K16"]
ENUM_T0 = ["case_ising50_T0", "case_rbm_s0", "case_rbm_s1"]


def _load(name):
  return fixtures.load(f"{fixtures.FIXTURES}/{name}.npz")


@pytest.mark.parametrize("name", ENUM_T_POS)
def test_forward_matches_reference_fixture(name):
  d = _load(name)
  g = bp_torch.EnumGraph(d["wiring"])
  f64 = lambda x: torch.as_tensor(np.asarray(x, dtype=np.float64))
  with torch.no_grad():
    out = g.run(f64(d["log_potentials"]), f64(d["evidence"]), f64(d["ftov_msgs_in"]),
                int(d["num_iters"]), float(d["damping"]), float(d["temperature"]))
    bel = g.beliefs(f64(d["evidence"]), out)
  # float32 reference vs float64 restatement
  np.testing.assert_allclose(out[0].numpy(), d["ftov_msgs_out"], atol=1e-5, rtol=0)
  np.testing.assert_allclose(bel[0].numpy(), d["flat_beliefs"], atol=2e-5, rtol=0)


@pytest.mark.parametrize("name", ENUM_T0)
def test_max_product_forward_matches_reference_fixture(name):
  """The float64 restatement's temperature-0 branch against the reference's float32 run (the
  float64 side of the per-configuration FP64 error)."""
  d = _load(name)
  g = bp_torch.EnumGraph(d["wiring"])
  f64 = lambda x: torch.as_tensor(np.asarray(x, dtype=np.float64))
  out = g.run(f64(d["log_potentials"]), f64(d["evidence"]), f64(d["ftov_msgs_in"]),
              int(d["num_iters"]), float(d["damping"]), 0.0)
  np.testing.assert_allclose(out[0].numpy(), d["ftov_msgs_out"], atol=1e-4, rtol=0)


def _loss(g, lp, ev, m, iters, damping, temperature, labels_w):
  out = g.run(lp, ev, m, iters, damping, temperature)
  bel = g.beliefs(ev, out)
  # per-state log-softmax weighted by fixed label weights (a smooth stand-in for -log p(label))
  return -(torch.log_softmax(bel.reshape(bel.shape[0], -1, g.k), dim=-1).reshape(bel.shape)
           * labels_w).sum() / bel.shape[0]


@pytest.mark.parametrize("name,batched_lp", [("case_ising12_T1", False), ("case_potts_K4", True)])
def test_autograd_matches_central_differences(name, batched_lp):
  d = _load(name)
  g = bp_torch.EnumGraph(d["wiring"])
  g.k = int(np.bincount(np.asarray(d["wiring"]["evidence_to_vars"])).max())
  rng = np.random.default_rng(7)
  B = 2
  lp = np.asarray(d["log_potentials"], np.float64)
  lp = np.stack([lp + 0.1 * rng.normal(size=lp.shape) for _ in range(B)]) if batched_lp else lp
  ev = np.asarray(d["evidence"], np.float64)[None] + rng.normal(size=(B,) + d["evidence"].shape)
  m = 0.3 * rng.normal(size=(B,) + d["ftov_msgs_in"].shape)
  labels_w = torch.as_tensor(rng.random(size=(B,) + d["evidence"].shape))
  iters, damping, temperature = 12, 0.5, float(d["temperature"])
  args = [torch.tensor(x, dtype=torch.float64, requires_grad=True) for x in (lp, ev, m)]
  loss = _loss(g, *args, iters, damping, temperature, labels_w)
  grads = torch.autograd.grad(loss, args)
  h = 1e-6
  for which, (x, gx) in enumerate(zip(args, grads)):
    flat = x.detach().reshape(-1)
    for idx in rng.choice(flat.numel(), size=6, replace=False):
      vals = []
      for sign in (1.0, -1.0):
        xs = [a.detach().clone() for a in args]
        xs[which].view(-1)[idx] += sign * h
        with torch.no_grad():
          vals.append(float(_loss(g, *xs, iters, damping, temperature, labels_w)))
      fd = (vals[0] - vals[1]) / (2 * h)
      assert abs(fd - float(gx.reshape(-1)[idx])) <= 1e-6 * max(1.0, abs(fd)), (which, idx)


# OR / AND / Pool factors (bp_torch.LogicalGraph): the forward against every reference fixture
# of graphs with these factors, and autograd against central differences.
LOGICAL = ["case_deconv_T1", "case_deconv_T0", "case_mixed_T1", "case_mixed_T0.3",
           "case_mixed_T0.001", "case_mixed_T0", "case_mixed_iters0", "case_mixed_iters1"]


@pytest.mark.parametrize("name", LOGICAL)
def test_logical_forward_matches_reference_fixture(name):
  d = _load(name)
  g = bp_torch.LogicalGraph(d["wiring"])
  f64 = lambda x: torch.as_tensor(np.asarray(x, dtype=np.float64))
  with torch.no_grad():
    out = g.run(f64(d["log_potentials"]), f64(d["evidence"]), f64(d["ftov_msgs_in"]),
                int(d["num_iters"]), float(d["damping"]), float(d["temperature"]))
  ref = d["ftov_msgs_out"]
  fin = np.isfinite(ref)
  np.testing.assert_array_equal(np.isfinite(out[0].numpy()), fin)
  # float32 reference vs float64 restatement
  np.testing.assert_allclose(out[0].numpy()[fin], ref[fin], atol=1e-5, rtol=0)


def test_logical_graph_equals_enum_graph_on_enum_only_graphs():
  d = _load("case_potts_K4")
  f64 = lambda x: torch.as_tensor(np.asarray(x, dtype=np.float64))
  args = (f64(d["log_potentials"]), f64(d["evidence"]), f64(d["ftov_msgs_in"]), 9, 0.5, 1.0)
  with torch.no_grad():
    a = bp_torch.EnumGraph(d["wiring"]).run(*args)
    b = bp_torch.LogicalGraph(d["wiring"]).run(*args)
  assert torch.equal(a, b)


@pytest.mark.parametrize("name,temperature", [("case_mixed_T1", 1.0), ("case_mixed_T1", 0.7),
                                              ("case_mixed_T1", 0.3), ("case_deconv_T1", 1.0)])
def test_logical_autograd_matches_central_differences(name, temperature):
  d = _load(name)
  g = bp_torch.LogicalGraph(d["wiring"])
  rng = np.random.default_rng(11)
  B = 2
  lp = np.asarray(d["log_potentials"], np.float64)
  lp = np.stack([lp + 0.1 * rng.normal(size=lp.shape) for _ in range(B)])
  ev = np.asarray(d["evidence"], np.float64)[None] + rng.normal(size=(B,) + d["evidence"].shape)
  m = 0.3 * rng.normal(size=(B,) + d["ftov_msgs_in"].shape)
  w = torch.as_tensor(rng.normal(size=(B,) + d["ftov_msgs_in"].shape))
  iters, damping = 8, 0.5

  def loss(*xs):
    out = g.run(*xs, iters, damping, temperature)
    return (torch.where(out > -1e30, out, torch.zeros_like(out)) * w).sum()

  args = [torch.tensor(x, dtype=torch.float64, requires_grad=True) for x in (lp, ev, m)]
  grads = torch.autograd.grad(loss(*args), args, allow_unused=True)
  h = 1e-6
  for which, (x, gx) in enumerate(zip(args, grads)):
    flat = x.detach().reshape(-1)
    gflat = gx.reshape(-1) if gx is not None else torch.zeros_like(flat)
    assert torch.isfinite(gflat).all()
    if flat.numel() == 0:  # the deconvolution graph has no potentials
      continue
    for idx in rng.choice(flat.numel(), size=6, replace=False):
      vals = []
      for sign in (1.0, -1.0):
        xs = [a.detach().clone() for a in args]
        xs[which].view(-1)[idx] += sign * h
        with torch.no_grad():
          vals.append(float(loss(*xs)))
      fd = (vals[0] - vals[1]) / (2 * h)
      assert abs(fd - float(gflat[idx])) <= 1e-5 * max(1.0, abs(fd)), (which, idx, fd,
                                                                         float(gflat[idx]))


def _closed_form_vjp_check(name, which, temperature):
  """Per factor closed-form VJP (oracle/closed_form_vjp.py) against autograd of one update."""
  from oracle import closed_form_vjp as cf  # pylint: disable=g-import-not-at-top
  d = _load(name)
  g = bp_torch.LogicalGraph(d["wiring"])
  a0, b0 = g.msgs_ranges[1 + which]
  n = b0 - a0
  rng = np.random.default_rng(3 + which)
  B = 2
  vt = torch.tensor(rng.normal(size=(B, n)) * 2.0, dtype=torch.float64, requires_grad=True)
  up = torch.tensor(rng.normal(size=(B, n)), dtype=torch.float64)
  if which < 2:
    out = g.logical_update(vt, which, temperature)
  else:
    out = g.pool_update(vt, temperature)
  (want,) = torch.autograd.grad((out * up).sum(), vt)
  got = np.zeros((B, n))
  v, u = vt.detach().numpy(), up.numpy()
  if which < 2:
    pfi, pmi, ch, off, F = g.logical[which]
    pfi, pmi, ch = pfi.numpy(), pmi.numpy(), ch.numpy()
    for b in range(B):
      for f in range(F):
        idx = np.nonzero(pfi == f)[0]
        dr, do, dcr, dco = cf.logical_factor_vjp(
            [v[b, pmi[i] + off] for i in idx], [v[b, pmi[i]] for i in idx], v[b, ch[f] + off],
            v[b, ch[f]], [u[b, pmi[i] + off] for i in idx], u[b, ch[f] + off], temperature)
        for k, i in enumerate(idx):
          got[b, pmi[i] + off] += dr[k]
          got[b, pmi[i]] += do[k]
        got[b, ch[f] + off] += dcr
        got[b, ch[f]] += dco
  else:
    cfi, cmi, ind, F = g.pool
    cfi, cmi, ind = cfi.numpy(), cmi.numpy(), ind.numpy()
    for b in range(B):
      for f in range(F):
        idx = np.nonzero(cfi == f)[0]
        dr, dz, dir_, diz = cf.pool_factor_vjp(
            [v[b, cmi[i] + 1] for i in idx], [v[b, cmi[i]] for i in idx], v[b, ind[f] + 1],
            v[b, ind[f]], [u[b, cmi[i] + 1] for i in idx], u[b, ind[f] + 1], temperature)
        for k, i in enumerate(idx):
          got[b, cmi[i] + 1] += dr[k]
          got[b, cmi[i]] += dz[k]
        got[b, ind[f] + 1] += dir_
        got[b, ind[f]] += diz
  np.testing.assert_allclose(got, want.numpy(), atol=1e-9, rtol=1e-9)


@pytest.mark.parametrize("temperature", [1.0, 0.7, 0.3, 0.2])
@pytest.mark.parametrize("name,which", [("case_mixed_T1", 0), ("case_mixed_T1", 1),
                                        ("case_mixed_T1", 2), ("case_deconv_T1", 0),
                                        ("case_deconv_T1", 1)])
def test_closed_form_vjps_match_autograd(name, which, temperature):
  _closed_form_vjp_check(name, which, temperature)
