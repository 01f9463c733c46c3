"""The warm-start network's CUDA kernels against the CPU float32 restatement (oracle/convnet_ref.py),
and what the trained network gains over cold-start BP.

Tolerances: BF16 outputs within 1e-2 relative of the largest value (one BF16 rounding of a float32
sum); FP32 weight gradients from BF16 operands within 1e-3 (the products are exact, only the
summation order differs); gradients through the whole network, whose intermediate gradients are
BF16, within 3e-2 (relative Frobenius norm).
"""

import numpy as np
import pytest

from oracle import convnet_ref as ref

pytestmark = pytest.mark.gpu

SHAPES = [(16, 64), (64, 64), (64, 32), (32, 64)]


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


def _rel(a, b):
  a = np.asarray(a, np.float64)
  b = np.asarray(b, np.float64)
  return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-12)


def _net():
  from pgmax_gb300.warmstart import convnet  # pylint: disable=g-import-not-at-top
  return convnet.ConvNet(seed=3)


@pytest.mark.parametrize("ci,co", SHAPES)
@pytest.mark.parametrize("out_f32,relu,masked", [(0, 1, 0), (1, 0, 0), (0, 0, 1)])
def test_conv3x3_matches_cpu(ci, co, out_f32, relu, masked):
  torch = _torch()
  net = _net()
  g = torch.Generator().manual_seed(ci * 100 + co)
  n, h, w = 2, 5, 32
  x = torch.randn(n, h, w, ci, generator=g).to(torch.bfloat16)
  wt = (0.2 * torch.randn(9, co, ci, generator=g)).to(torch.bfloat16)
  b = torch.randn(co, generator=g)
  mask = torch.randn(n, h, w, co, generator=g).to(torch.bfloat16) if masked else None
  out = net._conv(x.cuda(), wt.cuda(), b.cuda(), ci, co, out_f32=bool(out_f32), relu=bool(relu),  # pylint: disable=protected-access
                  mask=mask.cuda() if masked else None)
  want = ref.conv3x3(x.float(), wt.float(), b)
  if relu:
    want = torch.relu(want)
  if masked:
    want = want * (mask.float() > 0)
  got = out.float().cpu()
  assert _rel(got, want) < (1e-5 if out_f32 else 1e-2)


@pytest.mark.parametrize("ci,co", SHAPES)
def test_weight_gradient_matches_cpu(ci, co):
  torch = _torch()
  from pgmax_gb300 import native  # pylint: disable=g-import-not-at-top
  lib = native.load()
  g = torch.Generator().manual_seed(7 + ci + co)
  n, h, w = 3, 6, 32
  x = torch.randn(n, h, w, ci, generator=g).to(torch.bfloat16)
  dy = torch.randn(n, h, w, co, generator=g).to(torch.bfloat16)
  wt = torch.zeros(9, co, ci, requires_grad=True)
  bt = torch.zeros(co, requires_grad=True)
  (ref.conv3x3(x.float(), wt, bt) * dy.float()).sum().backward()
  dw = torch.empty(9, co, ci, device="cuda")
  db = torch.empty(co, device="cuda")
  nb = int(lib.pgbp_conv3x3_wgrad_workspace(ci, co))
  ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
  xc, dyc = x.cuda(), dy.cuda()
  stream = torch.cuda.current_stream().cuda_stream
  native.check(lib.pgbp_conv3x3_wgrad(stream, n, h, w, ci, co, xc.data_ptr(), dyc.data_ptr(),
                                      dw.data_ptr(), db.data_ptr(), ws.data_ptr(), nb), "wgrad")
  assert _rel(dw.cpu(), wt.grad) < 1e-3
  assert _rel(db.cpu(), bt.grad) < 1e-3


def test_network_gradients_match_cpu_autograd():
  torch = _torch()
  net = _net()
  g = torch.Generator().manual_seed(11)
  n, h, w = 2, 8, 16
  x = torch.randn(n, h, w, ref.LAYERS[0][0], generator=g).to(torch.bfloat16)
  y = torch.randn(n, h, w, 32, generator=g)
  pred, acts = net.forward(x.cuda(), keep=True)
  loss, gy = net.loss_and_grad(pred, y.cuda())
  dws, dbs = net.gradients(acts, gy)
  ws = [p.detach().cpu().clone().requires_grad_() for p in net.w]
  bs = [p.detach().cpu().clone().requires_grad_() for p in net.b]
  out = ref.forward(x.float(), ws, bs)
  lref = ref.center_mse(out, y)
  lref.backward()
  assert _rel(pred.cpu(), out.detach()) < 2e-2
  assert abs(float(loss) - float(lref.detach())) <= 2e-2 * float(lref.detach())
  for k in range(len(ws)):
    num = torch.linalg.norm(dws[k].cpu() - ws[k].grad) / torch.linalg.norm(ws[k].grad)
    assert float(num) < 3e-2, (k, float(num))
    num = torch.linalg.norm(dbs[k].cpu() - bs[k].grad) / max(float(torch.linalg.norm(bs[k].grad)),
                                                             1e-12)
    assert float(num) < 3e-2, (k, float(num))


def test_adam_step_matches_its_formula():
  torch = _torch()
  net = _net()
  g = [torch.randn_like(p) for p in net.w]
  gb = [torch.randn_like(p) for p in net.b]
  w0 = [p.clone() for p in net.w]
  net.adam(g, gb, lr=1e-2)
  for p, p0, gg in zip(net.w, w0, g):
    m = 0.1 * gg
    v = 0.001 * gg * gg
    want = p0 - 1e-2 * (m / 0.1) / (torch.sqrt(v / 0.001) + 1e-8)
    assert torch.allclose(p, want, atol=1e-6, rtol=1e-5)
  assert torch.equal(net.wb[0], net.w[0].to(torch.bfloat16))


def test_training_lowers_the_loss_and_the_learned_init_beats_a_cold_start():
  """The gain of the learned part over the method without it, on a 16 x 16 toroidal family: the
  trained correction lowers the loss below that of no correction, and warm starts need fewer
  iterations than cold starts at equal belief error."""
  torch = _torch()
  from pgmax_gb300.warmstart import convnet, train  # pylint: disable=g-import-not-at-top
  fam = train.Family(16, 8)
  x, y, info = train.make_dataset(fam, seed=5, n=4096, batch=1024, max_iters=2000)
  assert info["kept"] >= 4000
  yc = y.reshape(-1, 8)
  baseline = float(((yc - yc.mean(1, keepdim=True)) ** 2).mean())
  net = convnet.ConvNet(seed=0)
  losses = train.train(net, x, y, epochs=12, batch=32, lr=3e-4)
  assert losses[-1] < 0.95 * baseline, (losses, baseline)
  res = train.evaluate(fam, net, seed=6, n=256, batch=256, max_iters=2000)
  assert res["fallback_rate"] == 0.0
  assert res["warm_iters_mean"] < 0.9 * res["cold_iters_mean"], res
  assert res["warm_belief_err_mean"] <= 2 * res["cold_belief_err_mean"] + 1e-5, res


def test_packaged_weights_give_a_warm_start_on_the_96_family():
  import os  # pylint: disable=g-import-not-at-top
  from pgmax_gb300.warmstart import convnet, train  # pylint: disable=g-import-not-at-top
  path = os.path.join(os.path.dirname(convnet.__file__), "weights_potts96_k8.npz")
  net = convnet.ConvNet().load(dict(np.load(path)))
  fam = train.Family(96, 8)
  res = train.evaluate(fam, net, seed=9, n=32, batch=32, max_iters=2000)
  assert res["warm_iters_mean"] < res["cold_iters_mean"], res
  assert res["warm_iters_mean"] <= res["onestep_iters_mean"], res


def test_feature_kernel_matches_the_torch_restatement():
  torch = _torch()
  from pgmax_gb300.warmstart import potts  # pylint: disable=g-import-not-at-top
  for L in (3, 16, 96):
    J, u = potts.sample(L, 4, L, 8, 0.7)
    J = torch.as_tensor(J, device="cuda")
    u = torch.as_tensor(u, device="cuda")
    x, m1 = potts.features_and_messages(J, u, L, 8)
    want_m1 = potts.one_step_messages(J, u, L, 8)
    want_x = potts.features(J, u, L, 8)
    assert _rel(m1.cpu(), want_m1.cpu()) < 1e-5
    # BF16 features: one rounding of values within 1e-5 of each other
    assert _rel(x.float().cpu(), want_x.to(torch.bfloat16).float().cpu()) < 1e-2
