"""The warm-start network on the library's own CUDA kernels (include/pgbp_learn.h).

Six 3x3 convolutions with circular padding, 64 channels: five 64 -> 64 with ReLU, then 64 -> 32.
Input: per variable of the toroidal grid its K = 8 unaries, the couplings of its four edges and
the closed-form one-step messages of its four factors (potts.features); output: a correction to
those one-step messages, giving the 4 x 8 initial log-messages into the variable from its four
factors (potts.message_index). BF16 weights and activations, FP32
accumulation, FP32 master weights and Adam moments. Torch supplies device memory only; every
computation is a pgbp kernel.
"""

import ctypes
from typing import Dict, List

import numpy as np

from .. import native

LAYERS = [(64, 64), (64, 64), (64, 64), (64, 64), (64, 64), (64, 32)]


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


def _ptr(t):
  return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class ConvNet:
  """Parameters, forward, and one training step (loss, backward, Adam)."""

  def __init__(self, device=None, seed: int = 0):
    torch = _torch()
    self.lib = native.load()
    self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    rng = np.random.default_rng(seed)
    self.w, self.b, self.wb = [], [], []
    for layer, (ci, co) in enumerate(LAYERS):
      std = np.sqrt(2.0 / (9 * ci))
      if layer == len(LAYERS) - 1:
        std *= 0.01   # the correction starts near zero: the initial output is the one-step guess
      w = rng.normal(0.0, std, size=(9, co, ci)).astype(np.float32)
      self.w.append(torch.as_tensor(w, device=self.device))
      self.b.append(torch.zeros(co, dtype=torch.float32, device=self.device))
    self.wb = [w.to(torch.bfloat16) for w in self.w]
    self.m = [torch.zeros_like(p) for p in self.w + self.b]
    self.v = [torch.zeros_like(p) for p in self.w + self.b]
    self.step = 0
    # the network is trained on targets times target_scale (the corrections are ~1e-2):
    # messages = output / target_scale
    self.target_scale = 1.0

  # ----------------------------------------------------------------------------- helpers
  def _stream(self):
    return ctypes.c_void_p(_torch().cuda.current_stream(self.device).cuda_stream)

  def _conv(self, x, w, bias, ci, co, out_f32=False, relu=False, mask=None):
    torch = _torch()
    n, h, wd, _ = x.shape
    out = torch.empty((n, h, wd, co), dtype=torch.float32 if out_f32 else torch.bfloat16,
                      device=self.device)
    native.check(self.lib.pgbp_conv3x3(self._stream(), n, h, wd, ci, co, _ptr(x), _ptr(w),
                                       _ptr(bias), _ptr(out), int(out_f32), int(relu),
                                       _ptr(mask)), "pgbp_conv3x3")
    return out

  # ----------------------------------------------------------------------------- API
  def forward(self, x, keep: bool = False):
    """x [n, h, w, 64] (BF16, or float converted) -> [n, h, w, 32] FP32 (the correction)."""
    torch = _torch()
    a = x.to(device=self.device, dtype=torch.bfloat16).contiguous()
    acts = [a]
    for layer, (ci, co) in enumerate(LAYERS):
      last = layer == len(LAYERS) - 1
      a = self._conv(a, self.wb[layer], self.b[layer], ci, co, out_f32=last, relu=not last)
      acts.append(a)
    return (a, acts) if keep else a

  def loss_and_grad(self, pred, target):
    """Mean-centred squared error over groups of 8 states and its gradient (BF16)."""
    torch = _torch()
    grad = torch.empty(pred.shape, dtype=torch.bfloat16, device=self.device)
    loss = torch.zeros(1, dtype=torch.float64, device=self.device)
    groups = pred.numel() // 8
    native.check(self.lib.pgbp_center_mse(
        self._stream(), groups, 8, _ptr(pred), _ptr(target.contiguous()), _ptr(grad), _ptr(loss),
        ctypes.c_float(1.0 / pred.numel())), "pgbp_center_mse")
    return loss / pred.numel(), grad

  def gradients(self, acts: List, g):
    """Backward through the six layers from g = dL/d(output) (BF16): ([dW], [db]) FP32."""
    torch = _torch()
    dws, dbs = [None] * len(LAYERS), [None] * len(LAYERS)
    n, h, wd, _ = g.shape
    for layer in range(len(LAYERS) - 1, -1, -1):
      ci, co = LAYERS[layer]
      dw = torch.empty((9, co, ci), dtype=torch.float32, device=self.device)
      db = torch.empty(co, dtype=torch.float32, device=self.device)
      ws_bytes = int(self.lib.pgbp_conv3x3_wgrad_workspace(ci, co))
      ws = torch.empty(ws_bytes, dtype=torch.uint8, device=self.device)
      native.check(self.lib.pgbp_conv3x3_wgrad(self._stream(), n, h, wd, ci, co,
                                               _ptr(acts[layer]), _ptr(g), _ptr(dw), _ptr(db),
                                               _ptr(ws), ws_bytes), "pgbp_conv3x3_wgrad")
      dws[layer], dbs[layer] = dw, db
      if layer > 0:
        flipped = torch.empty((9, ci, co), dtype=torch.bfloat16, device=self.device)
        native.check(self.lib.pgbp_conv3x3_flip(self._stream(), ci, co, _ptr(self.wb[layer]),
                                                _ptr(flipped)), "pgbp_conv3x3_flip")
        # input gradient, times the ReLU derivative of the layer below (its output > 0)
        g = self._conv(g, flipped, None, co, ci, mask=acts[layer])
    return dws, dbs

  def adam(self, dws, dbs, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    self.step += 1
    grads = list(dws) + list(dbs)
    params = self.w + self.b
    copies = self.wb + [None] * len(self.b)
    for p, g, m, v, c in zip(params, grads, self.m, self.v, copies):
      native.check(self.lib.pgbp_adam(self._stream(), p.numel(), _ptr(p), _ptr(g), _ptr(m),
                                      _ptr(v), _ptr(c), ctypes.c_float(lr), ctypes.c_float(beta1),
                                      ctypes.c_float(beta2), ctypes.c_float(eps), self.step),
                   "pgbp_adam")

  def train_step(self, x, target, lr=1e-3):
    """One Adam step on the mean-centred squared error; returns the loss (device tensor)."""
    pred, acts = self.forward(x, keep=True)
    loss, g = self.loss_and_grad(pred, target)
    dws, dbs = self.gradients(acts, g)
    self.adam(dws, dbs, lr)
    return loss

  def messages(self, x):
    """The correction in message units (forward output / target_scale)."""
    return self.forward(x) * (1.0 / self.target_scale)

  def state(self) -> Dict[str, np.ndarray]:
    out = {"target_scale": np.float32(self.target_scale)}
    for k, (w, b) in enumerate(zip(self.w, self.b)):
      out[f"w{k}"] = w.cpu().numpy()
      out[f"b{k}"] = b.cpu().numpy()
    return out

  def load(self, state: Dict[str, np.ndarray]):
    torch = _torch()
    for k in range(len(LAYERS)):
      self.w[k] = torch.as_tensor(np.asarray(state[f"w{k}"], np.float32), device=self.device)
      self.b[k] = torch.as_tensor(np.asarray(state[f"b{k}"], np.float32), device=self.device)
    self.wb = [w.to(torch.bfloat16) for w in self.w]
    self.target_scale = float(state.get("target_scale", 1.0))
    return self
