"""CPU float32 restatement of the warm-start network. TEST INFRASTRUCTURE ONLY.

The checker of the network's CUDA kernels (include/pgbp_learn.h): the same six 3x3 convolutions
with circular padding, evaluated by torch on the CPU in float32 from the same BF16 weights and
inputs, with activations rounded to BF16 where the GPU stores them; gradients by torch autograd
(the BF16 roundings pass gradients through unchanged). Imported only by tests/.
"""

import torch
import torch.nn.functional as F

LAYERS = [(64, 64), (64, 64), (64, 64), (64, 64), (64, 64), (64, 32)]


def bf16(x):
  return x.to(torch.bfloat16).to(torch.float32)


def conv3x3(x, w, b=None):
  """x [n, h, w, ci], w [9, co, ci] (tap (dy + 1) * 3 + (dx + 1)), circular padding."""
  co, ci = w.shape[1], w.shape[2]
  k = w.reshape(3, 3, co, ci).permute(2, 3, 0, 1)        # [co, ci, ky, kx]
  xp = F.pad(x.permute(0, 3, 1, 2), (1, 1, 1, 1), mode="circular")
  return F.conv2d(xp, k, b).permute(0, 2, 3, 1)


def forward(x, ws, bs):
  """x [n, h, w, 64] (values exactly BF16), ws / bs float32 -> [n, h, w, 32] float32."""
  a = x
  for layer in range(len(LAYERS)):
    z = conv3x3(a, bf16(ws[layer]), bs[layer])
    a = bf16(torch.relu(z)) if layer < len(LAYERS) - 1 else z
  return a


def center_mse(pred, target, group=8):
  p = pred.reshape(-1, group)
  t = target.reshape(-1, group)
  d = (p - p.mean(1, keepdim=True)) - (t - t.mean(1, keepdim=True))
  return (d * d).sum() / pred.numel()
