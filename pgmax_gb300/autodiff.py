"""Differentiable BP: torch.autograd.Functions over the pgbp forward engine and its hand-written
adjoint.

The reference differentiates bp.run with jax.grad (examples/grid_mrf.ipynb cells 15-16: a loss on
get_marginals(get_beliefs(bp.run(bp.init(log_potentials_updates=...)))) is differentiated with
respect to the log potentials). Here the same chain is differentiable in torch:

* `run_with_diffs` runs the forward engine in chunks of `checkpoint_every` iterations, keeping
  the messages at each chunk start, and its backward calls pgbp_run_vjp, which recomputes each
  chunk with the forward engine and walks it backwards with the adjoint kernels. Gradients reach
  the log potentials, the evidence and the initial messages.
* `beliefs` is get_beliefs' flat scatter-add, whose backward is pgbp_beliefs_vjp (a gather).

Graphs must consist of EnumFactors (any config tables), OR and AND factors, and the temperature
must be > 0 (the adjoint's scope); Pool factors or temperature 0 raise ValueError at backward
time.
"""

from typing import Optional, Tuple


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


def wants_grad(*xs) -> bool:
  torch = _torch()
  return torch.is_grad_enabled() and any(
      isinstance(x, torch.Tensor) and x.requires_grad for x in xs)


def _sum_to(g, like_ndim: int):
  """Sums a batched [B, n] gradient over the batch when its input was shared ([n])."""
  if g is None:
    return None
  if like_ndim == 1 and g.ndim == 2:
    return g.sum(dim=0)
  return g


def _make_run_fn():
  torch = _torch()

  class RunFn(torch.autograd.Function):
    """(log_potentials, evidence, ftov_msgs) -> final messages of `num_iters` BP iterations."""

    @staticmethod
    def forward(ctx, log_potentials, evidence, ftov_msgs, plan, num_iters, damping, temperature,
                checkpoint_every):  # pylint: disable=arguments-differ
      msgs, deltas, ck = plan.run_checkpointed(log_potentials, evidence, ftov_msgs, num_iters,
                                               damping, temperature, checkpoint_every)
      ctx.plan = plan
      ctx.args = (int(num_iters), float(damping), float(temperature), int(checkpoint_every))
      ctx.ndims = (log_potentials.ndim, evidence.ndim, ftov_msgs.ndim)
      ctx.save_for_backward(log_potentials, evidence, ck)
      ctx.mark_non_differentiable(deltas)
      return msgs, deltas

    @staticmethod
    def backward(ctx, g_msgs, g_deltas):  # pylint: disable=arguments-differ
      del g_deltas  # residuals are not differentiated
      lp, ev, ck = ctx.saved_tensors
      num_iters, damping, temperature, k = ctx.args
      g = g_msgs if g_msgs is not None else torch.zeros(
          ck.shape[1:], dtype=torch.float32, device=ck.device)
      if g.ndim == 1:
        g = g.unsqueeze(0)
      g_lp, g_ev, g_m = ctx.plan.run_vjp(lp, ev, ck, num_iters, g.float().contiguous(), damping,
                                         temperature, k, want_msgs_in=ctx.needs_input_grad[2])
      if ctx.needs_input_grad[2]:
        g_m = _sum_to(g_m, ctx.ndims[2])
      lp_nd, ev_nd, _ = ctx.ndims
      if lp_nd == 1 and g_lp.ndim == 2:
        g_lp = g_lp.sum(dim=0)
      if ev_nd == 1 and g_ev.ndim == 2:
        g_ev = g_ev.sum(dim=0)
      return (g_lp.to(lp.dtype) if ctx.needs_input_grad[0] else None,
              g_ev.to(ev.dtype) if ctx.needs_input_grad[1] else None,
              g_m if ctx.needs_input_grad[2] else None, None, None, None, None, None)

  class BeliefsFn(torch.autograd.Function):
    """(evidence, ftov_msgs) -> flat beliefs (evidence + scatter-add of the messages)."""

    @staticmethod
    def forward(ctx, evidence, ftov_msgs, plan):  # pylint: disable=arguments-differ
      ctx.plan = plan
      ctx.ndims = (evidence.ndim, ftov_msgs.ndim)
      return plan.beliefs(evidence, ftov_msgs)

    @staticmethod
    def backward(ctx, g_beliefs):  # pylint: disable=arguments-differ
      g = g_beliefs.float().contiguous()
      g_ev = _sum_to(g, ctx.ndims[0]) if ctx.needs_input_grad[0] else None
      g_m = None
      if ctx.needs_input_grad[1]:
        g_m = _sum_to(ctx.plan.beliefs_vjp(g), ctx.ndims[1])
      return g_ev, g_m, None

  return RunFn, BeliefsFn


_FNS = None


def _fns():
  global _FNS
  if _FNS is None:
    _FNS = _make_run_fn()
  return _FNS


def _as_tensor(plan, x):
  torch = _torch()
  if isinstance(x, torch.Tensor):
    return x.to(device=f"cuda:{plan.device}", dtype=torch.float32)
  return plan._dev(x)  # pylint: disable=protected-access


def run_with_diffs(plan, log_potentials, evidence, ftov_msgs, num_iters: int,
                   damping: float = 0.5, temperature: float = 1.0,
                   checkpoint_every: int = 10) -> Tuple[object, object]:
  """Differentiable run_with_diffs: (messages, residuals); messages carry the autograd graph."""
  run_fn, _ = _fns()
  lp = _as_tensor(plan, log_potentials)
  if plan.num_potentials == 0:
    lp = lp.reshape(-1)[:0]
  return run_fn.apply(lp, _as_tensor(plan, evidence), _as_tensor(plan, ftov_msgs), plan,
                      num_iters, damping, temperature, checkpoint_every)


def beliefs(plan, evidence, ftov_msgs):
  """Differentiable flat beliefs."""
  _, beliefs_fn = _fns()
  return beliefs_fn.apply(_as_tensor(plan, evidence), _as_tensor(plan, ftov_msgs), plan)


def run(plan, log_potentials, evidence, ftov_msgs, num_iters: int, damping: float = 0.5,
        temperature: float = 1.0, checkpoint_every: Optional[int] = 10):
  return run_with_diffs(plan, log_potentials, evidence, ftov_msgs, num_iters, damping,
                        temperature, checkpoint_every)[0]
