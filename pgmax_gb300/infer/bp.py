"""BP: the drop-in for pgmax.infer.BP (pgmax/infer/bp.py:36-288), run by the pgbp CUDA engine.

`run_with_diffs(bp_arrays, num_iters, damping=0.5, temperature=T)` performs, on the GPU, exactly the
reference's loop: clip potentials to +-1e6, normalise and clip the initial messages, then
max(num_iters, 1) iterations of var-to-factor, factor-to-var for each type, damping,
normalisation, clipping and the max residual. BPArrays may carry a leading batch axis (what
`jax.vmap(bp.run)` computes); the whole batch runs in one call.
"""

import dataclasses
import warnings
from typing import Any, Callable, Dict, Hashable, Optional, Tuple

import numpy as np

from .. import autodiff, engine
from .bp_state import BPArrays, BPState
from .inferer import Beliefs, Inferer, InfererContext, unflatten_beliefs


def _is_torch(x):
  return type(x).__module__.startswith("torch")


@dataclasses.dataclass(frozen=True, eq=False)
class BeliefPropagation(Inferer):
  run_bp: Callable[..., BPArrays]
  run_with_diffs: Callable[..., Tuple[BPArrays, Any]]
  context: Any = None
  run_perturbed: Optional[Callable[..., BPArrays]] = None


def BP(bp_state: BPState, temperature: Optional[float] = 0.0,  # pylint: disable=invalid-name
       exec_flags: int = 0, checkpoint_every: int = 10) -> BeliefPropagation:
  """Returns the belief propagation functions of `bp_state`'s factor graph.

  Arguments not in PGMax: `exec_flags` forces an execution path of the engine
  (pgmax_gb300.native.FLAG_*); `checkpoint_every` is the message checkpoint interval of
  differentiable runs. A run whose BPArrays hold torch tensors that require grad (with grad
  enabled) is differentiable: torch autograd reaches the log potentials, evidence and initial
  messages through the hand-written adjoint (pgmax_gb300.autodiff), as jax.grad does through the
  reference's bp.run.
  """
  ctx = InfererContext(bp_state, exec_flags)
  default_t = temperature

  def run_with_diffs(bp_arrays: BPArrays, num_iters: int, damping: float = 0.5,
                     temperature: float = default_t):
    if autodiff.wants_grad(bp_arrays.log_potentials, bp_arrays.evidence, bp_arrays.ftov_msgs):
      msgs, deltas = autodiff.run_with_diffs(ctx.plan, bp_arrays.log_potentials,
                                             bp_arrays.evidence, bp_arrays.ftov_msgs, num_iters,
                                             damping, temperature, checkpoint_every)
    else:
      msgs, deltas = ctx.plan.run(bp_arrays.log_potentials, bp_arrays.evidence,
                                  bp_arrays.ftov_msgs, num_iters, damping, temperature)
    lp = bp_arrays.log_potentials
    ev = bp_arrays.evidence
    return BPArrays(log_potentials=lp if _is_torch(lp) else ctx.plan._dev(lp),  # pylint: disable=protected-access
                    ftov_msgs=msgs,
                    evidence=ev if _is_torch(ev) else ctx.plan._dev(ev)), deltas  # pylint: disable=protected-access

  def run(bp_arrays: BPArrays, num_iters: int, damping: float = 0.5,
          temperature: float = default_t) -> BPArrays:
    return run_with_diffs(bp_arrays, num_iters, damping, temperature)[0]

  def run_bp(bp_arrays: BPArrays, num_iters: int, damping: float = 0.5) -> BPArrays:
    warnings.warn("BP.run_bp is deprecated. Please consider using BP.run instead.")
    return run(bp_arrays, num_iters, damping, default_t)

  def run_perturbed(bp_arrays: BPArrays, num_iters: int, seed: int, batch: int,
                    noise_scale: float = 1.0, damping: float = 0.5,
                    temperature: float = default_t) -> BPArrays:
    """Perturb-and-MAP: `run` over `batch` samples whose evidence is bp_arrays.evidence plus
    noise_scale times fresh Gumbel(0, 1) noise (the stream of `seed`, pgmax_gb300.engine.gumbel)
    on every variable state, generated on the GPU inside the run. The returned BPArrays hold the
    batch's messages and its perturbed evidence [batch, N_vs], ready for get_beliefs. Not in
    PGMax, whose users draw the noise themselves and vmap run over update(evidence_updates=...)."""
    msgs, _, ev = ctx.plan.run_perturbed(bp_arrays.log_potentials, bp_arrays.evidence,
                                         bp_arrays.ftov_msgs, num_iters, seed, batch,
                                         noise_scale, damping, temperature, with_deltas=False)
    lp = bp_arrays.log_potentials
    return BPArrays(log_potentials=lp if _is_torch(lp) else ctx.plan._dev(lp),  # pylint: disable=protected-access
                    ftov_msgs=msgs, evidence=ev)

  return BeliefPropagation(init=ctx.init, update=ctx.update, to_bp_state=ctx.to_bp_state,
                           get_beliefs=ctx.get_beliefs, run=run, run_bp=run_bp,
                           run_with_diffs=run_with_diffs, context=ctx,
                           run_perturbed=run_perturbed)


def _softmax_last(x):
  if autodiff.wants_grad(x):
    # differentiable beliefs (torch autograd reaches them): torch's softmax carries the gradient
    if x.numel() == 0:
      return x
    return (x - x.logsumexp(dim=-1, keepdim=True)).exp()
  return engine.softmax_last(x)


def get_marginals(beliefs: Dict[Hashable, Any]) -> Dict[Hashable, Any]:
  """Per-variable softmax of the beliefs (pgmax/infer/bp.py:263-288) on the GPU. Beliefs from
  get_beliefs are normalised by the pgbp_marginals kernel over the flat array, any other belief
  arrays by pgbp_softmax_rows; padded states get probability 0. Beliefs that require grad go
  through torch's softmax so that autograd reaches them."""
  ctx = getattr(beliefs, "context", None)
  flat = getattr(beliefs, "flat", None)
  if (ctx is not None and flat is not None and ctx.num_variables > 0 and
      not autodiff.wants_grad(flat)):
    flat = ctx.plan.marginals(beliefs.flat)
    out = unflatten_beliefs(flat, ctx.bp_state.fg_state.variable_groups)

    def zero_pad(x):
      if isinstance(x, dict):
        return {k: zero_pad(v) for k, v in x.items()}
      return x.nan_to_num(nan=float("nan"), posinf=float("inf"), neginf=0.0)

    return {k: zero_pad(v) for k, v in out.items()}

  def tmap(t):
    return {k: tmap(v) for k, v in t.items()} if isinstance(t, dict) else _softmax_last(t)

  return tmap(beliefs)
