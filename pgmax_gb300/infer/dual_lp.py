"""The smooth dual LP-MAP solver: pgmax.infer.SDLP (pgmax/infer/dual_lp.py:60-463) on the pgbp
SDLP kernels (include/pgbp.h, pgbp_sdlp_run / pgbp_sdlp_objective).

Same functions and arguments as the reference: run_with_objvals / run (accelerated gradient
descent at logsumexp_temp > 0, subgradient descent at 0), decode_primal_unaries,
get_primal_upper_bound, get_map_lower_bound (minus the energy of a decoding, on pgbp_energy) and
get_bp_updates. BPArrays may carry a leading batch axis (what jax.vmap gives in the reference);
objective values are then [B, num_iters]. Results are device tensors.
"""

import dataclasses
from typing import Any, Callable, Dict, Hashable, Optional, Tuple

from . import energy as energy_mod
from .bp_state import BPArrays, BPState
from .inferer import Inferer, InfererContext, decode_map_states


@dataclasses.dataclass(frozen=True, eq=False)
class SmoothDualLP(Inferer):
  """Smooth Dual LP-MAP solver functions (dual_lp.py:33-57)."""
  run_with_objvals: Callable[..., Tuple[BPArrays, Any]]
  decode_primal_unaries: Callable[..., Tuple[Dict[Hashable, Any], Dict[Hashable, Any]]]
  get_primal_upper_bound: Callable[..., Any]
  get_map_lower_bound: Callable[..., Any]
  get_bp_updates: Callable[..., Tuple[Any, Any]]


def SDLP(bp_state: BPState) -> SmoothDualLP:  # pylint: disable=invalid-name
  """Returns the Smooth Dual LP-MAP functions for `bp_state` (dual_lp.py:60-463)."""
  ctx = InfererContext(bp_state)

  def run_with_objvals(sdlp_arrays: BPArrays, logsumexp_temp: float, num_iters: int,
                       lr: Optional[float] = None) -> Tuple[BPArrays, Any]:
    """num_iters (sub)gradient steps; returns the new BPArrays and the objective before each
    step (dual_lp.py:238-313)."""
    if logsumexp_temp < 0.0 or logsumexp_temp > 1.0:
      raise ValueError("The log sum-exp temperature of the Dual LP-MAP solver has to be between "
                       "0.0 and 1.0")
    if logsumexp_temp != 0.0 and lr is not None and lr > logsumexp_temp:
      raise ValueError("For gradient descent, the learning rate must be smaller than the log "
                       "sum-exp temperature.")
    if lr is None:
      lr = logsumexp_temp if logsumexp_temp != 0.0 else 0.01
    msgs, objvals = ctx.plan.sdlp_run(sdlp_arrays.log_potentials, sdlp_arrays.evidence,
                                      sdlp_arrays.ftov_msgs, int(num_iters),
                                      float(logsumexp_temp), float(lr))
    return BPArrays(log_potentials=sdlp_arrays.log_potentials, ftov_msgs=msgs,
                    evidence=sdlp_arrays.evidence), objvals

  def run(sdlp_arrays: BPArrays, logsumexp_temp: float, num_iters: int,
          lr: Optional[float] = None) -> BPArrays:
    return run_with_objvals(sdlp_arrays, logsumexp_temp, num_iters, lr)[0]

  def decode_primal_unaries(sdlp_arrays: BPArrays):
    """The local decoding of the primal unaries and the dual beliefs (dual_lp.py:330-352)."""
    dual_beliefs = ctx.get_beliefs(sdlp_arrays)
    return decode_map_states(dual_beliefs), dual_beliefs

  def get_primal_upper_bound(sdlp_arrays: BPArrays):
    """The Dual LP-MAP objective at temperature 0: an upper bound of the LP-MAP optimum
    (dual_lp.py:354-367)."""
    return ctx.plan.sdlp_objective(sdlp_arrays.log_potentials, sdlp_arrays.evidence,
                                   sdlp_arrays.ftov_msgs, 0.0)["objval"]

  def get_map_lower_bound(sdlp_arrays: BPArrays, decoded_primal_unaries: Dict[Hashable, Any],
                          debug_mode: bool = False):
    """Minus the energy of the decoding: a lower bound of the MAP optimum (dual_lp.py:369-417)."""
    return -energy_mod.compute_energy(bp_state, sdlp_arrays, decoded_primal_unaries,
                                      debug_mode=debug_mode)[0]

  def get_bp_updates(sdlp_arrays: BPArrays, logsumexp_temp: float):
    """(factor updates at -ftov, per-edge log-sum-exp of updates - ftov) (dual_lp.py:419-448)."""
    out = ctx.plan.sdlp_objective(sdlp_arrays.log_potentials, sdlp_arrays.evidence,
                                  sdlp_arrays.ftov_msgs, float(logsumexp_temp), updates=True,
                                  edge_lse=True)
    return out["updates"], out["edge_lse"]

  return SmoothDualLP(init=ctx.init, update=ctx.update, to_bp_state=ctx.to_bp_state,
                      get_beliefs=ctx.get_beliefs, run=run, run_with_objvals=run_with_objvals,
                      decode_primal_unaries=decode_primal_unaries,
                      get_primal_upper_bound=get_primal_upper_bound,
                      get_map_lower_bound=get_map_lower_bound, get_bp_updates=get_bp_updates)
