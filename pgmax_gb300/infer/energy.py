"""Energy of MAP decodings: pgmax.infer.compute_energy (pgmax/infer/energy.py:53-148) on the
pgbp_energy kernel.

`compute_energy(bp_state, bp_arrays, map_states)` returns `(energy, None, None)` like the
reference. The energy is a float32 device tensor: 0-d for one decoding, [B] when the decodings
(a leading batch axis on every group's states) or the BPArrays carry a batch axis, which is what
`jax.vmap(compute_energy)` gives in the reference (examples/rbm.ipynb evaluates the energies of a
batch of perturb-and-MAP samples this way). Lower is better; +inf marks a decoding that violates a
factor.
"""

from typing import Any, Dict, Hashable, Tuple

import numpy as np

from .bp_state import BPArrays, BPState


def _context(bp_state: BPState):
  """The context whose plan serves this graph: the one a BP object already compiled, else a new
  one (registered on the FactorGraphState, so later calls reuse it)."""
  from .inferer import InfererContext, register_context, registered_context  # pylint: disable=g-import-not-at-top
  ctx = registered_context(bp_state.fg_state)
  if ctx is None:
    ctx = InfererContext(bp_state)
    ctx.plan  # pylint: disable=pointless-statement
    register_context(ctx)
  return ctx


def _flat_states(variable_groups, map_states: Dict[Hashable, Any], device):
  """Per-variable states in evidence_to_vars order, int32 on `device`: [num_variables], or
  [B, num_variables] when a group's states carry a leading batch axis."""
  import torch  # pylint: disable=g-import-not-at-top
  tens = lambda v: (v if isinstance(v, torch.Tensor) else torch.as_tensor(np.asarray(v))).to(
      device=device, dtype=torch.int32)
  parts = []
  for vg in variable_groups:
    data = map_states[vg]
    if isinstance(data, dict):
      # VarDict: one state per name, or [B] states per name
      vals = [tens(data[name]) for name in vg.variable_names]
      vals = [v.reshape(()) if v.numel() == 1 else v.reshape(-1) for v in vals]
      if any(v.ndim == 1 for v in vals):
        B = max(v.shape[0] for v in vals if v.ndim == 1)
        vals = [v.expand(B) if v.ndim == 0 else v for v in vals]
      parts.append(torch.stack(vals, dim=-1))
    else:
      parts.append(tens(vg.flatten(data)))
  if any(p.ndim == 2 for p in parts):
    B = max(p.shape[0] for p in parts if p.ndim == 2)
    parts = [p if p.ndim == 2 else p.unsqueeze(0).expand(B, -1) for p in parts]
  if not parts:
    return torch.zeros(0, dtype=torch.int32, device=device)
  return torch.cat(parts, dim=-1).contiguous()


def compute_energy(bp_state: BPState, bp_arrays: BPArrays, map_states: Dict[Hashable, Any],
                   debug_mode: bool = False) -> Tuple[Any, Any, Any]:
  """Returns (energy, None, None): the energy of the decoding `map_states`, a dict from the
  VarGroups of the factor graph to their states, under the evidence and log potentials of
  `bp_arrays` (energy.py:53-148). The per-variable and per-factor breakdown of the reference's
  debug mode (energy.py:150-213, a host-side Python loop) is not provided."""
  if debug_mode:
    raise NotImplementedError(
        "compute_energy(debug_mode=True) (per-variable and per-factor energies) is not provided; "
        "the total energy is computed on the device with debug_mode=False")
  ctx = _context(bp_state)
  plan = ctx.plan
  groups = [vg for vg in bp_state.fg_state.variable_groups if int(np.prod(vg.num_states.shape)) > 0]
  states = _flat_states(groups, map_states, f"cuda:{plan.device}")
  energy = plan.energy(bp_arrays.log_potentials, bp_arrays.evidence, states)
  return energy, None, None
