"""Energy of MAP decodings: pgmax.infer.compute_energy (pgmax/infer/energy.py:53-204) on the
pgbp_energy / pgbp_energy_terms kernels.

`compute_energy(bp_state, bp_arrays, map_states)` returns `(energy, None, None)` like the
reference. The energy is a float32 device tensor: 0-d for one decoding, [B] when the decodings
(a leading batch axis on every group's states) or the BPArrays carry a batch axis, which is what
`jax.vmap(compute_energy)` gives in the reference (examples/rbm.ipynb evaluates the energies of a
batch of perturb-and-MAP samples this way). Lower is better; +inf marks a decoding that violates a
factor.

With `debug_mode=True` it returns `(energy, vars_energies, factors_energies)` as the reference's
debug mode does (energy.py:151-204): the energy as a Python float summed over the variables, then
the factors, in the reference's order; each variable's -evidence of its decoded state; each
factor's energy keyed by the frozenset of its variables. The terms come from one kernel launch.
"""

from typing import Any, Dict, Hashable, Tuple

import numpy as np

from .. import factor as factor_mod
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
  `bp_arrays` (energy.py:53-148). With debug_mode, (energy, vars_energies, factors_energies)
  (energy.py:151-204, see the module docstring)."""
  ctx = _context(bp_state)
  plan = ctx.plan
  groups = [vg for vg in bp_state.fg_state.variable_groups if int(np.prod(vg.num_states.shape)) > 0]
  states = _flat_states(groups, map_states, f"cuda:{plan.device}")
  if debug_mode:
    return _compute_energy_debug_mode(bp_state, bp_arrays, groups, states, plan)
  energy = plan.energy(bp_arrays.log_potentials, bp_arrays.evidence, states)
  return energy, None, None


def _compute_energy_debug_mode(bp_state, bp_arrays, groups, states, plan):
  """energy.py:151-204: the evidence of bp_arrays; the decoded configs from the device; the
  potentials of the factor objects themselves (in their own precision), as the reference's
  debug mode reads them."""
  ev_ndim = getattr(bp_arrays.evidence, "ndim", None)
  if states.ndim != 1 or (ev_ndim if ev_ndim is not None else np.ndim(bp_arrays.evidence)) != 1:
    raise ValueError("compute_energy(debug_mode=True) takes one decoding, without a batch axis")
  # states must be in [0, K): the reference raises for a state past the end (it indexes the
  # evidence with it), and a negative one, which its evidence lookup would count from the end
  # but its factor checks would not, is refused too
  k = np.concatenate([np.asarray(vg.num_states).reshape(-1) for vg in groups]) if groups else (
      np.zeros(0, np.int64))
  s = states.cpu().numpy().astype(np.int64)
  bad = np.nonzero((s < 0) | (s >= k))[0]
  if bad.size:
    raise IndexError(f"decoded state {int(s[bad[0]])} out of range for a variable with "
                     f"{int(k[bad[0]])} states")
  var_e, fac_c = plan.energy_terms(bp_arrays.evidence, states)
  var_e, fac_c = var_e.cpu().numpy(), fac_c.cpu().numpy()
  energy = 0.0
  vars_energies = {}
  i = 0
  for vg in groups:
    for var in vg.variables:
      e = float(var_e[i])
      vars_energies[var] = e
      energy += e
      i += 1
  # the factor's energy from its decoded config and its own potentials (enum.py:326-360), or
  # the verdict of an OR / AND / Pool factor (logical.py:378-406, pool.py:242-272)
  factors_energies = {}
  f = 0
  for factor_group in bp_state.fg_state.factor_group_to_potentials_starts:
    enum = factor_group.factor_type is factor_mod.EnumFactor
    for this_factor in factor_group.factors:
      c = int(fac_c[f])
      if c < 0:
        e = float(np.inf)
      elif enum:
        e = float(-np.asarray(this_factor.log_potentials)[c])
      else:
        e = 0.0
      energy += e
      factors_energies[frozenset(this_factor.variables)] = e
      f += 1
  return energy, vars_energies, factors_energies
