"""Inference: the drop-in for pgmax.infer (pgmax/infer/__init__.py)."""

from .bp import BP, BeliefPropagation, get_marginals
from .bp_state import BPArrays, BPState, Evidence, FToVMessages, LogPotentials
from .dual_lp import SDLP, SmoothDualLP
from .energy import compute_energy
from .inferer import Inferer, InfererContext, decode_map_states


def build_inferer(bp_state: BPState, backend: str) -> Inferer:
  """Builds a supported inferer (pgmax/infer/__init__.py:34-41)."""
  if backend == "bp":
    return BP(bp_state)
  if backend == "sdlp":
    return SDLP(bp_state)
  raise NotImplementedError(f"Inferer {backend} is not supported.")
