"""Differentiable float64 restatement of BP over EnumFactors in torch. TEST INFRASTRUCTURE ONLY.

The reference of the adjoint tests: torch autograd through this unrolled loop gives the gradient
that jax.grad gives through the reference's bp.run (which these tests cannot run without jax),
and it is itself checked against float64 central differences and, for its forward values,
against the golden fixtures recorded from the reference's code. Imported only by tests/.

Follows, over the flat wiring dict of oracle.py:
  run_with_diffs           pgmax/infer/bp.py:84-146 (potential clip, initial normalisation, loop)
  pass_var_to_fac_messages pgmax/infer/bp.py:191-219
  normalize_and_clip_msgs  pgmax/infer/bp.py:222-260
  pass_enum_fac_to_var_messages  pgmax/factor/enum.py:398-475 (temperature > 0: the shift M is
    detached, which leaves T log sum exp((s - M) / T) + M and its gradient unchanged; temperature
    0: the max-product branch, forward values only)
  get_beliefs              pgmax/infer/inferer.py:211-225
"""

import numpy as np
import torch

MSG_NEG_INF = -1e32
LOG_POTENTIAL_MAX_ABS = 1e6


class EnumGraph:
  """Index tensors of an Enum-only graph from the flat wiring (keys as in oracle.Wiring)."""

  def __init__(self, wiring, device="cpu"):
    mr = np.asarray(wiring["msgs_ranges"]).reshape(4, 2)
    if any(mr[t, 1] > mr[t, 0] for t in (1, 2, 3)):
      raise ValueError("bp_torch covers EnumFactors only")
    t = lambda k: torch.as_tensor(np.asarray(wiring[k], dtype=np.int64), device=device)
    self.vs = t("var_states_for_edge_states")
    self.edge = t("edge_indices_for_edge_states")
    self.cfg = t("enum.factor_configs_indices")
    self.cfg_es = t("enum.factor_configs_edge_states")
    self.num_cfg = int(wiring["enum.num_val_configs"])
    self.num_edges = int(wiring["num_edges"])
    self.num_var_states = int(wiring["num_var_states"])
    self.num_edge_states = int(self.vs.shape[0])
    pr = np.asarray(wiring["potentials_ranges"]).reshape(4, 2)
    self.lp_range = (int(pr[0, 0]), int(pr[0, 1]))

  def normalize(self, msgs):
    """msgs [B, E_s]: subtract each edge's max, clip at MSG_NEG_INF (bp.py:222-260)."""
    B = msgs.shape[0]
    mx = torch.full((B, self.num_edges), -float("inf"), dtype=msgs.dtype, device=msgs.device)
    mx = mx.scatter_reduce(1, self.edge.expand(B, -1), msgs, "amax", include_self=True)
    return torch.clamp(msgs - mx[:, self.edge], min=MSG_NEG_INF)

  def var_sums(self, msgs, evidence):
    return evidence.index_add(1, self.vs, msgs)

  def enum_update(self, vtof, lp, temperature):
    """Factor-to-variable messages of every EnumFactor (enum.py:398-475); temperature 0 is the
    max-product branch (forward only)."""
    B = vtof.shape[0]
    summary = torch.zeros((B, self.num_cfg), dtype=vtof.dtype, device=vtof.device)
    summary = summary.index_add(1, self.cfg, vtof[:, self.cfg_es]) + lp
    rows = summary[:, self.cfg]
    mx = torch.full((B, self.num_edge_states), -float("inf"), dtype=vtof.dtype, device=vtof.device)
    if temperature == 0:
      return mx.scatter_reduce(1, self.cfg_es.expand(B, -1), rows, "amax", include_self=True) - vtof
    mx = mx.scatter_reduce(1, self.cfg_es.expand(B, -1), rows.detach(), "amax", include_self=True)
    ex = torch.exp((rows - mx[:, self.cfg_es]) / temperature)
    se = torch.zeros_like(vtof).index_add(1, self.cfg_es, ex)
    return temperature * torch.log(se) + mx - vtof

  def iterate(self, msgs, lp, evidence, damping, temperature):
    vsum = self.var_sums(msgs, evidence)
    vtof = vsum[:, self.vs] - msgs
    f = self.enum_update(vtof, lp, temperature)
    return self.normalize(damping * msgs + (1.0 - damping) * f)

  def run(self, log_potentials, evidence, ftov_msgs, num_iters, damping=0.5, temperature=1.0,
          with_last_delta=False):
    """Final messages [B, E_s] of run_with_diffs; inputs [n] (shared) or [B, n]. With
    with_last_delta, also the last iteration's max |change| per instance (msgs_deltas[-1])."""
    if temperature < 0:
      raise ValueError("temperature must be >= 0")
    shapes = [x.shape[0] for x in (log_potentials, evidence, ftov_msgs) if x.ndim == 2]
    B = shapes[0] if shapes else 1
    lp = log_potentials if log_potentials.ndim == 2 else log_potentials.expand(B, -1)
    ev = evidence if evidence.ndim == 2 else evidence.expand(B, -1)
    m = ftov_msgs if ftov_msgs.ndim == 2 else ftov_msgs.expand(B, -1)
    lp = torch.clamp(lp, -LOG_POTENTIAL_MAX_ABS, LOG_POTENTIAL_MAX_ABS)
    lp = lp[:, self.lp_range[0]:self.lp_range[1]]
    m = self.normalize(m)
    for _ in range(max(int(num_iters), 1)):
      prev = m
      m = self.iterate(m, lp, ev, damping, temperature)
    if with_last_delta:
      return m, (m - prev).abs().amax(dim=1)
    return m

  def beliefs(self, evidence, msgs):
    B = msgs.shape[0]
    ev = evidence if evidence.ndim == 2 else evidence.expand(B, -1)
    return self.var_sums(msgs, ev)
