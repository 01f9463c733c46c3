"""Differentiable float64 restatement of BP in torch. TEST INFRASTRUCTURE ONLY.

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
  pass_logical_fac_to_var_messages  pgmax/factor/logical.py:492-779 (LogicalGraph)
  pass_pool_fac_to_var_messages     pgmax/factor/pool.py:276-474 (LogicalGraph)
  logaddexp / logminusexp / logsumexps_with_temp  pgmax/factor/update_utils.py:67-190

Gradients at the cutoffs. logminusexp_with_temp returns -inf where a < b + eps (update_utils.py
169-190), selected by jnp.where; autodiff through that where gives NaN when the unselected branch
is evaluated outside its domain. Here the unselected branch is evaluated at a safe argument, so
the gradient there is 0, the derivative of the constant that is returned: the convention the
adjoint kernels follow. Maxima and argmaxes (temperature < 0.5 lower bounds, top-2 of the
parent differences) pass the gradient to the element that attains them.
"""

import numpy as np
import torch

MSG_NEG_INF = -1e32
LOG_POTENTIAL_MAX_ABS = 1e6


class EnumGraph:
  """Index tensors of an Enum-only graph from the flat wiring (keys as in oracle.Wiring)."""

  def __init__(self, wiring, device="cpu", all_types=False):
    mr = np.asarray(wiring["msgs_ranges"]).reshape(4, 2)
    self.msgs_ranges = [(int(mr[t, 0]), int(mr[t, 1])) for t in range(4)]
    if not all_types and any(mr[t, 1] > mr[t, 0] for t in (1, 2, 3)):
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
    B, n = vtof.shape  # the Enum slice (the first in registry order: edge states 0 .. n - 1)
    summary = torch.zeros((B, self.num_cfg), dtype=vtof.dtype, device=vtof.device)
    summary = summary.index_add(1, self.cfg, vtof[:, self.cfg_es]) + lp
    rows = summary[:, self.cfg]
    mx = torch.full((B, n), -float("inf"), dtype=vtof.dtype, device=vtof.device)
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


STABILITY_THRE = 0.5  # TEMPERATURE_STABILITY_THRE, pgmax/factor/logical.py:33


def _lae(a, b, t):
  """logaddexp_with_temp (update_utils.py:150-166): t log(exp(a / t) + exp(b / t))."""
  return t * torch.logaddexp(a / t, b / t)


def _lme(a, b, t, eps):
  """logminusexp_with_temp (update_utils.py:169-190): t log(exp(a / t) - exp(b / t)) where
  a >= b + eps, else -inf (gradient 0 there; see the module docstring)."""
  ok = a >= b + eps
  x = torch.where(ok, (a - b) / t, torch.ones_like(a))
  # log1mexp (update_utils.py:134-147): log(1 - exp(-x)) for x > 0
  v = t * torch.where(x <= np.log(2.0), torch.log(-torch.expm1(-x)), torch.log1p(-torch.exp(-x))) + a
  return torch.where(ok, v, torch.full_like(v, -float("inf")))


def _seg_max_arg(x, seg, nseg):
  """Per segment: the max of x and the LAST index attaining it (get_maxes_and_argmaxes,
  update_utils.py:25-64), the index detached. Segments without elements give (-inf, -1)."""
  B, n = x.shape
  mx = torch.full((B, nseg), -float("inf"), dtype=x.dtype, device=x.device)
  mx = mx.scatter_reduce(1, seg.expand(B, -1), x, "amax", include_self=True)
  pos = torch.arange(n, device=x.device).expand(B, -1)
  hit = torch.where(x.detach() == mx.detach()[:, seg], pos, torch.full_like(pos, -1))
  arg = torch.full((B, nseg), -1, dtype=torch.int64, device=x.device)
  arg = arg.scatter_reduce(1, seg.expand(B, -1), hit, "amax", include_self=True)
  return mx, arg


def _at_arg(arg, n):
  """[B, n] mask of the argmax positions (arg >= 0)."""
  B = arg.shape[0]
  m = torch.zeros((B, n + 1), dtype=torch.bool, device=arg.device)
  idx = torch.where(arg >= 0, arg, torch.full_like(arg, n))
  m.scatter_(1, idx, True)
  return m[:, :n]


class LogicalGraph(EnumGraph):
  """EnumGraph with OR, AND and Pool factors too: the four types of FAC_TO_VAR_UPDATES in
  registry order, each on its own slice of the messages (normalize=True, as in bp.run)."""

  def __init__(self, wiring, device="cpu"):
    super().__init__(wiring, device, all_types=True)
    t = lambda k: torch.as_tensor(np.asarray(wiring[k], dtype=np.int64).reshape(-1), device=device)
    self.logical = []
    for key, off in (("or", 1), ("and", -1)):
      if f"{key}.parents_factor_indices" in wiring:
        pfi = t(f"{key}.parents_factor_indices")
        ch = t(f"{key}.children_edge_states")
        self.logical.append((pfi, t(f"{key}.parents_msg_indices"), ch, off, int(ch.shape[0])))
      else:
        self.logical.append(None)
    if "pool.pool_choices_factor_indices" in wiring:
      ind = t("pool.pool_indicators_edge_states")
      self.pool = (t("pool.pool_choices_factor_indices"), t("pool.pool_choices_msg_indices"), ind,
                   int(ind.shape[0]))
    else:
      self.pool = None

  def logical_update(self, vtof, which, temperature):
    """pass_logical_fac_to_var_messages (logical.py:492-779), normalize=True, on the type's
    slice vtof [B, n]."""
    pfi, pmi, ch, off, F = self.logical[which]
    B, n = vtof.shape
    P = pfi.shape[0]
    t = temperature
    p_rel, p_oth = vtof[:, pmi + off], vtof[:, pmi]
    c_rel, c_oth = vtof[:, ch + off], vtof[:, ch]
    diff = p_rel - p_oth
    zf = torch.zeros((B, F), dtype=vtof.dtype, device=vtof.device)
    fs_oth = zf.index_add(1, pfi, p_oth)
    max1, arg1 = _seg_max_arg(diff, pfi, F)
    at_arg = _at_arg(arg1, P)
    wo = torch.where(at_arg, torch.full_like(diff, -float("inf")), diff)
    max2 = torch.full((B, F), -float("inf"), dtype=vtof.dtype, device=vtof.device)
    max2 = max2.scatter_reduce(1, pfi.expand(B, -1), wo, "amax", include_self=True)
    if t == 0:
      mx = torch.maximum(p_oth, p_rel)
      fs_x = zf.index_add(1, pfi, mx)
      p_msg_rel = (fs_x[:, pfi] + c_rel[:, pfi]) - mx
      ch_rel = fs_x + torch.clamp(max1, max=0.0)
      opt1 = (c_oth[:, pfi] + fs_oth[:, pfi]) - p_oth
      m12 = torch.where(at_arg, max2[:, pfi], max1[:, pfi])
      opt2 = p_msg_rel + torch.clamp(m12, max=0.0)
      p_msg_oth = torch.maximum(opt1, opt2)
    else:
      lse = _lae(p_rel, p_oth, t)
      fs_x = zf.index_add(1, pfi, lse)
      fs_lse_wo = fs_x[:, pfi] - lse
      fs_oth_wo = fs_oth[:, pfi] - p_oth
      p_msg_rel = c_rel[:, pfi] + fs_lse_wo
      opt1 = c_oth[:, pfi] + fs_oth_wo
      opt2 = c_rel[:, pfi] + fs_lse_wo
      ch_rel = _lme(fs_x, fs_oth, t, 1e-4)
      if t < STABILITY_THRE:
        ch_rel = torch.maximum(ch_rel, _lae(fs_oth + max1, fs_oth + max2, t))
      p_msg_oth = _lme(_lae(opt1, opt2, t), c_rel[:, pfi] + fs_oth_wo, t, 1e-4)
      if t < STABILITY_THRE:
        fsp = fs_oth_wo + torch.where(at_arg, max2[:, pfi], max1[:, pfi])
        p_msg_oth = torch.maximum(p_msg_oth, _lae(opt1, c_rel[:, pfi] + fsp, t))
    # single-parent factors (logical.py:739-757)
    nump = torch.bincount(pfi, minlength=F)
    single = (nump[pfi] == 1).expand(B, -1)
    p_msg_rel = torch.where(single, c_rel[:, pfi], p_msg_rel)
    p_msg_oth = torch.where(single, c_oth[:, pfi], p_msg_oth)
    out = torch.zeros_like(vtof)
    out = out.index_put((torch.arange(B, device=vtof.device)[:, None], (pmi + off)[None]),
                        p_msg_rel - p_msg_oth)
    out = out.index_put((torch.arange(B, device=vtof.device)[:, None], (ch + off)[None]),
                        ch_rel - fs_oth)
    return out

  def pool_update(self, vtof, temperature):
    """pass_pool_fac_to_var_messages (pool.py:276-474), normalize=True, on the type's slice."""
    cfi, cmi, ind, F = self.pool
    B, n = vtof.shape
    P = cfi.shape[0]
    t = temperature
    pc_diff = vtof[:, cmi + 1] - vtof[:, cmi]
    pi_diff = vtof[:, ind + 1] - vtof[:, ind]
    max1, arg1 = _seg_max_arg(pc_diff, cfi, F)
    at_arg = _at_arg(arg1, P)
    ninf = lambda x: torch.full_like(x, -float("inf"))
    if t == 0:
      wo = torch.where(at_arg, ninf(pc_diff), pc_diff)
      max2 = ninf(max1).scatter_reduce(1, cfi.expand(B, -1), wo, "amax", include_self=True)
      pc_mdiff = torch.minimum(pi_diff[:, cfi], -torch.where(at_arg, max2[:, cfi], max1[:, cfi]))
      pi_mdiff = max1
    else:
      m1 = max1.detach()
      se = torch.zeros((B, F), dtype=vtof.dtype, device=vtof.device).index_add(
          1, cfi, torch.exp((pc_diff - m1[:, cfi]) / t))
      pi_mdiff = t * torch.log(se) + m1
      fl = _lae(pi_mdiff, -pi_diff, t)
      pc_mdiff = -_lme(fl[:, cfi], pc_diff, t, 1e-30)
      wo = torch.where(at_arg, -pi_diff[:, cfi], pc_diff)
      m2 = ninf(max1).scatter_reduce(1, cfi.expand(B, -1), wo, "amax", include_self=True).detach()
      se2 = torch.zeros((B, F), dtype=vtof.dtype, device=vtof.device).index_add(
          1, cfi, torch.exp((wo - m2[:, cfi]) / t))
      am = -(t * torch.log(se2) + m2)
      pc_mdiff = torch.where(at_arg, am[:, cfi], pc_mdiff)
    # single-choice factors (pool.py:430-450)
    num = torch.bincount(cfi, minlength=F)
    single = (num[cfi] == 1).expand(B, -1)
    pc_mdiff = torch.where(single, pi_diff[:, cfi], pc_mdiff)
    out = torch.zeros_like(vtof)
    rows = torch.arange(B, device=vtof.device)[:, None]
    out = out.index_put((rows, (cmi + 1)[None]), pc_mdiff)
    out = out.index_put((rows, (ind + 1)[None]), pi_mdiff)
    return out

  def iterate(self, msgs, lp, evidence, damping, temperature):
    vsum = self.var_sums(msgs, evidence)
    vtof = vsum[:, self.vs] - msgs
    parts = []
    for ti, (a, b) in enumerate(self.msgs_ranges):
      if b <= a:
        continue
      if ti == 0:
        parts.append(self.enum_update(vtof[:, a:b], lp, temperature))
      elif ti in (1, 2):
        parts.append(self.logical_update(vtof[:, a:b], ti - 1, temperature))
      else:
        parts.append(self.pool_update(vtof[:, a:b], temperature))
    f = torch.cat(parts, dim=1)
    return self.normalize(damping * msgs + (1.0 - damping) * f)
