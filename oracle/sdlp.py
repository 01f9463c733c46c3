"""NumPy restatement of PGMax's smooth dual LP-MAP solver. TEST INFRASTRUCTURE ONLY: the checker
of pgbp_sdlp_run / pgbp_sdlp_objective, imported by tests/ and bench.py's CPU-baseline arm; the
product never imports it.

Follows pgmax/infer/dual_lp.py: smooth_dual_objval_and_grad (65-236) and the accelerated
(sub)gradient loop of run_with_objvals (238-313), with get_maxes_and_argmaxes and
softmax_and_logsumexps_with_temp of pgmax/factor/update_utils.py:26-131. The factor updates are
the C oracle's (oracle.factor_update, normalize=False). Arrays are float32 with the reference's
operation order; scatters run in index order (np.*.at). The objective's two sums are float64 here
(float32 in the reference).
"""

import numpy as np

from . import oracle

F32 = np.float32


def _maxes_argmaxes(data, labels, n):
  """update_utils.py:26-64: per-label max (from -inf) and the LAST index attaining it."""
  maxes = np.full(n, -np.inf, F32)
  np.maximum.at(maxes, labels, data)
  N = data.shape[0]
  pos = np.arange(N, dtype=np.int64) - N * (data != maxes[labels]).astype(np.int64)
  arg = np.full(n, np.iinfo(np.int32).min, np.int64)
  np.maximum.at(arg, labels, pos)
  return maxes, arg


def _softmax_lse(data, labels, n, t):
  """update_utils.py:102-131 at temperature t > 0."""
  t = F32(t)
  maxes = np.full(n, -np.inf, F32)
  np.maximum.at(maxes, labels, data)
  with np.errstate(invalid="ignore", over="ignore"):
    exp_data = (t * np.exp((data - maxes[labels]) / t)).astype(F32)
  sums = np.zeros(n, F32)
  np.add.at(sums, labels, exp_data)
  with np.errstate(divide="ignore", invalid="ignore"):
    lse = (maxes + t * np.log(sums / t)).astype(F32)
    soft = (exp_data / sums[labels]).astype(F32)
  return soft, lse


class Problem:
  """The flat wiring of one graph (oracle.Wiring layout plus evidence_to_vars)."""

  def __init__(self, wiring):
    self.w = wiring
    self.cw = oracle.Wiring(wiring)
    self.vs = np.asarray(wiring["var_states_for_edge_states"], np.int64)
    self.ei = np.asarray(wiring["edge_indices_for_edge_states"], np.int64)
    self.fi = np.asarray(wiring["factor_indices_for_edge_states"], np.int64)
    self.e2v = np.asarray(wiring["evidence_to_vars"], np.int64)
    self.nvs = int(wiring["num_var_states"])
    self.nv = int(self.e2v.max(initial=-1)) + 1
    self.ne = int(wiring["num_edges"])
    self.nf = int(self.fi.max(initial=-1)) + 1
    self.mr = np.asarray(wiring["msgs_ranges"], np.int64).reshape(4, 2)
    self.pr = np.asarray(wiring["potentials_ranges"], np.int64).reshape(4, 2)

  def objective(self, log_potentials, evidence, ftov, temperature):
    """(objval, grad, bp_updates, per-edge lse or max): dual_lp.py:65-236."""
    lp = np.asarray(log_potentials, F32)
    ev = np.asarray(evidence, F32)
    ftov = np.asarray(ftov, F32)
    var_sums = ev.copy()
    np.add.at(var_sums, self.vs, ftov)
    bp = np.zeros_like(ftov)
    for t in range(4):
      m0, m1 = self.mr[t]
      if m1 > m0:
        p0, p1 = self.pr[t]
        bp[m0:m1] = oracle.factor_update(self.cw, t, -ftov[m0:m1], lp[p0:p1], temperature,
                                         normalize=False)
    data = (bp - ftov).astype(F32)
    if temperature == 0.0:
      maxes_var, arg_var = _maxes_argmaxes(var_sums, self.e2v, self.nv)
      plus = np.zeros(self.nvs, F32)
      plus[arg_var] = 1.0
      maxes_edge, arg_edge = _maxes_argmaxes(data, self.ei, self.ne)
      minus = np.zeros(ftov.shape[0], F32)
      minus[arg_edge] = -1.0
      grad = (plus[self.vs] + minus).astype(F32)
      var_obj, edge_obj = maxes_var, maxes_edge
    else:
      soft_var, lse_var = _softmax_lse(var_sums, self.e2v, self.nv, temperature)
      soft_edge, lse_edge = _softmax_lse(data, self.ei, self.ne, temperature)
      grad = (soft_var[self.vs] - soft_edge).astype(F32)
      var_obj, edge_obj = lse_var, lse_edge
    fac = np.full(self.nf, -np.inf, F32)
    np.maximum.at(fac, self.fi, edge_obj[self.ei])
    objval = float(np.sum(var_obj, dtype=np.float64) + np.sum(fac, dtype=np.float64))
    return objval, grad, bp, edge_obj

  def run_with_objvals(self, log_potentials, evidence, ftov, temperature, num_iters, lr=None):
    """(ftov after num_iters steps, objvals [num_iters]): dual_lp.py:238-313."""
    if lr is None:
      lr = temperature if temperature != 0.0 else 0.01
    lr = F32(lr)
    ftov = np.asarray(ftov, F32).copy()
    eta = ftov.copy()
    objvals = np.zeros(num_iters, np.float64)
    for it in range(num_iters):
      objvals[it], grad, _, _ = self.objective(log_potentials, evidence, ftov, temperature)
      itf = F32(it)
      if temperature > 0:
        new_eta = (ftov - lr * grad).astype(F32)
      else:
        new_eta = (ftov - (lr / np.sqrt(itf + F32(1.0))) * grad).astype(F32)
      coef = (itf + F32(1.0)) / (itf + F32(4.0))
      ftov = (new_eta + coef * (new_eta - eta)).astype(F32)
      eta = new_eta
    return ftov, objvals
