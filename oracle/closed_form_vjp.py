"""Closed-form VJPs of one OR / AND or Pool factor update. TEST INFRASTRUCTURE ONLY.

The derivations that the adjoint's logical kernels (and, for Pool, the next one) implement,
restated per factor in float64 Python. tests/test_adjoint_oracle.py checks them against torch
autograd through oracle/bp_torch.LogicalGraph, which is pinned to the reference's fixtures.
Updates are those of bp.run (normalize=True) at temperature t > 0:
  OR / AND  pgmax/factor/logical.py:645-779
  Pool      pgmax/factor/pool.py:390-460
  helpers   pgmax/factor/update_utils.py:67-190 (logaddexp, logminusexp, log1mexp)
At logminusexp's eps cutoff (which returns the constant -inf) the gradient is 0; through a
maximum it follows the selected branch or the element attaining it (the last one on ties).
"""

import math

STABILITY_THRE = 0.5


def lae(a, b, t):
  """t log(exp(a / t) + exp(b / t))."""
  mx, mn = max(a, b), min(a, b)
  if mx == -math.inf:
    return -math.inf
  return t * math.log1p(math.exp((mn - mx) / t)) + mx


def d_lae(a, b, t):
  l = lae(a, b, t)
  return math.exp((a - l) / t), math.exp((b - l) / t)


def lme(a, b, t, eps):
  """t log(exp(a / t) - exp(b / t)) where a >= b + eps, else -inf."""
  if not a >= b + eps:
    return -math.inf
  x = (a - b) / t
  return t * (math.log(-math.expm1(-x)) if x <= math.log(2.0) else math.log1p(-math.exp(-x))) + a


def d_lme(a, b, t, eps):
  if not a >= b + eps:
    return 0.0, 0.0
  e = math.exp((b - a) / t)
  return 1.0 / (1.0 - e), -e / (1.0 - e)


def logical_factor_vjp(r, o, cr, co, g, gc, t):
  """One OR / AND factor. r[i], o[i]: parent i's variable-to-factor messages of the relevant and
  other state; cr, co: the child's. g[i]: dL/d(parent i's relevant output), gc: dL/d(child's
  relevant output) (the other outputs are the constant 0). Returns (dr, do, dcr, dco)."""
  n = len(r)
  low = t < STABILITY_THRE
  d = [r[i] - o[i] for i in range(n)]
  fo = sum(o)
  l = [lae(r[i], o[i], t) for i in range(n)]
  fx = sum(l)
  max1 = max(d)
  a = max(i for i in range(n) if d[i] == max1)
  wo = [-math.inf if i == a else d[i] for i in range(n)]
  max2 = max(wo)
  a2 = max((i for i in range(n) if i != a and wo[i] == max2), default=-1)
  dr, do = [0.0] * n, [0.0] * n
  dcr = dco = dfx = dmax1 = dmax2 = 0.0
  dfo = -gc  # child output = ch_rel - fo
  dch = gc
  if low:
    xa, xb = fo + max1, fo + max2
    if lae(xa, xb, t) > lme(fx, fo, t, 1e-4):
      sa, sb = d_lae(xa, xb, t)
      dfo += dch * (sa + sb)
      dmax1 += dch * sa
      dmax2 += dch * sb
      dch = 0.0
  if dch != 0.0:
    pa, pb = d_lme(fx, fo, t, 1e-4)
    dfx += dch * pa
    dfo += dch * pb
  da, dO = [0.0] * n, [0.0] * n
  for i in range(n):
    if n == 1:  # single-parent rule: outputs (c_rel, c_oth)
      dcr += g[i]
      dco -= g[i]
      continue
    dpo = -g[i]
    A, O = fx - l[i], fo - o[i]
    o1, o2, o3 = co + O, cr + A, cr + O
    q = lae(o1, o2, t)
    if low:
      M = max2 if i == a else max1
      lbx = cr + O + M
      if lae(o1, lbx, t) > lme(q, o3, t, 1e-4):
        s1, s2 = d_lae(o1, lbx, t)
        dco += dpo * s1
        dO[i] += dpo * (s1 + s2)
        dcr += dpo * s2
        if i == a:
          dmax2 += dpo * s2
        else:
          dmax1 += dpo * s2
        dpo = 0.0
    if dpo != 0.0:
      pq, p3 = d_lme(q, o3, t, 1e-4)
      s1, s2 = d_lae(o1, o2, t)
      dq = dpo * pq
      dco += dq * s1
      dO[i] += dq * s1 + dpo * p3
      dcr += dq * s2 + dpo * p3
      da[i] += dq * s2
    dcr += g[i]  # relevant output = c_rel + A
    da[i] += g[i]
    dfx += da[i]
    dfo += dO[i]
  for i in range(n):
    dl = dfx - da[i]
    sr, so = d_lae(r[i], o[i], t)
    dr[i] += dl * sr
    do[i] += dl * so + dfo - dO[i]
  dr[a] += dmax1
  do[a] -= dmax1
  if a2 >= 0:
    dr[a2] += dmax2
    do[a2] -= dmax2
  return dr, do, dcr, dco


def pool_factor_vjp(r, z, ir, iz, g, gi, t):
  """One Pool factor. r[i], z[i]: choice i's variable-to-factor messages of states 1 and 0; ir,
  iz: the indicator's. g[i]: dL/d(choice i's state-1 output), gi: dL/d(indicator's state-1
  output). Returns (dr, dz, dir, diz)."""
  n = len(r)
  pcd = [r[i] - z[i] for i in range(n)]
  pid = ir - iz
  max1 = max(pcd)
  a = max(i for i in range(n) if pcd[i] == max1)
  s = sum(math.exp((x - max1) / t) for x in pcd)
  pim = t * math.log(s) + max1
  dpcd = [0.0] * n
  dpid = 0.0
  dpim = gi
  if n == 1:  # single-choice rule: the choice's output is the indicator difference
    dpid += g[0]
  else:
    fl = lae(pim, -pid, t)
    dfl = 0.0
    for i in range(n):
      if i == a:
        continue
      pa, pb = d_lme(fl, pcd[i], t, 1e-30)
      dfl -= g[i] * pa
      dpcd[i] -= g[i] * pb
    # argmax choice: -t log sum exp(wo / t), wo = pcd with the argmax replaced by -pid
    wo = [(-pid if i == a else pcd[i]) for i in range(n)]
    m2 = max(wo)
    lse = t * math.log(sum(math.exp((x - m2) / t) for x in wo)) + m2
    for j in range(n):
      w = -g[a] * math.exp((wo[j] - lse) / t)
      if j == a:
        dpid -= w
      else:
        dpcd[j] += w
    s1, s2 = d_lae(pim, -pid, t)
    dpim += dfl * s1
    dpid -= dfl * s2
  for j in range(n):  # pim = t log sum exp(pcd / t)
    dpcd[j] += dpim * math.exp((pcd[j] - pim) / t)
  dr = list(dpcd)
  dz = [-x for x in dpcd]
  return dr, dz, dpid, -dpid
