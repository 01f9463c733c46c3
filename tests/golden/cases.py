"""Seeded factor-graph builders shared by the golden-fixture generator and the tests.

Every builder takes `api`, a namespace with the modules `vgroup`, `fgroup`, `factor` and `fgraph`
(either PGMax's or `pgmax_gb300`'s, which expose the same classes), and returns
`(fg, variable_groups, evidence_updates)`. Because both libraries are driven by the same code and
the same seeds, the flat wiring they compile must be identical; the tests check exactly that.

The graphs follow the constructions in the reference's examples and tests:
  * `ising`: toroidal grid, right/down pairwise factors with 0.8*[[1,-1],[-1,1]]
    (tests/test_examples.py:24-47);
  * `rbm`: hidden/visible unary EnumFactorGroups + a PairwiseFactorGroup with [[0,0],[0,W_ij]]
    (benchmark/rbm_lib.py:135-171);
  * `potts`: open 4-neighbour grid with a shared J*I_K table (examples/grid_mrf.ipynb, cell 9);
  * `deconv`: AND(S, W -> SW) and OR(SW -> X) (examples/pmp_binary_deconvolution.ipynb, cell 14);
  * `mixed`: Enum, OR, AND and Pool factors in one graph over variables of 2, 3 and 4 states.
"""

import collections
import itertools

import numpy as np


def ising(api, n=50, seed=0, coupling=0.8):
  variables = api.vgroup.NDVarArray(num_states=2, shape=(n, n))
  fg = api.fgraph.FactorGraph(variable_groups=variables)
  variables_for_factors = []
  for ii in range(n):
    for jj in range(n):
      kk = (ii + 1) % n
      ll = (jj + 1) % n
      variables_for_factors.append([variables[ii, jj], variables[kk, jj]])
      variables_for_factors.append([variables[ii, jj], variables[ii, ll]])
  fg.add_factors(
      api.fgroup.PairwiseFactorGroup(
          variables_for_factors=variables_for_factors,
          log_potential_matrix=coupling * np.array([[1.0, -1.0], [-1.0, 1.0]]),
      )
  )
  rng = np.random.default_rng(seed)
  evidence = rng.gumbel(size=(n, n, 2)).astype(np.float32)
  return fg, [variables], {variables: evidence}


def rbm_params(nh, nv, seed=0, w_std=0.1, b_std=0.5):
  rng = np.random.default_rng(seed)
  W = rng.normal(0.0, w_std, size=(nh, nv)).astype(np.float32)
  bh = rng.normal(0.0, b_std, size=(nh,)).astype(np.float32)
  bv = rng.normal(0.0, b_std, size=(nv,)).astype(np.float32)
  return W, bh, bv


def rbm(api, nh=20, nv=30, seed=0, sample=0):
  """One perturb-and-MAP sample: evidence is fresh Gumbel noise on every unary state."""
  W, bh, bv = rbm_params(nh, nv, seed)
  hidden = api.vgroup.NDVarArray(num_states=2, shape=bh.shape)
  visible = api.vgroup.NDVarArray(num_states=2, shape=bv.shape)
  fg = api.fgraph.FactorGraph(variable_groups=[hidden, visible])
  hidden_unaries = api.fgroup.EnumFactorGroup(
      variables_for_factors=[[hidden[ii]] for ii in range(nh)],
      factor_configs=np.arange(2)[:, None],
      log_potentials=np.stack([np.zeros_like(bh), bh], axis=1),
  )
  visible_unaries = api.fgroup.EnumFactorGroup(
      variables_for_factors=[[visible[jj]] for jj in range(nv)],
      factor_configs=np.arange(2)[:, None],
      log_potentials=np.stack([np.zeros_like(bv), bv], axis=1),
  )
  log_potential_matrix = np.zeros(W.shape + (2, 2), dtype=np.float32).reshape((-1, 2, 2))
  log_potential_matrix[:, 1, 1] = W.ravel()
  pairwise = api.fgroup.PairwiseFactorGroup(
      variables_for_factors=[[hidden[ii], visible[jj]] for ii in range(nh) for jj in range(nv)],
      log_potential_matrix=log_potential_matrix,
  )
  fg.add_factors([hidden_unaries, visible_unaries, pairwise])
  rng = np.random.default_rng(seed * 1000003 + 17 + sample)
  ev_h = rng.gumbel(size=(nh, 2)).astype(np.float32)
  ev_v = rng.gumbel(size=(nv, 2)).astype(np.float32)
  return fg, [hidden, visible], {hidden: ev_h, visible: ev_v}


def potts(api, L=8, K=4, seed=0):
  rng = np.random.default_rng(seed)
  J = rng.uniform(0.0, 1.5)
  grid = api.vgroup.NDVarArray(num_states=K, shape=(L, L))
  fg = api.fgraph.FactorGraph(variable_groups=grid)
  top_down = [[grid[ii, jj], grid[ii + 1, jj]] for ii in range(L - 1) for jj in range(L)]
  left_right = [[grid[ii, jj], grid[ii, jj + 1]] for ii in range(L) for jj in range(L - 1)]
  table = (J * np.eye(K)).astype(np.float32)
  fg.add_factors(api.fgroup.PairwiseFactorGroup(variables_for_factors=top_down,
                                                log_potential_matrix=table))
  fg.add_factors(api.fgroup.PairwiseFactorGroup(variables_for_factors=left_right,
                                                log_potential_matrix=table))
  evidence = rng.normal(size=(L, L, K)).astype(np.float32)
  return fg, [grid], {grid: evidence}


def _logit(p):
  return np.log(p) - np.log1p(-p)


def deconv(api, n_feat=2, feat=3, im=6, seed=0, flip=0.05):
  """Binary deconvolution: X = OR over features of AND(S, W) (one image, one channel)."""
  rng = np.random.default_rng(seed)
  s_size = im - feat + 1
  W = api.vgroup.NDVarArray(num_states=2, shape=(1, n_feat, feat, feat))
  S = api.vgroup.NDVarArray(num_states=2, shape=(1, n_feat, s_size, s_size))
  SW = api.vgroup.NDVarArray(num_states=2, shape=(1, 1, im, im, n_feat, feat, feat))
  X = api.vgroup.NDVarArray(num_states=2, shape=(1, 1, im, im))
  fg = api.fgraph.FactorGraph(variable_groups=[S, W, SW, X])
  and_vars = []
  or_dict = collections.OrderedDict()
  for sh in range(s_size):
    for sw in range(s_size):
      for f in range(n_feat):
        for fh in range(feat):
          for fw in range(feat):
            sw_var = SW[0, 0, fh + sh, fw + sw, f, fh, fw]
            and_vars.append([S[0, f, sh, sw], W[0, f, fh, fw], sw_var])
            or_dict.setdefault(X[0, 0, fh + sh, fw + sw], []).append(sw_var)
  fg.add_factors(api.fgroup.ANDFactorGroup(and_vars))
  fg.add_factors(api.fgroup.ORFactorGroup([list(v) + [x] for x, v in or_dict.items()]))
  w_true = rng.random((1, n_feat, feat, feat)) < 0.25
  s_true = rng.random((1, n_feat, s_size, s_size)) < 0.1
  x_true = np.zeros((im, im), dtype=bool)
  for f in range(n_feat):
    for sh in range(s_size):
      for sw in range(s_size):
        if s_true[0, f, sh, sw]:
          x_true[sh:sh + feat, sw:sw + feat] |= w_true[0, f]
  x_obs = x_true ^ (rng.random((im, im)) < flip)
  uW = np.zeros(W.shape + (2,), dtype=np.float32)
  uW[..., 1] = _logit(0.25)
  uS = np.zeros(S.shape + (2,), dtype=np.float32)
  uS[..., 1] = _logit(0.02)
  uX = np.zeros(X.shape + (2,), dtype=np.float32)
  uX[0, 0, ..., 1] = np.where(x_obs, 4.0, -4.0)
  ev = {
      S: uS + rng.gumbel(size=uS.shape).astype(np.float32) * 0.1,
      W: uW + rng.gumbel(size=uW.shape).astype(np.float32) * 0.1,
      X: uX,
  }
  return fg, [S, W, SW, X], ev


def mixed(api, seed=0, vardict=True):
  """Enum (pairwise + ternary tables), OR, AND and Pool factors sharing variables. With
  vardict=False the five 3-state variables are an NDVarArray instead of a VarDict (the reference's
  compute_energy takes NDVarArrays only); the graph and the random draws are otherwise the same."""
  rng = np.random.RandomState(seed)
  nb = 24
  binary = api.vgroup.NDVarArray(num_states=2, shape=(nb,))
  ns = np.array([3, 4, 2, 3, 4, 3], dtype=np.int64)
  multi = api.vgroup.NDVarArray(num_states=ns, shape=(len(ns),))
  names = tuple(f"d{i}" for i in range(5))
  if vardict:
    vdict = api.vgroup.VarDict(variable_names=names, num_states=3)
    third = lambda i: vdict[names[i]]
  else:
    vdict = api.vgroup.NDVarArray(num_states=3, shape=(len(names),))
    third = lambda i: vdict[i]
  fg = api.fgraph.FactorGraph(variable_groups=[binary, multi, vdict])

  # Pairwise EnumFactors with per-factor tables between multi-state variables.
  pairs = [[multi[i], multi[(i + 1) % len(ns)]] for i in range(len(ns))]
  for v1, v2 in pairs:
    table = rng.normal(size=(v1[1], v2[1]))
    fg.add_factors(api.fgroup.PairwiseFactorGroup(variables_for_factors=[[v1, v2]],
                                                  log_potential_matrix=table))
  # A ternary EnumFactorGroup over the VarDict with a sparse config table.
  configs = np.array([c for c in itertools.product(range(3), repeat=3) if sum(c) % 2 == 0])
  fg.add_factors(
      api.fgroup.EnumFactorGroup(
          variables_for_factors=[[third(i), third(i + 1), third(i + 2)] for i in range(3)],
          factor_configs=configs,
          log_potentials=rng.normal(size=(3, configs.shape[0])),
      )
  )
  # Single EnumFactor linking a binary variable and a VarDict variable.
  fg.add_factors(
      api.factor.EnumFactor(
          variables=[binary[0], third(4)],
          factor_configs=np.array([[0, 0], [1, 1], [1, 2]]),
          log_potentials=rng.normal(size=(3,)),
      )
  )
  # OR, AND and Pool factors over the binary variables.
  fg.add_factors(api.fgroup.ORFactorGroup([[binary[1], binary[2], binary[3]],
                                           [binary[4], binary[5]],
                                           [binary[6], binary[7], binary[8], binary[9], binary[10]]]))
  fg.add_factors(api.fgroup.ANDFactorGroup([[binary[11], binary[12], binary[13]],
                                            [binary[2], binary[14]]]))
  fg.add_factors(api.factor.ANDFactor(variables=[binary[5], binary[9], binary[15]]))
  fg.add_factors(api.fgroup.PoolFactorGroup([[binary[16], binary[17], binary[18], binary[19]],
                                             [binary[20], binary[21]]]))
  fg.add_factors(api.factor.PoolFactor(variables=[binary[3], binary[12], binary[22], binary[23]]))
  ev = {
      binary: rng.gumbel(size=(nb, 2)),
      multi: np.where(np.arange(4)[None] < ns[:, None], rng.gumbel(size=(len(ns), 4)), 0.0),
  }
  for i in range(len(names)):
    ev[third(i)] = rng.gumbel(size=(3,))
  return fg, [binary, multi, vdict], ev


def mixed_ftov_updates(api, variable_groups, seed=0):
  """Per-variable initial messages, spread over every edge of the variable."""
  rng = np.random.RandomState(seed + 101)
  updates = {}
  for vg in variable_groups:
    for var in vg.variables:
      updates[var] = rng.normal(size=(int(var[1]),))
  return updates


def repair_decoding(w, m):
  """Sets OR / AND children and Pool indicators (and surplus Pool choices) so that a decoding
  satisfies every logical and Pool factor of the flat wiring `w`."""
  m = np.array(m, dtype=np.int64)
  e2v = np.asarray(w["evidence_to_vars"], np.int64)
  vs_of_es = np.asarray(w["var_states_for_edge_states"], np.int64)
  mr = np.asarray(w["msgs_ranges"], np.int64)
  var = lambda es: int(e2v[vs_of_es[es]])
  for _ in range(32):
    changed = False
    for t, name, r in ((1, "or", 0), (2, "and", 1)):
      m0 = mr[t][0]
      if mr[t][1] <= m0:
        continue
      pfi = np.asarray(w[f"{name}.parents_factor_indices"])
      pmi = np.asarray(w[f"{name}.parents_msg_indices"])
      ch = np.asarray(w[f"{name}.children_edge_states"])
      for f in range(ch.shape[0]):
        all_r = all(m[var(m0 + e)] == r for e in pmi[pfi == f])
        c = var(m0 + ch[f])
        want = r if all_r else 1 - r
        if m[c] != want:
          m[c], changed = want, True
    m0 = mr[3][0]
    if mr[3][1] > m0:
      cfi = np.asarray(w["pool.pool_choices_factor_indices"])
      cmi = np.asarray(w["pool.pool_choices_msg_indices"])
      ind = np.asarray(w["pool.pool_indicators_edge_states"])
      for f in range(ind.shape[0]):
        on = [var(m0 + e) for e in cmi[cfi == f] if m[var(m0 + e)] == 1]
        for v in on[1:]:
          m[v], changed = 0, True
        i = var(m0 + ind[f])
        want = 1 if on else 0
        if m[i] != want:
          m[i], changed = want, True
    if not changed:
      break
  return m.astype(np.int32)


BUILDERS = {
    "ising": ising,
    "rbm": rbm,
    "potts": potts,
    "deconv": deconv,
    "mixed": mixed,
}
