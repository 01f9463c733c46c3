"""NumPy restatement of PGMax's compute_energy. TEST INFRASTRUCTURE ONLY: the checker of
pgbp_energy, imported by tests/ and bench.py's CPU-baseline arm; the product never imports it.

Follows pgmax/infer/energy.py:53-148 (debug_mode=False) and, in compute_energy_configs /
compute_energy_terms, energy.py:151-204 (debug_mode=True) on the flat wiring of InfererContext (the
fixture layout of oracle.py), with the per-type terms of EnumFactor.compute_energy
(pgmax/factor/enum.py:276-323), LogicalFactor.compute_energy (pgmax/factor/logical.py:295-358)
and PoolFactor.compute_energy (pgmax/factor/pool.py:184-239). Sums are float64 (the reference
sums in float32); `map_flat` is one decoding, a state per variable in evidence_to_vars order.
"""

import numpy as np


def var_state_onehot(evidence_to_vars, map_flat):
  """One-hot decoding of every variable state (energy.py:104-124): state s of a K-state variable
  is decoded when map == s, a negative map taken once modulo K (JAX's index wrap); a map outside
  [0, K) decodes no state (JAX drops out-of-range scatters)."""
  e2v = np.asarray(evidence_to_vars, np.int64).reshape(-1)
  m = np.asarray(map_flat, np.int64).reshape(-1)
  nvs = e2v.shape[0]
  first = np.zeros(m.shape[0] + 1, np.int64)
  np.add.at(first, e2v + 1, 1)
  first = np.cumsum(first)
  k = (first[1:] - first[:-1])[e2v]
  local = np.arange(nvs, dtype=np.int64) - first[e2v]
  s = m[e2v]
  s = np.where(s < 0, s + k, s)
  return (s == local).astype(np.float64)


def compute_energy(wiring, log_potentials, evidence, map_flat):
  """Energy (float64) of one decoding; +inf for a decoding that a factor rules out."""
  ev = np.asarray(evidence, np.float64).reshape(-1)
  lp = np.asarray(log_potentials, np.float64).reshape(-1)
  onehot = var_state_onehot(wiring["evidence_to_vars"], map_flat)
  with np.errstate(invalid="ignore"):
    energy = -np.sum(onehot * ev)
  vs_of_es = np.asarray(wiring["var_states_for_edge_states"], np.int64)
  es_onehot = onehot[vs_of_es]
  mr = np.asarray(wiring["msgs_ranges"], np.int64).reshape(4, 2)
  pr = np.asarray(wiring["potentials_ranges"], np.int64).reshape(4, 2)
  fi = np.asarray(wiring["factor_indices_for_edge_states"], np.int64)
  i64 = lambda k: np.asarray(wiring[k], np.int64).reshape(-1)

  # EnumFactors (enum.py:306-322)
  m0, m1 = mr[0]
  if m1 > m0:
    oh = es_onehot[m0:m1]
    ncfg = int(np.asarray(wiring["enum.num_val_configs"]))
    decoded = np.ones(ncfg, dtype=bool)
    ci, ce = i64("enum.factor_configs_indices"), i64("enum.factor_configs_edge_states")
    np.logical_and.at(decoded, ci, oh[ce] != 0)
    num_factors = np.unique(fi[m0:m1]).shape[0]
    pot = lp[pr[0, 0]:pr[0, 1]]
    with np.errstate(invalid="ignore"):
      energy += np.inf if int(decoded.sum()) != num_factors else -np.sum(pot[:ncfg][decoded])

  # OR / AND factors (logical.py:343-357): all parents in the relevant state iff the child is
  for t, name in ((1, "or"), (2, "and")):
    m0, m1 = mr[t]
    if m1 <= m0:
      continue
    oh = es_onehot[m0:m1]
    ch = i64(f"{name}.children_edge_states")
    parents = np.ones(ch.shape[0])
    np.multiply.at(parents, i64(f"{name}.parents_factor_indices"),
                   oh[i64(f"{name}.parents_msg_indices")])
    energy += np.inf if np.any(parents != oh[ch]) else 0.0

  # Pool factors (pool.py:219-238): choices in state 1 must number the indicator's state 1
  m0, m1 = mr[3]
  if m1 > m0:
    oh = es_onehot[m0:m1]
    ind = i64("pool.pool_indicators_edge_states")
    on = np.zeros(ind.shape[0])
    np.add.at(on, i64("pool.pool_choices_factor_indices"),
              oh[i64("pool.pool_choices_msg_indices") + 1])
    energy += np.inf if np.any(on != oh[ind + 1]) else 0.0
  return float(energy)


def compute_energy_configs(wiring, evidence, map_flat):
  """What pgbp_energy_terms returns for one decoding (compute_energy's debug mode,
  pgmax/infer/energy.py:151-204, before the factors' own potentials are read): (variable terms
  [num_variables] float64 holding float32 values, factor configs [num_factors] int64).

  A variable's term is -evidence of its decoded state (a negative state wrapped once), NaN when
  the state is outside [0, K). An EnumFactor's config is the index, among the factor's configs,
  of the decoded one, the last of equal configs as the reference's dict keeps it, -1 when none is
  decoded (enum.py:326-360); an OR / AND (logical.py:378-406) or Pool (pool.py:242-272) factor's
  is 0 if the decoding satisfies it, else -1. Factors are numbered as in the flat wiring."""
  ev = np.asarray(evidence, np.float32).reshape(-1)
  e2v = np.asarray(wiring["evidence_to_vars"], np.int64).reshape(-1)
  m = np.asarray(map_flat, np.int64).reshape(-1)
  nv = m.shape[0]
  first = np.zeros(nv + 1, np.int64)
  np.add.at(first, e2v + 1, 1)
  first = np.cumsum(first)
  k = first[1:] - first[:-1]
  s = np.where(m < 0, m + k, m)
  ok = (s >= 0) & (s < k)
  var_terms = np.full(nv, np.nan)
  var_terms[ok] = -ev[first[:-1][ok] + s[ok]]
  onehot = var_state_onehot(wiring["evidence_to_vars"], map_flat)
  vs_of_es = np.asarray(wiring["var_states_for_edge_states"], np.int64)
  es_onehot = onehot[vs_of_es]
  mr = np.asarray(wiring["msgs_ranges"], np.int64).reshape(4, 2)
  fi = np.asarray(wiring["factor_indices_for_edge_states"], np.int64)
  nf = int(fi.max()) + 1 if fi.size else 0
  fac_cfg = np.zeros(nf, np.int64)
  i64 = lambda key: np.asarray(wiring[key], np.int64).reshape(-1)
  m0, m1 = mr[0]
  if m1 > m0:
    oh = es_onehot[m0:m1]
    ncfg = int(np.asarray(wiring["enum.num_val_configs"]))
    ci, ce = i64("enum.factor_configs_indices"), i64("enum.factor_configs_edge_states")
    decoded = np.ones(ncfg, dtype=bool)
    np.logical_and.at(decoded, ci, oh[ce] != 0)
    cfg_factor = np.full(ncfg, -1, np.int64)
    cfg_factor[ci] = fi[m0 + ce]
    first_cfg = np.full(nf, ncfg, np.int64)
    np.minimum.at(first_cfg, cfg_factor, np.arange(ncfg))
    fac_cfg[np.unique(fi[m0:m1])] = -1
    for c in np.nonzero(decoded)[0]:   # in config order: the last decoded config wins
      fac_cfg[cfg_factor[c]] = c - first_cfg[cfg_factor[c]]
  for t, name in ((1, "or"), (2, "and")):
    m0, m1 = mr[t]
    if m1 <= m0:
      continue
    oh = es_onehot[m0:m1]
    ch = i64(f"{name}.children_edge_states")
    parents = np.ones(ch.shape[0])
    np.multiply.at(parents, i64(f"{name}.parents_factor_indices"),
                   oh[i64(f"{name}.parents_msg_indices")])
    fac_cfg[fi[m0 + ch]] = np.where(parents != oh[ch], -1, 0)
  m0, m1 = mr[3]
  if m1 > m0:
    oh = es_onehot[m0:m1]
    ind = i64("pool.pool_indicators_edge_states")
    on = np.zeros(ind.shape[0])
    np.add.at(on, i64("pool.pool_choices_factor_indices"),
              oh[i64("pool.pool_choices_msg_indices") + 1])
    fac_cfg[fi[m0 + ind]] = np.where(on != oh[ind + 1], -1, 0)
  return var_terms, fac_cfg


def compute_energy_terms(wiring, factor_potentials, evidence, map_flat):
  """compute_energy's debug mode: (variable terms, factor terms), float64. factor_potentials
  holds the Enum factors' own potentials, concatenated in factor order (the flat wiring's Enum
  config order), in their own precision, as the reference's factor objects keep them."""
  var_terms, fac_cfg = compute_energy_configs(wiring, evidence, map_flat)
  pot = np.asarray(factor_potentials, np.float64).reshape(-1)
  mr = np.asarray(wiring["msgs_ranges"], np.int64).reshape(4, 2)
  fi = np.asarray(wiring["factor_indices_for_edge_states"], np.int64)
  fac_terms = np.where(fac_cfg < 0, np.inf, 0.0)
  m0, m1 = mr[0]
  if m1 > m0:
    ci = np.asarray(wiring["enum.factor_configs_indices"], np.int64).reshape(-1)
    ce = np.asarray(wiring["enum.factor_configs_edge_states"], np.int64).reshape(-1)
    ncfg = int(np.asarray(wiring["enum.num_val_configs"]))
    cfg_factor = np.full(ncfg, -1, np.int64)
    cfg_factor[ci] = fi[m0 + ce]
    first_cfg = np.full(fac_cfg.shape[0], ncfg, np.int64)
    np.minimum.at(first_cfg, cfg_factor, np.arange(ncfg))
    for f in np.unique(fi[m0:m1]):
      if fac_cfg[f] >= 0:
        fac_terms[f] = -pot[first_cfg[f] + fac_cfg[f]]
  return var_terms, fac_terms


def compute_energy_batch(wiring, log_potentials, evidence, maps):
  """[B] energies; log_potentials / evidence are [B, n] or [n] (shared), maps [B, num_variables]."""
  maps = np.asarray(maps)
  lp = np.asarray(log_potentials)
  ev = np.asarray(evidence)
  out = np.empty(maps.shape[0], np.float64)
  for b in range(maps.shape[0]):
    out[b] = compute_energy(wiring, lp[b] if lp.ndim == 2 else lp, ev[b] if ev.ndim == 2 else ev,
                            maps[b])
  return out
