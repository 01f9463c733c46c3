"""NumPy restatement of PGMax's compute_energy. TEST INFRASTRUCTURE ONLY: the checker of
pgbp_energy, imported by tests/ and bench.py's CPU-baseline arm; the product never imports it.

Follows pgmax/infer/energy.py:53-148 (debug_mode=False) on the flat wiring of InfererContext (the
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
