"""GPU parity of pgbp_energy (compute_energy on the device) through the C ABI and the host API.

Against the reference: every recorded compute_energy call (tests/golden/fixtures/energy_*.npz,
from the reference's tests and the seeded cases). Against the oracle (oracle/energy.py, pinned to
those fixtures by test_energy_oracle.py): batches of random, repaired and BP decodings with batched
and shared evidence / potentials. Infinite and nan energies must match exactly; finite ones within
2e-6 of the sum of |evidence| and |log potentials| (the kernel sums in double, the reference in
float32).
"""

import types

import numpy as np
import pytest

import cases
import fixtures
from oracle import energy as oracle_energy
from test_energy_oracle import assert_energy_close, scale_of

pytestmark = pytest.mark.gpu

ENERGIES = fixtures.energy_fixture_paths()


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


def _plan(wiring):
  from pgmax_gb300 import engine  # pylint: disable=g-import-not-at-top
  w = dict(wiring)
  w["num_variables"] = int(np.max(w["evidence_to_vars"], initial=-1)) + 1
  return engine.Plan(w)


def _api():
  from pgmax_gb300 import factor, fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  return types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer,
                               vgroup=vgroup)


@pytest.mark.parametrize("path", ENERGIES, ids=fixtures.fixture_id)
def test_energy_matches_reference(path):
  fx = fixtures.load(path)
  plan = _plan(fx["wiring"])
  got = float(plan.energy(fx["log_potentials"], fx["evidence"], fx["map_flat"]).cpu())
  scale = scale_of(fx)
  assert_energy_close(got, float(fx["energy"]), scale)
  want = oracle_energy.compute_energy(fx["wiring"], fx["log_potentials"], fx["evidence"],
                                      fx["map_flat"])
  assert_energy_close(got, want, scale)


def _case_wiring(builder, **kw):
  api = _api()
  fg, groups, ev = cases.BUILDERS[builder](api, **kw)
  ctx = api.infer.InfererContext(fg.bp_state)
  w = ctx.flat_wiring()
  return fg, groups, ev, w


def _decodings(w, rng, B):
  nstates = np.bincount(np.asarray(w["evidence_to_vars"], np.int64))
  maps = []
  for b in range(B):
    m = (rng.random(nstates.shape[0]) * nstates).astype(np.int32)
    maps.append(cases.repair_decoding(w, m) if b % 2 else m)
  maps = np.stack(maps)
  maps[B - 1, 0] = nstates[0]        # out of range: no state of variable 0 decoded
  maps[B - 2, ::5] -= nstates[::5]   # negative states wrap once
  return maps


@pytest.mark.parametrize("builder,kw", [
    ("mixed", dict(seed=0, vardict=False)),
    ("mixed", dict(seed=3)),
    ("deconv", dict(seed=1)),
    ("rbm", dict(nh=20, nv=30, seed=2, sample=0)),
    ("potts", dict(L=7, K=5, seed=4)),
    ("ising", dict(n=9, seed=5)),
])
@pytest.mark.parametrize("batched_arrays", [False, True])
def test_batched_energies_match_oracle(builder, kw, batched_arrays):
  torch = _torch()
  _, _, _, w = _case_wiring(builder, **kw)
  plan = _plan(w)
  rng = np.random.default_rng(17)
  B = 37
  maps = _decodings(w, rng, B)
  nvs = int(w["num_var_states"])
  npot = int(np.asarray(w["potentials_ranges"])[:, 1].max())
  if batched_arrays:
    ev = rng.normal(size=(B, nvs)).astype(np.float32)
    lp = rng.normal(size=(B, npot)).astype(np.float32)
  else:
    ev = rng.normal(size=(nvs,)).astype(np.float32)
    lp = rng.normal(size=(npot,)).astype(np.float32)
  got = plan.energy(torch.as_tensor(lp), torch.as_tensor(ev), torch.as_tensor(maps)).cpu().numpy()
  want = oracle_energy.compute_energy_batch(w, lp, ev, maps)
  assert got.shape == (B,)
  finite = 0
  for b in range(B):
    scale = np.abs(ev[b] if batched_arrays else ev).sum() + np.abs(
        lp[b] if batched_arrays else lp).sum()
    assert_energy_close(float(got[b]), float(want[b]), scale)
    finite += bool(np.isfinite(want[b]))
  assert finite > 0


def test_one_decoding_for_every_instance_and_determinism():
  torch = _torch()
  _, _, _, w = _case_wiring("mixed", seed=1, vardict=False)
  plan = _plan(w)
  rng = np.random.default_rng(3)
  m = cases.repair_decoding(w, _decodings(w, rng, 4)[1])
  nvs = int(w["num_var_states"])
  npot = int(np.asarray(w["potentials_ranges"])[:, 1].max())
  ev = rng.normal(size=(9, nvs)).astype(np.float32)
  lp = rng.normal(size=(npot,)).astype(np.float32)
  got = plan.energy(torch.as_tensor(lp), torch.as_tensor(ev), torch.as_tensor(m))
  again = plan.energy(torch.as_tensor(lp), torch.as_tensor(ev), torch.as_tensor(m))
  assert got.shape == (9,)
  assert torch.equal(got, again)
  for b in range(9):
    want = oracle_energy.compute_energy(w, lp, ev[b], m)
    assert_energy_close(float(got[b]), want, np.abs(ev[b]).sum() + np.abs(lp).sum())


def test_large_batch_is_deterministic():
  """Batches of 16 or more score the dense pairwise terms with the instances on the lanes:
  repeated calls give the same bits, and every instance matches its single-instance call."""
  torch = _torch()
  _, _, _, w = _case_wiring("rbm", nh=20, nv=30, seed=6, sample=0)
  plan = _plan(w)
  rng = np.random.default_rng(8)
  maps = _decodings(w, rng, 45)
  nvs = int(w["num_var_states"])
  npot = int(np.asarray(w["potentials_ranges"])[:, 1].max())
  ev = rng.normal(size=(nvs,)).astype(np.float32)
  lp = rng.normal(size=(npot,)).astype(np.float32)
  got = plan.energy(torch.as_tensor(lp), torch.as_tensor(ev), torch.as_tensor(maps))
  assert torch.equal(got, plan.energy(torch.as_tensor(lp), torch.as_tensor(ev),
                                      torch.as_tensor(maps)))
  for b in (0, 31, 32, 44):
    one = plan.energy(torch.as_tensor(lp), torch.as_tensor(ev), torch.as_tensor(maps[b:b + 1]))
    assert_energy_close(float(got[b]), float(one[0]), np.abs(ev).sum() + np.abs(lp).sum())


def test_shared_tables_and_implicit_rows_match_explicit_plan():
  """A K = 16 grid with one shared table and implied rows against the same grid with per-factor
  tables and explicit rows (the potentials expanded), for the same decodings."""
  torch = _torch()
  from pgmax_gb300 import batch  # pylint: disable=g-import-not-at-top
  L, K = 12, 16
  wc = batch.grid_wiring(L, K, shared_table=True, implicit_rows=True)
  we = batch.grid_wiring(L, K)
  pc, pe = _plan(wc), _plan(we)
  rng = np.random.default_rng(5)
  F = 2 * L * (L - 1)
  table = rng.normal(size=(K * K,)).astype(np.float32)
  lp_full = np.tile(table, F)
  ev = rng.normal(size=(L * L * K,)).astype(np.float32)
  maps = rng.integers(0, K, size=(16, L * L)).astype(np.int32)
  maps[3, 7] = K + 2
  a = pc.energy(torch.as_tensor(table), torch.as_tensor(ev), torch.as_tensor(maps)).cpu().numpy()
  b = pe.energy(torch.as_tensor(lp_full), torch.as_tensor(ev), torch.as_tensor(maps)).cpu().numpy()
  assert np.array_equal(a, b)
  want = oracle_energy.compute_energy_batch(we, lp_full, ev, maps)
  for k in range(16):
    assert_energy_close(float(a[k]), float(want[k]), np.abs(ev).sum() + np.abs(lp_full).sum())
  assert np.isinf(a[3])


# ------------------------------------------------------------------ drop-in host API
# The scenarios of the reference's tests/test_energy.py, on pgmax_gb300's API.

def test_energy_empty_vgroup():
  api = _api()
  variables = api.vgroup.NDVarArray(num_states=2, shape=(2, 2))
  variables_empty = api.vgroup.NDVarArray(num_states=2, shape=(0, 2))
  fg = api.fgraph.FactorGraph(variable_groups=[variables, variables_empty])
  fg.add_factors(api.fgroup.EnumFactorGroup(
      variables_for_factors=[[variables[0, 0], variables[0, 1]]],
      factor_configs=np.zeros((1, 2), int)))
  bp = api.infer.build_inferer(fg.bp_state, backend="bp")
  bp_arrays = bp.init()
  map_states = api.infer.decode_map_states(bp.get_beliefs(bp_arrays))
  energy, v, f = api.infer.compute_energy(fg.bp_state, bp_arrays, map_states)
  assert float(energy) == 0 and v is None and f is None


def test_energy_single_state():
  api = _api()
  variables = api.vgroup.NDVarArray(num_states=2, shape=(2, 2))
  single = api.vgroup.NDVarArray(num_states=1, shape=(1, 2))
  fg = api.fgraph.FactorGraph(variable_groups=[variables, single])
  fg.add_factors(api.fgroup.EnumFactorGroup(
      variables_for_factors=[[variables[0, 0], variables[0, 1]]],
      factor_configs=np.zeros((1, 2), int)))
  bp = api.infer.build_inferer(fg.bp_state, backend="bp")
  bp_arrays = bp.init()
  map_states = api.infer.decode_map_states(bp.get_beliefs(bp_arrays))
  assert float(api.infer.compute_energy(fg.bp_state, bp_arrays, map_states)[0]) == 0


@pytest.mark.parametrize("table,want", [
    (np.array([[-np.inf, -np.inf], [-np.inf, 0.0]]), 0.0),
    (np.array([[-np.inf, -np.inf], [-np.inf, -np.inf]]), np.inf),
])
def test_energy_infinite_log_potentials(table, want):
  api = _api()
  variables = api.vgroup.NDVarArray(num_states=2, shape=(2,))
  fg = api.fgraph.FactorGraph(variable_groups=[variables])
  fg.add_factors(api.fgroup.PairwiseFactorGroup(variables_for_factors=[[variables[0],
                                                                        variables[1]]],
                                                log_potential_matrix=table))
  bp = api.infer.build_inferer(fg.bp_state, backend="bp")
  bp_arrays = bp.run(bp.init(), num_iters=1, temperature=0)
  map_states = api.infer.decode_map_states(bp.get_beliefs(bp_arrays))
  if np.isfinite(want):
    assert np.array_equal(np.asarray(map_states[variables].cpu()), [1, 1])
  assert float(api.infer.compute_energy(fg.bp_state, bp_arrays, map_states)[0]) == want


def test_host_api_batched_decodings_match_oracle():
  """Perturb-and-MAP style: a batch of evidence samples runs, decodes and is scored in one call
  per step; every energy matches the oracle on the same flat arrays."""
  torch = _torch()
  api = _api()
  fg, groups, ev, w = _case_wiring("rbm", nh=12, nv=18, seed=1, sample=0)
  hidden, visible = groups
  bp = api.infer.BP(fg.bp_state, temperature=0.0)
  rng = np.random.default_rng(8)
  B = 24
  base = bp.init(evidence_updates=ev)
  ev_b = base.evidence.unsqueeze(0) + torch.as_tensor(
      rng.gumbel(size=(B, base.evidence.shape[0])).astype(np.float32), device=base.evidence.device)
  arrays = api.infer.BPArrays(log_potentials=base.log_potentials, ftov_msgs=base.ftov_msgs,
                              evidence=ev_b)
  out = bp.run(arrays, num_iters=30, damping=0.5)
  map_states = api.infer.decode_map_states(bp.get_beliefs(out))
  energy, _, _ = api.infer.compute_energy(fg.bp_state, out, map_states)
  assert tuple(energy.shape) == (B,)
  flat = torch.cat([map_states[hidden].reshape(B, -1), map_states[visible].reshape(B, -1)],
                   dim=1).cpu().numpy()
  want = oracle_energy.compute_energy_batch(w, out.log_potentials.cpu().numpy(),
                                            out.evidence.cpu().numpy(), flat)
  scale = float(np.abs(out.evidence.cpu().numpy()).sum(1).max() +
                np.abs(out.log_potentials.cpu().numpy()).sum())
  for b in range(B):
    assert_energy_close(float(energy[b]), float(want[b]), scale)


def test_host_api_or_factors_score_like_their_enum_form():
  """The energy check of the reference's tests/factor/test_or.py: an ORFactor graph and the same
  constraint as an EnumFactor give equal energies for the same decoding."""
  import itertools  # pylint: disable=g-import-not-at-top
  api = _api()
  rng = np.random.default_rng(2)
  n = 4
  energies = []
  parents = rng.integers(0, 2, size=n)
  ev = rng.normal(size=(n + 1, 2)).astype(np.float32)
  for form in ("or", "enum"):
    v = api.vgroup.NDVarArray(num_states=2, shape=(n + 1,))
    fg = api.fgraph.FactorGraph(variable_groups=[v])
    vars_ = [v[i] for i in range(n + 1)]
    if form == "or":
      fg.add_factors(api.fgroup.ORFactorGroup([vars_]))
    else:
      configs = np.array([list(c) + [int(any(c))] for c in itertools.product((0, 1), repeat=n)])
      fg.add_factors(api.fgroup.EnumFactorGroup(variables_for_factors=[vars_],
                                                factor_configs=configs))
    bp = api.infer.BP(fg.bp_state)
    arrays = bp.init(evidence_updates={v: ev})
    for child in (int(parents.any()), 1 - int(parents.any())):
      states = np.concatenate([parents, [child]]).astype(np.int32)
      energies.append(float(api.infer.compute_energy(fg.bp_state, arrays, {v: states})[0]))
  # [or valid, or invalid, enum valid, enum invalid]
  assert np.isfinite(energies[0]) and np.isinf(energies[1])
  assert np.isinf(energies[3])
  assert abs(energies[0] - energies[2]) <= 1e-5


DEBUG = [p for p in ENERGIES if "debug_energy" in np.load(p).files]


def _bits_equal(got, want):
  got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
  return got.shape == want.shape and np.array_equal(got, want, equal_nan=True)


@pytest.mark.parametrize("path", DEBUG, ids=fixtures.fixture_id)
def test_energy_terms_match_reference_debug_mode(path):
  """pgbp_energy_terms against the reference's debug mode (energy.py:151-204): the variable
  terms bit for bit, the decoded configs as the oracle finds them (pinned to the same fixtures),
  and the factor terms and total they give with the factors' own potentials."""
  fx = fixtures.load(path)
  plan = _plan(fx["wiring"])
  var_e, fac_c = plan.energy_terms(fx["evidence"], fx["map_flat"])
  var_e, fac_c = var_e.cpu().numpy(), fac_c.cpu().numpy()
  assert _bits_equal(var_e, fx["debug_var_terms"])
  _, want_cfg = oracle_energy.compute_energy_configs(fx["wiring"], fx["evidence"], fx["map_flat"])
  np.testing.assert_array_equal(fac_c, want_cfg)
  _, fac_t = oracle_energy.compute_energy_terms(fx["wiring"], fx["debug_factor_potentials"],
                                                fx["evidence"], fx["map_flat"])
  assert _bits_equal(fac_t, fx["debug_fac_terms"])


@pytest.mark.parametrize("builder,kw", [
    ("mixed", dict(seed=0, vardict=False)),
    ("mixed", dict(seed=3)),
    ("deconv", dict(seed=1)),
    ("potts", dict(L=7, K=5, seed=4)),
])
def test_energy_terms_batched_match_oracle(builder, kw):
  """Batches of random, repaired, negative and out-of-range decodings: every instance's terms
  and configs as the oracle's."""
  torch = _torch()
  _, _, _, w = _case_wiring(builder, **kw)
  plan = _plan(w)
  rng = np.random.default_rng(23)
  B = 21
  maps = _decodings(w, rng, B)
  ev = rng.normal(size=(B, int(w["num_var_states"]))).astype(np.float32)
  var_e, fac_c = plan.energy_terms(torch.as_tensor(ev), torch.as_tensor(maps))
  var_e, fac_c = var_e.cpu().numpy(), fac_c.cpu().numpy()
  for b in range(B):
    want_v, want_c = oracle_energy.compute_energy_configs(w, ev[b], maps[b])
    assert _bits_equal(var_e[b], want_v)
    np.testing.assert_array_equal(fac_c[b], want_c)


@pytest.mark.parametrize("builder,kw", [
    ("mixed", dict(seed=1, vardict=False)),
    ("mixed", dict(seed=2)),
    ("rbm", dict(nh=12, nv=18, seed=3, sample=0)),
])
def test_compute_energy_debug_mode_through_the_api(builder, kw):
  """infer.compute_energy(debug_mode=True) returns the reference's structure: the total as a
  float summed over the variables then the factors, each variable's term keyed by the variable,
  each factor's keyed by the frozenset of its variables, with the factors' own potentials."""
  api = _api()
  fg, groups, ev = cases.BUILDERS[builder](api, **kw)
  bp = api.infer.BP(fg.bp_state, temperature=0.0)
  arrays = bp.run(bp.init(evidence_updates=ev), num_iters=15)
  decoded = api.infer.decode_map_states(bp.get_beliefs(arrays))
  total, var_en, fac_en = api.infer.compute_energy(fg.bp_state, arrays, decoded, debug_mode=True)
  assert isinstance(total, float)
  w = bp.context.flat_wiring()
  from pgmax_gb300.infer import energy as energy_mod  # pylint: disable=g-import-not-at-top
  live = [vg for vg in fg.bp_state.fg_state.variable_groups
          if int(np.prod(vg.num_states.shape)) > 0]
  m = energy_mod._flat_states(live, decoded, "cpu").numpy()  # pylint: disable=protected-access
  ev_flat = np.asarray(arrays.evidence.cpu() if hasattr(arrays.evidence, "cpu") else
                       arrays.evidence, np.float32)
  pots = [np.asarray(f.log_potentials, np.float64).reshape(-1)
          for g in fg.bp_state.fg_state.factor_group_to_potentials_starts
          if g.factor_type is api.factor.EnumFactor for f in g.factors]
  pots = np.concatenate(pots) if pots else np.zeros(0)
  want_v, want_f = oracle_energy.compute_energy_terms(w, pots, ev_flat, m)
  variables = [v for vg in live for v in vg.variables]
  assert list(var_en) == variables
  assert _bits_equal([var_en[v] for v in variables], want_v)
  factors = [f for g in fg.bp_state.fg_state.factor_group_to_potentials_starts for f in g.factors]
  assert len(fac_en) == len({frozenset(f.variables) for f in factors})
  got_f = [fac_en[frozenset(f.variables)] for f in factors]
  assert _bits_equal(got_f, want_f)
  want_total = 0.0
  for x in list(want_v) + list(want_f):
    want_total += float(x)
  assert total == want_total or (np.isnan(total) and np.isnan(want_total))
  # and the non-debug energy agrees with the total
  e = float(api.infer.compute_energy(fg.bp_state, arrays, decoded)[0].cpu())
  if np.isfinite(want_total):
    assert abs(e - want_total) <= 2e-6 * (np.abs(want_v).sum() + np.abs(want_f).sum()) + 1e-6
  else:
    assert e == want_total
