"""Regenerates the golden fixtures in tests/golden/fixtures/ from the reference PGMax code itself.

Run from the repository root:  python tests/golden/make_golden.py [--reference PATH]

The reference (google-deepmind/PGMax 0.6.1, pure Python over JAX) is imported unmodified from its
source tree, with `jax_shim` standing in for jax/numba (neither is installed here). Every call to
`BP(...).run / run_with_diffs / run_bp` made while this script runs is intercepted and saved with
the flat wiring that `InfererContext` compiled (pgmax/infer/inferer.py:65-118), the input BPArrays,
the run parameters and the reference's outputs (messages, per-iteration deltas, flat beliefs and
the MAP decode). Two sources of runs are captured:
  1. the reference's own tests (tests/test_pgmax.py, tests/test_clipping.py,
     tests/factor/test_{or,and,pool}.py, tests/fgraph/test_fgraph.py), executed as-is; the
     84-message golden vector of tests/test_pgmax.py:63-152 is captured from its `jnp.allclose`;
  2. the seeded graphs of `cases.py` (Ising 50x50 at 1000 iterations, small RBM, Potts,
     deconvolution, a mixed Enum/OR/AND/Pool graph), which the tests rebuild with pgmax_gb300 to
     check that the host-side wiring is identical.
It also records single factor-update calls (`FAC_TO_VAR_UPDATES[type](...)`, normalize True and
False, several temperatures) on the mixed graph, and every `infer.compute_energy` call
(pgmax/infer/energy.py:53-148, debug_mode=False) made by the reference's energy, OR, AND and Pool
tests and by `energy_cases` (BP decodings, random decodings, random decodings repaired to satisfy
the OR / AND / Pool factors, out-of-range and negative states, infinite evidence) as
`energy_*.npz`: the flat wiring, the BPArrays' log potentials and evidence, the decoding (a state
per variable, evidence_to_vars order) and the reference's energy.

The smooth dual LP-MAP solver (`infer.SDLP`, pgmax/infer/dual_lp.py) is recorded the same way as
`sdlp_*.npz`: every `run_with_objvals` / `run` (inputs, output messages, objective values),
`get_bp_updates` (factor updates and per-edge log-sum-exp) and `get_primal_upper_bound` call of the
reference's tests/lp/test_bp_for_lp.py and of `sdlp_cases` (the seeded graphs of cases.py with
cold and random initial messages, temperatures 0 to 1, default and explicit learning rates).

`get_marginals` (pgmax/infer/bp.py:263-288) is recorded as `marginals_*.npz`: for seeded graphs
of cases.py (including the mixed graph, whose variables of 2, 3 and 4 states make the unflattened
beliefs padded with -inf), the run's output messages, the flat and unflattened beliefs and the
reference's marginals leaf by leaf; and `marginals_direct.npz`: get_marginals called on hand-made
belief arrays (-inf states, a variable whose states are all -inf, large magnitudes, an empty
array).

`--energy-only` / `--sdlp-only` / `--marginals-only` regenerate those fixtures alone and leave the
others untouched. `--reference` names the PGMax source tree (or set PGMAX_REFERENCE).
"""

import argparse
import importlib
import json
import os
import sys
import traceback
import types
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "fixtures")
TYPE_NAMES = ("enum", "or", "and", "pool")


def _np(x, dtype=None):
  a = np.asarray(x)
  return a.astype(dtype) if dtype is not None else a


def wiring_arrays(ctx, fg_state):
  """Flat wiring exactly as the reference's InfererContext holds it."""
  from pgmax.factor import FAC_TO_VAR_UPDATES  # pylint: disable=g-import-not-at-top
  d = {
      "var_states_for_edge_states": _np(ctx.var_states_for_edge_states, np.int32),
      "edge_indices_for_edge_states": _np(ctx.edge_indices_for_edge_states, np.int32),
      "factor_indices_for_edge_states": _np(ctx.factor_indices_for_edge_states, np.int32),
      "num_edges": np.int64(ctx.num_edges),
      "num_factors": np.int64(ctx.num_factors),
      "num_var_states": np.int64(fg_state.num_var_states),
      "evidence_to_vars": _np(fg_state.evidence_to_vars, np.int32),
  }
  msgs_ranges, pot_ranges = [], []
  for ftype, name in zip(FAC_TO_VAR_UPDATES, TYPE_NAMES):
    msgs_ranges.append(ctx.factor_type_to_msgs_range[ftype])
    pot_ranges.append(ctx.factor_type_to_potentials_range[ftype])
    args = ctx.inference_arguments[ftype]
    for k, v in args.items():
      if isinstance(v, (int, np.integer)):
        d[f"{name}.{k}"] = np.int64(v)
      else:
        d[f"{name}.{k}"] = _np(v, np.int32)
  d["msgs_ranges"] = np.array(msgs_ranges, dtype=np.int64).reshape(4, 2)
  d["potentials_ranges"] = np.array(pot_ranges, dtype=np.int64).reshape(4, 2)
  return d


class Recorder:

  def __init__(self):
    self.runs = []
    self.energies = []
    self.sdlp = []
    self.allclose_args = []
    self.current = "unnamed"
    self.meta = {}


REC = Recorder()


def install_capture(pgmax):
  """Wraps pgmax.infer.BP so that every run is recorded."""
  bp_mod = importlib.import_module("pgmax.infer.bp")
  inferer_mod = importlib.import_module("pgmax.infer.inferer")
  orig_bp = bp_mod.BP

  def BP(bp_state, temperature=0.0):  # pylint: disable=invalid-name
    bp = orig_bp(bp_state, temperature)
    ctx = inferer_mod.InfererContext(bp_state)
    wiring = wiring_arrays(ctx, bp_state.fg_state)
    groups = bp_state.fg_state.variable_groups

    def run_with_diffs(bp_arrays, num_iters, damping=0.5, temperature=temperature):
      out, deltas = bp.run_with_diffs(bp_arrays, num_iters, damping, temperature)
      flat_beliefs = np.asarray(
          importlib.import_module("jax").numpy.array(bp_arrays.evidence)
          .at[ctx.var_states_for_edge_states].add(out.ftov_msgs), dtype=np.float32)
      beliefs = bp.get_beliefs(out)
      decoded = inferer_mod.decode_map_states(beliefs)
      map_flat = []
      for vg in groups:
        m = decoded[vg]
        if isinstance(m, dict):
          map_flat += [int(np.asarray(m[n]).reshape(-1)[0]) for n in vg.variable_names]
        else:
          map_flat += list(np.asarray(m).reshape(-1).astype(np.int64))
      REC.runs.append({
          "source": REC.current,
          "meta": dict(REC.meta),
          "wiring": wiring,
          "log_potentials": _np(bp_arrays.log_potentials, np.float32),
          "evidence": _np(bp_arrays.evidence, np.float32),
          "ftov_msgs_in": _np(bp_arrays.ftov_msgs, np.float32),
          "num_iters": np.int64(num_iters),
          "damping": np.float64(damping),
          "temperature": np.float64(temperature),
          "ftov_msgs_out": _np(out.ftov_msgs, np.float32),
          "deltas": _np(deltas, np.float32),
          "flat_beliefs": flat_beliefs,
          "map_flat": np.array(map_flat, dtype=np.int32),
      })
      return out, deltas

    def run(bp_arrays, num_iters, damping=0.5, temperature=temperature):
      return run_with_diffs(bp_arrays, num_iters, damping, temperature)[0]

    def run_bp(bp_arrays, num_iters, damping=0.5):
      return run(bp_arrays, num_iters, damping, temperature)

    return bp_mod.BeliefPropagation(
        init=bp.init, update=bp.update, to_bp_state=bp.to_bp_state,
        get_beliefs=bp.get_beliefs, run=run, run_bp=run_bp, run_with_diffs=run_with_diffs)

  bp_mod.BP = BP
  infer_pkg = importlib.import_module("pgmax.infer")
  infer_pkg.BP = BP

  jnp = importlib.import_module("jax.numpy")
  orig_allclose = jnp.allclose

  def allclose(a, b, *args, **kwargs):
    REC.allclose_args.append((REC.current, np.asarray(a), np.asarray(b), kwargs))
    return orig_allclose(a, b, *args, **kwargs)

  jnp.allclose = allclose


def flat_map(groups, map_states):
  """A decoding dict {VarGroup: states} as one state per variable, variable-group order."""
  out = []
  for vg in groups:
    m = map_states[vg]
    if isinstance(m, dict):
      out += [int(np.asarray(m[n]).reshape(-1)[0]) for n in vg.variable_names]
    else:
      out += list(np.asarray(m).reshape(-1).astype(np.int64))
  return np.array(out, dtype=np.int32)


def unflat_map(groups, flat):
  """Inverse of flat_map for NDVarArray groups."""
  out, k = {}, 0
  for vg in groups:
    n = int(np.prod(vg.shape))
    out[vg] = np.asarray(flat[k:k + n], dtype=np.int32).reshape(vg.shape)
    k += n
  return out


def install_energy_capture():
  """Wraps pgmax.infer.compute_energy so that every non-debug call is recorded."""
  energy_mod = importlib.import_module("pgmax.infer.energy")
  inferer_mod = importlib.import_module("pgmax.infer.inferer")
  factor_mod = importlib.import_module("pgmax.factor")
  orig = energy_mod.compute_energy

  def compute_energy(bp_state, bp_arrays, map_states, debug_mode=False):
    res = orig(bp_state, bp_arrays, map_states, debug_mode)
    if not debug_mode:
      ctx = inferer_mod.InfererContext(bp_state)
      rec = {
          "source": REC.current,
          "meta": dict(REC.meta),
          "wiring": wiring_arrays(ctx, bp_state.fg_state),
          "log_potentials": _np(bp_arrays.log_potentials, np.float32),
          "evidence": _np(bp_arrays.evidence, np.float32),
          "map_flat": flat_map(bp_state.fg_state.variable_groups, map_states),
          "energy": np.float32(np.asarray(res[0])),
      }
      # the same decoding in debug mode (energy.py:151-204), when every state is in [0, K): the
      # terms in variable order and in factor order, and the total as the reference sums it
      nstates = np.bincount(np.asarray(rec["wiring"]["evidence_to_vars"], np.int64))
      m = rec["map_flat"]
      debug = None
      if m.shape[0] == nstates.shape[0] and np.all((m >= 0) & (m < nstates)):
        try:
          with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            debug = orig(bp_state, bp_arrays, map_states, True)
        except AttributeError:
          # the reference's debug mode reads factor_configs, which a SingleFactorGroup (a factor
          # added on its own) and the logical groups lack: such graphs get no debug record
          debug = None
      if debug is not None:
        total, var_e, fac_e = debug
        fg_state = bp_state.fg_state
        rec["debug_var_terms"] = np.array(
            [var_e[v] for vg in fg_state.variable_groups for v in vg.variables], np.float64)
        rec["debug_fac_terms"] = np.array(
            [fac_e[frozenset(f.variables)] for g in fg_state.factor_group_to_potentials_starts
             for f in g.factors], np.float64)
        rec["debug_energy"] = np.float64(total)
        # the potentials debug mode reads: the Enum factor objects' own, in their own precision,
        # concatenated in factor order (the flat wiring's Enum config order)
        enum_pots = [np.asarray(f.log_potentials, np.float64).reshape(-1)
                     for g in fg_state.factor_group_to_potentials_starts
                     if g.factor_type is factor_mod.EnumFactor for f in g.factors]
        rec["debug_factor_potentials"] = (np.concatenate(enum_pots) if enum_pots
                                          else np.zeros(0, np.float64))
      REC.energies.append(rec)
    return res

  energy_mod.compute_energy = compute_energy
  importlib.import_module("pgmax.infer").compute_energy = compute_energy


def energy_cases(api):
  """compute_energy on the seeded graphs of cases.py for several kinds of decodings."""
  sys.path.insert(0, HERE)
  import cases  # pylint: disable=g-import-not-at-top
  inferer_mod = importlib.import_module("pgmax.infer.inferer")
  plans = [
      ("ising12", "ising", dict(n=12, seed=3), dict(num_iters=50, temperature=0.0)),
      ("rbm", "rbm", dict(nh=20, nv=30, seed=0, sample=0), dict(num_iters=30, temperature=0.0)),
      ("potts_K4", "potts", dict(L=6, K=4, seed=1), dict(num_iters=20, temperature=0.0)),
      ("deconv", "deconv", dict(seed=0), dict(num_iters=40, temperature=0.0)),
      ("mixed0", "mixed", dict(seed=0, vardict=False), dict(num_iters=7, temperature=0.0)),
      ("mixed1", "mixed", dict(seed=1, vardict=False), dict(num_iters=7, temperature=1.0)),
  ]
  for name, builder, bkw, rkw in plans:
    fg, groups, ev = cases.BUILDERS[builder](api, **bkw)
    bp = api.infer.BP(fg.bp_state, temperature=rkw["temperature"])
    bp_arrays = bp.run(bp.init(evidence_updates=ev), num_iters=rkw["num_iters"])
    decoded = api.infer.decode_map_states(bp.get_beliefs(bp_arrays))
    flat = flat_map(groups, decoded)
    w = wiring_arrays(inferer_mod.InfererContext(fg.bp_state), fg.bp_state.fg_state)
    nstates = np.bincount(np.asarray(w["evidence_to_vars"], np.int64))
    rng = np.random.default_rng(len(name) * 1000 + bkw.get("seed", 0))
    decodings = [("decode", flat)]
    for k in range(3):
      rand = (rng.random(flat.shape[0]) * nstates).astype(np.int32)
      decodings.append((f"random{k}", rand))
      decodings.append((f"repaired{k}", cases.repair_decoding(w, rand)))
    bad = flat.copy()
    bad[flat.shape[0] // 2] = nstates[flat.shape[0] // 2]
    decodings.append(("out_of_range", bad))
    neg = cases.repair_decoding(w, flat)
    neg[::7] -= nstates[::7]
    decodings.append(("negative", neg))
    for kind, m in decodings:
      REC.current = f"energy_case::{name}::{kind}"
      REC.meta = {"case": name, "builder": builder, "builder_kwargs": bkw, "kind": kind}
      api.infer.compute_energy(fg.bp_state, bp_arrays, unflat_map(groups, m))
    # infinite evidence on a state that the decoding does not pick: 0 * inf is nan
    g0 = groups[0]
    ev_inf = np.zeros(tuple(g0.shape) + (int(np.max(g0.num_states)),), np.float32)
    ev_inf[(0,) * len(g0.shape) + (1,)] = -np.inf
    arrays_inf = bp.update(bp_arrays=bp_arrays, evidence_updates={g0: ev_inf})
    m = flat.copy()
    m[0] = 0
    REC.current = f"energy_case::{name}::evidence_inf"
    REC.meta = {"case": name, "builder": builder, "builder_kwargs": bkw, "kind": "evidence_inf"}
    api.infer.compute_energy(fg.bp_state, arrays_inf, unflat_map(groups, m))


def save_energies():
  counts = {}
  for rec in REC.energies:
    src = rec["source"].replace("::", "__").replace(".", "_")
    counts[src] = counts.get(src, 0) + 1
    arrays = {"w." + k: v for k, v in rec["wiring"].items()}
    for k in ("log_potentials", "evidence", "map_flat", "energy", "debug_var_terms",
              "debug_fac_terms", "debug_energy", "debug_factor_potentials"):
      if k in rec:
        arrays[k] = rec[k]
    arrays["meta"] = np.array(json.dumps({"source": rec["source"], **rec["meta"]}))
    np.savez_compressed(os.path.join(OUT, f"energy_{src}_{counts[src]:02d}.npz"), **arrays)
  return len(REC.energies)


def install_sdlp_capture():
  """Wraps pgmax.infer.SDLP so that the solver calls of every SDLP object are recorded."""
  dual_mod = importlib.import_module("pgmax.infer.dual_lp")
  inferer_mod = importlib.import_module("pgmax.infer.inferer")
  infer_pkg = importlib.import_module("pgmax.infer")
  orig = dual_mod.SDLP

  def SDLP(bp_state):  # pylint: disable=invalid-name
    sd = orig(bp_state)
    wiring = wiring_arrays(inferer_mod.InfererContext(bp_state), bp_state.fg_state)

    def arrays_of(a):
      return {"log_potentials": _np(a.log_potentials, np.float32),
              "evidence": _np(a.evidence, np.float32),
              "ftov_msgs_in": _np(a.ftov_msgs, np.float32)}

    def record(kind, a, extra):
      REC.sdlp.append({"source": REC.current, "meta": dict(REC.meta, call=kind),
                       "wiring": wiring, **arrays_of(a), **extra})

    def run_with_objvals(sdlp_arrays, logsumexp_temp, num_iters, lr=None):
      out, objvals = sd.run_with_objvals(sdlp_arrays, logsumexp_temp, num_iters, lr)
      record("run_with_objvals", sdlp_arrays, {
          "logsumexp_temp": np.float64(logsumexp_temp), "num_iters": np.int64(num_iters),
          "lr": np.float64(-1.0 if lr is None else lr),
          "ftov_msgs_out": _np(out.ftov_msgs, np.float32),
          "objvals": _np(objvals, np.float32).reshape(-1)})
      return out, objvals

    def run(sdlp_arrays, logsumexp_temp, num_iters, lr=None):
      return run_with_objvals(sdlp_arrays, logsumexp_temp, num_iters, lr)[0]

    def get_bp_updates(sdlp_arrays, logsumexp_temp):
      upd, lse = sd.get_bp_updates(sdlp_arrays, logsumexp_temp)
      record("get_bp_updates", sdlp_arrays, {
          "logsumexp_temp": np.float64(logsumexp_temp), "bp_updates": _np(upd, np.float32),
          "edge_lse": _np(lse, np.float32)})
      return upd, lse

    def get_primal_upper_bound(sdlp_arrays):
      ub = sd.get_primal_upper_bound(sdlp_arrays)
      record("get_primal_upper_bound", sdlp_arrays, {
          "logsumexp_temp": np.float64(0.0), "objval": np.float32(np.asarray(ub))})
      return ub

    return dual_mod.SmoothDualLP(
        init=sd.init, update=sd.update, to_bp_state=sd.to_bp_state, get_beliefs=sd.get_beliefs,
        run=run, run_with_objvals=run_with_objvals, decode_primal_unaries=sd.decode_primal_unaries,
        get_primal_upper_bound=get_primal_upper_bound, get_map_lower_bound=sd.get_map_lower_bound,
        get_bp_updates=get_bp_updates)

  dual_mod.SDLP = SDLP
  infer_pkg.SDLP = SDLP


def sdlp_cases(api):
  """SDLP on the seeded graphs of cases.py."""
  sys.path.insert(0, HERE)
  import cases  # pylint: disable=g-import-not-at-top
  bp_state_mod = importlib.import_module("pgmax.infer.bp_state")
  jnp = importlib.import_module("jax.numpy")
  plans = [
      ("ising6", "ising", dict(n=6, seed=2)),
      ("potts_K3", "potts", dict(L=5, K=3, seed=4)),
      ("rbm", "rbm", dict(nh=8, nv=12, seed=1, sample=0)),
      ("deconv", "deconv", dict(seed=0)),
      ("mixed", "mixed", dict(seed=0)),
  ]
  runs = [(0.0, 1, None), (0.0, 60, None), (0.0, 40, 0.05), (1e-3, 60, None), (0.05, 40, None),
          (0.05, 40, 0.01), (0.3, 25, 0.1), (1.0, 30, None)]
  for name, builder, bkw in plans:
    fg, _, ev = cases.BUILDERS[builder](api, **bkw)
    sdlp = api.infer.build_inferer(fg.bp_state, backend="sdlp")
    cold = sdlp.init(evidence_updates=ev)
    rng = np.random.default_rng(len(name))
    warm = bp_state_mod.BPArrays(
        log_potentials=cold.log_potentials,
        ftov_msgs=jnp.asarray(rng.normal(size=cold.ftov_msgs.shape).astype(np.float32)),
        evidence=cold.evidence)
    for init_name, arrays in (("cold", cold), ("random", warm)):
      REC.meta = {"case": name, "builder": builder, "builder_kwargs": bkw, "init": init_name}
      for temp, iters, lr in runs:
        REC.current = f"sdlp_case::{name}::{init_name}::T{temp}_n{iters}"
        out = sdlp.run(arrays, logsumexp_temp=temp, num_iters=iters, lr=lr)
      REC.current = f"sdlp_case::{name}::{init_name}::bounds"
      sdlp.get_primal_upper_bound(out)
      for temp in (0.0, 1e-3, 0.2, 1.0):
        REC.current = f"sdlp_case::{name}::{init_name}::updates_T{temp}"
        sdlp.get_bp_updates(out, logsumexp_temp=temp)


def save_sdlp():
  counts = {}
  for rec in REC.sdlp:
    src = rec["source"].replace("::", "__").replace(".", "_")
    counts[src] = counts.get(src, 0) + 1
    arrays = {"w." + k: v for k, v in rec["wiring"].items()}
    for k, v in rec.items():
      if k not in ("source", "meta", "wiring"):
        arrays[k] = v
    arrays["meta"] = np.array(json.dumps({"source": rec["source"], **rec["meta"]}))
    np.savez_compressed(os.path.join(OUT, f"sdlp_{src}_{counts[src]:02d}.npz"), **arrays)
  return len(REC.sdlp)


def _leaves(tree, prefix=()):
  """(key path, array) of the leaves of a beliefs / marginals dict."""
  out = []
  for k, v in tree.items():
    if isinstance(v, dict):
      out += _leaves(v, prefix + (k,))
    else:
      out.append((prefix + (k,), np.asarray(v)))
  return out


def marginals_cases(api):
  """get_marginals of the beliefs of seeded runs, and of hand-made belief arrays."""
  sys.path.insert(0, HERE)
  import cases  # pylint: disable=g-import-not-at-top
  inferer_mod = importlib.import_module("pgmax.infer.inferer")
  bp_mod = importlib.import_module("pgmax.infer.bp")
  plans = [
      ("ising12_T1", "ising", dict(n=12, seed=3), dict(num_iters=50, damping=0.5, temperature=1.0)),
      ("rbm_T0", "rbm", dict(nh=20, nv=30, seed=0, sample=0), dict(num_iters=40, damping=0.5, temperature=0.0)),
      ("potts_K4", "potts", dict(L=8, K=4, seed=1), dict(num_iters=30, damping=0.5, temperature=1.0)),
      ("potts_K16", "potts", dict(L=4, K=16, seed=3), dict(num_iters=20, damping=0.5, temperature=0.5)),
      ("deconv_T1", "deconv", dict(seed=0), dict(num_iters=40, damping=0.5, temperature=1.0)),
      ("mixed_T0", "mixed", dict(seed=0), dict(num_iters=7, damping=0.5, temperature=0.0)),
      ("mixed_T1", "mixed", dict(seed=1), dict(num_iters=9, damping=0.5, temperature=1.0)),
      ("mixed_T0.3", "mixed", dict(seed=2), dict(num_iters=9, damping=0.3, temperature=0.3)),
  ]
  n = 0
  for name, builder, bkw, rkw in plans:
    fg, groups, ev = cases.BUILDERS[builder](api, **bkw)
    bp = api.infer.BP(fg.bp_state, temperature=rkw["temperature"])
    arrays = bp.init(evidence_updates=ev)
    out = bp.run(arrays, num_iters=rkw["num_iters"], damping=rkw["damping"],
                 temperature=rkw["temperature"])
    ctx = inferer_mod.InfererContext(fg.bp_state)
    beliefs = bp.get_beliefs(out)
    marg = bp_mod.get_marginals(beliefs)
    keyed = lambda t: {groups.index(g): v for g, v in t.items()}
    bl = sorted(_leaves(keyed(beliefs)), key=lambda x: str(x[0]))
    md = dict(_leaves(keyed(marg)))
    ml = [(path, md[path]) for path, _ in bl]
    rec = {"w." + k: v for k, v in wiring_arrays(ctx, fg.bp_state.fg_state).items()}
    rec["evidence"] = _np(out.evidence, np.float32)
    rec["ftov_msgs"] = _np(out.ftov_msgs, np.float32)
    rec["log_potentials"] = _np(out.log_potentials, np.float32)
    rec["flat_beliefs"] = np.asarray(
        importlib.import_module("jax").numpy.array(out.evidence)
        .at[ctx.var_states_for_edge_states].add(out.ftov_msgs), dtype=np.float32)
    for k, ((path, b), (_, m)) in enumerate(zip(bl, ml)):
      rec[f"leaf{k}.beliefs"] = b.astype(np.float32)
      rec[f"leaf{k}.marginals"] = m.astype(np.float32)
    rec["num_leaves"] = np.int64(len(bl))
    rec["meta"] = np.array(json.dumps({
        "source": "get_marginals", "case": name, "builder": builder, "builder_kwargs": bkw,
        "run_kwargs": rkw, "leaf_paths": [[p[0]] + [str(x) for x in p[1:]] for p, _ in bl]}))
    np.savez_compressed(os.path.join(OUT, f"marginals_{name}.npz"), **rec)
    n += 1
  # hand-made beliefs: -inf states (probability 0), a variable with every state -inf (nan, as
  # exp(-inf - logsumexp) is), magnitudes of 1e4, a row of equal values, an empty array
  rng = np.random.default_rng(4)
  a = (rng.normal(size=(6, 5)) * 3).astype(np.float32)
  a[0, 1] = -np.inf
  a[1, :3] = -np.inf
  a[2, :] = -np.inf
  a[3, :] = 7.0
  b = (rng.normal(size=(4, 3, 2)) * 1e4).astype(np.float32)
  c = np.zeros((0, 4), np.float32)
  d = rng.normal(size=(7, 64)).astype(np.float32)
  direct = {"in0": a, "in1": b, "in2": c, "in3": d}
  res = bp_mod.get_marginals({k: importlib.import_module("jax").numpy.array(v)
                              for k, v in direct.items()})
  rec = dict(direct)
  for k in direct:
    rec["out" + k[2:]] = np.asarray(res[k], dtype=np.float32)
  rec["meta"] = np.array(json.dumps({"source": "get_marginals", "case": "direct"}))
  np.savez_compressed(os.path.join(OUT, "marginals_direct.npz"), **rec)
  return n + 1


def save_run(path, run, extra=None):
  arrays = {}
  for k, v in run["wiring"].items():
    arrays["w." + k] = v
  for k in ("log_potentials", "evidence", "ftov_msgs_in", "num_iters", "damping", "temperature",
            "ftov_msgs_out", "deltas", "flat_beliefs", "map_flat"):
    arrays[k] = run[k]
  meta = {"source": run["source"], **run["meta"]}
  arrays["meta"] = np.array(json.dumps(meta))
  if extra:
    arrays.update(extra)
  np.savez_compressed(path, **arrays)


def run_reference_tests(ref, modules=None):
  """Runs selected reference test functions unmodified; returns {name: error or None}."""
  status = {}
  modules = modules or {
      "test_pgmax": ["test_e2e_sanity_check", "test_e2e_heretic"],
      "test_clipping": None,
      "factor.test_or": None,
      "factor.test_and": None,
      "factor.test_pool": None,
      "fgraph.test_fgraph": ["test_bp_state", "test_bp", "test_bp_different_num_states"],
  }
  for mod_name, fns in modules.items():
    mod = importlib.import_module("tests." + mod_name)
    names = fns or [n for n in dir(mod) if n.startswith("test_")]
    for n in names:
      if not hasattr(mod, n):
        continue
      REC.current = f"{mod_name}::{n}"
      REC.meta = {}
      try:
        getattr(mod, n)()
        status[REC.current] = None
      except Exception as e:  # pylint: disable=broad-except
        status[REC.current] = f"{type(e).__name__}: {e}"[:300]
        traceback.print_exc()
  return status


def run_cases(api):
  sys.path.insert(0, HERE)
  import cases  # pylint: disable=g-import-not-at-top
  plans = [
      ("ising50_T1", "ising", dict(n=50, seed=0), dict(num_iters=1000, damping=0.5, temperature=1.0)),
      ("ising50_T0", "ising", dict(n=50, seed=0), dict(num_iters=1000, damping=0.5, temperature=0.0)),
      ("ising12_T1", "ising", dict(n=12, seed=3), dict(num_iters=50, damping=0.5, temperature=1.0)),
      ("rbm_s0", "rbm", dict(nh=20, nv=30, seed=0, sample=0), dict(num_iters=100, damping=0.5, temperature=0.0)),
      ("rbm_s1", "rbm", dict(nh=20, nv=30, seed=0, sample=1), dict(num_iters=100, damping=0.5, temperature=0.0)),
      ("potts_K4", "potts", dict(L=8, K=4, seed=1), dict(num_iters=30, damping=0.5, temperature=1.0)),
      ("potts_K8", "potts", dict(L=6, K=8, seed=2), dict(num_iters=30, damping=0.5, temperature=1.0)),
      ("potts_K16", "potts", dict(L=4, K=16, seed=3), dict(num_iters=20, damping=0.5, temperature=0.5)),
      ("deconv_T1", "deconv", dict(seed=0), dict(num_iters=40, damping=0.5, temperature=1.0)),
      ("deconv_T0", "deconv", dict(seed=0), dict(num_iters=40, damping=0.5, temperature=0.0)),
      ("mixed_T0", "mixed", dict(seed=0), dict(num_iters=7, damping=0.5, temperature=0.0)),
      ("mixed_T1", "mixed", dict(seed=0), dict(num_iters=7, damping=0.5, temperature=1.0)),
      ("mixed_T0.3", "mixed", dict(seed=1), dict(num_iters=7, damping=0.3, temperature=0.3)),
      ("mixed_T0.001", "mixed", dict(seed=2), dict(num_iters=5, damping=0.5, temperature=0.001)),
      ("mixed_iters0", "mixed", dict(seed=3), dict(num_iters=0, damping=0.5, temperature=1.0)),
      ("mixed_iters1", "mixed", dict(seed=3), dict(num_iters=1, damping=0.9, temperature=0.7)),
  ]
  saved = []
  for name, builder, bkw, rkw in plans:
    fg, groups, ev = cases.BUILDERS[builder](api, **bkw)
    bp = api.infer.BP(fg.bp_state, temperature=rkw["temperature"])
    init_kw = {"evidence_updates": ev}
    if builder == "mixed":
      init_kw["ftov_msgs_updates"] = cases.mixed_ftov_updates(api, groups, seed=bkw["seed"])
    bp_arrays = bp.init(**init_kw)
    REC.current = f"case::{name}"
    REC.meta = {"case": name, "builder": builder, "builder_kwargs": bkw, "run_kwargs": rkw}
    bp.run_with_diffs(bp_arrays, **rkw)
    saved.append(name)
  return saved


def factor_update_fixtures(api):
  """Direct calls of each factor-type update on the mixed graph."""
  sys.path.insert(0, HERE)
  import cases  # pylint: disable=g-import-not-at-top
  from pgmax.factor import FAC_TO_VAR_UPDATES  # pylint: disable=g-import-not-at-top
  inferer_mod = importlib.import_module("pgmax.infer.inferer")
  fg, _, _ = cases.mixed(api, seed=5)
  bp_state = fg.bp_state
  ctx = inferer_mod.InfererContext(bp_state)
  wiring = wiring_arrays(ctx, bp_state.fg_state)
  lp = np.asarray(bp_state.log_potentials.value, dtype=np.float32)
  rng = np.random.RandomState(7)
  n_es = wiring["var_states_for_edge_states"].shape[0]
  out = {}
  idx = 0
  for temperature in (0.0, 0.001, 0.05, 0.3, 1.0, 2.5):
    for normalize in (True, False):
      vtof = rng.normal(size=(n_es,)).astype(np.float32) * 2.0
      out[f"upd{idx}.vtof"] = vtof
      out[f"upd{idx}.temperature"] = np.float64(temperature)
      out[f"upd{idx}.normalize"] = np.int64(normalize)
      for t, (ftype, tname) in enumerate(zip(FAC_TO_VAR_UPDATES, TYPE_NAMES)):
        ms, me = ctx.factor_type_to_msgs_range[ftype]
        ps, pe = ctx.factor_type_to_potentials_range[ftype]
        if ms == me:
          continue
        res = FAC_TO_VAR_UPDATES[ftype](
            vtof_msgs=vtof[ms:me], log_potentials=lp[ps:pe], temperature=temperature,
            normalize=normalize, **ctx.inference_arguments[ftype])
        out[f"upd{idx}.{tname}"] = np.asarray(res, dtype=np.float32)
      idx += 1
  arrays = {"w." + k: v for k, v in wiring.items()}
  arrays.update(out)
  arrays["log_potentials"] = lp
  arrays["num_updates"] = np.int64(idx)
  arrays["meta"] = np.array(json.dumps({"source": "factor_updates", "case": "mixed", "seed": 5}))
  np.savez_compressed(os.path.join(OUT, "factor_updates_mixed.npz"), **arrays)


def main():
  ap = argparse.ArgumentParser()
  ap.add_argument("--reference", default=os.environ.get("PGMAX_REFERENCE"),
                  help="the PGMax source tree (default: $PGMAX_REFERENCE)")
  ap.add_argument("--energy-only", action="store_true")
  ap.add_argument("--sdlp-only", action="store_true")
  ap.add_argument("--marginals-only", action="store_true")
  args = ap.parse_args()
  if not args.reference:
    ap.error("name the PGMax source tree with --reference or PGMAX_REFERENCE")
  sys.path.insert(0, HERE)
  import jax_shim  # pylint: disable=g-import-not-at-top
  jax_shim.install()
  sys.path.insert(0, args.reference)
  import pgmax  # pylint: disable=g-import-not-at-top
  from pgmax import factor, fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  install_capture(pgmax)
  install_energy_capture()
  install_sdlp_capture()
  api = types.SimpleNamespace(factor=factor, fgraph=fgraph, fgroup=fgroup, infer=infer,
                              vgroup=vgroup)
  os.makedirs(OUT, exist_ok=True)
  energy_tests = {"test_energy": None, "factor.test_or": None, "factor.test_and": None,
                  "factor.test_pool": None}
  sdlp_tests = {"lp.test_bp_for_lp": None}
  if args.sdlp_only:
    for f in os.listdir(OUT):
      if f.startswith("sdlp_") and f.endswith(".npz"):
        os.remove(os.path.join(OUT, f))
    status = run_reference_tests(args.reference, sdlp_tests)
    sdlp_cases(api)
    n = save_sdlp()
    print(json.dumps({"sdlp_reference_tests": status, "sdlp_fixtures": n}, indent=1))
    return
  if args.marginals_only:
    for f in os.listdir(OUT):
      if f.startswith("marginals_") and f.endswith(".npz"):
        os.remove(os.path.join(OUT, f))
    n = marginals_cases(api)
    print(json.dumps({"marginals_fixtures": n}, indent=1))
    return
  if args.energy_only:
    for f in os.listdir(OUT):
      if f.startswith("energy_") and f.endswith(".npz"):
        os.remove(os.path.join(OUT, f))
    status = run_reference_tests(args.reference, energy_tests)
    energy_cases(api)
    n = save_energies()
    print(json.dumps({"energy_reference_tests": status, "energy_fixtures": n}, indent=1))
    return
  for f in os.listdir(OUT):
    if f.endswith(".npz"):
      os.remove(os.path.join(OUT, f))

  status = run_reference_tests(args.reference)
  n_ref = len(REC.runs)
  run_cases(api)
  factor_update_fixtures(api)
  REC.energies = [r for r in REC.energies if r["source"].startswith("factor.")]
  status.update(run_reference_tests(args.reference, {"test_energy": None}))
  energy_cases(api)
  save_energies()
  REC.sdlp = []
  status.update(run_reference_tests(args.reference, sdlp_tests))
  sdlp_cases(api)
  save_sdlp()
  n_runs = len(REC.runs)
  marginals_cases(api)
  del REC.runs[n_runs:]  # the marginals cases' own runs are saved in their fixtures

  # Golden vector of tests/test_pgmax.py: the (messages, expected) pair of its allclose call.
  golden = [a for a in REC.allclose_args if a[0] == "test_pgmax::test_e2e_sanity_check"]
  extra_golden = {}
  if golden:
    extra_golden = {"golden_expected": golden[0][2].astype(np.float32),
                    "golden_atol": np.float64(golden[0][3].get("atol", 1e-8))}

  counts = {}
  for i, run in enumerate(REC.runs):
    src = run["source"].replace("::", "__").replace(".", "_")
    if run["meta"].get("case"):
      fname = f"case_{run['meta']['case']}.npz"
    else:
      counts[src] = counts.get(src, 0) + 1
      fname = f"ref_{src}_{counts[src]:02d}.npz"
    extra = extra_golden if run["source"] == "test_pgmax::test_e2e_sanity_check" else None
    save_run(os.path.join(OUT, fname), run, extra)
  manifest = {
      "reference_tests": status,
      "captured_runs_from_reference_tests": n_ref,
      "captured_runs_total": len(REC.runs),
      "golden_vector_captured": bool(golden),
  }
  with open(os.path.join(OUT, "MANIFEST.json"), "w") as f:
    json.dump(manifest, f, indent=1, sort_keys=True)
  print(json.dumps(manifest, indent=1))


if __name__ == "__main__":
  main()
