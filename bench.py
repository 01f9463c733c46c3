"""Benchmark: RBM perturb-and-MAP, the headline BP workload, on the pgbp CUDA engine.

Workload (one "step"): a 784-visible x 500-hidden binary RBM - unary EnumFactorGroups with biases
N(0, 0.5^2), a PairwiseFactorGroup of 392,000 2x2 tables [[0, 0], [0, W_ij]] with W ~ N(0, 0.1^2)
(built like the reference's benchmark/rbm_lib.py:135-171) - and a batch of 128 perturb-and-MAP
samples, each with fresh Gumbel(0, 1) evidence on every unary state. One step runs BP for 200
iterations at temperature 0, damping 0.5 over the whole batch, then computes beliefs and MAP-decodes
every sample (the reference benchmark's timed region, rbm_lib.py:180-187, minus JAX compilation).
Every step draws fresh noise: BP.run_perturbed generates it on the GPU inside the run
(pgbp_run_perturbed) from a new seed.
Data are synthetic and seeded (the reference's own numbers are for other RBM sizes on a V100).

Metric: edge-message updates per second = batch x num_edges x iterations / time, num_edges =
2*392,000 + 1,284 = 785,284.
  value  device-resident inputs; CUDA events on the launching stream around K steps.
  e2e    the public API (pgmax_gb300.infer.BP): every step runs BP.run_perturbed from a new seed
         (nothing is copied in: the noise is made on the GPU), decodes, and copies the MAP states
         back to pinned host memory. `e2e_host_noise` is the same with the Gumbel evidence drawn
         on the host and copied in from pinned memory every step (BP.run).
Roofline: the dense pairwise Enum kernel dominates; its per-launch algorithmic bytes are
  B*4*(2*E_pairwise) message reads + writes + B*4*N_vs variable sums + 4*P_pairwise shared potentials,
timed per launch with CUDA events (pgbp_profile_*) inside the timed region.
`--impl reference` times the reference algorithm on the host CPU (the C oracle, a float32
restatement of PGMax's run_with_diffs: PGMax itself needs jax, which is not installed) on a bounded
sample of the same workload with all host cores.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NH, NV, BATCH, ITERS, DAMPING, TEMPERATURE = 500, 784, 128, 200, 0.5, 0.0
NUM_EDGES = 2 * NH * NV + NH + NV
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "pairwise_kernel_rbm_b128.md")
ENERGY_TRAFFIC_FILE = os.path.join(ROOT, "profiles", "energy_pairwise_rbm_b128.md")
TC_TRAFFIC_FILE = os.path.join(ROOT, "profiles", "tc_pairwise_k64_multigraph64.md")


def rbm_params(seed=0):
  rng = np.random.default_rng(seed)
  W = rng.normal(0.0, 0.1, size=(NH, NV)).astype(np.float32)
  bh = rng.normal(0.0, 0.5, size=(NH,)).astype(np.float32)
  bv = rng.normal(0.0, 0.5, size=(NV,)).astype(np.float32)
  return W, bh, bv


def build_rbm(seed=0):
  from pgmax_gb300 import fgraph, fgroup, vgroup  # pylint: disable=g-import-not-at-top
  W, bh, bv = rbm_params(seed)
  hidden = vgroup.NDVarArray(num_states=2, shape=(NH,))
  visible = vgroup.NDVarArray(num_states=2, shape=(NV,))
  fg = fgraph.FactorGraph(variable_groups=[hidden, visible])
  hu = fgroup.EnumFactorGroup(variables_for_factors=[[hidden[i]] for i in range(NH)],
                              factor_configs=np.arange(2)[:, None],
                              log_potentials=np.stack([np.zeros_like(bh), bh], axis=1))
  vu = fgroup.EnumFactorGroup(variables_for_factors=[[visible[j]] for j in range(NV)],
                              factor_configs=np.arange(2)[:, None],
                              log_potentials=np.stack([np.zeros_like(bv), bv], axis=1))
  lpm = np.zeros((NH * NV, 2, 2), dtype=np.float32)
  lpm[:, 1, 1] = W.ravel()
  hv = hidden.variables
  vv = visible.variables
  pw = fgroup.PairwiseFactorGroup(variables_for_factors=[[hv[i], vv[j]] for i in range(NH)
                                                         for j in range(NV)],
                                  log_potential_matrix=lpm)
  fg.add_factors([hu, vu, pw])
  return fg, hidden, visible


def build_ising(n=50, coupling=0.8):
  """Toroidal n x n Ising grid, right/down pairwise factors (the reference's
  tests/test_examples.py:24-40 construction)."""
  from pgmax_gb300 import fgraph, fgroup, vgroup  # pylint: disable=g-import-not-at-top
  variables = vgroup.NDVarArray(num_states=2, shape=(n, n))
  fg = fgraph.FactorGraph(variable_groups=variables)
  vff = []
  for ii in range(n):
    for jj in range(n):
      vff.append([variables[ii, jj], variables[(ii + 1) % n, jj]])
      vff.append([variables[ii, jj], variables[ii, (jj + 1) % n]])
  fg.add_factors(fgroup.PairwiseFactorGroup(
      variables_for_factors=vff,
      log_potential_matrix=coupling * np.array([[1.0, -1.0], [-1.0, 1.0]])))
  return fg, variables


def run_ising(args):
  """50x50 toroidal Ising, B=1: one step = 1000 iterations at T=1 (beliefs, marginals) plus 1000
  at T=0 (MAP decode), damping 0.5. Latency-bound: reported with ns per iteration."""
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer, native  # pylint: disable=g-import-not-at-top
  n, iters = 50, 1000
  fg, variables = build_ising(n)
  flags = {"auto": 0, "multi": native.FLAG_NO_SMALL_GRAPH, "small": native.FLAG_PATH_SMALL,
           "cluster": native.FLAG_PATH_CLUSTER}[args.exec_path]
  bp = infer.BP(fg.bp_state, exec_flags=flags)
  rng = np.random.default_rng(0)
  ev = rng.gumbel(size=(n, n, 2)).astype(np.float32)
  arrays = bp.init(evidence_updates={variables: ev})
  num_edges = 4 * n * n
  dev = torch.device("cuda", 0)
  stream = torch.cuda.current_stream(dev)

  def step():
    a1 = bp.run(arrays, num_iters=iters, damping=0.5, temperature=1.0)
    marg = infer.get_marginals(bp.get_beliefs(a1))
    a0 = bp.run(arrays, num_iters=iters, damping=0.5, temperature=0.0)
    return marg, infer.decode_map_states(bp.get_beliefs(a0))

  for _ in range(args.warmup):
    step()
  torch.cuda.synchronize()
  s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  with ClockSampler(0) as clocks:
    s0.record(stream)
    for _ in range(args.steps):
      step()
    s1.record(stream)
    torch.cuda.synchronize()
  ms = s0.elapsed_time(s1)
  native.profile_read()
  native.profile_enable(True)
  for _ in range(args.steps):
    step()
  torch.cuda.synchronize()
  native.profile_enable(False)
  prof = native.profile_read()
  units = num_edges * 2 * iters * args.steps
  info = bp.context.plan.info
  iter_ns = ms * 1e6 / (2 * iters * args.steps)
  line = {
      "metric": "edge-msg updates/s", "value": units / (ms / 1e3), "unit": "edge-msg updates/s",
      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
      "data": "synthetic (Gumbel(0,1) evidence, seed 0)",
      "config": {"workload": "ising50x50_toroidal", "batch": 1, "num_iters": iters,
                 "temperatures": [1.0, 0.0], "damping": 0.5, "num_edges": num_edges,
                 "exec_path": args.exec_path},
      "ns_per_iteration": iter_ns,
      "kernel_time_share": {k: v[1] for k, v in prof.items() if v[0]},
      "roofline": {"bound": "latency (2 block barriers per iteration)",
                   "bytes_per_iter": 4 * (3 * info["num_slots"] + 3 * n * n * 2)
                                     + 4 * int(bp.context.plan.num_potentials)},
      "clocks": clocks.summary(),
  }
  if not args.no_cpu_baseline:
    from oracle import oracle  # pylint: disable=g-import-not-at-top
    w = oracle.Wiring(bp.context.flat_wiring())
    lp = np.asarray(fg.fg_state.log_potentials, np.float32)
    evf = arrays.evidence.cpu().numpy()
    m0 = np.zeros(fg.fg_state.total_factor_num_states, np.float32)
    t0 = time.perf_counter()
    oracle.run(w, lp, evf, m0, iters, 0.5, 1.0)
    oracle.run(w, lp, evf, m0, iters, 0.5, 0.0)
    dt = time.perf_counter() - t0
    line["cpu_baseline"] = {"value": num_edges * 2 * iters / dt, "unit": "edge-msg updates/s",
                            "cores": 1, "kind": "port",
                            "sample": f"one full step (2 x {iters} iterations), C oracle, {dt:.2f} s"}
  print(json.dumps(line))
  return 0


ENUM_VARS, ENUM_K, ENUM_FACTORS, ENUM_B, ENUM_ITERS = 2000, 10, 3000, 128, 50


def build_enum(seed=0):
  """Higher-order EnumFactors: 3,000 ternary factors over random triples of 2,000 variables of 10
  states, each with the full 1,000-config table (one shared config list, per-factor potentials
  N(0, 1)); every variable also gets Gumbel evidence in the runs."""
  import itertools  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import fgraph, fgroup, vgroup  # pylint: disable=g-import-not-at-top
  rng = np.random.default_rng(seed)
  var = vgroup.NDVarArray(num_states=ENUM_K, shape=(ENUM_VARS,))
  fg = fgraph.FactorGraph(variable_groups=[var])
  seen, triples = set(), []
  while len(triples) < ENUM_FACTORS:
    t = tuple(sorted(rng.choice(ENUM_VARS, size=3, replace=False).tolist()))
    if t not in seen:
      seen.add(t)
      triples.append(t)
  configs = np.array(list(itertools.product(range(ENUM_K), repeat=3)), dtype=np.int64)
  fg.add_factors(fgroup.EnumFactorGroup(
      variables_for_factors=[[var[i] for i in t] for t in triples], factor_configs=configs,
      log_potentials=rng.normal(size=(ENUM_FACTORS, configs.shape[0])).astype(np.float32)))
  return fg, var


def run_enum(args):
  """Perturb-and-MAP on a graph of higher-order EnumFactors (generic config tables, the staged or
  per-thread generic kernel as the tuner picks): 128 samples, 50 iterations at T = 0 per step,
  Gumbel noise generated on the GPU inside the run. Messages: 90,000 edge states x 128 samples
  (46 MB) per buffer; the config rows and potentials (24 MB) are shared by the batch."""
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer, native  # pylint: disable=g-import-not-at-top
  fg, var = build_enum()
  bp = infer.BP(fg.bp_state)
  base = bp.init()
  dev = torch.device("cuda", 0)
  stream = torch.cuda.current_stream(dev)
  seeds = iter(range(1 << 40, 1 << 62))
  map_h = torch.empty((ENUM_B, ENUM_VARS), dtype=torch.int32).pin_memory()
  flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # larger than the 129 MB L2

  def step():
    out = bp.run_perturbed(base, ENUM_ITERS, next(seeds), ENUM_B, damping=0.5, temperature=0.0)
    return infer.decode_map_states(bp.get_beliefs(out))

  for _ in range(args.warmup):
    step()
  torch.cuda.synchronize()
  s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  ms = 0.0
  with ClockSampler(0) as clocks:
    for _ in range(args.steps):
      flush.zero_()
      s0.record(stream)
      step()
      s1.record(stream)
      torch.cuda.synchronize()
      ms += s0.elapsed_time(s1)
  # end to end: the MAP states of every sample copied to pinned host memory each step
  e2e_ms = 0.0
  for _ in range(args.steps):
    flush.zero_()
    s0.record(stream)
    map_h.copy_(step()[var], non_blocking=True)
    s1.record(stream)
    torch.cuda.synchronize()
    e2e_ms += s0.elapsed_time(s1)
  native.profile_read()
  native.profile_enable(True)
  for _ in range(args.steps):
    step()
  torch.cuda.synchronize()
  native.profile_enable(False)
  prof = native.profile_read()
  plan = bp.context.plan
  num_edges = 3 * ENUM_FACTORS
  units = num_edges * ENUM_ITERS * ENUM_B * args.steps
  n_es = plan.num_edge_states
  gen_launches, gen_ms = prof["enum_generic"]
  gen_launch_ms = gen_ms / max(gen_launches, 1)
  # per launch: each (factor, instance) reads its 30 messages and 30 variable sums and writes 30
  # messages; the config rows (3 int32 per config) and the potentials are read once
  alg_bytes = ENUM_B * n_es * 4 * 3 + ENUM_FACTORS * 1000 * (3 * 4 + 4)
  peak, peak_kind = peaks()
  # shared-memory bound of the staged kernel: every (config, variable) pair read twice per
  # (factor, instance), once for the config sums and once for the maxima, at 128 B per clock
  # per SM (nominal) at the sampled SM clock
  smem_bytes = 2 * ENUM_FACTORS * 1000 * 3 * ENUM_B * 4
  csum = clocks.summary()
  sm_mhz = csum.get("sm_mhz") or 2070
  smem_peak_gbs = 128 * 152 * sm_mhz * 1e6 / 1e9
  line = {
      "metric": "edge-msg updates/s", "value": units / (ms / 1e3), "unit": "edge-msg updates/s",
      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
      "data": "synthetic (seeded ternary 10-state tables N(0,1), Gumbel(0,1) noise on the GPU)",
      "config": {"workload": "enum_ternary10_3000f_b128", "batch": ENUM_B,
                 "num_iters": ENUM_ITERS, "temperature": 0.0, "damping": 0.5,
                 "factors": ENUM_FACTORS, "configs_per_factor": 1000, "num_edges": num_edges,
                 "edge_states": n_es, "l2": "flushed before every step (256 MB written)"},
      "e2e": {"value": units / (e2e_ms / 1e3), "unit": "edge-msg updates/s",
              "h2d_bytes_per_step": 0, "d2h_bytes_per_step": ENUM_B * ENUM_VARS * 4,
              "noise": "Gumbel(0,1) generated on the GPU inside the run (pgbp_run_perturbed)"},
      "gpu_launches": int(sum(v[0] for v in prof.values())),
      "kernel_time_share": {k: v[1] / max(sum(x[1] for x in prof.values()), 1e-9)
                            for k, v in prof.items() if v[0]},
      "generic_kernel": _generic_site_choice(plan, ENUM_B),
      "roofline": {"bound": "hbm", "kernel": "generic EnumFactor kernel",
                   "achieved": alg_bytes / (gen_launch_ms / 1e3) / 1e9, "peak": peak,
                   "unit": "GB/s", "frac": alg_bytes / (gen_launch_ms / 1e3) / 1e9 / peak,
                   "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({peak_kind})",
                   "traffic": None, "algorithmic_bytes_per_launch": alg_bytes,
                   "launch_ms": gen_launch_ms,
                   "note": "not HBM-bound: the config loops bound it (smem_estimate)"},
      "smem_estimate": {"bytes_per_launch": smem_bytes,
                        "peak_gbs_nominal": smem_peak_gbs,
                        "frac": smem_bytes / (gen_launch_ms / 1e3) / 1e9 / smem_peak_gbs},
      "clocks": csum,
  }
  if not args.no_cpu_baseline:
    from oracle import oracle  # pylint: disable=g-import-not-at-top
    w = oracle.Wiring(bp.context.flat_wiring())
    lp = np.asarray(fg.fg_state.log_potentials, np.float32)
    rng = np.random.default_rng(1)
    nvs = fg.fg_state.num_var_states
    n_cpu = 4
    evs = rng.gumbel(size=(n_cpu, nvs)).astype(np.float32)
    m0 = np.zeros((n_es,), np.float32)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.run_batch(w, lp, evs, m0, ENUM_ITERS, 0.5, 0.0, num_threads=threads)
    dt = time.perf_counter() - t0
    line["cpu_baseline"] = {"value": num_edges * ENUM_ITERS * n_cpu / dt,
                            "unit": "edge-msg updates/s", "cores": min(threads, n_cpu),
                            "kind": "port",
                            "sample": f"{n_cpu} samples x {ENUM_ITERS} iterations, C oracle, "
                                      f"{dt:.2f} s"}
  print(json.dumps(line))
  return 0


def _generic_site_choice(plan, batch):
  """The tuned generic-Enum kernel at this batch (T = 0): per-thread, staged or the rule."""
  for e in plan.tuning():
    if e["batch"] == batch and e["temperature0"] and e["sites"]:
      return {0: "per-thread", 1: "staged", -1: "rule"}.get(e["sites"][-1], "rule")
  return "rule"


ADJ_N, ADJ_B, ADJ_ITERS, ADJ_CKPT, ADJ_FLIP = 64, 32, 100, 10, 0.1
SDLP_TEMP, SDLP_ITERS = 1e-3, 200


def run_sdlp(args):
  """Smooth dual LP-MAP on the RBM perturb-and-MAP batch: 784 x 500 RBM, 128 Gumbel-perturbed
  evidence samples, logsumexp_temp 1e-3 at the default learning rate, 200 accelerated gradient
  steps per step (pgbp_sdlp_run), the objective recorded every step. Messages (804 MB per
  buffer) are larger than L2."""
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer, native  # pylint: disable=g-import-not-at-top
  dev = torch.device("cuda", 0)
  nb = args.batch
  fg, _, _ = build_rbm(seed=0)
  sdlp = infer.build_inferer(fg.bp_state, backend="sdlp")
  nvs = fg.fg_state.num_var_states
  n_es = fg.fg_state.total_factor_num_states
  ev_host = gumbel_evidence(nvs, nb, 1000)
  lp_dev = torch.as_tensor(np.asarray(fg.fg_state.log_potentials, np.float32), device=dev)
  ev_dev = torch.as_tensor(ev_host, device=dev)
  msgs0 = torch.zeros((nb, n_es), dtype=torch.float32, device=dev)
  arrays = infer.BPArrays(log_potentials=lp_dev, ftov_msgs=msgs0, evidence=ev_dev)
  stream = torch.cuda.current_stream(dev)

  def step():
    return sdlp.run_with_objvals(arrays, logsumexp_temp=SDLP_TEMP, num_iters=SDLP_ITERS)

  for _ in range(args.warmup):
    out, objvals = step()
  torch.cuda.synchronize()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  with ClockSampler(0) as clocks:
    e0.record(stream)
    for _ in range(args.steps):
      out, objvals = step()
    e1.record(stream)
    torch.cuda.synchronize()
  ms = e0.elapsed_time(e1)
  native.profile_read()
  native.profile_enable(True)
  step()
  torch.cuda.synchronize()
  native.profile_enable(False)
  prof = native.profile_read()
  # the same steps as subgradient descent (logsumexp_temp 0: max-product updates, no exp / log)
  sdlp.run_with_objvals(arrays, logsumexp_temp=0.0, num_iters=SDLP_ITERS)
  torch.cuda.synchronize()
  e0.record(stream)
  for _ in range(args.steps):
    sdlp.run_with_objvals(arrays, logsumexp_temp=0.0, num_iters=SDLP_ITERS)
  e1.record(stream)
  torch.cuda.synchronize()
  ms_t0 = e0.elapsed_time(e1)
  units = nb * n_es * SDLP_ITERS * args.steps
  # per step and instance: messages read by the variable sums and the factor pass, eta read and
  # written, the next messages written; variable sums written and read, the variable softmax
  # written and gathered once per edge state; the evidence; potentials shared by the batch
  iter_bytes = nb * 4 * (5 * n_es + 4 * nvs) + 4 * int(lp_dev.numel())
  achieved = iter_bytes * SDLP_ITERS * args.steps / (ms / 1e3) / 1e9
  peak, peak_kind = peaks()
  line = {
      "metric": "edge-state updates/s", "value": units / (ms / 1e3),
      "unit": "edge-state updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
      "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
      "vs_baseline": None, "dtype": "f32",
      "data": "synthetic (seeded RBM, Gumbel(0,1) evidence per sample)",
      "config": {"workload": f"sdlp_rbm784x500_b{nb}", "batch": nb, "num_iters": SDLP_ITERS,
                 "logsumexp_temp": SDLP_TEMP, "edge_states": n_es,
                 "l2": "inputs larger than L2 (804 MB of messages per buffer)"},
      "final_objval_mean": float(objvals[:, -1].mean()),
      "temp0": {"ms_per_step": ms_t0 / args.steps, "value": units / (ms_t0 / 1e3),
                "frac_of_hbm": iter_bytes * SDLP_ITERS * args.steps / (ms_t0 / 1e3) / 1e9 / peak},
      "kernel_time_share": {k: v[1] for k, v in prof.items() if v[0]},
      "gpu_launches": sum(v[0] for v in prof.values()) * args.steps,
      "roofline": {"bound": "hbm", "kernel": "one SDLP step (all launches)", "achieved": achieved,
                   "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                   "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({peak_kind})",
                   "algorithmic_bytes_per_iteration": iter_bytes, "traffic": None},
      "clocks": clocks.summary(),
  }
  if not args.no_cpu_baseline:
    from oracle import sdlp as oracle_sdlp  # pylint: disable=g-import-not-at-top
    problem = oracle_sdlp.Problem(sdlp_context(fg).flat_wiring())
    lp_h = lp_dev.cpu().numpy()
    n, t_start = 0, time.perf_counter()
    msgs = np.zeros(n_es, np.float32)
    while time.perf_counter() - t_start < 10.0 and n < SDLP_ITERS:
      msgs, _ = problem.run_with_objvals(lp_h, ev_host[0], msgs, SDLP_TEMP, 1)
      n += 1
    dt = time.perf_counter() - t_start
    line["cpu_baseline"] = {"value": n * n_es / dt, "unit": "edge-state updates/s", "cores": 1,
                            "kind": "port",
                            "sample": f"{n} steps of sample 0, NumPy + C oracle, {dt:.1f} s"}
  print(json.dumps(line))
  return 0


def sdlp_context(fg):
  from pgmax_gb300 import infer  # pylint: disable=g-import-not-at-top
  return infer.InfererContext(fg.bp_state)


def run_energy(args):
  """compute_energy of the RBM perturb-and-MAP batch: the 128 MAP decodings of one 200-iteration
  T = 0 run (784 x 500 RBM, Gumbel evidence per sample) scored in one pgbp_energy launch against
  their own evidence and the shared potentials. A step is one launch; L2 is flushed (a 512 MB
  write) before each, and only the launches are timed (CUDA events around each)."""
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer, native  # pylint: disable=g-import-not-at-top
  dev = torch.device("cuda", 0)
  fg, hidden, visible = build_rbm(seed=0)
  bp = infer.BP(fg.bp_state, temperature=TEMPERATURE)
  plan = bp.context.plan
  nvs = fg.fg_state.num_var_states
  ev_host = gumbel_evidence(nvs, BATCH, 1000)
  lp_dev = torch.as_tensor(np.asarray(fg.fg_state.log_potentials, np.float32), device=dev)
  ev_dev = torch.as_tensor(ev_host, device=dev)
  msgs0 = torch.zeros(fg.fg_state.total_factor_num_states, dtype=torch.float32, device=dev)
  arrays = infer.BPArrays(log_potentials=lp_dev, ftov_msgs=msgs0, evidence=ev_dev)
  out = bp.run(arrays, num_iters=ITERS, damping=DAMPING, temperature=TEMPERATURE)
  dec = infer.decode_map_states(bp.get_beliefs(out))
  maps = torch.cat([dec[hidden].reshape(BATCH, -1), dec[visible].reshape(BATCH, -1)],
                   dim=1).to(torch.int32).contiguous()
  stream = torch.cuda.current_stream(dev)
  flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
  for _ in range(args.warmup):
    energies = plan.energy(lp_dev, ev_dev, maps)
  torch.cuda.synchronize()
  evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
         for _ in range(args.steps)]
  with ClockSampler(0) as clocks:
    for e0, e1 in evs:
      flush.zero_()
      e0.record(stream)
      energies = plan.energy(lp_dev, ev_dev, maps)
      e1.record(stream)
    torch.cuda.synchronize()
  ms = sum(e0.elapsed_time(e1) for e0, e1 in evs)
  info = plan.info
  nv = NH + NV
  n_factors = info["num_enum_factors"]
  terms = BATCH * (n_factors + nv)
  # bytes one launch must bring from HBM (cold L2): the decodings and per-sample evidence, the
  # shared potentials, and the plan's index arrays it walks (int4 record + first potential per
  # pairwise factor; unary factors: 7 int32 per factor and 1 per config row; var_off, var_of_vs)
  f_pw = info["num_enum_pairwise_factors"]
  algo_bytes = (BATCH * 4 * (nv + nvs) + 4 * int(plan.num_potentials) + 20 * f_pw
                + 4 * (7 * (n_factors - f_pw) + 2 * (n_factors - f_pw)) + 4 * (nv + 1 + nvs))
  launch_s = ms / 1e3 / args.steps
  peak, peak_kind = peaks()
  achieved = algo_bytes / launch_s / 1e9
  # end to end through the public API: host decodings in, host energies out
  maps_pinned = maps.cpu().pin_memory()
  ev_pinned = torch.as_tensor(ev_host).pin_memory()
  en_host = torch.empty(BATCH, dtype=torch.float32).pin_memory()
  host_arrays = infer.BPArrays(log_potentials=lp_dev, ftov_msgs=msgs0, evidence=ev_dev)
  map_states = {hidden: None, visible: None}

  def step_e2e():
    m = maps_pinned.to(dev, non_blocking=True)
    e = ev_pinned.to(dev, non_blocking=True)
    map_states[hidden] = m[:, :NH]
    map_states[visible] = m[:, NH:]
    a = infer.BPArrays(log_potentials=lp_dev, ftov_msgs=msgs0, evidence=e)
    en, _, _ = infer.compute_energy(fg.bp_state, a, map_states)
    en_host.copy_(en, non_blocking=True)

  del host_arrays
  for _ in range(args.warmup):
    step_e2e()
  torch.cuda.synchronize()
  t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  t0.record(stream)
  for _ in range(args.steps):
    step_e2e()
  t1.record(stream)
  torch.cuda.synchronize()
  e2e_ms = t0.elapsed_time(t1)
  line = {
      "metric": "energy terms/s", "value": terms * args.steps / (ms / 1e3),
      "unit": "energy terms/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
      "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
      "vs_baseline": None, "dtype": "f64 sums of f32",
      "data": "synthetic (seeded RBM, Gumbel(0,1) evidence; the decodings of a 200-iteration run)",
      "config": {"workload": "energy_rbm784x500_b128", "batch": BATCH,
                 "terms_per_decoding": n_factors + nv, "l2": "flushed before every launch"},
      "decodings_per_s": BATCH * args.steps / (ms / 1e3),
      "e2e": {"value": terms * args.steps / (e2e_ms / 1e3), "unit": "energy terms/s",
              "h2d_bytes_per_step": int(maps_pinned.numel() * 4 + ev_pinned.numel() * 4),
              "d2h_bytes_per_step": int(en_host.numel() * 4)},
      # per call: the decodings' transpose, the partial kernel (variables, unary factors), the
      # dense pairwise kernel (one bucket) and the final per-instance sum
      "gpu_launches": 4 * args.steps,
      "roofline": {"bound": "hbm", "kernel": "pgbp_energy (all four launches of one call)",
                   "achieved": achieved,
                   "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                   "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({peak_kind})",
                   "algorithmic_bytes_per_launch": algo_bytes,
                   "traffic": read_traffic(ENERGY_TRAFFIC_FILE, "traffic_bytes_per_launch:"),
                   "traffic_kernel": "energy_pairwise_kernel (ncu, one launch; the transpose, "
                                     "partial and final launches move about 2 MB more)"},
      "clocks": clocks.summary(),
  }
  if not args.no_cpu_baseline:
    from oracle import energy as oracle_energy  # pylint: disable=g-import-not-at-top
    w = bp.context.flat_wiring()
    lp_h = lp_dev.cpu().numpy()
    maps_h = maps.cpu().numpy()
    n, t_start = 0, time.perf_counter()
    while n < BATCH and time.perf_counter() - t_start < 10.0:
      got = oracle_energy.compute_energy(w, lp_h, ev_host[n], maps_h[n])
      want = float(energies[n])
      assert (np.isinf(got) and np.isinf(want)) or abs(got - want) <= 1e-4 * max(1.0, abs(got))
      n += 1
    dt = time.perf_counter() - t_start
    line["cpu_baseline"] = {"value": n * (n_factors + nv) / dt, "unit": "energy terms/s",
                            "cores": 1, "kind": "port",
                            "sample": f"{n} of the {BATCH} decodings, NumPy oracle, {dt:.1f} s"}
  print(json.dumps(line))
  return 0


def shape_images(n, batch, seed, flip):
  """`batch` binary n x n images, each the union of 2-6 random axis-aligned rectangles and
  ellipses, and their observations with every pixel flipped with probability `flip`."""
  rng = np.random.default_rng(seed)
  yy, xx = np.mgrid[0:n, 0:n]
  clean = np.zeros((batch, n, n), dtype=np.int64)
  for b in range(batch):
    for _ in range(rng.integers(2, 7)):
      cy, cx = rng.uniform(0, n, size=2)
      hy, hx = rng.uniform(n / 16, n / 4, size=2)
      if rng.random() < 0.5:
        clean[b] |= ((np.abs(yy - cy) <= hy) & (np.abs(xx - cx) <= hx))
      else:
        clean[b] |= (((yy - cy) / hy) ** 2 + ((xx - cx) / hx) ** 2 <= 1.0)
  noisy = clean ^ (rng.random(clean.shape) < flip)
  return clean, noisy


def build_grid(n):
  """Open n x n binary grid with top-down and left-right PairwiseFactorGroups."""
  from pgmax_gb300 import fgraph, fgroup, vgroup  # pylint: disable=g-import-not-at-top
  grid = vgroup.NDVarArray(num_states=2, shape=(n, n))
  fg = fgraph.FactorGraph(variable_groups=grid)
  td = fgroup.PairwiseFactorGroup(
      variables_for_factors=[[grid[i, j], grid[i + 1, j]] for i in range(n - 1) for j in range(n)],
      log_potential_matrix=np.zeros((2, 2)))
  lr = fgroup.PairwiseFactorGroup(
      variables_for_factors=[[grid[i, j], grid[i, j + 1]] for i in range(n) for j in range(n - 1)],
      log_potential_matrix=np.zeros((2, 2)))
  fg.add_factors([td, lr])
  return fg, grid, td, lr


def run_adjoint(args):
  """Differentiable loopy BP: one step = forward + hand-written backward of the mean negative
  log-marginal of the clean labels of 32 noisy 64x64 binary images with respect to a shared
  top-down 2x2 log potential, a shared left-right one and a unary scale (100 iterations at
  temperature 1, damping 0.5, messages checkpointed every 10 iterations), through the drop-in
  API: bp.init -> bp.run -> get_beliefs -> get_marginals -> loss.backward()."""
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer, native  # pylint: disable=g-import-not-at-top
  n, B, iters = ADJ_N, ADJ_B, ADJ_ITERS
  fg, grid, td, lr = build_grid(n)
  bp = infer.BP(fg.bp_state, temperature=1.0, checkpoint_every=ADJ_CKPT)
  num_edges = 2 * 2 * n * (n - 1)
  dev = torch.device("cuda", 0)
  stream = torch.cuda.current_stream(dev)
  clean, noisy = shape_images(n, B, 0, ADJ_FLIP)
  noisy_host = torch.as_tensor(noisy.astype(np.float32)).pin_memory()
  labels = torch.as_tensor(clean, device=dev)
  w_td = torch.tensor([[0.5, -0.5], [-0.5, 0.5]], device=dev, requires_grad=True)
  w_lr = torch.tensor([[0.5, -0.5], [-0.5, 0.5]], device=dev, requires_grad=True)
  scale = torch.tensor(1.0, device=dev, requires_grad=True)
  lo, hi = float(np.log(ADJ_FLIP)), float(np.log1p(-ADJ_FLIP))
  loss_host = torch.empty((), dtype=torch.float32).pin_memory()

  def forward(obs):
    # log p(observed | state): rows state 0 / state 1 of every pixel
    logp = torch.stack([torch.where(obs == 0, hi, lo), torch.where(obs == 1, hi, lo)], dim=-1)
    arrays = bp.init(log_potentials_updates={td: w_td, lr: w_lr},
                     evidence_updates={grid: scale * logp})
    arrays = bp.run(arrays, num_iters=iters, damping=0.5, temperature=1.0)
    marg = infer.get_marginals(bp.get_beliefs(arrays))[grid]
    return -torch.log(torch.gather(marg, -1, labels[..., None])).mean()

  obs_static = noisy_host.to(dev)

  def step(events=None):
    if events:
      events[0].record(torch.cuda.current_stream(dev))
    loss = forward(obs_static)
    if events:
      events[1].record(torch.cuda.current_stream(dev))
    for p in (w_td, w_lr, scale):
      p.grad = None
    loss.backward()
    if events:
      events[2].record(torch.cuda.current_stream(dev))
    return loss

  # warm-up on a side stream (what CUDA-graph capture of an autograd step requires), eager timing
  side = torch.cuda.Stream(dev)
  side.wait_stream(stream)
  with torch.cuda.stream(side):
    for _ in range(args.warmup):
      step()
    ev_pairs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)]
                for _ in range(args.steps)]
    for k in range(args.steps):
      step(events=ev_pairs[k])
  stream.wait_stream(side)
  torch.cuda.synchronize()
  fwd_ms = sum(e[0].elapsed_time(e[1]) for e in ev_pairs) / args.steps
  bwd_ms = sum(e[1].elapsed_time(e[2]) for e in ev_pairs) / args.steps
  # the step captured once in a CUDA graph: every replay runs every kernel of the step again
  graph = torch.cuda.CUDAGraph()
  with torch.cuda.graph(graph):
    loss_static = step()
  graph.replay()
  torch.cuda.synchronize()
  s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  with ClockSampler(0) as clocks:
    s0.record(stream)
    for _ in range(args.steps):
      graph.replay()
    s1.record(stream)
    torch.cuda.synchronize()
  ms = s0.elapsed_time(s1)
  # end to end: observations copied from pinned host memory and the loss read back every step
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record(stream)
  for _ in range(args.steps):
    obs_static.copy_(noisy_host, non_blocking=True)
    graph.replay()
    loss_host.copy_(loss_static.detach(), non_blocking=True)
  e1.record(stream)
  torch.cuda.synchronize()
  e2e_ms = e0.elapsed_time(e1)
  native.profile_read()
  native.profile_enable(True)
  step()
  torch.cuda.synchronize()
  native.profile_enable(False)
  prof = native.profile_read()
  units = B * num_edges * iters
  # kernels of one step: the forward engine's (profiled per launch) plus the adjoint's, counted
  # from its structure (per chunk: normalise, k variable sums, k - 1 factor passes; per iteration
  # backwards: factor pass + variable-sum pass; one batch reduction of the shared potentials)
  n_buckets = bp.context.plan.info["num_pairwise_buckets"]
  n_ck = -(-iters // ADJ_CKPT)
  adj_kernels = (n_ck * (1 + ADJ_CKPT + (ADJ_CKPT - 1) * n_buckets) + iters * (n_buckets + 1) + 1)
  fwd_kernels = sum(v[0] for kk, v in prof.items() if kk != "adjoint")
  line = {
      "metric": "edge-msg updates/s (forward + backward)", "value": units * args.steps / (ms / 1e3),
      "unit": "edge-msg updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
      "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
      "vs_baseline": None, "dtype": "f32",
      "data": "synthetic (rectangles/ellipses, 10% pixel flips, seed 0)",
      "config": {"workload": "adjoint_grid64_b32", "batch": B, "num_iters": iters,
                 "temperature": 1.0, "damping": 0.5, "checkpoint_every": ADJ_CKPT,
                 "num_edges": num_edges, "step": "forward + backward, captured in a CUDA graph",
                 "l2": "inputs smaller than L2 (no flush)"},
      "eager_ms_per_step": fwd_ms + bwd_ms,
      "forward_ms_eager": fwd_ms, "backward_ms_eager": bwd_ms,
      "kernel_time_share": {k: v[1] for k, v in prof.items() if v[0]},
      "gpu_launches": int((fwd_kernels + adj_kernels) * args.steps),
      "e2e": {"value": units * args.steps / (e2e_ms / 1e3), "unit": "edge-msg updates/s",
              "h2d_bytes_per_step": int(noisy_host.numel() * 4), "d2h_bytes_per_step": 4},
      "clocks": clocks.summary(),
      "loss": float(loss_static.detach()),
  }
  if not args.no_cpu_baseline:
    from oracle import bp_torch  # pylint: disable=g-import-not-at-top
    g = bp_torch.EnumGraph(bp.context.flat_wiring())
    nb = 2
    cores = torch.get_num_threads()
    lp = bp.init(log_potentials_updates={td: w_td.detach().cpu(), lr: w_lr.detach().cpu()}
                 ).log_potentials.detach().cpu().double()
    wt = lp.clone().requires_grad_()
    obs = torch.as_tensor(noisy[:nb])
    logp = torch.stack([torch.where(obs == 0, hi, lo), torch.where(obs == 1, hi, lo)], -1)
    ev = logp.reshape(nb, -1).double().requires_grad_()
    t0 = time.perf_counter()
    out = g.run(wt, ev, torch.zeros(g.num_edge_states, dtype=torch.float64), iters, 0.5, 1.0)
    bel = g.beliefs(ev, out).reshape(nb, n, n, 2)
    loss = -torch.log_softmax(bel, -1).gather(-1, torch.as_tensor(clean[:nb])[..., None]).mean()
    loss.backward()
    dt = time.perf_counter() - t0
    line["cpu_baseline"] = {
        "value": nb * num_edges * iters / dt, "unit": "edge-msg updates/s", "cores": cores,
        "kind": "port",
        "sample": f"{nb} of the {B} images, full {iters} iterations, forward + autograd backward "
                  f"of the float64 torch restatement on CPU ({dt:.1f} s)"}
  print(json.dumps(line))
  return 0


MG_GRAPHS, MG_ITERS = 256, 200


def deconv_template(n_feat=5, feat=6, im=14):
  """The 2D binary deconvolution graph (the reference's examples/pmp_binary_deconvolution.ipynb
  construction): features W (1, n_feat, feat, feat), activations S (1, n_feat, s, s),
  s = im - feat + 1, auxiliaries SW = AND(S, W) and pixels X = OR of the SW covering them."""
  from pgmax_gb300 import fgraph, fgroup, infer, vgroup  # pylint: disable=g-import-not-at-top
  s_size = im - feat + 1
  W = vgroup.NDVarArray(num_states=2, shape=(1, n_feat, feat, feat))
  S = vgroup.NDVarArray(num_states=2, shape=(1, n_feat, s_size, s_size))
  SW = vgroup.NDVarArray(num_states=2, shape=(1, 1, im, im, n_feat, feat, feat))
  X = vgroup.NDVarArray(num_states=2, shape=(1, 1, im, im))
  fg = fgraph.FactorGraph(variable_groups=[S, W, SW, X])
  and_vars, or_parents = [], {}
  for sh in range(s_size):
    for sw in range(s_size):
      for f in range(n_feat):
        for fh in range(feat):
          for fw in range(feat):
            aux = SW[0, 0, fh + sh, fw + sw, f, fh, fw]
            and_vars.append([S[0, f, sh, sw], W[0, f, fh, fw], aux])
            or_parents.setdefault((fh + sh, fw + sw), []).append(aux)
  fg.add_factors(fgroup.ANDFactorGroup(and_vars))
  fg.add_factors(fgroup.ORFactorGroup([v + [X[0, 0, r, c]] for (r, c), v in or_parents.items()]))
  wiring = infer.InfererContext(fg.bp_state).flat_wiring()
  return wiring, (S.shape, W.shape, SW.shape, X.shape), (n_feat, feat, im, s_size)


def deconv_evidence(shapes, dims, rng):
  """Seeded evidence of one deconvolution graph: W clamped to Bernoulli(0.25) masks (+-100),
  S prior Bernoulli(0.02) log-odds, X the OR of the true activations' features with 5% of the
  pixels flipped, observed at +-4 log-odds."""
  (s_shape, w_shape, sw_shape, x_shape), (n_feat, feat, im, s_size) = shapes, dims
  w_true = rng.random(w_shape) < 0.25
  s_true = rng.random(s_shape) < 0.02
  x = np.zeros((im, im), bool)
  for f in range(n_feat):
    for r, c in zip(*np.nonzero(s_true[0, f])):
      x[r:r + feat, c:c + feat] |= w_true[0, f]
  x ^= rng.random((im, im)) < 0.05
  ev_s = np.zeros(s_shape + (2,), np.float32)
  ev_s[..., 1] = np.log(0.02) - np.log(0.98)
  ev_w = np.zeros(w_shape + (2,), np.float32)
  ev_w[..., 1] = np.where(w_true, 100.0, -100.0)
  ev_sw = np.zeros(sw_shape + (2,), np.float32)
  ev_x = np.zeros(x_shape + (2,), np.float32)
  ev_x[0, 0, ..., 1] = np.where(x, 4.0, -4.0)
  return np.concatenate([a.reshape(-1) for a in (ev_s, ev_w, ev_sw, ev_x)])


def build_multigraph(seed=0, n_graphs=MG_GRAPHS):
  """256 graphs, family g mod 3: (a) open Potts grids L ~ U{16..128}, K ~ U{2,4,8,16}, one table
  J * I_K per graph, J ~ U(0, 1.5), unaries N(0, 1); (b) the same at K = 64 with one table
  ~ N(0, 0.5^2) per graph; (c) binary deconvolution graphs. Returns the wirings (grids with shared
  tables and implicit config rows), per-graph potentials and evidence, and the family sizes."""
  from pgmax_gb300 import batch  # pylint: disable=g-import-not-at-top
  rng = np.random.default_rng(seed)
  dec_w, dec_shapes, dec_dims = deconv_template()
  cache, wirings, tables, evs, fam = {}, [], [], [], {"a": 0, "b": 0, "c": 0}
  for g in range(n_graphs):
    kind = "abc"[g % 3]
    fam[kind] += 1
    if kind == "c":
      wirings.append(dec_w)
      tables.append(np.zeros(0, np.float32))
      evs.append(deconv_evidence(dec_shapes, dec_dims, rng))
      continue
    L = int(rng.integers(16, 129))
    if kind == "a":
      K = int(rng.choice([2, 4, 8, 16]))
      table = (rng.uniform(0.0, 1.5) * np.eye(K)).astype(np.float32).reshape(-1)
    else:
      K = 64
      table = rng.normal(0.0, 0.5, size=K * K).astype(np.float32)
    if (L, K) not in cache:
      cache[(L, K)] = batch.grid_wiring(L, K, shared_table=True, implicit_rows=True)
    wirings.append(cache[(L, K)])
    tables.append(table)
    evs.append(rng.normal(size=L * L * K).astype(np.float32))
  return wirings, tables, evs, fam


def multigraph_cpu_baseline(wirings, tables, evs, sample, iters):
  """The C oracle on a sample of the batch's graphs, one host thread per graph (ctypes releases
  the GIL): edge-message updates per second over the sample."""
  import concurrent.futures  # pylint: disable=g-import-not-at-top
  from oracle import oracle  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import batch  # pylint: disable=g-import-not-at-top
  jobs = []
  for g in sample:
    w = wirings[g]
    if w.get("enum.implicit_rows"):   # the oracle reads explicit rows and per-factor tables
      L = int(round(np.sqrt(w["num_variables"])))
      K = int(round(np.sqrt(tables[g].shape[0])))
      w, lp = batch.grid_wiring(L, K), np.tile(tables[g], 2 * L * (L - 1))
    else:
      lp = tables[g]
    jobs.append((oracle.Wiring(w), lp, evs[g], int(w["num_edges"]),
                 np.zeros(w["var_states_for_edge_states"].shape[0], np.float32)))
  cores = len(os.sched_getaffinity(0))
  t0 = time.perf_counter()
  with concurrent.futures.ThreadPoolExecutor(min(cores, len(jobs))) as ex:
    list(ex.map(lambda j: oracle.run(j[0], j[1], j[2], j[4], iters, 0.5, 1.0), jobs))
  dt = time.perf_counter() - t0
  edges = sum(j[3] for j in jobs)
  return {"value": edges * iters / dt, "unit": "edge-msg updates/s", "cores": min(cores, len(jobs)),
          "kind": "port",
          "sample": f"graphs {list(sample)} of the batch (families a, b, c), {iters} of the "
                    f"{MG_ITERS} iterations each, C oracle, one host thread per graph ({dt:.1f} s)"}


def run_multigraph(args):
  """Config 3: the 256-graph uneven batch as one union plan, 200 iterations at T=1, damping 0.5
  (one step = one run over every graph). The step is captured once in a CUDA graph and replayed
  (value); the same step launched eagerly is reported beside it."""
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import batch, native  # pylint: disable=g-import-not-at-top
  t0 = time.perf_counter()
  wirings, tables, evs, fam = build_multigraph(n_graphs=args.graphs)
  t_gen = time.perf_counter() - t0
  t0 = time.perf_counter()
  gb = batch.GraphBatch(wirings)
  torch.cuda.synchronize()
  t_plan = time.perf_counter() - t0
  dev = torch.device("cuda", 0)
  stream = torch.cuda.current_stream(dev)
  lp = torch.as_tensor(gb.concat(tables), device=dev)
  ev = torch.as_tensor(gb.concat(evs), device=dev)
  n_es = int(gb.layout.perm.shape[0])
  m0 = torch.zeros(n_es, device=dev)
  u = gb.wiring
  num_edges, n_vs = int(u["num_edges"]), int(u["num_var_states"])
  iters = MG_ITERS

  def step():
    out, _ = gb.run(lp, ev, m0, iters, 0.5, 1.0)
    return out

  def timed(fn):
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(args.steps):
      fn()
    s1.record(stream)
    torch.cuda.synchronize()
    return s0.elapsed_time(s1) / args.steps

  for _ in range(args.warmup):   # also settles the autotuner's choices for this batch
    step()
  eager_ms = timed(step)
  # the whole 200-iteration step as one CUDA graph (captured on a side stream, as torch asks)
  graph = torch.cuda.CUDAGraph()
  side = torch.cuda.Stream(dev)
  side.wait_stream(stream)
  with torch.cuda.stream(side):
    step()
  stream.wait_stream(side)
  with torch.cuda.graph(graph):
    captured_out = step()
  for _ in range(args.warmup):
    graph.replay()
  with ClockSampler(0) as clocks:
    ms = timed(graph.replay)
  ref_out = step()
  torch.cuda.synchronize()
  replay_equal = bool(torch.equal(captured_out, ref_out))
  # end to end: host evidence in, beliefs and MAP states out
  ev_host = torch.as_tensor(gb.concat(evs)).pin_memory()
  map_host = torch.empty(int(u["num_variables"]), dtype=torch.int32).pin_memory()

  def step_e2e():
    evd = ev_host.to(dev, non_blocking=True)
    out, _ = gb.run(lp, evd, m0, iters, 0.5, 1.0)
    map_host.copy_(gb.decode(gb.beliefs(evd, out)), non_blocking=True)

  e2e_ms = timed(step_e2e)
  native.profile_read()
  native.profile_enable(True)
  step()
  torch.cuda.synchronize()
  native.profile_enable(False)
  prof = native.profile_read()
  peak, src = peaks()
  p_distinct = int(lp.numel())
  bytes_iter = 4 * (2 * n_es + n_vs) + 4 * p_distinct
  # the K = 64 tcgen05 kernel (family b): per launch every factor's two 64-state messages read
  # and written and each of its variables' 64 sums read once (distinct), plus the tables
  fb = [g for g in range(len(wirings)) if g % 3 == 1]
  side_b = [int(round(np.sqrt(wirings[g]["num_variables"]))) for g in fb]
  f64 = sum(2 * L * (L - 1) for L in side_b)
  v64 = sum(L * L for L in side_b)
  k64_bytes = 4 * (2 * 2 * 64 * f64 + 64 * v64) + 4 * 64 * 64 * len(fb)
  n_k64, k64_ms = prof["pairwise_exp"]
  k64_launch_ms = k64_ms / max(n_k64, 1)
  k64_gbs = k64_bytes / (k64_launch_ms / 1e3) / 1e9 if n_k64 else None
  line = {
      "metric": "edge-msg updates/s", "value": num_edges * iters / (ms / 1e3),
      "unit": "edge-msg updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
      "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
      "dtype": "f32", "data": "synthetic (seed 0)",
      "config": {"workload": f"multigraph{args.graphs}_potts_potts64_deconv", "graphs": args.graphs,
                 "families": fam, "num_iters": iters, "temperature": 1.0, "damping": 0.5,
                 "num_edges": num_edges, "edge_states": n_es, "var_states": n_vs,
                 "shared_table_floats": p_distinct,
                 "execution": "one CUDA graph per step (the 200 iterations captured once, replayed)",
                 "l2": "inputs larger than L2 (%d MB of messages)" % (4 * n_es >> 20)},
      "eager": {"ms_per_step": eager_ms, "value": num_edges * iters / (eager_ms / 1e3)},
      "captured_replay_equals_eager": replay_equal,
      "setup_s": {"generate": round(t_gen, 2), "plan": round(t_plan, 2)},
      "kernel_ms_per_step": {k: v[1] for k, v in prof.items() if v[0]},
      "gpu_launches": int(sum(v[0] for v in prof.values()) * args.steps),
      "roofline": {"bound": "hbm",
                   "kernel": "tc::pairwise_kernel (K = 64 shared tables, tcgen05.mma tf32, TMEM "
                             "accumulators)",
                   "achieved": k64_gbs, "peak": peak, "unit": "GB/s",
                   "frac": k64_gbs / peak if k64_gbs else None,
                   "peak_source": src,
                   "traffic": (lambda r: r * k64_bytes if r else None)(
                       read_traffic(TC_TRAFFIC_FILE, "traffic_per_algorithmic_byte:")),
                   "traffic_note": "ncu DRAM bytes per algorithmic byte of a 64-graph launch "
                                   "(profiles/tc_pairwise_k64_multigraph64.md) x this launch's",
                   "algorithmic_bytes_per_launch": k64_bytes, "launch_ms": k64_launch_ms,
                   "factors": f64},
      "iteration_roofline": {"bytes_per_iter": bytes_iter,
                             "achieved_gbs": bytes_iter * iters / (ms / 1e3) / 1e9,
                             "peak_gbs": peak, "frac": bytes_iter * iters / (ms / 1e3) / 1e9 / peak,
                             "peak_source": src},
      "e2e": {"value": num_edges * iters / (e2e_ms / 1e3), "unit": "edge-msg updates/s",
              "h2d_bytes_per_step": int(ev_host.numel() * 4),
              "d2h_bytes_per_step": int(map_host.numel() * 4)},
      "clocks": clocks.summary(),
  }
  if not args.no_cpu_baseline:
    line["cpu_baseline"] = multigraph_cpu_baseline(wirings, tables, evs, range(min(6, len(wirings))),
                                                   5)
  print(json.dumps(line))
  return 0


WS_WEIGHTS = os.path.join(ROOT, "pgmax_gb300", "warmstart", "weights_potts96_k8.npz")


def run_warmstart(args):
  """Config 5: learned warm start vs cold-start plain BP on 2,000 held-out 96 x 96 toroidal
  spin-glass Potts instances (K = 8, J_e ~ N(0, 0.7^2), unaries N(0, 1), T = 1, damping 0.5), each
  run to max message residual 1e-4 in batches of 250 (residual checked every iteration). The
  network's weights were trained on 20,000 instances of the family (pgmax_gb300.warmstart.train,
  seed 1) and are loaded from the package; the held-out instances use seed 2."""
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300.warmstart import convnet, train  # pylint: disable=g-import-not-at-top
  fam = train.Family(96, 8)
  net = convnet.ConvNet().load(dict(np.load(WS_WEIGHTS)))
  n_eval = 2000
  train.evaluate(fam, net, seed=3, n=250, batch=250)  # warm-up (compilation of paths, caches)
  torch.cuda.synchronize()
  with ClockSampler(0) as clocks:
    res = train.evaluate(fam, net, seed=2, n=n_eval, batch=250)
  per_warm = res["warm_ms"] / res["instances"]
  per_cold = res["cold_ms"] / res["instances"]
  line = {
      "metric": "time to max message residual 1e-4, learned init (ms per instance)",
      "value": per_warm, "unit": "ms/instance", "n_gpus": 1, "steps": 1, "warmup": 1,
      "ms_per_step": res["warm_ms"], "higher_is_better": False, "scaling": "weak",
      "vs_baseline": None, "dtype": "f32 BP, bf16 network",
      "data": "synthetic (seeded spin-glass Potts; held-out seed 2, training seed 1)",
      "config": {"workload": "warmstart_potts96_k8", "instances": res["instances"], "batch": 250,
                 "tolerance": 1e-4, "temperature": 1.0, "damping": 0.5},
      "cold_ms_per_instance": per_cold, "speedup_vs_cold": res["speedup"],
      "iterations": {"cold_mean": res["cold_iters_mean"], "warm_mean": res["warm_iters_mean"],
                     "one_step_init_mean": res["onestep_iters_mean"]},
      "belief_error_vs_converged": {"cold_mean": res["cold_belief_err_mean"],
                                    "cold_max": res["cold_belief_err_max"],
                                    "warm_mean": res["warm_belief_err_mean"],
                                    "warm_max": res["warm_belief_err_max"]},
      "fallback_rate": res["fallback_rate"],
      "clocks": clocks.summary(),
  }
  print(json.dumps(line))
  return 0


def gumbel_evidence(num_var_states, batch, seed):
  rng = np.random.default_rng(seed)
  return rng.gumbel(size=(batch, num_var_states)).astype(np.float32)


class ClockSampler:
  """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

  FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
            "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
            "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

  def __init__(self, device_index):
    self.device_index = device_index
    self.samples = []
    self._stop = threading.Event()
    self._thread = None

  def _run(self):
    while not self._stop.is_set():
      try:
        out = subprocess.run(["nvidia-smi", f"--id={self.device_index}",
                              f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"],
                             capture_output=True, text=True, timeout=5).stdout.strip()
        if out:
          self.samples.append([x.strip() for x in out.split(",")])
      except Exception:  # pylint: disable=broad-except
        return
      self._stop.wait(0.2)

  def __enter__(self):
    self._thread = threading.Thread(target=self._run, daemon=True)
    self._thread.start()
    return self

  def __exit__(self, *exc):
    self._stop.set()
    if self._thread:
      self._thread.join(timeout=10)

  def summary(self):
    if not self.samples:
      return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
    mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    reasons = sorted({names[i] for s in self.samples for i in range(4)
                      if len(s) > 5 + i and s[5 + i].lower() == "active"})
    return {"sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
            "samples": len(self.samples)}


def read_traffic(path=None, key="traffic_bytes_per_full_launch:"):
  """Per-launch DRAM bytes of a kernel from its committed ncu summary (default: the RBM
  pairwise kernel), if any."""
  try:
    for line in open(path or TRAFFIC_FILE):
      if line.startswith(key):
        return float(line.split(":")[1].split()[0])
  except OSError:
    pass
  return None


def peaks():
  try:
    with open(PEAKS) as f:
      p = json.load(f)
    return float(p["hbm_gbs"]), "measured"
  except Exception:  # pylint: disable=broad-except
    return 6800.0, "fallback"


def cpu_baseline(wiring, lp, ev, target_s=12.0):
  """The C oracle on a bounded sample (all host cores, one thread per instance)."""
  from oracle import oracle  # pylint: disable=g-import-not-at-top
  w = oracle.Wiring(wiring)
  cores = len(os.sched_getaffinity(0))
  samples = min(cores, ev.shape[0])
  msgs = np.zeros(w.num_edge_states, np.float32)
  t0 = time.perf_counter()
  oracle.run_batch(w, lp, ev[:samples], msgs, 2, DAMPING, TEMPERATURE, num_threads=cores)
  per_iter = (time.perf_counter() - t0) / 2
  iters = int(max(2, min(ITERS, target_s / max(per_iter, 1e-6))))
  t0 = time.perf_counter()
  oracle.run_batch(w, lp, ev[:samples], msgs, iters, DAMPING, TEMPERATURE, num_threads=cores)
  dt = time.perf_counter() - t0
  return {
      "value": samples * NUM_EDGES * iters / dt,
      "unit": "edge-msg updates/s",
      "cores": cores,
      "kind": "port",
      "sample": f"{samples} of the {BATCH} samples x {iters} of the {ITERS} iterations "
                f"({dt:.1f} s, C oracle, one OpenMP thread per sample)",
  }


def dist_setup(n_gpus):
  """Replicas: one process per GPU under torchrun, each with its own batch (weak scaling)."""
  from pgmax_gb300 import distributed  # pylint: disable=g-import-not-at-top
  del n_gpus
  return distributed.init("nccl")


def run_reference(args):
  world, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
  if rank != 0:
    return 0
  from pgmax_gb300 import infer  # pylint: disable=g-import-not-at-top
  from oracle import oracle  # pylint: disable=g-import-not-at-top
  fg, _, _ = build_rbm()
  ctx = infer.InfererContext(fg.bp_state)
  w = oracle.Wiring(ctx.flat_wiring())
  lp = np.asarray(fg.fg_state.log_potentials, np.float32)
  ev = gumbel_evidence(fg.fg_state.num_var_states, BATCH, 1)
  cores = len(os.sched_getaffinity(0))
  samples = min(cores, BATCH)
  msgs = np.zeros(w.num_edge_states, np.float32)
  iters = 4
  times = []
  for step in range(args.warmup + args.steps):
    t0 = time.perf_counter()
    oracle.run_batch(w, lp, ev[:samples], msgs, iters, DAMPING, TEMPERATURE, num_threads=cores)
    dt = time.perf_counter() - t0
    if step >= args.warmup:
      times.append(dt)
  total = sum(times)
  value = samples * NUM_EDGES * iters * len(times) / total
  sample = (f"each step: {samples} of the {BATCH} samples x {iters} of the {ITERS} iterations "
            f"(C oracle, float32 restatement of PGMax run_with_diffs; PGMax itself needs jax, "
            f"absent here)")
  line = {
      "impl": "reference", "metric": "edge-msg updates/s", "value": value,
      "unit": "edge-msg updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
      "ms_per_step": 1e3 * total / len(times), "higher_is_better": True, "scaling": "weak",
      "vs_baseline": None, "dtype": "f32", "data": "synthetic",
      "config": {"workload": "rbm784x500_perturb_and_map", "batch": BATCH, "num_iters": ITERS,
                 "temperature": TEMPERATURE, "damping": DAMPING, "parallelism": "cpu"},
      "cpu_baseline": {"value": value, "unit": "edge-msg updates/s", "cores": cores,
                       "kind": "port", "sample": sample},
      "e2e": {"value": value, "unit": "edge-msg updates/s", "h2d_bytes_per_step": 0,
              "d2h_bytes_per_step": 0},
  }
  print(json.dumps(line))
  return 0


def main():
  ap = argparse.ArgumentParser()
  ap.add_argument("--gpus", type=int, default=1)
  ap.add_argument("--steps", type=int, default=10)
  ap.add_argument("--warmup", type=int, default=3)
  ap.add_argument("--impl", default="pgbp", choices=["pgbp", "reference"])
  ap.add_argument("--no-cpu-baseline", action="store_true")
  ap.add_argument("--graphs", type=int, default=MG_GRAPHS,
                  help="graphs of the multigraph workload (256; fewer for small profiling cases)")
  ap.add_argument("--batch", type=int, default=BATCH,
                  help="samples of the sdlp and energy workloads (128; fewer for profiling cases)")
  ap.add_argument("--exec-path", default="auto", choices=["auto", "multi", "small", "cluster"],
                  help="execution path of the ising workload (auto: timed choice)")
  ap.add_argument("--workload", default="rbm",
                  choices=["rbm", "ising", "adjoint", "multigraph", "warmstart", "energy", "sdlp",
                           "enum"],
                  help="rbm: the headline RBM perturb-and-MAP batch (default); ising: the 50x50 "
                       "toroidal Ising configuration; adjoint: differentiable BP on 64x64 grids; "
                       "multigraph: the 256-graph uneven batch; warmstart: learned init vs "
                       "cold-start BP; energy: compute_energy of the RBM batch's decodings; "
                       "sdlp: the smooth dual LP-MAP solver on the RBM batch; enum: "
                       "perturb-and-MAP on 3,000 ternary 10-state EnumFactors")
  args = ap.parse_args()
  if args.warmup < 3:
    args.warmup = 3
  if args.impl == "reference":
    return run_reference(args)
  if args.workload == "ising":
    return run_ising(args)
  if args.workload == "adjoint":
    return run_adjoint(args)
  if args.workload == "multigraph":
    return run_multigraph(args)
  if args.workload == "warmstart":
    return run_warmstart(args)
  if args.workload == "energy":
    return run_energy(args)
  if args.workload == "sdlp":
    return run_sdlp(args)
  if args.workload == "enum":
    return run_enum(args)

  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import infer, native  # pylint: disable=g-import-not-at-top

  world, rank, local = dist_setup(args.gpus)
  torch.cuda.set_device(local)
  dev = torch.device("cuda", local)

  fg, hidden, visible = build_rbm(seed=0)
  bp = infer.BP(fg.bp_state, temperature=TEMPERATURE)
  ctx = bp.context
  plan = ctx.plan
  nvs = fg.fg_state.num_var_states
  n_es = fg.fg_state.total_factor_num_states

  ev_host = gumbel_evidence(nvs, BATCH, 1000 + rank)
  lp_dev = torch.as_tensor(np.asarray(fg.fg_state.log_potentials, np.float32), device=dev)
  msgs0 = torch.zeros(n_es, dtype=torch.float32, device=dev)
  # the unperturbed evidence (zero: the biases are in the unary factors' potentials)
  base = bp.init()
  seeds = iter(range((rank + 1) << 40, 1 << 62))

  def step_device():
    # fresh Gumbel noise on every unary state of every sample, generated inside the run
    out = bp.run_perturbed(base, ITERS, next(seeds), BATCH, damping=DAMPING,
                           temperature=TEMPERATURE)
    beliefs = bp.get_beliefs(out)
    return infer.decode_map_states(beliefs)

  stream = torch.cuda.current_stream(dev)

  from pgmax_gb300 import distributed  # pylint: disable=g-import-not-at-top

  def barrier():
    distributed.barrier()
    torch.cuda.synchronize(dev)

  def max_over_ranks(x):
    return distributed.max_over_ranks(x, device=dev)

  for _ in range(args.warmup):
    step_device()
  barrier()
  start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  with ClockSampler(local) as clocks:
    barrier()
    start.record(stream)
    for _ in range(args.steps):
      step_device()
    stop.record(stream)
    barrier()
  ms = max_over_ranks(start.elapsed_time(stop))
  ms_per_step = ms / args.steps
  units = BATCH * NUM_EDGES * ITERS * args.steps * world
  value = units / (ms / 1e3)

  # per-kernel device time: the same K steps again, every launch bracketed by CUDA events
  # (pgbp_profile_*); kept out of the headline timing above because the events add device time
  native.profile_read()
  native.profile_enable(True)
  barrier()
  for _ in range(args.steps):
    step_device()
  barrier()
  native.profile_enable(False)
  prof = native.profile_read()

  # end to end through the public API: the seed in (the noise is made on the GPU), every
  # sample's MAP states copied back to pinned host memory
  map_h = torch.empty((BATCH, NH), dtype=torch.int32).pin_memory()
  map_v = torch.empty((BATCH, NV), dtype=torch.int32).pin_memory()

  def step_e2e():
    out = bp.run_perturbed(base, ITERS, next(seeds), BATCH, damping=DAMPING,
                           temperature=TEMPERATURE)
    dec = infer.decode_map_states(bp.get_beliefs(out))
    map_h.copy_(dec[hidden], non_blocking=True)
    map_v.copy_(dec[visible], non_blocking=True)

  # the same with the noise drawn on the host and copied in every step (bp.run on host evidence)
  ev_pinned = torch.as_tensor(ev_host).pin_memory()

  def step_e2e_host_noise():
    ev_d = ev_pinned.to(dev, non_blocking=True)
    a = infer.BPArrays(log_potentials=lp_dev, ftov_msgs=msgs0, evidence=ev_d)
    out = bp.run(a, num_iters=ITERS, damping=DAMPING, temperature=TEMPERATURE)
    dec = infer.decode_map_states(bp.get_beliefs(out))
    map_h.copy_(dec[hidden], non_blocking=True)
    map_v.copy_(dec[visible], non_blocking=True)

  def timed(fn):
    for _ in range(args.warmup):
      fn()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
      fn()
    e1.record(stream)
    barrier()
    return max_over_ranks(e0.elapsed_time(e1))

  e2e_ms = timed(step_e2e)
  e2e_value = units / (e2e_ms / 1e3)
  host_noise_ms = timed(step_e2e_host_noise)

  # roofline of the dominant kernel (dense pairwise Enum, binary edges stored as one slot each):
  # its average launch time comes from the profiled repetition of the timed steps.
  # per launch it must read and write 2 slots per (factor, instance), read the 2 + 2 variable sums
  # of each factor (N_vs distinct per instance) and the shared tables once.
  info = plan.info
  f_pw = info["num_enum_pairwise_factors"]
  algo_bytes = BATCH * 4 * (2 * 2 * f_pw) + BATCH * 4 * nvs + 4 * (4 * f_pw)
  n_launch, pw_ms = prof["pairwise"]
  achieved = algo_bytes / (pw_ms / max(n_launch, 1) / 1e3) / 1e9 if n_launch else None
  peak, peak_kind = peaks()
  total_prof_ms = sum(v[1] for v in prof.values())
  gpu_launches = sum(v[0] for v in prof.values())
  n_slots = info["num_slots"]
  p_total = int(plan.num_potentials)
  # whole iteration: variable sums read every slot; the factor pass reads and writes every slot
  iter_bytes = BATCH * 4 * (3 * n_slots + 3 * nvs) + 4 * p_total
  # the same iteration counted as the uncompressed formula B*4*(2*E_s + N_vs) + 4*P
  iter_bytes_uncompressed = BATCH * 4 * (2 * n_es + nvs) + 4 * p_total
  iter_s = (ms / 1e3) / (ITERS * args.steps)

  line = {
      "metric": "edge-msg updates/s",
      "value": value,
      "unit": "edge-msg updates/s",
      "n_gpus": world,
      "steps": args.steps,
      "warmup": args.warmup,
      "ms_per_step": ms_per_step,
      "higher_is_better": True,
      "scaling": "weak",
      "vs_baseline": None,
      "dtype": "f32",
      "data": "synthetic (seeded RBM weights N(0,0.1^2), biases N(0,0.5^2), Gumbel(0,1) evidence)",
      "config": {"workload": "rbm784x500_perturb_and_map", "batch": BATCH, "num_iters": ITERS,
                 "temperature": TEMPERATURE, "damping": DAMPING, "num_edges": NUM_EDGES,
                 "edge_states": n_es, "parallelism": "replicas" if world > 1 else "single",
                 "l2": "inputs larger than L2 (804 MB of messages per buffer)"},
      "e2e": {"value": e2e_value, "unit": "edge-msg updates/s",
              "h2d_bytes_per_step": 0,
              "d2h_bytes_per_step": int((map_h.numel() + map_v.numel()) * 4),
              "noise": "Gumbel(0,1) generated on the GPU inside the run (pgbp_run_perturbed)"},
      "e2e_host_noise": {"value": units / (host_noise_ms / 1e3), "unit": "edge-msg updates/s",
                         "h2d_bytes_per_step": int(ev_pinned.numel() * 4),
                         "d2h_bytes_per_step": int((map_h.numel() + map_v.numel()) * 4),
                         "noise": "drawn on the host, copied in every step (bp.run)"},
      "gpu_launches": gpu_launches,
      "roofline": {
          "bound": "hbm",
          "kernel": "pairwise22_x4_kernel<T0> (dense 2x2 pairwise Enum, fused damping/normalise/clip)",
          "achieved": achieved, "peak": peak, "unit": "GB/s",
          "frac": (achieved / peak) if achieved else None,
          "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({peak_kind})",
          "traffic": read_traffic(),
          "algorithmic_bytes_per_launch": algo_bytes,
          "launch_ms": pw_ms / max(n_launch, 1),
      },
      "kernel_time_share": {k: (v[1] / total_prof_ms if total_prof_ms else None)
                            for k, v in prof.items() if v[0]},
      "iteration_roofline": {
          "bytes_per_iter": iter_bytes,
          "achieved_gbs": iter_bytes / iter_s / 1e9,
          "frac": iter_bytes / iter_s / 1e9 / peak,
          "bytes_per_iter_uncompressed_formula": iter_bytes_uncompressed,
          "uncompressed_equivalent_gbs": iter_bytes_uncompressed / iter_s / 1e9,
      },
  }
  line["clocks"] = clocks.summary()
  if rank == 0 and not args.no_cpu_baseline:
    lp = np.asarray(fg.fg_state.log_potentials, np.float32)
    line["cpu_baseline"] = cpu_baseline(ctx.flat_wiring(), lp, ev_host)
  if rank == 0:
    print(json.dumps(line))
  if world > 1:
    import torch.distributed as dist  # pylint: disable=g-import-not-at-top
    dist.destroy_process_group()
  return 0


if __name__ == "__main__":
  sys.exit(main())
