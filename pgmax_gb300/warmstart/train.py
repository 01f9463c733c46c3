"""Data, training and evaluation of the learned warm start on the spin-glass Potts family.

  run_to_tolerance   plain BP (pgbp_run) in chunks until every instance's max message residual
                     is below a tolerance; per-instance iteration counts
  make_dataset       instances run to residual 1e-5 from a cold start: network inputs, and the
                     converged messages minus the closed-form one-step messages as targets
  train              Adam on the mean-centred squared error of the predicted correction
  evaluate           held-out instances run to 1e-4 from the learned init and from a cold start:
                     wall time (the warm start's features, one-step messages and network
                     included), iterations, belief error against the converged solution, and the
                     fallback rate (warm starts that miss the tolerance are rerun cold)

`python -m pgmax_gb300.warmstart.train --out weights.npz` trains on the GPU and saves the weights.
"""

import argparse
import dataclasses
import time
from typing import Dict, Optional

import numpy as np

from . import convnet, potts

L_DEFAULT, K_DEFAULT, SIGMA = 96, 8, 0.7
DAMPING, TEMPERATURE = 0.5, 1.0


def _torch():
  import torch  # pylint: disable=g-import-not-at-top
  return torch


@dataclasses.dataclass
class Family:
  """The compiled graph of one (L, K) toroidal Potts family and its index maps."""
  L: int
  K: int

  def __post_init__(self):
    from .. import engine  # pylint: disable=g-import-not-at-top
    torch = _torch()
    self.wiring = potts.torus_wiring(self.L, self.K)
    self.plan = engine.Plan(self.wiring)
    self.index = torch.as_tensor(potts.message_index(self.L, self.K), device="cuda")
    self.n_es = int(self.wiring["var_states_for_edge_states"].shape[0])

  def problems(self, seed: int, n: int):
    """(couplings J [n, 2 L^2], unaries u [n, L^2 K], potentials [n, P], evidence [n, N_vs]) of n
    instances, on the GPU."""
    torch = _torch()
    J, u = potts.sample(seed, n, self.L, self.K, SIGMA)
    J = torch.as_tensor(J, device="cuda")
    u = torch.as_tensor(u, device="cuda")
    return J, u, potts.potentials(J, self.K).contiguous(), u

  def warm_inputs(self, J, u):
    """The network's input features [n, L, L, 64] (BF16) and the closed-form one-step messages
    [n, L, L, 32] it corrects (one pgbp_potts_features launch): the part of a warm start computed
    before the network runs."""
    return potts.features_and_messages(J, u, self.L, self.K)

  def instances(self, seed: int, n: int):
    """(features [n, L, L, 64] BF16, one-step messages [n, L, L, 32], potentials [n, P],
    evidence [n, N_vs]) on the GPU."""
    J, u, lp, ev = self.problems(seed, n)
    x, m1 = self.warm_inputs(J, u)
    return x, m1, lp, ev

  def to_channels(self, msgs):
    """Flat messages [n, E_s] -> network layout [n, L, L, 4 K]."""
    return msgs[:, self.index].reshape(msgs.shape[0], self.L, self.L, 4 * self.K)

  def from_channels(self, out):
    """Network output [n, L, L, 4 K] -> flat messages [n, E_s]."""
    torch = _torch()
    msgs = torch.empty((out.shape[0], self.n_es), dtype=torch.float32, device=out.device)
    msgs[:, self.index] = out.reshape(out.shape[0], -1)
    return msgs


def run_to_tolerance(plan, lp, ev, msgs, tol: float, max_iters: int, chunk: int = 1):
  """BP from `msgs` until every instance's residual is below `tol` or `max_iters` iterations ran
  (pgbp_run_to_tolerance, residual tested every `chunk` iterations). Returns (messages,
  iterations [B] to reach tol (-1 if never), iterations run)."""
  out, first, ran = plan.run_to_tolerance(lp, ev, msgs, tol, max_iters, DAMPING, TEMPERATURE,
                                          check_every=chunk)
  return out, first.to(_torch().int64), ran


def make_dataset(fam: Family, seed: int, n: int, batch: int = 256, tol: float = 1e-5,
                 max_iters: int = 3000):
  """Network inputs and targets for n instances: the converged messages (cold starts run to
  tol) minus the one-step messages, i.e. the correction the network learns. Instances that do not
  converge within max_iters are dropped."""
  torch = _torch()
  xs, ys, kept, iters = [], [], 0, []
  for k in range(0, n, batch):
    m = min(batch, n - k)
    x, m1, lp, ev = fam.instances(seed * 1_000_003 + k, m)
    msgs0 = torch.zeros((m, fam.n_es), device="cuda")
    msgs, first, _ = run_to_tolerance(fam.plan, lp, ev, msgs0, tol, max_iters, chunk=10)
    ok = (first >= 0).to("cuda")
    xs.append(x[ok])
    ys.append((fam.to_channels(msgs) - m1)[ok])
    kept += int(ok.sum())
    iters.append(first[first >= 0])
  return torch.cat(xs), torch.cat(ys), {"kept": kept, "requested": n,
                                         "median_iters_to_tol": float(torch.cat(iters).float().median())}


def train(net: convnet.ConvNet, x, y, epochs: int = 8, batch: int = 32, lr: float = 1e-3,
          seed: int = 0, log=None, target_scale: float = 30.0):
  """Adam epochs over (x, y); the network learns y * target_scale. Returns per-epoch losses in
  message units squared."""
  torch = _torch()
  n = x.shape[0]
  net.target_scale = target_scale
  g = torch.Generator().manual_seed(seed)
  losses = []
  for epoch in range(epochs):
    order = torch.randperm(n, generator=g)
    total, steps = 0.0, 0
    for k in range(0, n - batch + 1, batch):
      idx = order[k:k + batch].to("cuda")
      # the learning rate halves three times over the run
      loss = net.train_step(x[idx], y[idx] * target_scale,
                            lr * (0.5 ** (epoch // max(1, epochs // 4))))
      total += float(loss) / target_scale ** 2
      steps += 1
    losses.append(total / max(steps, 1))
    if log:
      log(f"epoch {epoch}: loss {losses[-1]:.5f}")
  return losses


def evaluate(fam: Family, net: Optional[convnet.ConvNet], seed: int, n: int, batch: int = 250,
             tol: float = 1e-4, max_iters: int = 3000, chunk: int = 1) -> Dict:
  """Warm (learned init: one-step messages plus the network's correction) vs cold (zeros) runs
  to `tol` on n held-out instances; also the one-step messages alone as the init ("onestep")."""
  torch = _torch()
  res = {"cold_ms": 0.0, "warm_ms": 0.0, "cold_iters": [], "warm_iters": [], "fallbacks": 0,
         "instances": 0, "cold_belief_err": [], "warm_belief_err": [], "skipped": 0,
         "onestep_iters": []}
  for k in range(0, n, batch):
    m = min(batch, n - k)
    J, u, lp, ev = fam.problems(seed * 1_000_003 + k, m)
    zeros = torch.zeros((m, fam.n_es), device="cuda")
    # the converged plain solution (the judge of belief error)
    ref, ref_first, _ = run_to_tolerance(fam.plan, lp, ev, zeros, 1e-5, max_iters, chunk=10)
    ok = ref_first >= 0
    res["skipped"] += int((~ok).sum())
    ref_m = fam.plan.marginals(fam.plan.beliefs(ev, ref))
    # cold start
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cold, cold_first, _ = run_to_tolerance(fam.plan, lp, ev, zeros, tol, max_iters, chunk)
    torch.cuda.synchronize()
    res["cold_ms"] += 1e3 * (time.perf_counter() - t0)
    # one-step init alone (iterations only)
    _, m1_only = fam.warm_inputs(J, u)
    _, one_first, _ = run_to_tolerance(fam.plan, lp, ev, fam.from_channels(m1_only), tol,
                                       max_iters, chunk)
    res["onestep_iters"].append(one_first[ok & (one_first >= 0)])
    # learned warm start, its inputs included; instances that miss the tolerance fall back to a
    # cold start
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if net is not None:
      x, m1 = fam.warm_inputs(J, u)
      init = fam.from_channels(m1 + net.messages(x))
    else:
      init = zeros
    warm, warm_first, _ = run_to_tolerance(fam.plan, lp, ev, init, tol, max_iters, chunk)
    miss = warm_first < 0
    if bool(miss.any()):
      idx = miss.nonzero().squeeze(1).to("cuda")
      fb, fb_first, _ = run_to_tolerance(fam.plan, lp[idx], ev[idx], zeros[idx], tol, max_iters,
                                         chunk)
      warm[idx] = fb
      warm_first[miss] = fb_first.cpu() + max_iters
      res["fallbacks"] += int(miss.sum())
    torch.cuda.synchronize()
    res["warm_ms"] += 1e3 * (time.perf_counter() - t0)
    for name, msgs, first in (("cold", cold, cold_first), ("warm", warm, warm_first)):
      mg = fam.plan.marginals(fam.plan.beliefs(ev, msgs))
      err = (mg - ref_m).abs().max(dim=1).values.cpu()
      res[f"{name}_belief_err"].append(err[ok])
      res[f"{name}_iters"].append(first[ok])
    res["instances"] += m
  out = {k: v for k, v in res.items() if not isinstance(v, list)}
  for name in ("cold", "warm"):
    it = torch.cat(res[f"{name}_iters"]).float()
    err = torch.cat(res[f"{name}_belief_err"])
    out[f"{name}_iters_mean"] = float(it.mean())
    out[f"{name}_iters_median"] = float(it.median())
    out[f"{name}_belief_err_mean"] = float(err.mean())
    out[f"{name}_belief_err_max"] = float(err.max())
  out["onestep_iters_mean"] = float(torch.cat(res["onestep_iters"]).float().mean())
  out["speedup"] = out["cold_ms"] / max(out["warm_ms"], 1e-9)
  out["fallback_rate"] = out["fallbacks"] / max(out["instances"], 1)
  return out


def main(argv=None):
  ap = argparse.ArgumentParser()
  ap.add_argument("--out", required=True)
  ap.add_argument("--L", type=int, default=L_DEFAULT)
  ap.add_argument("--train", type=int, default=20000)
  ap.add_argument("--eval", type=int, default=2000)
  ap.add_argument("--epochs", type=int, default=12)
  ap.add_argument("--batch", type=int, default=32)
  ap.add_argument("--lr", type=float, default=3e-4)
  ap.add_argument("--target-scale", type=float, default=30.0)
  args = ap.parse_args(argv)
  fam = Family(args.L, K_DEFAULT)
  t0 = time.perf_counter()
  x, y, info = make_dataset(fam, seed=1, n=args.train)
  print(f"dataset: {info} in {time.perf_counter() - t0:.1f} s", flush=True)
  net = convnet.ConvNet(seed=0)
  t0 = time.perf_counter()
  losses = train(net, x, y, epochs=args.epochs, batch=args.batch, lr=args.lr,
                 log=lambda s: print(s, flush=True), target_scale=args.target_scale)
  print(f"training: {time.perf_counter() - t0:.1f} s, losses {losses}", flush=True)
  np.savez(args.out, **net.state())
  res = evaluate(fam, net, seed=2, n=args.eval)
  print(res, flush=True)


if __name__ == "__main__":
  main()
