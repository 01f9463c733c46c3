"""Replicas over several GPUs: one process per GPU, each running its own share of the instances.

Belief propagation over a batch of independent instances (perturb-and-MAP samples, graphs of a
multi-graph batch) shards with no data-path collective: rank r runs instances
[shard_range(n, world, r)) and the only communication is collecting results and the slowest
rank's time. Single-process use (world 1) needs no torch.distributed at all.
"""

import os
from typing import Callable, List, Sequence, Tuple


def world_info() -> Tuple[int, int, int]:
  """(world size, rank, local rank) from the torchrun environment (1, 0, 0 without it)."""
  return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
          int(os.environ.get("LOCAL_RANK", "0")))


def shard_range(n: int, world: int, rank: int) -> Tuple[int, int]:
  """Contiguous, as-even-as-possible split of n instances: the first n % world ranks get one more."""
  if world <= 0 or not 0 <= rank < world:
    raise ValueError(f"rank {rank} of world {world}")
  base, extra = divmod(n, world)
  start = rank * base + min(rank, extra)
  return start, start + base + (1 if rank < extra else 0)


def init(backend: str = "nccl") -> Tuple[int, int, int]:
  """Joins the process group when launched under torchrun with more than one process."""
  world, rank, local = world_info()
  if world > 1:
    import torch.distributed as dist  # pylint: disable=g-import-not-at-top
    if not dist.is_initialized():
      dist.init_process_group(backend)
  return world, rank, local


def barrier() -> None:
  import torch.distributed as dist  # pylint: disable=g-import-not-at-top
  if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
    dist.barrier()


def max_over_ranks(x: float, device=None) -> float:
  """The maximum of a per-rank number (e.g. elapsed time: the job is as slow as its slowest rank)."""
  import torch  # pylint: disable=g-import-not-at-top
  import torch.distributed as dist  # pylint: disable=g-import-not-at-top
  if not (dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1):
    return x
  t = torch.tensor([x], dtype=torch.float64, device=device)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  return float(t.item())


def gather_rows(local, n_total: int, device=None):
  """Concatenates every rank's [n_r, ...] rows (n_r from shard_range) into the full [n_total, ...]
  array, on every rank."""
  import torch  # pylint: disable=g-import-not-at-top
  import torch.distributed as dist  # pylint: disable=g-import-not-at-top
  if not (dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1):
    return local
  world = dist.get_world_size()
  sizes = [shard_range(n_total, world, r) for r in range(world)]
  width = max(b - a for a, b in sizes)
  padded = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
  padded[:local.shape[0]] = local
  parts = [torch.empty_like(padded) for _ in range(world)]
  dist.all_gather(parts, padded)
  return torch.cat([p[:b - a] for p, (a, b) in zip(parts, sizes)], dim=0)


def run_sharded(run_fn: Callable, inputs: Sequence, n_total: int):
  """Runs `run_fn` on this rank's rows of every input ([n_total, ...] arrays) and gathers the
  [n_total, ...] result on every rank."""
  import torch.distributed as dist  # pylint: disable=g-import-not-at-top
  world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
  rank = dist.get_rank() if world > 1 else 0
  a, b = shard_range(n_total, world, rank)
  out = run_fn(*[x[a:b] for x in inputs])
  return gather_rows(out, n_total)
