"""Replica logic over two ranks (gloo, CPU): sharding, gathering, slowest-rank timing.

BP instances are independent, so N GPUs run N disjoint shards of the batch with no collective in
the data path; these tests run that host logic with world_size 2 on CPU, with a host stand-in for
the per-rank computation (no GPU is involved).
"""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pgmax_gb300 import distributed


def test_shard_range_covers_every_instance_once():
  for n in (0, 1, 5, 128, 1000):
    for world in (1, 2, 3, 8):
      seen = []
      for r in range(world):
        a, b = distributed.shard_range(n, world, r)
        assert 0 <= a <= b <= n
        seen.extend(range(a, b))
      assert seen == list(range(n))
  with pytest.raises(ValueError):
    distributed.shard_range(4, 2, 2)


def _free_port():
  s = socket.socket()
  s.bind(("127.0.0.1", 0))
  port = s.getsockname()[1]
  s.close()
  return port


def _worker(rank, world, port, n_total, q):
  os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                     "WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank)})
  try:
    w, r, _ = distributed.init("gloo")
    assert (w, r) == (world, rank)
    rng = np.random.default_rng(0)
    evidence = torch.as_tensor(rng.normal(size=(n_total, 6)).astype(np.float32))
    # host stand-in for one shard's BP run: any per-instance function of the instance's rows
    out = distributed.run_sharded(lambda ev: ev.cumsum(dim=1) * 2.0, [evidence], n_total)
    slowest = distributed.max_over_ranks(float(rank + 1))
    distributed.barrier()
    q.put((rank, out.numpy(), slowest))
  finally:
    if dist.is_initialized():
      dist.destroy_process_group()


@pytest.mark.parametrize("n_total", [7, 128])
def test_two_replicas_gather_the_single_process_result(n_total):
  ctx = mp.get_context("spawn")
  q = ctx.Queue()
  port = _free_port()
  procs = [ctx.Process(target=_worker, args=(r, 2, port, n_total, q)) for r in range(2)]
  for p in procs:
    p.start()
  results = [q.get(timeout=120) for _ in procs]
  for p in procs:
    p.join(timeout=60)
    assert p.exitcode == 0
  rng = np.random.default_rng(0)
  evidence = torch.as_tensor(rng.normal(size=(n_total, 6)).astype(np.float32))
  want = (evidence.cumsum(dim=1) * 2.0).numpy()
  for _, out, slowest in results:
    np.testing.assert_array_equal(out, want)
    assert slowest == 2.0
