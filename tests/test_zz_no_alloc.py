"""pgbp_run_static_scratch: BP for callers that cannot allocate device memory while running.

Such callers (code inside a host framework that owns all device memory, services with a fixed
budget reserved at start-up) get the run's scratch from one static device array instead of a
workspace. This test calls the entry point through the C ABI twice in a row, on different inputs,
and checks each result against pgbp_run with a caller workspace: the same kernels run on the same
inputs, so messages and residuals must be identical bit for bit. It also checks that a run needing
more scratch than the static array holds is refused with a clear error, and that the caller's
current device is the same after a call as before it. The file is named to be collected last; it
also passes when run on its own.
"""

import ctypes

import numpy as np
import pytest

import fixtures

pytestmark = pytest.mark.gpu


def _setup(name):
  import torch  # pylint: disable=g-import-not-at-top
  from pgmax_gb300 import engine, native  # pylint: disable=g-import-not-at-top
  f = fixtures.load(f"{fixtures.FIXTURES}/{name}.npz")
  plan = engine.Plan(f["wiring"])
  return torch, native, plan, f


def _reference_run(torch, native, plan, lp, ev, msgs, B, iters, damping, temperature):
  out = torch.empty((B, plan.num_edge_states), device="cuda", dtype=torch.float32)
  deltas = torch.empty((B, max(iters, 1)), device="cuda", dtype=torch.float32)
  ws_bytes = int(plan.lib.pgbp_workspace_size(plan.handle, B, iters))
  ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
  native.check(plan.lib.pgbp_run(plan.handle, plan._stream(), B, lp.data_ptr(), lp.stride(0),  # pylint: disable=protected-access
                                 ev.data_ptr(), ev.stride(0), msgs.data_ptr(), msgs.stride(0),
                                 out.data_ptr(), deltas.data_ptr(), iters, damping, temperature,
                                 ws.data_ptr(), ws_bytes), "pgbp_run")
  return out, deltas


def _static_run(torch, native, plan, lp, ev, msgs, B, iters, damping, temperature):
  out = torch.full((B, plan.num_edge_states), float("nan"), device="cuda", dtype=torch.float32)
  deltas = torch.full((B, max(iters, 1)), float("nan"), device="cuda", dtype=torch.float32)
  native.check(plan.lib.pgbp_run_static_scratch(
      plan.handle, plan._stream(), B, lp.data_ptr(), lp.stride(0), ev.data_ptr(), ev.stride(0),  # pylint: disable=protected-access
      msgs.data_ptr(), msgs.stride(0), out.data_ptr(), deltas.data_ptr(), iters, damping,
      temperature), "pgbp_run_static_scratch")
  return out, deltas


@pytest.mark.parametrize("name", ["case_mixed_T1", "case_deconv_T0"])
def test_static_scratch_matches_workspace_run_twice(name):
  torch, native, plan, f = _setup(name)
  torch.cuda.set_device(0)
  rng = np.random.default_rng(11)
  B, iters = 9, 12
  T = float(f["temperature"])
  for call in range(2):
    ev = torch.as_tensor((f["evidence"][None] + rng.gumbel(size=(B,) + f["evidence"].shape))
                         .astype(np.float32), device="cuda")
    msgs = torch.as_tensor((f["ftov_msgs_in"][None] + rng.normal(
        size=(B,) + f["ftov_msgs_in"].shape)).astype(np.float32), device="cuda")
    lp = torch.as_tensor((f["log_potentials"][None] + 0.1 * rng.normal(
        size=(B,) + f["log_potentials"].shape)).astype(np.float32), device="cuda")
    want, want_d = _reference_run(torch, native, plan, lp, ev, msgs, B, iters, 0.5, T)
    got, got_d = _static_run(torch, native, plan, lp, ev, msgs, B, iters, 0.5, T)
    torch.cuda.synchronize()
    assert torch.cuda.current_device() == 0
    np.testing.assert_array_equal(got.cpu().numpy(), want.cpu().numpy(), err_msg=f"call {call}")
    np.testing.assert_array_equal(got_d.cpu().numpy(), want_d.cpu().numpy(),
                                  err_msg=f"call {call}")


def test_static_scratch_rejects_runs_larger_than_the_array():
  torch, native, plan, f = _setup("case_ising50_T0")
  B = 512  # 2 x 20,000 edge states x 512 instances of messages alone exceed 32 MiB
  lp = torch.as_tensor(f["log_potentials"], device="cuda")[None].expand(B, -1)
  ev = torch.as_tensor(f["evidence"], device="cuda")[None].expand(B, -1)
  msgs = torch.as_tensor(f["ftov_msgs_in"], device="cuda")[None].expand(B, -1)
  out = torch.empty((B, plan.num_edge_states), device="cuda")
  rc = plan.lib.pgbp_run_static_scratch(plan.handle, plan._stream(), B, lp.data_ptr(), 0,  # pylint: disable=protected-access
                                        ev.data_ptr(), 0, msgs.data_ptr(), 0, out.data_ptr(), None,
                                        5, 0.5, 0.0)
  assert rc == 5
  assert b"PGBP_STATIC_SCRATCH_BYTES" in plan.lib.pgbp_last_error()
