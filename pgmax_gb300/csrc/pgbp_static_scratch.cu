// pgbp_run_static_scratch: belief propagation without any device allocation.
//
// Some callers of this library cannot call cudaMalloc at the time they run inference, and cannot
// hand over a scratch buffer either: code executing inside a host framework that owns all device
// memory (a custom call or plugin that is given only its input and output buffers), and services
// that reserve a fixed memory budget at start-up and forbid allocation afterwards. For them this
// entry point runs exactly the computation of pgbp_run, with its scratch taken from one
// statically sized array in device memory that every GPU loading this library holds until the
// process exits.
//
// Contract (see include/pgbp.h):
//   * scratch is the file-scope array below, PGBP_STATIC_SCRATCH_BYTES (32 MiB) on each device;
//     a call whose scratch need (pgbp_workspace_size) exceeds it is rejected with
//     PGBP_ERR_WORKSPACE before anything is enqueued;
//   * no cudaMalloc, cudaFree or allocating library routine is called;
//   * the first call on a device looks up the array's device address with cudaGetSymbolAddress
//     (with that device current) and caches it; make that first call before any stream capture.
//     A device reset frees the array together with every plan, so the cached address, like the
//     plans, must not be used across a cudaDeviceReset;
//   * the caller's current device is the same after the call as before it;
//   * every call shares the one array: calls that overlap on the GPU (different streams, or
//     different host threads without ordering) race on it. The part that must start at zero (the
//     per-iteration residual accumulators) is cleared by every call; everything else is written
//     before it is read.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "pgbp_internal.h"

namespace {

constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[PGBP_STATIC_SCRATCH_BYTES];

std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_static_scratch on `device` (current); looked up once per device.
int scratch_address(int device, void** out) {
  if (device < 0 || device >= kMaxDevices) {
    return pgbp::set_last_error(PGBP_ERR_INVALID_ARGUMENT, "device index out of range");
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (g_scratch_ptr[device] == nullptr) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
      char msg[256];
      snprintf(msg, sizeof(msg), "cudaGetSymbolAddress(static scratch): %s",
               cudaGetErrorString(e));
      return pgbp::set_last_error(PGBP_ERR_CUDA, msg);
    }
    g_scratch_ptr[device] = ptr;
  }
  *out = g_scratch_ptr[device];
  return PGBP_OK;
}

}  // namespace

extern "C" int pgbp_run_static_scratch(const pgbp_plan* plan, void* stream, int64_t batch,
                                       const float* log_potentials, int64_t lp_stride,
                                       const float* evidence, int64_t ev_stride,
                                       const float* msgs_in, int64_t msgs_stride, float* msgs_out,
                                       float* deltas, int64_t num_iters, double damping,
                                       double temperature) {
  if (!plan) return pgbp::set_last_error(PGBP_ERR_INVALID_ARGUMENT, "null plan");
  if (batch <= 0) return pgbp::set_last_error(PGBP_ERR_INVALID_ARGUMENT, "batch must be positive");
  if (lp_stride < 0 || ev_stride < 0 || msgs_stride < 0)
    return pgbp::set_last_error(PGBP_ERR_INVALID_ARGUMENT, "negative stride");
  const size_t need = pgbp::workspace_bytes(plan->p, batch, num_iters, ev_stride != 0,
                                            lp_stride != 0);
  if (need > (size_t)PGBP_STATIC_SCRATCH_BYTES) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "this run needs %zu bytes of scratch; pgbp_run_static_scratch has %zu "
             "(PGBP_STATIC_SCRATCH_BYTES): use pgbp_run with a caller workspace",
             need, (size_t)PGBP_STATIC_SCRATCH_BYTES);
    return pgbp::set_last_error(PGBP_ERR_WORKSPACE, msg);
  }
  // the caller's current device is given back when the call returns
  pgbp::DeviceGuard guard(plan->p.device);
  if (guard.status() != cudaSuccess)
    return pgbp::set_last_error(PGBP_ERR_CUDA, cudaGetErrorString(guard.status()));
  void* scratch = nullptr;
  const int rc = scratch_address(plan->p.device, &scratch);
  if (rc != PGBP_OK) return rc;
  // pgbp_run validates the remaining arguments and launches the same kernels.
  return pgbp_run(plan, stream, batch, log_potentials, lp_stride, evidence, ev_stride, msgs_in,
                  msgs_stride, msgs_out, deltas, num_iters, damping, temperature, scratch,
                  (size_t)PGBP_STATIC_SCRATCH_BYTES);
}
