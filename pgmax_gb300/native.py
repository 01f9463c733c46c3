"""Builds and loads libpgbp.so, the C-ABI engine of pgmax_gb300 (declared in include/pgbp.h).

The library is compiled in-tree for sm_103a only (`nvcc -gencode arch=compute_103a,code=sm_103a`)
into pgmax_gb300/_build/. There is no CPU fallback: if the library is missing or cannot load, every
BP entry point raises.
"""

import concurrent.futures
import ctypes
import os
import shutil
import subprocess
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libpgbp.so")

SOURCES = ["pgbp_kernels.cu", "pgbp_plan.cpp", "pgbp_static_scratch.cu", "pgbp_adjoint.cu",
           "pgbp_expgemm.cu", "pgbp_conv.cu", "pgbp_energy.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no multiply-add contraction, so every float32 op rounds as the reference's does.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I" + INCLUDE]


def _nvcc():
  exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
  if not os.path.exists(exe):
    raise RuntimeError("nvcc not found: the pgbp CUDA library cannot be built")
  return exe


def _stale():
  if not os.path.exists(LIB):
    return True
  t = os.path.getmtime(LIB)
  deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "pgbp.h")]
  return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
  """Compiles every translation unit in parallel and links libpgbp.so. Returns its path."""
  if not force and not _stale():
    return LIB
  os.makedirs(BUILD, exist_ok=True)
  nvcc = _nvcc()

  def compile_one(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
      cmd = [nvcc, "-x", "cu"] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
      raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
      print(r.stderr)
    return obj

  with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
    objs = list(ex.map(compile_one, SOURCES))
  tmp = LIB + ".tmp"
  cmd = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
  r = subprocess.run(cmd, capture_output=True, text=True)
  if r.returncode != 0:
    raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
  os.replace(tmp, LIB)
  return LIB


_lock = threading.Lock()
_lib = None

_i64 = ctypes.c_int64
_p = ctypes.c_void_p
_d = ctypes.c_double


class WiringDesc(ctypes.Structure):
  """Mirror of pgbp_wiring_desc (include/pgbp.h)."""
  _p32 = ctypes.POINTER(ctypes.c_int32)
  _fields_ = [
      ("num_edge_states", _i64), ("num_var_states", _i64), ("num_edges", _i64),
      ("var_states_for_edge_states", _p32), ("edge_indices_for_edge_states", _p32),
      ("factor_indices_for_edge_states", _p32),
      ("msgs_range", (_i64 * 2) * 4), ("potentials_range", (_i64 * 2) * 4),
      ("enum_num_rows", _i64), ("enum_factor_configs_indices", _p32),
      ("enum_factor_configs_edge_states", _p32), ("enum_num_val_configs", _i64),
      ("logical_num_parents", _i64 * 2), ("logical_parents_factor_indices", _p32 * 2),
      ("logical_parents_msg_indices", _p32 * 2), ("logical_num_factors", _i64 * 2),
      ("logical_children_edge_states", _p32 * 2),
      ("pool_num_choices", _i64), ("pool_choices_factor_indices", _p32),
      ("pool_choices_msg_indices", _p32), ("pool_num_factors", _i64),
      ("pool_indicators_edge_states", _p32),
      ("num_variables", _i64), ("evidence_to_vars", _p32),
      ("flags", _i64),
      ("enum_num_factors", _i64),
      ("enum_factor_potential_offsets", ctypes.POINTER(ctypes.c_int32)),
  ]


class PlanInfo(ctypes.Structure):
  _fields_ = [(n, _i64) for n in (
      "num_edge_states", "num_var_states", "num_edges", "num_variables", "num_potentials",
      "num_enum_factors", "num_enum_pairwise_factors", "num_or_factors", "num_and_factors",
      "num_pool_factors", "num_pairwise_buckets", "device_bytes", "num_slots",
      "small_graph_smem_bytes")]

FLAG_NO_SMALL_GRAPH = 1
FLAG_PATH_SMALL = 2
FLAG_PATH_CLUSTER = 4
FLAG_PATH_MULTI = 8
FLAG_ENUM_IMPLICIT_ROWS = 16


PROFILE_CLASSES = ("varsum", "pairwise", "enum_generic", "or", "and", "pool", "layout", "readout",
                   "small_graph", "adjoint", "pairwise_exp")


class Profile(ctypes.Structure):
  _fields_ = [("launches", _i64 * len(PROFILE_CLASSES)),
              ("milliseconds", ctypes.c_double * len(PROFILE_CLASSES))]

# (name, restype, argtypes) of every symbol include/pgbp.h declares
SIGNATURES = [
    ("pgbp_plan_create", ctypes.c_int, [ctypes.POINTER(WiringDesc), ctypes.c_int,
                                        ctypes.POINTER(_p)]),
    ("pgbp_plan_destroy", ctypes.c_int, [_p]),
    ("pgbp_plan_get_info", ctypes.c_int, [_p, ctypes.POINTER(PlanInfo)]),
    ("pgbp_workspace_size", ctypes.c_size_t, [_p, _i64, _i64]),
    ("pgbp_run", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _p, _i64, _d, _d,
                                _p, ctypes.c_size_t]),
    ("pgbp_run_static_scratch", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p,
                                               _p, _i64, _d, _d]),
    ("pgbp_run_perturbed", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, ctypes.c_uint64, _d,
                                          _p, _i64, _p, _p, _p, _i64, _d, _d, _p,
                                          ctypes.c_size_t]),
    ("pgbp_gumbel", ctypes.c_int, [_p, ctypes.c_uint64, _i64, _p]),
    ("pgbp_factor_update", ctypes.c_int, [_p, _p, ctypes.c_int, _i64, _p, _i64, _p, _i64, _d,
                                          ctypes.c_int, _p, _i64]),
    ("pgbp_run_checkpointed", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _p,
                                             _i64, _i64, _d, _d, _p, _p, ctypes.c_size_t]),
    ("pgbp_run_to_tolerance", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _d,
                                             _i64, _i64, _d, _d, _p, _p, _p, ctypes.c_size_t]),
    ("pgbp_vjp_workspace_size", ctypes.c_size_t, [_p, _i64, _i64, _i64]),
    ("pgbp_run_vjp", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _i64, _d, _d, _p,
                                    _p, _p, _p, _p, ctypes.c_size_t]),
    ("pgbp_beliefs_vjp", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p]),
    ("pgbp_beliefs", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p]),
    ("pgbp_decode", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p]),
    ("pgbp_marginals", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p]),
    ("pgbp_softmax_rows", ctypes.c_int, [_p, _i64, _i64, _p, _p]),
    ("pgbp_argmax_rows", ctypes.c_int, [_p, _i64, _i64, _p, _p]),
    ("pgbp_plan_tuning_count", _i64, [_p]),
    ("pgbp_plan_tuning_get", ctypes.c_int, [_p, _p, _i64]),
    ("pgbp_plan_tuning_set", ctypes.c_int, [_p, _p, _i64]),
    ("pgbp_plan_signature", ctypes.c_int, [_p, ctypes.c_char_p, ctypes.c_size_t]),
    ("pgbp_sdlp_workspace_size", ctypes.c_size_t, [_p, _i64]),
    ("pgbp_sdlp_objective", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _d, _p, _p,
                                           _p, _p, _p, ctypes.c_size_t]),
    ("pgbp_sdlp_run", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _p, _i64, _d,
                                     _d, _p, ctypes.c_size_t]),
    ("pgbp_energy_workspace_size", ctypes.c_size_t, [_p, _i64]),
    ("pgbp_energy", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _p,
                                   ctypes.c_size_t]),
    ("pgbp_energy_terms", ctypes.c_int, [_p, _p, _i64, _p, _i64, _p, _i64, _p, _p]),
    # include/pgbp_learn.h
    ("pgbp_conv3x3", ctypes.c_int, [_p, _i64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, _p, _p, _p, _p, ctypes.c_int, ctypes.c_int, _p]),
    ("pgbp_conv3x3_wgrad_workspace", ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    ("pgbp_conv3x3_wgrad", ctypes.c_int, [_p, _i64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, _p, _p, _p, _p, _p, ctypes.c_size_t]),
    ("pgbp_conv3x3_flip", ctypes.c_int, [_p, ctypes.c_int, ctypes.c_int, _p, _p]),
    ("pgbp_center_mse", ctypes.c_int, [_p, _i64, ctypes.c_int, _p, _p, _p, _p, ctypes.c_float]),
    ("pgbp_adam", ctypes.c_int, [_p, _i64, _p, _p, _p, _p, _p, ctypes.c_float, ctypes.c_float,
                                 ctypes.c_float, ctypes.c_float, _i64]),
    ("pgbp_potts_features", ctypes.c_int, [_p, _i64, ctypes.c_int, ctypes.c_int, _p, _p, _p, _p]),
    ("pgbp_profile_enable", ctypes.c_int, [ctypes.c_int]),
    ("pgbp_profile_read", ctypes.c_int, [ctypes.POINTER(Profile)]),
    ("pgbp_wait_timeouts", ctypes.c_int, [ctypes.POINTER(_i64)]),
    ("pgbp_plan_check", ctypes.c_int, [_p]),
    ("pgbp_debug_set", ctypes.c_int, [ctypes.c_int, _i64]),
    ("pgbp_last_error", ctypes.c_char_p, []),
    ("pgbp_version", ctypes.c_int, []),
]


def load(build_if_missing=True):
  """Loads libpgbp.so (building it first when stale). Raises if that is impossible."""
  global _lib
  with _lock:
    if _lib is None:
      if build_if_missing:
        build()
      if not os.path.exists(LIB):
        raise RuntimeError(f"{LIB} is missing; run pgmax_gb300.native.build()")
      lib = ctypes.CDLL(LIB)
      for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
      _lib = lib
    return _lib


class PgbpError(RuntimeError):
  pass


def check(code, what=""):
  if code != 0:
    msg = load().pgbp_last_error().decode(errors="replace")
    if code in (1, 2, 3, 5):
      raise ValueError(f"{what}: {msg} (pgbp status {code})")
    raise PgbpError(f"{what}: {msg} (pgbp status {code})")


def profile_enable(on=True):
  load().pgbp_profile_enable(1 if on else 0)


TUNE_MAX_SITES = 64


class TuningEntry(ctypes.Structure):
  _fields_ = [("batch", _i64), ("temperature0", ctypes.c_int32), ("path", ctypes.c_int32),
              ("num_sites", ctypes.c_int32), ("site", ctypes.c_int32 * TUNE_MAX_SITES)]


def wait_timeouts():
  """Bounded device waits that gave up since the last call (pgbp_wait_timeouts); 0 normally."""
  n = _i64(0)
  rc = load().pgbp_wait_timeouts(ctypes.byref(n))
  if rc not in (0, 6):  # PGBP_OK, PGBP_ERR_TIMEOUT
    check(rc, "pgbp_wait_timeouts")
  return int(n.value)


DEBUG_WAIT_LIMIT_NS = 1
DEBUG_SKIP_TABLE_COPY = 2
DEBUG_LEGACY_MMA = 3
DEBUG_ENUM_KERNEL = 4


def debug_set(knob, value):
  """Process-wide debug setting (pgbp_debug_set): DEBUG_WAIT_LIMIT_NS (0 = the built-in 2 s),
  DEBUG_SKIP_TABLE_COPY (1 = the exp-domain kernels' table wait runs out with no copy issued) or
  DEBUG_LEGACY_MMA (1 = shared 64 x 64 tables of one instance on the mma.sync kernel) or
  DEBUG_ENUM_KERNEL (generic EnumFactors: 1 = per-thread kernel, 2 = staged kernel, 0 = tuned /
  rule)."""
  check(load().pgbp_debug_set(int(knob), int(value)), "pgbp_debug_set")


def profile_read():
  """{class: (launches, total ms)} of the launches recorded since the last read."""
  p = Profile()
  check(load().pgbp_profile_read(ctypes.byref(p)), "pgbp_profile_read")
  return {name: (int(p.launches[i]), float(p.milliseconds[i]))
          for i, name in enumerate(PROFILE_CLASSES)}
