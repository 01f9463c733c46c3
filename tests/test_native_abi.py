"""The C ABI library: it builds for sm_103a, loads, and exports every symbol the headers in
include/ declare. No kernel is launched here (no GPU needed)."""

import ctypes
import glob
import os
import re

import pytest

from pgmax_gb300 import native

HEADERS = sorted(glob.glob(os.path.join(native.ROOT, "include", "*.h")))


def declared_functions():
  text = "".join(open(h).read() for h in HEADERS)
  return sorted(set(re.findall(r"^\s*(?:int|int64_t|size_t|const char\*)\s+(pgbp_\w+)\s*\(",
                              text, re.M)))


def test_header_declares_expected_entry_points():
  names = declared_functions()
  for n in ("pgbp_plan_create", "pgbp_plan_destroy", "pgbp_run", "pgbp_factor_update",
            "pgbp_beliefs", "pgbp_decode", "pgbp_marginals", "pgbp_workspace_size",
            "pgbp_last_error"):
    assert n in names


def test_library_builds_loads_and_exports_every_declared_symbol():
  lib = native.load()
  for n in declared_functions():
    assert hasattr(lib, n), n
  assert {s[0] for s in native.SIGNATURES} == set(declared_functions())
  assert lib.pgbp_version() >= 100


def test_null_arguments_are_rejected_with_a_status():
  lib = native.load()
  assert lib.pgbp_plan_create(None, 0, None) == 1
  assert b"null" in lib.pgbp_last_error()
  assert lib.pgbp_run(None, None, 1, None, 0, None, 0, None, 0, None, None, 1, 0.5, 0.0, None, 0) == 1
  assert lib.pgbp_workspace_size(None, 1, 1) == 0
  assert lib.pgbp_plan_destroy(None) == 0


def test_debug_settings_validate_their_values():
  """pgbp_debug_set needs no GPU: each knob accepts its documented range, rejects the rest with
  status 1 (invalid argument), and 0 restores the default."""
  lib = native.load()
  for knob, good, bad in ((native.DEBUG_SKIP_TABLE_COPY, (0, 1), (2, -1)),
                          (native.DEBUG_LEGACY_MMA, (0, 1), (2,)),
                          (native.DEBUG_ENUM_KERNEL, (0, 1, 2), (3, -1)),
                          (native.DEBUG_WAIT_LIMIT_NS, (0, 1000000), (-1, 10000000001))):
    for v in good:
      assert lib.pgbp_debug_set(knob, v) == 0, (knob, v)
    for v in bad:
      assert lib.pgbp_debug_set(knob, v) == 1, (knob, v)
    assert lib.pgbp_debug_set(knob, 0) == 0
  assert lib.pgbp_debug_set(99, 0) == 1
  assert b"unknown debug knob" in lib.pgbp_last_error()
