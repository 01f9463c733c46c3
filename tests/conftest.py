import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests", "golden")):
  if p not in sys.path:
    sys.path.insert(0, p)


def pytest_configure(config):
  config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


def pytest_collection_modifyitems(config, items):
  try:
    import torch
    has_gpu = torch.cuda.is_available()
  except Exception:  # pylint: disable=broad-except
    has_gpu = False
  if has_gpu:
    return
  skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
  for item in items:
    if "gpu" in item.keywords:
      item.add_marker(skip)
