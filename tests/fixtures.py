"""Loading helpers for the golden fixtures in tests/golden/fixtures/ (see make_golden.py)."""

import glob
import json
import os

import numpy as np

FIXTURES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fixtures")


def run_fixture_paths():
  return sorted(p for p in glob.glob(os.path.join(FIXTURES, "*.npz"))
                if not os.path.basename(p).startswith(("factor_updates", "energy_", "sdlp_",
                                                       "marginals_")))


def energy_fixture_paths():
  """compute_energy calls of the reference: wiring, log_potentials, evidence, map_flat, energy."""
  return sorted(glob.glob(os.path.join(FIXTURES, "energy_*.npz")))


def load(path):
  z = np.load(path, allow_pickle=False)
  d = {k: z[k] for k in z.files}
  d["meta"] = json.loads(str(d["meta"]))
  d["wiring"] = {k[2:]: v for k, v in d.items() if k.startswith("w.")}
  d["name"] = os.path.basename(path)[:-4]
  return d


def fixture_id(path):
  return os.path.basename(path)[:-4]


def sdlp_fixture_paths():
  """SDLP calls of the reference: wiring, BPArrays, call kind and its outputs."""
  return sorted(glob.glob(os.path.join(FIXTURES, "sdlp_*.npz")))


def marginals_fixture_paths():
  """get_marginals calls of the reference after seeded runs: wiring, evidence, messages, flat
  beliefs and, leaf by leaf, the unflattened beliefs and the reference's marginals."""
  return sorted(p for p in glob.glob(os.path.join(FIXTURES, "marginals_*.npz"))
                if not p.endswith("marginals_direct.npz"))
