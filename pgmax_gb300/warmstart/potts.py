"""The spin-glass Potts family: L x L toroidal grids of K-state variables, one pairwise factor per
grid edge with table J_e * I_K, J_e ~ N(0, sigma^2), unaries N(0, 1).

Factor order: the L * L down factors ((i, j), (i + 1 mod L, j)), row-major, then the L * L right
factors ((i, j), (i, j + 1 mod L)); the flat wiring is the one FactorGraph compiles for two
PairwiseFactorGroups in that order (checked in the tests). Also here: the network's input
features (with the closed-form one-step messages the network corrects) and the map from its
outputs to flat messages.
"""

from typing import Dict, Tuple

import numpy as np

FEATURES = 64  # K centred unaries, 4 couplings, 4 K one-step messages, zero padding


def torus_wiring(L: int, K: int) -> Dict:
  """Flat wiring of the toroidal Potts grid (explicit config rows, one table per factor)."""
  i, j = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
  down = np.stack([i * L + j, ((i + 1) % L) * L + j], -1).reshape(-1, 2)
  right = np.stack([i * L + j, i * L + (j + 1) % L], -1).reshape(-1, 2)
  pairs = np.concatenate([down, right]).astype(np.int64)
  F = pairs.shape[0]
  s = np.arange(K, dtype=np.int64)
  vs = (pairs[:, :, None] * K + s).reshape(-1)
  es = np.arange(2 * K * F, dtype=np.int64)
  a, b = np.meshgrid(s, s, indexing="ij")
  base = (2 * K * np.arange(F))[:, None, None]
  E = 2 * K * F
  P = F * K * K
  return {
      "var_states_for_edge_states": vs.astype(np.int32),
      "edge_indices_for_edge_states": (es // K).astype(np.int32),
      "factor_indices_for_edge_states": (es // (2 * K)).astype(np.int32),
      "num_edges": 2 * F, "num_factors": F, "num_var_states": L * L * K,
      "evidence_to_vars": np.repeat(np.arange(L * L), K).astype(np.int32),
      "num_variables": L * L,
      "msgs_ranges": np.array([[0, E], [E, E], [E, E], [E, E]], np.int64),
      "potentials_ranges": np.array([[0, P], [P, P], [P, P], [P, P]], np.int64),
      "enum.factor_configs_indices": np.repeat(np.arange(P, dtype=np.int32), 2),
      "enum.factor_configs_edge_states": np.stack([base + a, base + K + b], -1).reshape(-1).astype(
          np.int32),
      "enum.num_val_configs": P,
  }


def sample(seed: int, n: int, L: int, K: int, sigma: float = 0.7) -> Tuple[np.ndarray, np.ndarray]:
  """n instances: couplings J [n, 2 L^2] (down factors, then right) and unaries [n, L^2 K]."""
  rng = np.random.default_rng(seed)
  J = rng.normal(0.0, sigma, size=(n, 2 * L * L)).astype(np.float32)
  u = rng.normal(size=(n, L * L * K)).astype(np.float32)
  return J, u


def potentials(J, K: int):
  """Flat log-potentials [n, F K^2] of tables J_f * I_K (torch or numpy)."""
  eye = np.eye(K, dtype=np.float32).reshape(-1)
  if type(J).__module__.startswith("torch"):
    import torch  # pylint: disable=g-import-not-at-top
    return (J[:, :, None] * torch.as_tensor(eye, device=J.device)).reshape(J.shape[0], -1)
  return (J[:, :, None] * eye).reshape(J.shape[0], -1)


def _neighbours(J, u, L: int, K: int):
  """Per variable, for its down, right, up and left factor: the coupling [n, L, L] and the
  other variable's unaries [n, L, L, K] (torch)."""
  import torch  # pylint: disable=g-import-not-at-top
  n = J.shape[0]
  jd = J[:, :L * L].reshape(n, L, L)
  jr = J[:, L * L:].reshape(n, L, L)
  uu = u.reshape(n, L, L, K)
  couplings = [jd, jr, torch.roll(jd, 1, 1), torch.roll(jr, 1, 2)]
  others = [torch.roll(uu, -1, 1), torch.roll(uu, -1, 2), torch.roll(uu, 1, 1),
            torch.roll(uu, 1, 2)]
  return couplings, others, uu


def one_step_messages(J, u, L: int, K: int):
  """The message every factor sends its variables after one undamped BP iteration from zero
  messages, normalised per edge, in network channel layout [n, L, L, 4 K]: for the factor shared
  with neighbour k, log sum_t exp(J_k [s == t] + u_k(t)), with u_k the neighbour's unaries. A
  closed-form function of the unaries and couplings (torch)."""
  import torch  # pylint: disable=g-import-not-at-top
  couplings, others, _ = _neighbours(J, u, L, K)
  out = []
  for jk, a in zip(couplings, others):
    lse = torch.logsumexp(a, -1, keepdim=True)
    m = torch.log(torch.exp(lse) + torch.expm1(jk)[..., None] * torch.exp(a))
    out.append(m - m.max(-1, keepdim=True).values)
  return torch.cat(out, -1)


def features(J, u, L: int, K: int):
  """Network input [n, L, L, FEATURES] (torch): each variable's unaries (centred), the couplings
  of its down, right, up and left edges, the one-step messages of those four factors, zeros."""
  import torch  # pylint: disable=g-import-not-at-top
  couplings, _, uu = _neighbours(J, u, L, K)
  parts = [uu - uu.mean(-1, keepdim=True)] + [c[..., None] for c in couplings]
  parts.append(one_step_messages(J, u, L, K))
  n = J.shape[0]
  pad = FEATURES - K - 4 - 4 * K
  parts.append(torch.zeros((n, L, L, pad), dtype=u.dtype, device=u.device))
  return torch.cat(parts, -1)


def features_and_messages(J, u, L: int, K: int):
  """(features [n, L, L, FEATURES] BF16, one-step messages [n, L, L, 4 K] FP32) of CUDA tensors
  J [n, 2 L^2] and u [n, L^2 K], in one pgbp_potts_features launch: the values of features() and
  one_step_messages() above (which restate them in torch, for checking)."""
  import ctypes  # pylint: disable=g-import-not-at-top
  import torch  # pylint: disable=g-import-not-at-top
  from .. import native  # pylint: disable=g-import-not-at-top
  J = J.to(torch.float32).contiguous()
  u = u.to(torch.float32).contiguous()
  n = J.shape[0]
  x = torch.empty((n, L, L, FEATURES), dtype=torch.bfloat16, device=J.device)
  m1 = torch.empty((n, L, L, 4 * K), dtype=torch.float32, device=J.device)
  stream = ctypes.c_void_p(torch.cuda.current_stream(J.device).cuda_stream)
  native.check(native.load().pgbp_potts_features(stream, n, L, K, ctypes.c_void_p(J.data_ptr()),
                                                 ctypes.c_void_p(u.data_ptr()),
                                                 ctypes.c_void_p(x.data_ptr()),
                                                 ctypes.c_void_p(m1.data_ptr())),
               "pgbp_potts_features")
  return x, m1


def message_index(L: int, K: int) -> np.ndarray:
  """[L * L * 4 * K] flat edge state of output channel (k, s) of pixel (i, j): the message into
  variable (i, j), state s, from its down (k=0), right (1), up (2) and left (3) factor."""
  i, j = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
  f_down = i * L + j
  f_right = L * L + i * L + j
  f_up = ((i - 1) % L) * L + j
  f_left = L * L + i * L + (j - 1) % L
  s = np.arange(K)
  first = np.stack([2 * K * f_down, 2 * K * f_right, 2 * K * f_up + K, 2 * K * f_left + K], -1)
  return (first[..., None] + s).reshape(-1).astype(np.int64)
