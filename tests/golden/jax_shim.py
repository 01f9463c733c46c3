"""Test-only NumPy stand-in for the subset of `jax`, `jaxlib` and `numba` that PGMax 0.6.1 uses.

This module exists so that the unmodified PGMax package (pure Python over JAX) can be imported and
run in a container that has neither `jax` nor `numba`. It is used only by `make_golden.py` in this
folder, to execute the reference's own code and record its inputs and outputs as fixtures. It is
never imported by the product package, by `bench.py` or by any GPU test.

Semantics reproduced (JAX with `jax_enable_x64` off, the PGMax default):
  * arrays are float32 / int32 ("canonical" dtypes); float64 / int64 inputs are narrowed at every
    `jnp.*` call, at `jax.device_put` and at `jax.jit` boundaries;
  * `x.at[idx].add/max/min/multiply/set` are functional scatters. `add`, `max`, `min` and
    `multiply` apply updates serially in index order (`np.ufunc.at`), which is the order XLA:CPU's
    scatter loop uses; out-of-range indices (on any axis of a tuple of integer index arrays,
    after one negative wrap) are dropped (JAX's default scatter mode);
  * `jax.jit`, `jax.checkpoint` and `numba.jit` are identity decorators; `jax.lax.scan` is a loop;
  * `jax.tree_util` handles dicts, lists, tuples, None and classes registered with
    `register_pytree_node_class`.
Transcendental functions are NumPy's float32 implementations, so results differ from XLA:CPU at
the ulp level; the reference's own golden vector (`tests/test_pgmax.py`, atol 1e-6) is the check
that this is close enough.
"""

import dataclasses
import functools
import sys
import types

import numpy as np
import scipy.special


def _canon_dtype(dt):
  dt = np.dtype(dt)
  if dt == np.float64 or dt == np.float16 or dt == np.longdouble:
    return np.dtype(np.float32)
  if dt == np.int64 or dt == np.int16 or dt == np.int8:
    return np.dtype(np.int32)
  if dt == np.uint64:
    return np.dtype(np.uint32)
  return dt


def _canon_in(x):
  """Narrows an ufunc input; python scalars stay weakly typed."""
  if isinstance(x, np.ndarray):
    base = x.view(np.ndarray) if type(x) is not np.ndarray else x
    cd = _canon_dtype(base.dtype)
    return base.astype(cd) if cd != base.dtype else base
  if isinstance(x, np.generic):
    cd = _canon_dtype(x.dtype)
    return x.astype(cd)
  return x


def _wrap(x):
  if isinstance(x, np.ndarray):
    cd = _canon_dtype(x.dtype)
    if cd != x.dtype:
      x = x.astype(cd)
    return x.view(Arr)
  if isinstance(x, np.generic):
    return np.asarray(x).astype(_canon_dtype(x.dtype)).view(Arr)
  return x


def asarr(x, dtype=None):
  """Canonical float32/int32 array (a copy), like jnp.array."""
  if isinstance(x, (list, tuple)):
    x = np.array([np.asarray(v) for v in x]) if x and isinstance(x[0], np.ndarray) else np.array(x)
  a = np.array(x.view(np.ndarray) if isinstance(x, Arr) else x, copy=True)
  if dtype is not None:
    a = a.astype(dtype)
  cd = _canon_dtype(a.dtype)
  if cd != a.dtype:
    a = a.astype(cd)
  return a.view(Arr)


class _AtRef:

  def __init__(self, arr, idx):
    self._arr = arr
    self._idx = idx

  def _prep(self):
    out = np.array(self._arr.view(np.ndarray), copy=True)
    idx = self._idx
    if isinstance(idx, np.ndarray):
      idx = idx.view(np.ndarray)
      if np.issubdtype(idx.dtype, np.integer):
        n = out.shape[0]
        keep = (idx < n) & (idx >= -n)
        return out, idx, keep
    if isinstance(idx, tuple) and idx and all(
        isinstance(i, (np.ndarray, int, np.integer)) and np.issubdtype(np.asarray(i).dtype, np.integer)
        for i in idx):
      # advanced indexing with integer arrays on the leading axes: an update whose index is out of
      # range on any axis (after one negative wrap) is dropped
      parts = np.broadcast_arrays(*[np.asarray(i).view(np.ndarray) for i in idx])
      keep = np.ones(parts[0].shape, dtype=bool)
      for a, n in zip(parts, out.shape):
        keep &= (a < n) & (a >= -n)
      return out, tuple(parts), keep
    return out, idx, None

  @staticmethod
  def _select(idx, keep):
    if isinstance(idx, tuple):
      return tuple(a[keep] for a in idx)
    return idx[keep]

  def _apply(self, ufunc, values):
    out, idx, keep = self._prep()
    vals = _canon_in(values)
    if isinstance(vals, np.ndarray):
      vals = vals.astype(out.dtype, copy=False)
    if keep is not None and not keep.all():
      if isinstance(vals, np.ndarray) and vals.ndim > 0:
        vals = np.broadcast_to(vals, keep.shape)[keep]
      idx = self._select(idx, keep)
    ufunc.at(out, idx, vals)
    return out.view(Arr)

  def add(self, values):
    return self._apply(np.add, values)

  def max(self, values):
    return self._apply(np.maximum, values)

  def min(self, values):
    return self._apply(np.minimum, values)

  def multiply(self, values):
    return self._apply(np.multiply, values)

  def set(self, values):
    out, idx, keep = self._prep()
    vals = _canon_in(values)
    if keep is not None and not keep.all():
      if isinstance(vals, np.ndarray) and vals.ndim > 0:
        vals = np.broadcast_to(vals, keep.shape)[keep]
      idx = self._select(idx, keep)
    out[idx] = vals
    return out.view(Arr)

  def get(self):
    return _wrap(self._arr.view(np.ndarray)[self._idx])


class _AtIndexer:

  def __init__(self, arr):
    self._arr = arr

  def __getitem__(self, idx):
    if isinstance(idx, Arr):
      idx = idx.view(np.ndarray)
    return _AtRef(self._arr, idx)


class Arr(np.ndarray):
  """A NumPy array with JAX's functional `.at[]` updates and 32-bit dtype promotion."""

  @property
  def at(self):
    return _AtIndexer(self)

  def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
    if kwargs.get("out") is not None:
      raise TypeError("in-place ufuncs are not supported on jax arrays")
    ins = [_canon_in(x) for x in inputs]
    kwargs = {k: (_canon_in(v) if isinstance(v, np.ndarray) else v) for k, v in kwargs.items()}
    res = getattr(ufunc, method)(*ins, **kwargs)
    if isinstance(res, tuple):
      return tuple(_wrap(r) for r in res)
    return _wrap(res)

  # jax arrays are immutable: augmented assignment rebinds to a new array.
  def __iadd__(self, other):
    return self + other

  def __isub__(self, other):
    return self - other

  def __imul__(self, other):
    return self * other

  def __itruediv__(self, other):
    return self / other

  def block_until_ready(self):
    return self

  def __hash__(self):  # jax arrays are unhashable too; keep numpy's behaviour explicit
    raise TypeError("unhashable type: 'Array'")


# ----------------------------------------------------------------------------- pytrees

_REGISTERED = set()


class _TreeDef:

  def __init__(self, kind, meta, children):
    self.kind = kind
    self.meta = meta
    self.children = children



def _is_registered(x):
  return type(x) in _REGISTERED


def _sorted_keys(d):
  keys = list(d.keys())
  try:
    return sorted(keys)
  except TypeError:
    return keys


def _flatten(x):
  if x is None:
    return [], _TreeDef("none", None, [])
  if isinstance(x, dict):
    keys = _sorted_keys(x)
    leaves, defs = [], []
    for k in keys:
      l, d = _flatten(x[k])
      leaves += l
      defs.append(d)
    return leaves, _TreeDef("dict", keys, defs)
  if isinstance(x, (list, tuple)) and not hasattr(x, "_fields"):
    leaves, defs = [], []
    for v in x:
      l, d = _flatten(v)
      leaves += l
      defs.append(d)
    return leaves, _TreeDef("list" if isinstance(x, list) else "tuple", None, defs)
  if _is_registered(x):
    children, aux = x.tree_flatten()
    leaves, child_defs = [], []
    for c in children:
      l, d = _flatten(c)
      leaves += l
      child_defs.append(d)
    return leaves, _TreeDef("custom_list", (type(x), aux), child_defs)
  return [x], _TreeDef("leaf", None, [])


def _unflatten(treedef, leaves):
  def build(td, leaves):
    if td.kind == "leaf":
      return leaves[0], leaves[1:]
    if td.kind == "none":
      return None, leaves
    vals = []
    for c in td.children:
      v, leaves = build(c, leaves)
      vals.append(v)
    if td.kind == "dict":
      return dict(zip(td.meta, vals)), leaves
    if td.kind == "list":
      return vals, leaves
    if td.kind == "tuple":
      return tuple(vals), leaves
    if td.kind == "custom_list":
      cls, aux = td.meta
      return cls.tree_unflatten(aux, vals), leaves
    raise ValueError(td.kind)

  out, rest = build(treedef, list(leaves))
  assert not rest
  return out


class _PublicTreeDef:

  def __init__(self, td):
    self._td = td

  def unflatten(self, leaves):
    return _unflatten(self._td, leaves)


def tree_flatten(x):
  leaves, td = _flatten(x)
  return leaves, _PublicTreeDef(td)


def tree_leaves(x):
  return _flatten(x)[0]


def tree_map(f, tree, *rest):
  leaves, td = _flatten(tree)
  others = [_flatten(r)[0] for r in rest]
  return _unflatten(td, [f(*xs) for xs in zip(leaves, *others)])


def register_pytree_node_class(cls):
  _REGISTERED.add(cls)
  return cls


# ----------------------------------------------------------------------------- jax.numpy


def _ufunc(npf):
  def f(*args, **kwargs):
    return _wrap(npf(*[_canon_in(a) for a in args], **kwargs))

  f.__name__ = npf.__name__
  return f


def _default_float(dtype):
  return np.float32 if dtype is None else _canon_dtype(dtype)


def zeros(shape, dtype=None):
  return np.zeros(shape, dtype=_default_float(dtype)).view(Arr)


def ones(shape, dtype=None):
  return np.ones(shape, dtype=_default_float(dtype)).view(Arr)


def empty(shape, dtype=None):
  return zeros(shape, dtype)


def full(shape, fill_value, dtype=None):
  if dtype is None:
    if isinstance(fill_value, (bool, np.bool_)):
      dtype = np.bool_
    elif isinstance(fill_value, (int, np.integer)):
      dtype = np.int32
    else:
      dtype = np.float32
  return np.full(shape, fill_value, dtype=_canon_dtype(dtype)).view(Arr)


def zeros_like(x, dtype=None):
  return np.zeros(np.shape(x), dtype=_canon_dtype(dtype or np.asarray(x).dtype)).view(Arr)


def arange(*args, dtype=None):
  return _wrap(np.arange(*args, dtype=dtype))


def where(cond, x=None, y=None):
  if x is None:
    return tuple(_wrap(a) for a in np.where(_canon_in(cond)))
  return _wrap(np.where(_canon_in(cond), _canon_in(x), _canon_in(y)))


def clip(a, a_min=None, a_max=None):
  out = _canon_in(a)
  if a_min is not None:
    out = np.maximum(out, _canon_in(a_min))
  if a_max is not None:
    out = np.minimum(out, _canon_in(a_max))
  return _wrap(out)


def concatenate(arrays, axis=0):
  return _wrap(np.concatenate([_canon_in(np.asarray(a) if not isinstance(a, np.ndarray) else a)
                               for a in arrays], axis=axis))


def bincount(x, weights=None, minlength=0, length=None):
  n = length if length is not None else minlength
  out = np.bincount(np.asarray(x).view(np.ndarray), weights=weights, minlength=n)
  if length is not None:
    out = out[:length]
  return _wrap(out)


def _reduction(npf):
  def f(a, *args, **kwargs):
    kwargs = {k: (_canon_in(v) if isinstance(v, np.ndarray) else v) for k, v in kwargs.items()}
    return _wrap(npf(_canon_in(np.asarray(a) if not isinstance(a, np.ndarray) else a), *args,
                     **kwargs))

  return f


def tile(a, reps):
  return _wrap(np.tile(_canon_in(a), reps))


def broadcast_to(a, shape):
  return _wrap(np.broadcast_to(_canon_in(a), shape))


def copy(a):
  return asarr(a)


def meshgrid(*xs, **kw):
  return [_wrap(m) for m in np.meshgrid(*[_canon_in(x) for x in xs], **kw)]


def allclose(a, b, rtol=1e-05, atol=1e-08, equal_nan=False):
  return bool(np.allclose(np.asarray(a), np.asarray(b), rtol=rtol, atol=atol, equal_nan=equal_nan))


def _logsumexp(a, axis=None, b=None, keepdims=False, return_sign=False):
  return _wrap(scipy.special.logsumexp(_canon_in(a), axis=axis, b=b, keepdims=keepdims,
                                       return_sign=return_sign))


def device_put(x, *args, **kwargs):
  return tree_map(lambda l: asarr(l) if isinstance(l, (np.ndarray, np.generic, list)) else l, x)


def _canon_arg(x):
  if isinstance(x, np.ndarray) and not isinstance(x, Arr):
    return asarr(x)
  if isinstance(x, dict):
    return {k: _canon_arg(v) for k, v in x.items()}
  if isinstance(x, (list, tuple)) and not hasattr(x, "_fields"):
    return type(x)(_canon_arg(v) for v in x)
  return x


def jit(fun=None, **jit_kwargs):
  if fun is None:
    return lambda f: jit(f, **jit_kwargs)

  @functools.wraps(fun)
  def wrapped(*args, **kwargs):
    return fun(*[_canon_arg(a) for a in args], **{k: _canon_arg(v) for k, v in kwargs.items()})

  return wrapped


def checkpoint(fun=None, **kwargs):
  if fun is None:
    return lambda f: f
  return fun


def scan(f, init, xs, length=None):
  n = length if length is not None else len(xs)
  carry = init
  ys = []
  for i in range(n):
    carry, y = f(carry, None if xs is None else xs[i])
    ys.append(y)
  if ys and ys[0] is not None:
    return carry, _wrap(np.stack([np.asarray(y) for y in ys]))
  return carry, None


def vmap(fun, in_axes=0, out_axes=0):
  raise NotImplementedError("vmap is not needed by the PGMax code paths exercised here")


def install():
  """Registers fake `jax`, `jax.numpy`, `jax.lax`, `jax.tree_util`, `jax.scipy.special`,
  `jax.lib.xla_bridge` and `numba` modules in sys.modules."""
  if "jax" in sys.modules and getattr(sys.modules["jax"], "__shim__", False):
    return sys.modules["jax"]

  jnp = types.ModuleType("jax.numpy")
  jnp.ndarray = Arr
  jnp.array = asarr
  jnp.asarray = asarr
  for name in ["zeros", "ones", "empty", "full", "zeros_like", "arange", "where", "clip",
               "concatenate", "bincount", "tile", "broadcast_to", "copy", "meshgrid",
               "allclose"]:
    setattr(jnp, name, globals()[name])
  for name in ["maximum", "minimum", "exp", "log", "log1p", "expm1", "abs", "sign", "isinf",
               "isnan", "logical_and", "logical_or", "sqrt", "square", "equal", "not_equal"]:
    setattr(jnp, name, _ufunc(getattr(np, name)))
  for name in ["sum", "max", "min", "all", "any", "argmax", "argmin", "cumsum", "mean",
               "prod", "reshape", "stack"]:
    setattr(jnp, name, _reduction(getattr(np, name)))
  jnp.stack = lambda arrays, axis=0: _wrap(np.stack([_canon_in(a) for a in arrays], axis=axis))
  jnp.iinfo = np.iinfo
  jnp.finfo = np.finfo
  jnp.int32 = np.int32
  jnp.float32 = np.float32
  jnp.bool_ = np.bool_
  jnp.inf = np.inf
  jnp.nan = np.nan

  tree_util = types.ModuleType("jax.tree_util")
  tree_util.tree_map = tree_map
  tree_util.tree_flatten = tree_flatten
  tree_util.tree_leaves = tree_leaves
  tree_util.register_pytree_node_class = register_pytree_node_class

  lax = types.ModuleType("jax.lax")
  lax.scan = scan

  special = types.ModuleType("jax.scipy.special")
  special.logsumexp = _logsumexp
  jscipy = types.ModuleType("jax.scipy")
  jscipy.special = special

  xla_bridge = types.ModuleType("jax.lib.xla_bridge")
  xla_bridge.get_backend = lambda *a: types.SimpleNamespace(platform="cpu")
  jlib = types.ModuleType("jax.lib")
  jlib.xla_bridge = xla_bridge

  jax = types.ModuleType("jax")
  jax.__shim__ = True
  jax.numpy = jnp
  jax.tree_util = tree_util
  jax.lax = lax
  jax.scipy = jscipy
  jax.lib = jlib
  jax.jit = jit
  jax.checkpoint = checkpoint
  jax.device_put = device_put
  jax.vmap = vmap
  jax.Array = Arr

  numba = types.ModuleType("numba")
  numba.jit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
  numba.njit = numba.jit
  numba.prange = range

  sys.modules.update({
      "jax": jax, "jax.numpy": jnp, "jax.tree_util": tree_util, "jax.lax": lax,
      "jax.scipy": jscipy, "jax.scipy.special": special, "jax.lib": jlib,
      "jax.lib.xla_bridge": xla_bridge, "numba": numba,
  })
  return jax
