"""NumPy stand-in for the subset of ``jax`` that Mahakala imports.

Test infrastructure only: ``make_golden.py`` installs these modules into
``sys.modules`` so that the UNMODIFIED reference package (``mahakala``) can be
imported and executed on a machine without jax, to produce golden vectors.

Semantics mirrored (all FP64, as ``jax_enable_x64`` is set by
``mahakala/__init__.py:22-23``):

* ``jit``            -> identity (also usable as a decorator).
* ``vmap``           -> a Python loop over the mapped axis, outputs stacked.
* ``jacfwd(f)``      -> Jacobian w.r.t. the first argument by complex step
                        (exact to rounding for the analytic ``metric``); the
                        derivative index is appended last, as jacfwd does.
* ``lax.scan``       -> a Python loop; stacked per-step outputs.
* ``lax.select``     -> ``np.where``.
* ``jnp.linalg.inv`` -> ``np.linalg.inv`` (LAPACK LU, as XLA's CPU path).
* ``x.at[idx].set(v)`` -> returns a modified COPY (functional update), so a
  discarded result is a no-op exactly as in jax.
* ``jnp.floor_divide`` / ``%`` on floats follow Python/NumPy divmod rules,
  which are the rules jax implements for floating point.

Nothing under this file is part of the shipped package.
"""

import sys
import types

import numpy as np


class JArray(np.ndarray):
    """ndarray with jax's functional ``.at[...]`` update syntax."""

    def __array_finalize__(self, obj):
        pass

    @property
    def at(self):
        return _AtIndexer(self)

    def __getitem__(self, idx):
        # jax gathers clamp out-of-range integer-array indices (after
        # normalising negative ones) instead of raising; mirror that.
        items = idx if isinstance(idx, tuple) else (idx,)
        if any(it is Ellipsis for it in items) or not any(
                isinstance(it, np.ndarray) and it.dtype.kind in "iu"
                for it in items):
            return super().__getitem__(idx)
        out = []
        axis = 0
        for it in items:
            if it is None:
                out.append(it)
                continue
            if isinstance(it, np.ndarray) and it.dtype.kind in "iu":
                dim = self.shape[axis]
                it = np.asarray(it)
                it = np.where(it < 0, it + dim, it)
                it = np.clip(it, 0, dim - 1)
            out.append(it)
            axis += 1
        return super().__getitem__(tuple(out))


class _AtIndexer:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtUpdate(self._arr, idx)


class _AtUpdate:
    def __init__(self, arr, idx):
        self._arr = arr
        self._idx = idx

    def set(self, value):
        out = np.array(self._arr, copy=True)
        idx = self._idx
        if isinstance(idx, np.ndarray):
            idx = np.asarray(idx)
        out[idx] = value
        return out.view(JArray)


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, JArray):
        return x.view(JArray)
    if isinstance(x, (np.floating, np.integer, np.bool_, np.complexfloating)):
        return np.asarray(x).view(JArray)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    return x


def _wrapped(fn):
    def inner(*args, **kwargs):
        return _wrap(fn(*args, **kwargs))
    inner.__name__ = getattr(fn, "__name__", "fn")
    return inner


def _array(obj, dtype=None, **kwargs):
    if isinstance(obj, (list, tuple)):
        parts = [np.asarray(o) for o in obj]
        if parts and all(p.ndim == 0 for p in parts):
            arr = np.array([p[()] for p in parts], dtype=dtype)
        else:
            arr = np.array(obj, dtype=dtype)
    else:
        arr = np.array(obj, dtype=dtype)
    if arr.dtype == np.float32:
        arr = arr.astype(np.float64)
    return arr.view(JArray)


def _linspace(start, stop, num=50, endpoint=True, dtype=None):
    """jnp.linspace's own formula: start*(1 - i/div) + stop*(i/div), with the
    endpoint written exactly (it differs from np.linspace in the last ulp)."""
    start = np.float64(start)
    stop = np.float64(stop)
    div = (num - 1) if endpoint else num
    if num > 1:
        step = np.arange(div, dtype=np.float64) / np.float64(div)
        out = start * (1.0 - step) + stop * step
        if endpoint:
            out = np.concatenate([out, [stop]])
    elif num == 1:
        out = np.array([start])
    else:
        out = np.zeros(0)
    return out.view(JArray)


def _select(condlist, choicelist, default=0):
    return _wrap(np.select([np.asarray(c) for c in condlist],
                           [np.asarray(c) for c in choicelist], default))


def _make_jnp():
    jnp = types.ModuleType("jax.numpy")
    passthrough = [
        "isclose", "heaviside", "sqrt", "minimum", "maximum", "concatenate",
        "diag", "ones", "zeros", "meshgrid", "cross", "zeros_like",
        "logical_or", "isnan", "abs", "broadcast_to", "all", "argmax",
        "arange", "exp", "sin", "cos", "arccos", "einsum", "stack",
        "ones_like", "floor_divide", "remainder", "multiply",
        "add", "subtract", "divide", "where", "sum", "dot", "matmul",
    ]
    for name in passthrough:
        setattr(jnp, name, _wrapped(getattr(np, name)))
    jnp.array = _array
    jnp.asarray = _array
    jnp.select = _select
    jnp.linspace = _linspace
    jnp.newaxis = None
    jnp.pi = np.pi
    jnp.nan = np.nan
    jnp.inf = np.inf
    linalg = types.ModuleType("jax.numpy.linalg")
    linalg.inv = _wrapped(np.linalg.inv)
    jnp.linalg = linalg
    return jnp, linalg


def jit(fn=None, **kwargs):
    if fn is None:
        return lambda f: f
    return fn


def vmap(fn, in_axes=0, out_axes=0):
    def mapped(*args):
        axes = in_axes
        if not isinstance(axes, (tuple, list)):
            axes = (axes,) * len(args)
        n = None
        for arg, ax in zip(args, axes):
            if ax is not None:
                n = np.shape(arg)[ax]
                break
        outs = []
        for i in range(n):
            call = []
            for arg, ax in zip(args, axes):
                if ax is None:
                    call.append(arg)
                else:
                    call.append(_wrap(np.take(np.asarray(arg), i, axis=ax)))
            outs.append(fn(*call))
        if isinstance(outs[0], tuple):
            return tuple(_wrap(np.stack([np.asarray(o[k]) for o in outs]))
                         for k in range(len(outs[0])))
        return _wrap(np.stack([np.asarray(o) for o in outs]))
    return mapped


_CSTEP = 1e-100


def jacfwd(fn):
    """Jacobian of ``fn`` w.r.t. its first argument by complex step."""
    def jac(x, *rest):
        x = np.asarray(x, dtype=np.float64)
        cols = []
        for c in range(x.shape[0]):
            xc = x.astype(np.complex128)
            xc[c] += 1j * _CSTEP
            cols.append(np.imag(np.asarray(fn(xc, *rest))) / _CSTEP)
        return _wrap(np.stack(cols, axis=-1))
    return jac


def _scan(f, init, xs, length=None):
    carry = init
    ys = []
    if xs is None:
        xs = range(length)
    for x in xs:
        carry, y = f(carry, x)
        ys.append(y)
    if not ys or ys[0] is None:
        return carry, None
    if isinstance(ys[0], tuple):
        stacked = tuple(_wrap(np.stack([np.asarray(y[k]) for y in ys]))
                        for k in range(len(ys[0])))
        return carry, stacked
    return carry, _wrap(np.stack([np.asarray(y) for y in ys]))


def _lax_select(pred, on_true, on_false):
    return _wrap(np.where(np.asarray(pred), on_true, on_false))


class _Config:
    def update(self, key, value):
        pass


class _Backend:
    platform = "cpu (numpy stand-in for jax)"


class _FakeH5File:
    """Minimal ``h5py.File`` over an in-memory dict (see ``register_h5``)."""

    registry = {}

    def __init__(self, name, mode="r"):
        data = self.registry[name]
        self._data = data["datasets"]
        self.attrs = data["attrs"]

    def __getitem__(self, key):
        return self._data[key]

    def close(self):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def register_h5(name, datasets, attrs):
    _FakeH5File.registry[name] = {"datasets": datasets, "attrs": attrs}


def install():
    """Install ``jax``, ``jax.numpy``, ``jax.lax``, ``jax.lib`` and ``h5py``."""
    jax = types.ModuleType("jax")
    jnp, linalg = _make_jnp()
    lax = types.ModuleType("jax.lax")
    lax.scan = _scan
    lax.select = _lax_select
    lib = types.ModuleType("jax.lib")
    xla_bridge = types.ModuleType("jax.lib.xla_bridge")
    xla_bridge.get_backend = lambda: _Backend()
    lib.xla_bridge = xla_bridge
    jax.numpy = jnp
    jax.lax = lax
    jax.lib = lib
    jax.jit = jit
    jax.vmap = vmap
    jax.jacfwd = jacfwd
    jax.config = _Config()
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp
    sys.modules["jax.numpy.linalg"] = linalg
    sys.modules["jax.lax"] = lax
    sys.modules["jax.lib"] = lib
    sys.modules["jax.lib.xla_bridge"] = xla_bridge
    h5py = types.ModuleType("h5py")
    h5py.File = _FakeH5File
    sys.modules["h5py"] = h5py
