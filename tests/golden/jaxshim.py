"""A numpy stand-in for the parts of ``jax`` the reference library uses.

Used ONLY by ``make_golden.py`` to import and run the reference's own source
files in a container without JAX, to generate golden vectors.  It is not used
by the tests at run time, and never by the engine.

* ``jax.numpy`` is numpy, with array results wrapped in ``AtArray`` (an
  ndarray subclass that provides JAX's functional ``.at[idx].set/add/divide``).
* ``X64 = False`` emulates JAX's default 32-bit mode: float64 inputs to
  ``jnp.array``/``jnp.asarray`` become float32 and int64 becomes int32.
* ``vmap``, ``lax.map``, ``lax.scan`` are python loops; ``jit`` is the identity.
* ``jvp``/``value_and_grad``/``random`` raise if called (no autodiff here).
"""

import sys
import types

import numpy as np

X64 = True


class _AtOp:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx

    def set(self, v):
        out = np.array(self.arr, copy=True).view(AtArray)
        out[self.idx] = v
        return out

    def add(self, v):
        out = np.array(self.arr, copy=True).view(AtArray)
        np.add.at(out, self.idx, v)
        return out

    def divide(self, v):
        out = np.array(self.arr, copy=True).view(AtArray)
        np.divide.at(out, self.idx, v)
        return out


class _AtIndexer:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtOp(self.arr, idx)


class AtArray(np.ndarray):
    @property
    def at(self):
        return _AtIndexer(self)


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, AtArray):
        return x.view(AtArray)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    return x


def _canon(a):
    a = np.asarray(a)
    if not X64:
        if a.dtype == np.float64:
            a = a.astype(np.float32)
        elif a.dtype == np.int64:
            a = a.astype(np.int32)
    return a


def _array(x, dtype=None, **kw):
    if dtype is not None:
        if dtype is float:
            dtype = np.float64 if X64 else np.float32
        elif dtype is int:
            dtype = np.int64 if X64 else np.int32
        return np.array(x, dtype=dtype).view(AtArray)
    return _canon(np.array(x)).view(AtArray)


def _dtype_kw(kw):
    d = kw.get("dtype", None)
    if d is float:
        kw["dtype"] = np.float64 if X64 else np.float32
    elif d is int:
        kw["dtype"] = np.int64 if X64 else np.int32
    return kw


class _JNP(types.ModuleType):
    ndarray = np.ndarray
    pi = np.pi

    def __getattr__(self, name):
        obj = getattr(np, name)
        if callable(obj) and not isinstance(obj, type):
            def f(*a, **kw):
                kw = _dtype_kw(kw)
                out = obj(*a, **kw)
                if name in ("zeros", "ones", "full", "arange", "linspace", "eye") and "dtype" not in kw:
                    out = _canon(out)
                return _wrap(out)
            return f
        return obj


jnp = _JNP("jax.numpy")
jnp.array = _array
jnp.asarray = _array


# ---------------------------------------------------------------- pytrees

def tree_map(f, tree, *rest, is_leaf=None):
    if is_leaf is not None and is_leaf(tree):
        return f(tree, *rest)
    if isinstance(tree, dict):
        return {k: tree_map(f, tree[k], *[r[k] for r in rest], is_leaf=is_leaf) for k in tree}
    if isinstance(tree, (list, tuple)) and not hasattr(tree, "_fields"):
        return type(tree)(tree_map(f, t, *[r[i] for r in rest], is_leaf=is_leaf)
                          for i, t in enumerate(tree))
    if tree is None:
        return None
    return f(tree, *rest)


def tree_leaves(tree):
    out = []
    tree_map(lambda x: out.append(x), tree)
    return out


def _map_axes(spec, arg, b):
    if spec is None:
        return arg
    if spec == 0 and not isinstance(spec, (dict, list, tuple)):
        return tree_map(lambda a: a[b], arg)
    if isinstance(spec, dict):
        return {k: _map_axes(spec[k], arg[k], b) for k in arg}
    if isinstance(spec, (list, tuple)):
        return type(arg)(_map_axes(s, a, b) for s, a in zip(spec, arg))
    raise ValueError(spec)


def _batch_size(spec, arg):
    if spec is None:
        return None
    if spec == 0 and not isinstance(spec, (dict, list, tuple)):
        ls = tree_leaves(arg)
        return ls[0].shape[0] if ls else None
    items = spec.items() if isinstance(spec, dict) else enumerate(spec)
    for k, s in items:
        n = _batch_size(s, arg[k])
        if n is not None:
            return n
    return None


def vmap(fun, in_axes=0):
    def vf(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        B = None
        for s, a in zip(axes, args):
            B = _batch_size(s, a)
            if B is not None:
                break
        outs = [fun(*[_map_axes(s, a, b) for s, a in zip(axes, args)]) for b in range(B)]
        return tree_map(lambda *xs: _wrap(np.stack(xs)), outs[0], *outs[1:])
    return vf


def jit(fun=None, **kw):
    if fun is None:
        return lambda f: f
    return fun


def _unavailable(*a, **k):
    raise NotImplementedError("autodiff / PRNG are not available in the numpy stand-in")


def segment_sum(data, segment_ids, num_segments=None, indices_are_sorted=False):
    out = np.zeros((num_segments,) + tuple(np.shape(data)[1:]), dtype=np.asarray(data).dtype)
    np.add.at(out, np.asarray(segment_ids), data)
    return _wrap(out)


def lax_map(f, xs):
    n = tree_leaves(xs)[0].shape[0]
    outs = [f(tree_map(lambda a: a[i], xs)) for i in range(n)]
    return tree_map(lambda *v: _wrap(np.stack(v)), outs[0], *outs[1:])


def lax_scan(f, init, xs):
    n = tree_leaves(xs)[0].shape[0]
    carry, ys = init, []
    for i in range(n):
        carry, y = f(carry, tree_map(lambda a: a[i], xs))
        ys.append(y)
    return carry, None


def dynamic_slice(operand, start, sizes):
    sl = tuple(slice(int(s), int(s) + int(z)) for s, z in zip(start, sizes))
    return _wrap(np.asarray(operand)[sl])


class _Stub(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _StubObj()


class _StubObj:
    def __call__(self, *a, **k):
        return _StubObj()

    def __getattr__(self, name):
        return _StubObj()


def install():
    """Register the stand-in modules in ``sys.modules``."""
    jax = types.ModuleType("jax")
    jax.numpy = jnp
    jax.jit = jit
    jax.vmap = vmap
    jax.jvp = _unavailable
    jax.value_and_grad = _unavailable
    nn = types.ModuleType("jax.nn")
    nn.tanh = lambda x: _wrap(np.tanh(x))
    nn.sigmoid = lambda x: _wrap(1 / (1 + np.exp(-np.asarray(x))))
    jax.nn = nn
    rnd = _Stub("jax.random")
    jax.random = rnd
    tu = types.ModuleType("jax.tree_util")
    tu.tree_map = tree_map
    tu.tree_leaves = tree_leaves
    tu.tree_flatten = _unavailable
    tu.tree_unflatten = _unavailable
    jax.tree_util = tu
    ops = types.ModuleType("jax.ops")
    ops.segment_sum = segment_sum
    jax.ops = ops
    lax = types.ModuleType("jax.lax")
    lax.map = lax_map
    lax.scan = lax_scan
    lax.dynamic_slice = dynamic_slice
    jax.lax = lax
    mods = {"jax": jax, "jax.numpy": jnp, "jax.nn": nn, "jax.random": rnd, "jax.tree_util": tu,
            "jax.ops": ops, "jax.lax": lax}
    for name in ["optax", "matplotlib", "matplotlib.pyplot", "matplotlib.collections",
                 "IPython", "IPython.display", "tensorboardX", "PIL", "PIL.Image"]:
        mods[name] = _Stub(name)
    sys.modules.update(mods)
