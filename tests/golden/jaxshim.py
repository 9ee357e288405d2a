"""A minimal numpy-backed stand-in for the JAX API used by jax-powspec's
src/mas.py and src/correlations.py (P(k) part), so that the reference's own
source can be imported and run here (JAX is not installed) to produce golden
fixtures.  Test infrastructure only -- used by make_golden.py.

Semantics restated from JAX's published behaviour with 64-bit mode off:
  * dtypes are canonicalised to bool / int32 / float32 / complex64;
  * promotion: bool < int < float < complex; int32 with float32 gives
    float32; Python scalars are "weak" and take the other operand's type;
    arguments of a jitted function that are Python scalars become weak
    0-d arrays (as jax.jit traces them);
  * ``x.at[idx].add(v)`` / ``.set(v)``: updates applied in order; a negative
    index counts once from the end; an update with any index still outside
    [0, n) is dropped (FILL_OR_DROP);
  * ``jnp.histogram`` with array bins: searchsorted(bins, a, 'right'), values
    equal to the last edge go to the last bin, then
    ``zeros(len(bins), weights.dtype).at[idx].add(weights)[1:]``;
  * ``jnp.sinc`` = sin(pi x)/(pi x) with value 1 at x == 0, in float32;
  * ``jnp.fft.rfftn`` / ``irfftn`` in complex64 / float32 (scipy.fft single
    precision; irfftn normalised by 1/N like numpy and JAX);
  * ``lax.cond`` / ``lax.scan`` evaluated eagerly.
"""
from __future__ import annotations

import sys
import types

import numpy as np
import scipy.fft

_CANON = {np.dtype(np.float64): np.dtype(np.float32), np.dtype(np.int64): np.dtype(np.int32),
          np.dtype(np.complex128): np.dtype(np.complex64), np.dtype(np.uint64): np.dtype(np.uint32),
          np.dtype(np.float16): np.dtype(np.float32)}
_RANK = {"b": 0, "u": 1, "i": 1, "f": 2, "c": 3}
_DEFAULT = {0: np.dtype(bool), 1: np.dtype(np.int32), 2: np.dtype(np.float32), 3: np.dtype(np.complex64)}
_FLOAT_UFUNCS = {np.true_divide, np.sqrt, np.sin, np.cos, np.tan, np.exp, np.log, np.arctan2, np.arcsin,
                 np.arccos, np.arctan, np.log10, np.expm1, np.log1p, np.sinh, np.cosh, np.tanh}


def canon(dt) -> np.dtype:
    dt = np.dtype(dt)
    return _CANON.get(dt, dt)


class JArray(np.ndarray):
    """ndarray with JAX's promotion, a weak-type flag and the ``.at`` helper."""

    weak = False

    def __array_finalize__(self, obj):
        self.weak = False

    @property
    def at(self):
        return _At(self)

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        out = kwargs.pop("out", None)
        if out is not None:
            # in-place update (`a *= b`): jax rebinds instead; compute then copy back
            res = self.__array_ufunc__(ufunc, method, *inputs, **kwargs)
            target = out[0] if isinstance(out, tuple) else out
            np.copyto(target.view(np.ndarray), np.asarray(res).astype(target.dtype))
            return target
        if method != "__call__":
            inputs = tuple(np.asarray(x) if isinstance(x, JArray) else x for x in inputs)
            return getattr(ufunc, method)(*inputs, **kwargs)
        if ufunc is np.power and len(inputs) == 2 and isinstance(inputs[1], int) and not isinstance(inputs[1], bool) \
                and inputs[1] >= 0:
            return _integer_pow(inputs[0], inputs[1])
        common = promote(*inputs)
        if ufunc in _FLOAT_UFUNCS and _RANK[common.kind] < 2:
            common = np.dtype(np.float32)
        args = [np.asarray(x).astype(common) if not _is_pyscalar(x) else np.asarray(x, dtype=common)
                for x in inputs]
        res = ufunc(*args, **kwargs)
        all_weak = all(_is_weak(x) for x in inputs)
        return wrap(res, weak=all_weak)

    def __getitem__(self, item):
        return wrap(np.ndarray.__getitem__(self.view(np.ndarray), item))


def _integer_pow(x, y: int):
    """lax.integer_pow: binary exponentiation by repeated multiplication."""
    x = x if isinstance(x, JArray) else wrap(np.asarray(x))
    if y == 0:
        return wrap(np.ones_like(np.asarray(x)), weak=x.weak)
    acc = None
    while y > 0:
        if y & 1:
            acc = x if acc is None else acc * x
        y >>= 1
        if y > 0:
            x = x * x
    return acc


def _is_pyscalar(x) -> bool:
    return isinstance(x, (bool, int, float, complex)) and not isinstance(x, np.generic)


def _is_weak(x) -> bool:
    return _is_pyscalar(x) or (isinstance(x, JArray) and x.weak)


def _kind_of_pyscalar(x) -> int:
    if isinstance(x, bool):
        return 0
    if isinstance(x, int):
        return 1
    if isinstance(x, float):
        return 2
    return 3


def promote(*xs) -> np.dtype:
    strong, weak_rank = [], -1
    for x in xs:
        if _is_pyscalar(x):
            weak_rank = max(weak_rank, _kind_of_pyscalar(x))
        elif isinstance(x, JArray) and x.weak:
            weak_rank = max(weak_rank, _RANK[x.dtype.kind])
        else:
            strong.append(canon(np.asarray(x).dtype))
    if not strong:
        return _DEFAULT[max(weak_rank, 0)]
    rank = max(_RANK[d.kind] for d in strong)
    same = [d for d in strong if _RANK[d.kind] == rank]
    best = max(same, key=lambda d: d.itemsize)
    if weak_rank > rank:
        return _DEFAULT[weak_rank]
    return best


def wrap(a, weak: bool = False) -> JArray:
    a = np.asarray(a)
    a = a.astype(canon(a.dtype), copy=False)
    out = a.view(JArray)
    out.weak = bool(weak)
    return out


def weak_scalar(v) -> JArray:
    return wrap(np.asarray(v, dtype=_DEFAULT[_kind_of_pyscalar(v)]), weak=True)


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIndex(self.arr, idx)


class _AtIndex:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx if isinstance(idx, tuple) else (idx,)

    def _norm(self):
        arr = self.arr
        parts, ok = [], None
        full = len(self.idx) == arr.ndim
        for k, a in enumerate(self.idx):
            a = np.asarray(a)
            if a.dtype.kind not in "iu":
                raise TypeError("only integer indices are supported")
            n = arr.shape[k]
            a = a.astype(np.int64)
            a = np.where(a < 0, a + n, a)
            good = (a >= 0) & (a < n)
            ok = good if ok is None else (ok & good)
            parts.append(a)
        if not full:
            raise TypeError("partial indexing is not supported by this shim")
        shape = np.broadcast(*parts).shape
        parts = [np.broadcast_to(p, shape).ravel() for p in parts]
        ok = np.broadcast_to(ok, shape).ravel()
        return parts, ok, shape

    def _basic(self) -> bool:
        return any(isinstance(a, slice) or a is Ellipsis for a in self.idx)

    def add(self, vals):
        out = np.array(self.arr, copy=True)
        if self._basic():
            np.add.at(out, self.idx, np.asarray(vals).astype(out.dtype))
            return wrap(out)
        parts, ok, shape = self._norm()
        v = np.broadcast_to(np.asarray(vals).astype(out.dtype), shape).ravel()
        np.add.at(out, tuple(p[ok] for p in parts), v[ok])
        return wrap(out)

    def set(self, vals):
        out = np.array(self.arr, copy=True)
        if self._basic():
            out[self.idx] = np.asarray(vals).astype(out.dtype)
            return wrap(out)
        parts, ok, shape = self._norm()
        v = np.broadcast_to(np.asarray(vals).astype(out.dtype), shape).ravel()
        sel = tuple(p[ok] for p in parts)
        out[sel] = v[ok]          # numpy keeps the last of duplicate indices (in-order writes)
        return wrap(out)


class _Caster:
    """jnp.int32 / jnp.float32: usable as a dtype and as a converting function."""

    def __init__(self, dt):
        self.dtype = np.dtype(dt)

    def __call__(self, x):
        return wrap(np.asarray(x).astype(self.dtype))


def _dt(dtype):
    if dtype is None:
        return None
    return dtype.dtype if isinstance(dtype, _Caster) else canon(dtype)


def _build_jnp():
    jnp = types.ModuleType("jax.numpy")
    jnp.pi = np.pi
    jnp.inf = np.inf
    jnp.int32 = _Caster(np.int32)
    jnp.float32 = _Caster(np.float32)
    jnp.complex64 = _Caster(np.complex64)

    def asarray(x, dtype=None):
        if _is_pyscalar(x) and dtype is None:
            return weak_scalar(x)
        a = np.asarray(x)
        return wrap(a if dtype is None else a.astype(_dt(dtype)))

    jnp.asarray = asarray
    jnp.array = asarray
    jnp.zeros = lambda shape, dtype=None: wrap(np.zeros(shape, dtype=_dt(dtype) or np.float32))
    jnp.ones = lambda shape, dtype=None: wrap(np.ones(shape, dtype=_dt(dtype) or np.float32))
    jnp.ones_like = lambda a, dtype=None: wrap(np.ones_like(np.asarray(a), dtype=_dt(dtype)))
    jnp.zeros_like = lambda a, dtype=None: wrap(np.zeros_like(np.asarray(a), dtype=_dt(dtype)))

    def arange(*args, dtype=None):
        if dtype is None and all(isinstance(a, int) for a in args):
            return wrap(np.arange(*args, dtype=np.int32))
        fargs = [np.float32(a) if not isinstance(a, np.ndarray) else a for a in args]
        return wrap(np.arange(*fargs, dtype=_dt(dtype) or np.float32))

    jnp.arange = arange

    def where(c, a, b):
        dt = promote(a, b)
        return wrap(np.where(np.asarray(c), np.asarray(a, dtype=dt) if _is_pyscalar(a) else np.asarray(a).astype(dt),
                             np.asarray(b, dtype=dt) if _is_pyscalar(b) else np.asarray(b).astype(dt)))

    jnp.where = where
    jnp.broadcast_to = lambda a, shape: wrap(np.broadcast_to(np.asarray(a), shape))
    jnp.logical_and = lambda a, b: wrap(np.logical_and(np.asarray(a), np.asarray(b)))
    jnp.nansum = lambda a: wrap(np.asarray(np.nansum(np.asarray(a))))   # keeps the input's float dtype

    def _unary(fn):
        def f(x):
            x = asarray(x) if not isinstance(x, JArray) else x
            return fn(x)
        return f

    jnp.sqrt = _unary(np.sqrt)
    jnp.sin = _unary(np.sin)
    jnp.cos = _unary(np.cos)
    jnp.exp = _unary(np.exp)
    jnp.abs = _unary(np.abs)

    def sinc(x):
        x = asarray(x)
        if _RANK[x.dtype.kind] < 2:
            x = wrap(np.asarray(x).astype(np.float32))
        eq0 = np.asarray(x == 0)
        pix = np.pi * x
        safe = where(eq0, 1, pix)
        return where(eq0, 1.0, np.sin(safe) / safe)

    jnp.sinc = sinc

    def histogram(a, bins=10, range=None, weights=None, density=None):
        if range is not None or density:
            raise NotImplementedError
        a = asarray(a).ravel()
        edges = asarray(bins)
        if _RANK[edges.dtype.kind] < 2:
            edges = wrap(np.asarray(edges).astype(np.float32))
        if weights is None:
            weights = wrap(np.ones(a.shape, dtype=promote(a, 1.0)))
        idx = np.searchsorted(np.asarray(edges), np.asarray(a), side="right")
        idx = np.where(np.asarray(a) == np.asarray(edges)[-1], edges.size - 1, idx)
        counts = wrap(np.zeros(edges.size, dtype=canon(np.asarray(weights).dtype)))
        counts = counts.at[idx].add(asarray(weights).ravel())
        return counts[1:], edges

    jnp.histogram = histogram

    fft = types.ModuleType("jax.numpy.fft")

    def rfftn(x, s=None, axes=None):
        x = np.asarray(x)
        if x.dtype.kind != "f":
            x = x.astype(np.float32)
        return wrap(scipy.fft.rfftn(x.astype(np.float32), s=s, axes=axes).astype(np.complex64))

    def irfftn(x, s=None, axes=None):
        x = np.asarray(x).astype(np.complex64)
        return wrap(scipy.fft.irfftn(x, s=s, axes=axes).astype(np.float32))

    fft.rfftn = rfftn
    fft.irfftn = irfftn
    jnp.fft = fft
    return jnp


def _jit(fn=None, **kw):
    if fn is None:
        return lambda f: _jit(f, **kw)

    def traced(*args):
        args = [weak_scalar(a) if _is_pyscalar(a) else (a if isinstance(a, JArray) else wrap(np.asarray(a)))
                for a in args]
        return fn(*args)

    traced.__wrapped__ = fn
    return traced


def _cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(np.asarray(pred)) else false_fun(*operands)


def _scan(f, init, xs, length=None):
    carry = init
    leaves = xs if isinstance(xs, (tuple, list)) else (xs,)
    n = len(leaves[0])
    ys = []
    for i in range(n):
        step = tuple(wrap(np.asarray(leaf)[i]) for leaf in leaves)
        step = step if isinstance(xs, (tuple, list)) else step[0]
        carry, y = f(carry, step)
        ys.append(y)
    if ys and isinstance(ys[0], tuple):
        stacked = tuple(wrap(np.stack([np.asarray(y[k]) for y in ys])) for k in range(len(ys[0])))
    else:
        stacked = wrap(np.stack([np.asarray(y) for y in ys])) if ys else None
    return carry, stacked


def install() -> None:
    """Register the shim as `jax` (and stub what the reference imports but never uses)."""
    jax = types.ModuleType("jax")
    jnp = _build_jnp()
    lax = types.ModuleType("jax.lax")
    lax.cond = _cond
    lax.scan = _scan
    experimental = types.ModuleType("jax.experimental")
    loops = types.ModuleType("jax.experimental.loops")       # imported by the reference, unused on this path
    experimental.loops = loops
    jax.numpy, jax.lax, jax.experimental = jnp, lax, experimental
    jax.jit = _jit
    sys.modules.update({"jax": jax, "jax.numpy": jnp, "jax.numpy.fft": jnp.fft, "jax.lax": lax,
                        "jax.experimental": experimental, "jax.experimental.loops": loops})
    # src/correlations.py:1 imports a private numpy helper that numpy 2 no longer has.
    import numpy.core.defchararray as dca
    if not hasattr(dca, "_join_dispatcher"):
        dca._join_dispatcher = lambda *a, **k: a
