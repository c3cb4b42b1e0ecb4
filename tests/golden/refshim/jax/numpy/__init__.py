"""numpy-backed stand-in for the ``jax.numpy`` subset the reference uses.

All floating arrays are float32 and all integer arrays int32 (JAX with x64
disabled).  Reductions are sequential float32 folds.  See ../README.md.
"""
import builtins as _bi

import numpy as _np

float32 = _np.float32
float64 = _np.float64
int32 = _np.int32
int64 = _np.int64
bool_ = _np.bool_
newaxis = None
ndarray = _np.ndarray


def _canon_dtype(dt):
    dt = _np.dtype(dt)
    if dt.kind == "f":
        return _np.dtype(_np.float32)
    if dt.kind in "iu":
        return _np.dtype(_np.int32)
    return dt


def _plain(x):
    if isinstance(x, JArray):
        return x.view(_np.ndarray)
    if isinstance(x, (tuple, list)):
        return type(x)(_plain(v) for v in x)
    return x


def _wrap(x):
    if isinstance(x, _np.ndarray):
        dt = _canon_dtype(x.dtype)
        if x.dtype != dt:
            x = x.astype(dt)
        return x.view(JArray)
    if isinstance(x, _np.generic):
        dt = _canon_dtype(x.dtype)
        return _np.asarray(x, dtype=dt).view(JArray)
    return x


def _is_py_scalar(x):
    return isinstance(x, (_bi.int, _bi.float, _bi.bool)) and not isinstance(x, _np.generic)


def _promote(args):
    """JAX-style promotion: if any operand is floating (array or Python
    float), integer/bool arrays are cast to float32."""
    any_float = False
    for a in args:
        if isinstance(a, (_np.ndarray, _np.generic)):
            if _np.dtype(a.dtype).kind == "f":
                any_float = True
        elif isinstance(a, _bi.float):
            any_float = True
    out = []
    for a in args:
        if isinstance(a, (_np.ndarray, _np.generic)):
            a = _np.asarray(a)
            dt = _canon_dtype(a.dtype)
            if any_float and dt.kind in "iub":
                dt = _np.dtype(_np.float32)
            a = a.astype(dt, copy=False)
        out.append(a)
    return out


def _integer_pow(x, k):
    """lax.integer_pow: binary exponentiation by repeated squaring."""
    if k == 0:
        return _np.ones_like(x)
    neg = k < 0
    k = abs(k)
    acc = None
    while k > 0:
        if k & 1:
            acc = x if acc is None else acc * x
        k >>= 1
        if k > 0:
            x = x * x
    return 1 / acc if neg else acc


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtSet(self._arr, idx)


class _AtSet:
    def __init__(self, arr, idx):
        self._arr, self._idx = arr, idx

    def set(self, value):
        out = _np.array(self._arr.view(_np.ndarray), copy=True)
        out[_plain(self._idx)] = _plain(value)
        return _wrap(out)


class JArray(_np.ndarray):
    """ndarray subclass with JAX dtype promotion and ``.at[].set``."""

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        if kwargs.get("out") is not None:
            raise NotImplementedError("out= is not supported")
        ins = [_plain(i) for i in inputs]
        if method == "__call__" and ufunc is _np.power and len(ins) == 2 and isinstance(ins[1], _bi.int):
            base = _promote([ins[0]])[0]
            return _wrap(_np.asarray(_integer_pow(base, ins[1])))
        if method == "__call__":
            ins = _promote(ins)
            if ufunc in (_np.sqrt, _np.cos, _np.sin, _np.exp, _np.log, _np.arccos) and \
                    _np.asarray(ins[0]).dtype.kind in "iub":
                ins[0] = _np.asarray(ins[0]).astype(_np.float32)
        res = getattr(ufunc, method)(*ins, **kwargs)
        if isinstance(res, tuple):
            return tuple(_wrap(_np.asarray(r)) for r in res)
        return _wrap(_np.asarray(res))

    @property
    def at(self):
        return _At(self)

    def __getitem__(self, idx):
        r = _np.ndarray.__getitem__(self.view(_np.ndarray), _plain(idx))
        return _wrap(r) if isinstance(r, (_np.ndarray, _np.generic)) else r

    def __bool__(self):
        return bool(self.view(_np.ndarray))


def _infer_dtype(x):
    a = _np.asarray(_plain(x))
    return _canon_dtype(a.dtype)


def array(x, dtype=None, copy=True):
    x = _plain(x)
    if hasattr(x, "__jax_array__"):
        x = _plain(x.__jax_array__())
    if dtype is None:
        a = _np.array(x)
        dtype = _canon_dtype(a.dtype)
    else:
        dtype = _canon_dtype(dtype)
    return _wrap(_np.array(x, dtype=dtype))


def asarray(x, dtype=None):
    return array(x, dtype)


def zeros(shape, dtype=None):
    return _wrap(_np.zeros(shape, dtype=_canon_dtype(dtype or _np.float32)))


def ones(shape, dtype=None):
    return _wrap(_np.ones(shape, dtype=_canon_dtype(dtype or _np.float32)))


def zeros_like(x, dtype=None):
    return _wrap(_np.zeros(_np.shape(_plain(x)), dtype=_canon_dtype(dtype or _infer_dtype(x))))


def ones_like(x, dtype=None):
    return _wrap(_np.ones(_np.shape(_plain(x)), dtype=_canon_dtype(dtype or _infer_dtype(x))))


def full(shape, fill_value, dtype=None):
    return _wrap(_np.full(shape, fill_value, dtype=_canon_dtype(dtype or _np.float32)))


def arange(*args, dtype=None):
    a = _np.arange(*args)
    return _wrap(a.astype(_canon_dtype(dtype or a.dtype)))


def repeat(a, repeats, axis=None):
    return _wrap(_np.repeat(_plain(a), repeats, axis=axis))


def _fold(x, axis):
    """Sequential left fold along ``axis`` in the array's (canonical) dtype."""
    x = _np.moveaxis(x, axis, 0)
    acc = x[0].copy()
    for i in range(1, x.shape[0]):
        acc = acc + x[i]
    return acc


def sum(a, axis=None, keepdims=False):
    x = _promote([_plain(a)])[0]
    x = _np.asarray(x)
    if axis is None:
        flat = x.reshape(-1)
        acc = _fold(flat, 0) if flat.size else _np.zeros((), x.dtype)
        r = _np.asarray(acc)
        if keepdims:
            r = r.reshape((1,) * x.ndim)
        return _wrap(r)
    axis = axis % x.ndim
    r = _np.asarray(_fold(x, axis)) if x.shape[axis] else _np.zeros(
        x.shape[:axis] + x.shape[axis + 1:], x.dtype)
    if keepdims:
        r = _np.expand_dims(r, axis)
    return _wrap(r)


def mean(a, axis=None, keepdims=False):
    x = _np.asarray(_promote([_plain(a)])[0])
    if x.dtype.kind in "iub":
        x = x.astype(_np.float32)
    n = x.size if axis is None else x.shape[axis]
    s = _np.asarray(sum(x, axis=axis, keepdims=keepdims).view(_np.ndarray))
    return _wrap(s / _np.asarray(n, dtype=s.dtype))


def dot(a, b):
    a, b = _promote([_plain(a), _plain(b)])
    a = _np.asarray(a)
    b = _np.asarray(b)
    if a.ndim == 1 and b.ndim == 1:
        prods = a * b
        return _wrap(_np.asarray(_fold(prods, 0)))
    if a.ndim == 2 and b.ndim == 1:
        prods = a * b[None, :]
        return _wrap(_np.asarray(_fold(prods, 1)))
    if a.ndim == 1 and b.ndim == 2:
        prods = a[:, None] * b
        return _wrap(_np.asarray(_fold(prods, 0)))
    if a.ndim == 2 and b.ndim == 2:
        prods = a[:, :, None] * b[None, :, :]
        return _wrap(_np.asarray(_fold(prods, 1)))
    raise NotImplementedError("dot for ndim", a.ndim, b.ndim)


def where(cond, x=None, y=None):
    cond = _plain(cond)
    if x is None and y is None:
        return tuple(_wrap(i) for i in _np.nonzero(cond))
    x, y = _plain(x), _plain(y)
    arrs = _promote([x, y])
    return _wrap(_np.asarray(_np.where(cond, arrs[0], arrs[1])))


def sqrt(x):
    x = _np.asarray(_promote([_plain(x)])[0])
    if x.dtype.kind in "iub":
        x = x.astype(_np.float32)
    return _wrap(_np.sqrt(x))


def cos(x):
    x = _np.asarray(_promote([_plain(x)])[0])
    if x.dtype.kind in "iub":
        x = x.astype(_np.float32)
    return _wrap(_np.cos(x))


def concatenate(arrs, axis=0):
    arrs = _promote([_np.asarray(_plain(a)) for a in arrs])
    return _wrap(_np.concatenate(arrs, axis=axis))


def stack(arrs, axis=0):
    arrs = _promote([_np.asarray(_plain(a)) for a in arrs])
    return _wrap(_np.stack(arrs, axis=axis))


def pad(a, pad_width, mode="constant", constant_values=0):
    return _wrap(_np.pad(_plain(a), pad_width, mode=mode, constant_values=constant_values))


def unique(a):
    return _wrap(_np.unique(_plain(a)))


def argwhere(a):
    return _wrap(_np.argwhere(_plain(a)))


def max(a, axis=None):
    return _wrap(_np.asarray(_np.max(_plain(a), axis=axis)))


def min(a, axis=None):
    return _wrap(_np.asarray(_np.min(_plain(a), axis=axis)))


def shape(a):
    return _np.shape(_plain(a))
