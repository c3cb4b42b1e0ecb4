"""numpy-backed stand-in for the ``jax`` subset the reference imports:
``jit`` (identity), ``vmap`` (loop over the mapped axis), ``lax.select``,
``tree_util.register_pytree_node_class`` (identity).  See ../README.md."""
import numpy as _np

from . import numpy  # noqa: F401
from . import lax, tree_util, typing  # noqa: F401
from .numpy import JArray as Array, _wrap, _plain


def jit(fun=None, **kwargs):
    if fun is None:
        return lambda f: f
    return fun


def _take(a, i, axis):
    if axis == 0:
        return a[i]
    return _wrap(_np.take(_plain(a), i, axis=axis))


def _stack(outs):
    first = outs[0]
    if isinstance(first, tuple):
        return tuple(_stack([o[k] for o in outs]) for k in range(len(first)))
    return _wrap(_np.stack([_np.asarray(_plain(o)) for o in outs]))


def vmap(fun, in_axes=0, out_axes=0):
    def wrapped(*args):
        axes = tuple(in_axes) if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = None
        for a, ax in zip(args, axes):
            if ax is not None:
                n = _np.shape(_plain(a))[ax]
                break
        if not n:
            raise ValueError("vmap over an empty axis is not supported by the stand-in")
        outs = [fun(*[a if ax is None else _take(a, i, ax) for a, ax in zip(args, axes)])
                for i in range(n)]
        return _stack(outs)
    return wrapped
