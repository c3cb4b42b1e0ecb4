"""lax.select stand-in (element-wise select; both branches already evaluated)."""
import numpy as _np

from .numpy import _plain, _wrap


def select(pred, on_true, on_false):
    return _wrap(_np.asarray(_np.where(_plain(pred), _plain(on_true), _plain(on_false))))
