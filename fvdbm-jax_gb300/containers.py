"""Host-side ``Cells``/``Faces``/``Nodes`` containers with the reference's
attribute names, shapes and dtypes (reference ``src/containers.py:18-408``).

They are plain numpy holders: ``Mesher.to_env`` fills them, the boundary
setters mutate them, and ``Environment.init`` uploads them to the device.
Once an ``Environment`` owns them, the dynamic leaves (``pdf``, ``rho``,
``vel``, ``pdf_eq``) read through to the device state and writes to them are
uploaded before the next step; the static leaves are frozen at ``init``.

Reference containers (JAX pytrees) are accepted too: ``from_any`` copies any
object exposing the same attributes into these classes.
"""
from __future__ import annotations

import numpy as np

from .dynamics import D2Q9, as_lattice

F32, I32 = np.float32, np.int32

FLUX_SCHEMES = ("upwind", "lax_wendroff")


class _Container:
    _dynamic: tuple = ("pdf",)

    def __init__(self, size: int, dynamics):
        self.dynamics = dynamics
        object.__setattr__(self, "_owner", None)
        self.pdf = np.repeat(dynamics.rest_pdf()[None, :], size, axis=0).astype(F32)

    def __getattribute__(self, name):
        if name in type(self)._dynamic:
            owner = object.__getattribute__(self, "_owner")
            if owner is not None:
                owner._pull(self, name)
        return object.__getattribute__(self, name)

    def __setattr__(self, name, value):
        if name in type(self)._dynamic:
            owner = object.__getattribute__(self, "_owner")
            value = np.array(value, dtype=F32, copy=True)
            object.__setattr__(self, name, value)
            if owner is not None:
                owner._push(self, name)
            return
        object.__setattr__(self, name, value)

    def init(self):
        """Reference ``Container.init`` converts padded builders into arrays;
        here the arrays are already final."""
        return None

    def __repr__(self):
        keys = [k for k in self.__dict__ if not k.startswith("_")]
        return f"{type(self).__name__}({', '.join(keys)})"


class Cells(_Container):
    """Cells: dynamic ``pdf [N,9]``, ``rho [N,1]``, ``vel [N,2]``,
    ``pdf_eq [N,9]``; static ``face_indices [N,K]`` and ``face_normals [N,K]``
    (signs), reference ``src/containers.py:47-134``."""

    _dynamic = ("pdf", "rho", "vel", "pdf_eq")

    def __init__(self, size: int, dynamics):
        super().__init__(size, dynamics)
        self.rho = np.zeros((size, 1), F32)
        self.vel = np.zeros((size, dynamics.DIM), F32)
        self.pdf_eq = np.zeros((size, dynamics.NUM_QUIVERS), F32)
        self.face_indices = -np.ones((size, 1), I32)
        self.face_normals = -np.ones((size, 1), I32)


class Faces(_Container):
    """Faces: dynamic ``pdf [F,9]`` (the flux); static ``nodes_index [F,2]``,
    ``stencil_cells_index [F,2]`` (-1 = ghost), ``stencil_dists [F,2]``,
    ``n [F,2]``, ``L [F,1]``, ``flux_scheme``; reference
    ``src/containers.py:136-291``.  ``alpha [F,1]`` (cos-weighted
    cell-centre stencil, ``src/faces.py:10-74``) and ``npq [F,2]``
    (xi-ratio stencil, ``src/faces.py:76-141``) are set for those variants."""

    def __init__(self, size: int, dynamics, flux_scheme: str = "upwind"):
        super().__init__(size, dynamics)
        self.nodes_index = -np.ones((size, 2), I32)
        self.stencil_cells_index = -np.ones((size, 2), I32)
        self.stencil_dists = -np.ones((size, 2), F32)
        self.n = np.zeros((size, dynamics.DIM), F32)
        self.L = np.zeros((size, 1), F32)
        self.flux_scheme = flux_scheme
        self.stencil_variant = None   # None, "cos" (CCStencilFaces) or "ksi" (CCStencilKsiFaces)
        self.alpha = None
        self.npq = None


class Nodes(_Container):
    """Nodes: dynamic ``pdf [P,9]``, ``rho [P,1]``, ``vel [P,2]``; static
    ``type [P,1]`` (0 none, 1 velocity, 2 density), ``cells_index [P,K]`` and
    ``cell_dists [P,K]`` (-1 padded); reference ``src/containers.py:293-408``."""

    _dynamic = ("pdf", "rho", "vel")

    def __init__(self, size: int, dynamics):
        super().__init__(size, dynamics)
        self.rho = np.zeros((size, 1), F32)
        self.vel = np.zeros((size, dynamics.DIM), F32)
        self.type = np.zeros((size, 1), I32)
        self.cells_index = -np.ones((size, 1), I32)
        self.cell_dists = -np.ones((size, 1), F32)


def _arr(x, dtype):
    return np.array(np.asarray(x), dtype=dtype, copy=True)


def _rows(a, n: int):
    """a as [n, k]; a 2-D array keeps its k (also when n is 0, where
    reshape(0, -1) has no answer)."""
    if a.ndim == 2 and a.shape[0] == n:
        return a
    if n == 0:
        return a.reshape(0, a.shape[-1] if a.ndim >= 2 else 1)
    return a.reshape(n, -1)


def from_any(cells, faces, nodes, dynamics=None):
    """Copy reference (or these) containers into fresh host containers; the
    originals are never modified.
    Flux-scheme variants are recognised by the reference's class names
    ``CCStencilFaces`` (``alpha``) and ``CCStencilKsiFaces`` (``npq``)."""
    dyn = dynamics or getattr(cells, "dynamics", None)
    if dyn is None:
        raise ValueError("containers carry no dynamics; pass dynamics=")
    dyn = as_lattice(dyn)
    Q = dyn.NUM_QUIVERS
    N = int(np.shape(cells.pdf)[0])
    F = int(np.shape(faces.pdf)[0])
    P = int(np.shape(nodes.pdf)[0])
    c = Cells(N, dyn)
    c.pdf = _arr(cells.pdf, F32)
    c.rho = _arr(cells.rho, F32).reshape(N, 1)
    c.vel = _arr(cells.vel, F32).reshape(N, 2)
    c.pdf_eq = _arr(cells.pdf_eq, F32).reshape(N, Q)
    c.face_indices = _rows(_arr(cells.face_indices, I32), N)
    c.face_normals = _rows(_arr(cells.face_normals, I32), N)
    for extra in ("centroids", "areas"):
        if getattr(cells, extra, None) is not None:
            setattr(c, extra, _arr(getattr(cells, extra), F32))

    f = Faces(F, dyn, getattr(faces, "flux_scheme", "upwind"))
    f.pdf = _arr(faces.pdf, F32)
    f.nodes_index = _arr(faces.nodes_index, I32).reshape(F, 2)
    f.stencil_cells_index = _arr(faces.stencil_cells_index, I32).reshape(F, 2)
    f.stencil_dists = _arr(faces.stencil_dists, F32).reshape(F, 2)
    f.n = _arr(faces.n, F32).reshape(F, 2)
    f.L = _arr(faces.L, F32).reshape(F, 1)
    variant = getattr(faces, "stencil_variant", None)
    cls = type(faces).__name__
    if variant == "cos" or cls == "CCStencilFaces":
        f.stencil_variant, f.alpha = "cos", _arr(faces.alpha, F32).reshape(F, 1)
    elif variant == "ksi" or cls == "CCStencilKsiFaces":
        f.stencil_variant, f.npq = "ksi", _arr(faces.npq, F32).reshape(F, 2)

    n = Nodes(P, dyn)
    n.pdf = _arr(nodes.pdf, F32)
    n.rho = _arr(nodes.rho, F32).reshape(P, 1)
    n.vel = _arr(nodes.vel, F32).reshape(P, 2)
    n.type = _arr(nodes.type, I32).reshape(P, 1)
    n.cells_index = _rows(_arr(nodes.cells_index, I32), P)
    n.cell_dists = _rows(_arr(nodes.cell_dists, F32), P)
    return c, f, n
