"""``Environment``: drop-in for the reference's ``Environment``
(``src/environment.py:10-68``) backed by the CUDA kernels of libfvdbm.

    env = Environment(cells, faces, nodes)   # src/environment.py:15-18
    env.init()                               # :38-42 (uploads, builds tables)
    for _ in range(n):
        env = env.step()                     # :55-65, returns self

The environment holds its own copies of the containers (the caller's objects
are never modified, as with the reference's jitted step).  After ``step``
``env.cells``/``env.faces``/``env.nodes`` read through to the device: ``cells.pdf`` is
the updated pdf; ``cells.rho``, ``cells.vel``, ``cells.pdf_eq`` and
``faces.pdf`` (the fluxes) are those of the pdf before the last update, as
the reference leaves them; ``nodes.pdf/rho/vel`` are the node state.
Writing a dynamic leaf (``cells.pdf``, ``nodes.pdf/rho/vel``) uploads it
before the next step, as replacing a pytree leaf does in the reference.

``step(n)`` runs n steps in one call (replayed from a captured CUDA graph).
Errors are Python exceptions: an unknown ``flux_scheme`` raises
``ValueError`` as ``Faces.calc_fluxes`` does (``src/containers.py:202-203``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from .containers import Cells, Faces, Nodes, _Container, from_any
from .dynamics import D2Q9, as_lattice

F32, I32 = np.float32, np.int32

_ORDER = {"none": nat.ORDER_NONE, "rcm": nat.ORDER_RCM, "morton": nat.ORDER_MORTON}
_KERNEL = {"auto": nat.KERNEL_AUTO, "staged": nat.KERNEL_STAGED, "fused": nat.KERNEL_FUSED,
           "tile": nat.KERNEL_TILE, "tile_split": nat.KERNEL_TILE_SPLIT, "one": nat.KERNEL_ONE,
           "fused_nodes": nat.KERNEL_FUSED_NODES, "persist": nat.KERNEL_PERSIST,
           "fast": nat.KERNEL_FAST}


def _face_scale(faces):
    """Flux multipliers of the cell-centre stencil classes, float32 as the
    reference computes them (``src/faces.py:71-72``, ``:136-138``)."""
    v = getattr(faces, "stencil_variant", None)
    if v == "cos":
        return nat.VARIANT_FACE_SCALE, np.ascontiguousarray(
            np.cos(np.asarray(faces.alpha, F32).reshape(-1)), F32)
    if v == "ksi":
        ksi = D2Q9.KSI.astype(F32)
        n = np.asarray(faces.n, F32)
        npq = np.asarray(faces.npq, F32).reshape(-1, 2)
        num = ksi[None, 1:, 0] * n[:, None, 0] + ksi[None, 1:, 1] * n[:, None, 1]
        den = ksi[None, 1:, 0] * npq[:, None, 0] + ksi[None, 1:, 1] * npq[:, None, 1]
        with np.errstate(divide="ignore", invalid="ignore"):
            r = np.concatenate([np.zeros((n.shape[0], 1), F32), num / den], axis=1)
        return nat.VARIANT_FACE_Q_SCALE, np.ascontiguousarray(r, F32)
    return nat.VARIANT_NONE, None


def pack(c, f, n, *, ordering="auto", kernel="auto", device=0, finite_volume=False):
    """The C-ABI mesh and parameter structs of one case (``fvdbm_mesh_t``,
    ``fvdbm_params_t``), the arrays they point into (keep them alive), the
    sizes (N, F, P) and the case's D2Q9 dynamics."""
    if f.flux_scheme not in ("upwind", "lax_wendroff"):
        raise ValueError(f"Unknown flux scheme: {f.flux_scheme}")
    dyn = as_lattice(c.dynamics)
    a = {
        "cfi": np.ascontiguousarray(c.face_indices, I32),
        "cfs": np.ascontiguousarray(c.face_normals, I32),
        "fc": np.ascontiguousarray(f.stencil_cells_index, I32),
        "fd": np.ascontiguousarray(f.stencil_dists, F32),
        "fn_": np.ascontiguousarray(f.nodes_index, I32),
        "fnrm": np.ascontiguousarray(f.n, F32),
        "fL": np.ascontiguousarray(np.asarray(f.L, F32).reshape(-1)),
        "nt": np.ascontiguousarray(np.asarray(n.type, I32).reshape(-1)),
        "nc": np.ascontiguousarray(n.cells_index, I32),
        "nd": np.ascontiguousarray(n.cell_dists, F32),
    }
    N, F, P = a["cfi"].shape[0], a["fc"].shape[0], a["nt"].shape[0]
    if a["nc"].shape[0] != P or a["nd"].shape != a["nc"].shape:
        raise ValueError("Nodes.cells_index / cell_dists shapes disagree")
    if a["cfs"].shape != a["cfi"].shape:
        raise ValueError("Cells.face_indices / face_normals shapes disagree")
    variant, scale = _face_scale(f)
    a["scale"] = scale
    xy = getattr(c, "centroids", None)
    a["xy"] = None if xy is None else np.ascontiguousarray(xy, F32)
    a["ia"] = None
    area = getattr(c, "areas", None)
    a["area"] = None if area is None else np.ascontiguousarray(np.asarray(area, F32).reshape(-1), F32)
    if finite_volume:
        area = getattr(c, "areas", None)
        if area is None:
            raise ValueError("finite_volume=True needs cell areas (cells.areas)")
        a["ia"] = np.ascontiguousarray(F32(1) / np.asarray(area, F32).reshape(-1), F32)
    order = ordering
    if order == "auto":
        order = "morton" if a["xy"] is not None else "rcm"
    mesh = nat.Mesh(N, F, P, a["cfi"].shape[1] if N else 0, a["nc"].shape[1] if P else 0,
                    nat.iptr(a["cfi"]), nat.iptr(a["cfs"]), nat.iptr(a["fc"]), nat.fptr(a["fd"]),
                    nat.iptr(a["fn_"]), nat.fptr(a["fnrm"]), nat.fptr(a["fL"]), nat.fptr(a["scale"]),
                    nat.iptr(a["nt"]), nat.iptr(a["nc"]), nat.fptr(a["nd"]), nat.fptr(a["xy"]),
                    nat.fptr(a["ia"]), nat.fptr(a["area"]))
    params = nat.Params(nat.FVDBM_UPWIND if f.flux_scheme == "upwind" else nat.FVDBM_LAX_WENDROFF,
                        variant, float(dyn.inv_tau), float(dyn.dt32), float(dyn.c2),
                        float(dyn.c4x2), float(dyn.c2x2), _ORDER[order], _KERNEL[kernel],
                        int(device), int(dyn.NUM_QUIVERS), float(dyn.c6x2))
    return mesh, params, a, (N, F, P), dyn


class Environment:
    """GB300 FVDBM environment (reference ``Environment``)."""

    dynamics = None  # class attribute used by ``create``, as in the reference

    def __init__(self, cells, faces, nodes, *, ordering: str = "auto", kernel: str = "auto",
                 device: int = 0, finite_volume: bool = False):
        # private copies: like the reference's jitted step, stepping never
        # modifies the containers the caller passed in
        cells, faces, nodes = from_any(cells, faces, nodes)
        self.cells, self.faces, self.nodes = cells, faces, nodes
        self.ordering, self.kernel, self.device = ordering, kernel, device
        self.finite_volume = finite_volume
        self._h = None
        self._steps = 0
        self._version = 0
        self._fresh = {}

    # reference factory methods (src/environment.py:20-36)
    @classmethod
    def create(cls, num_cells, num_faces, num_nodes):
        if cls.dynamics is None:
            raise ValueError("Environment.create needs the class attribute Environment.dynamics")
        return cls(Cells(num_cells, cls.dynamics), Faces(num_faces, cls.dynamics),
                   Nodes(num_nodes, cls.dynamics))

    @classmethod
    def define(cls, cells, faces, nodes):
        return cls(cells, faces, nodes)

    # ------------------------------------------------------------------
    def init(self):
        """Validate, renumber and upload (``src/environment.py:38-42``)."""
        c, f, n = self.cells, self.faces, self.nodes
        for cont in (c, f, n):
            cont.init()
        mesh, params, keep, (N, F, P), dyn = pack(c, f, n, ordering=self.ordering, kernel=self.kernel,
                                                  device=self.device, finite_volume=self.finite_volume)
        L = nat.lib()
        self.close()
        h = C.c_void_p()
        rc = L.fvdbm_create(C.byref(mesh), C.byref(params), C.byref(h))
        if rc != 0:
            msg = L.fvdbm_last_error(None)
            msg = msg.decode() if msg else ""
            if rc == -1:
                raise ValueError(msg)
            raise nat.FvdbmError(f"fvdbm_create failed ({rc}): {msg}")
        self._h = h
        self._dyn = dyn
        self._Q = int(dyn.NUM_QUIVERS)
        self._N, self._F, self._P = N, F, P
        self._upload_all()
        for cont in (c, f, n):
            object.__setattr__(cont, "_owner", self)
        self._version += 1
        return None

    def _upload_all(self):
        c, n = self.cells, self.nodes
        pdf = np.ascontiguousarray(object.__getattribute__(c, "pdf"), F32)
        npdf = np.ascontiguousarray(object.__getattribute__(n, "pdf"), F32)
        nrho = np.ascontiguousarray(np.asarray(object.__getattribute__(n, "rho"), F32).reshape(-1))
        nvel = np.ascontiguousarray(object.__getattribute__(n, "vel"), F32)
        nat.check(nat.lib().fvdbm_set_state(self._h, nat.fptr(pdf), nat.fptr(npdf), nat.fptr(nrho),
                                            nat.fptr(nvel)), self._h)

    # ------------------------------------------------------------------
    def step(self, n_steps: int = 1):
        """``n_steps`` FVDBM steps (``src/environment.py:55-65``); returns self.

        Unlike the reference's jitted ``step``, which returns a new pytree and
        leaves the old ``env`` as it was, this advances ``self`` in place (the
        state lives on the device) and returns it: ``env = env.step()`` reads
        the same, but after ``env2 = env.step()`` both names refer to the
        stepped environment.  Keep an earlier state with ``to_pickle`` or by
        copying ``env.cells.pdf`` / ``env.nodes.*`` before stepping."""
        if self._h is None:
            self.init()
        nat.check(nat.lib().fvdbm_step(self._h, int(n_steps)), self._h)
        if n_steps:
            self._steps += int(n_steps)
            self._version += 1
        return self

    def residual(self):
        """(res_u, mass) of the current state in double: the velocity change
        since the previous call per unit time, relative to the previous
        velocity norm, and sum(rho * area) (``fvdbm_residual``)."""
        if self._h is None:
            self.init()
        r, m = C.c_double(), C.c_double()
        nat.check(nat.lib().fvdbm_residual(self._h, C.byref(r), C.byref(m)), self._h)
        return r.value, m.value

    def run_to_steady(self, threshold: float = 1e-6, check_every: int = 100, max_steps: int = 1_000_000):
        """Step until the residual falls below ``threshold`` (checked every
        ``check_every`` steps) or ``max_steps``; returns (steps, res_u).
        res_u == 0 means the float32 state froze (no cell's velocity changed
        over the last check).  A NaN residual (the run diverged) raises
        ``NonFiniteError`` after the steps taken are recorded."""
        if self._h is None:
            self.init()
        n, r = C.c_int64(), C.c_double()
        rc = nat.lib().fvdbm_run_to_steady(self._h, float(threshold), int(check_every), int(max_steps),
                                           C.byref(n), C.byref(r))
        if n.value:
            self._steps += n.value
            self._version += 1
        nat.check(rc, self._h)
        return n.value, r.value

    def sync(self):
        if self._h is not None:
            nat.check(nat.lib().fvdbm_sync(self._h), self._h)
        return self

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        inf = nat.Info()
        nat.check(nat.lib().fvdbm_get_info(self._h, C.byref(inf)), self._h)
        return {k: getattr(inf, k) for k, _ in nat.Info._fields_}

    @property
    def stream_ptr(self) -> int:
        return int(nat.lib().fvdbm_stream(self._h) or 0)

    def close(self):
        if getattr(self, "_h", None) is not None:
            nat.lib().fvdbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------
    # checkpoints: pickling keeps the containers with the current state (as
    # the reference pickles its pytree, src/mesher.py:600-608); the device
    # handle is not kept, and the next step re-initialises from that state,
    # continuing the run exactly
    def __getstate__(self):
        import copy
        if self._h is not None:
            for cont, names in ((self.cells, ("pdf", "rho", "vel", "pdf_eq")), (self.faces, ("pdf",)),
                                (self.nodes, ("pdf",))):
                for nm in names:
                    getattr(cont, nm)  # read the leaves back from the device
        st = {k: v for k, v in self.__dict__.items() if k not in ("_h", "_fresh")}
        for k in ("cells", "faces", "nodes"):
            c = copy.copy(self.__dict__[k])
            object.__setattr__(c, "_owner", None)
            st[k] = c
        st["_h"], st["_fresh"] = None, {}
        return st

    def __setstate__(self, st):
        self.__dict__.update(st)

    # ------------------------------------------------------------------
    # read-through of the dynamic leaves
    def _pull(self, cont: _Container, name: str):
        key = (id(cont), name)
        if self._fresh.get(key) == self._version:
            return
        self._fresh[key] = self._version
        L = nat.lib()
        if cont is self.cells:
            N = self._N
            if name == "pdf":
                out = np.empty((N, self._Q), F32)
                nat.check(L.fvdbm_get_cells(self._h, nat.fptr(out), None, None, None), self._h)
            elif self._steps == 0:
                return
            elif name == "rho":
                out = np.empty((N, 1), F32)
                nat.check(L.fvdbm_get_cells(self._h, None, nat.fptr(out), None, None), self._h)
            elif name == "vel":
                out = np.empty((N, 2), F32)
                nat.check(L.fvdbm_get_cells(self._h, None, None, nat.fptr(out), None), self._h)
            else:
                out = np.empty((N, self._Q), F32)
                nat.check(L.fvdbm_get_cells(self._h, None, None, None, nat.fptr(out)), self._h)
        elif cont is self.faces:
            if self._steps == 0:
                return
            out = np.empty((self._F, self._Q), F32)
            nat.check(L.fvdbm_get_face_fluxes(self._h, nat.fptr(out)), self._h)
        else:
            P = self._P
            pdf, rho, vel = np.empty((P, self._Q), F32), np.empty((P, 1), F32), np.empty((P, 2), F32)
            nat.check(L.fvdbm_get_nodes(self._h, nat.fptr(pdf), nat.fptr(rho), nat.fptr(vel)), self._h)
            for k, v in (("pdf", pdf), ("rho", rho), ("vel", vel)):
                object.__setattr__(cont, k, v)
                self._fresh[(id(cont), k)] = self._version
            return
        object.__setattr__(cont, name, out)

    def _push(self, cont: _Container, name: str):
        if self._h is None:
            return
        L = nat.lib()
        if cont is self.cells and name == "pdf":
            pdf = np.ascontiguousarray(object.__getattribute__(cont, "pdf"), F32)
            if pdf.shape != (self._N, self._Q):
                raise ValueError(f"cells.pdf must be [{self._N},{self._Q}]")
            nat.check(L.fvdbm_set_state(self._h, nat.fptr(pdf), None, None, None), self._h)
            self._version += 1
            self._fresh[(id(cont), "pdf")] = self._version
        elif cont is self.nodes:
            new = np.ascontiguousarray(object.__getattribute__(cont, name), F32)
            self._version += 1
            self._pull(cont, "pdf")   # refresh all three from the device
            object.__setattr__(cont, name, new)
            n = cont
            pdf = np.ascontiguousarray(object.__getattribute__(n, "pdf"), F32)
            rho = np.ascontiguousarray(np.asarray(object.__getattribute__(n, "rho"), F32).reshape(-1))
            vel = np.ascontiguousarray(object.__getattribute__(n, "vel"), F32)
            nat.check(L.fvdbm_set_state(self._h, None, nat.fptr(pdf), nat.fptr(rho), nat.fptr(vel)),
                      self._h)
            self._version += 1
            for k in ("pdf", "rho", "vel"):
                self._fresh[(id(n), k)] = self._version
        else:
            # outputs of the last step (cells.rho/vel/pdf_eq, faces.pdf): the
            # next step overwrites them; keep the host value until then
            self._fresh[(id(cont), name)] = self._version

    def __repr__(self):
        return f"Environment(cells={self.cells}, faces={self.faces}, nodes={self.nodes})"
