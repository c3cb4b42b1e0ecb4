"""Vectorised mesh preprocessing: the geometry and connectivity that the
reference's ``Mesher`` computes with per-element Python loops
(``src/mesher.py:20-742``), restated with whole-array numpy so that a
1M-triangle case is prepared in seconds.

Every quantity follows the reference's definition and float64 arithmetic,
then ``to_env`` casts to float32 / int32 exactly as the reference does (x64
is never enabled there, so its ``jnp.float64`` requests yield float32):

* CCW enforcement by signed area (``:63-78``);
* boundary faces flipped so their left normal points out (``:80-110``);
* centroids (``:113-120``), face centres/normals/lengths (``:172-195``);
* per-cell faces in the order (c0,c1),(c1,c2),(c2,c0) with outward normals
  and signs against the face normal (``:122-169``);
* stencil norms (``:506-541``) and face-stencil angles (``:543-558``);
* face->cell slots: the first cell listing the face, re-ordered so that slot 0
  has the smaller normal-projected offset, distances made absolute
  (``:197-266``), ghost distances mirrored (``:268-283``);
* point->cell lists in cell order with Euclidean distances, padded with -1
  (``:286-316``).

Integer outputs match the reference exactly.  Float outputs can differ from
it in the last float64 bit where the reference's ``np.dot``/``np.linalg.norm``
use fused multiply-adds; after the float32 cast that is at most one ulp.
"""
from __future__ import annotations

import io
import time
from types import SimpleNamespace

import numpy as np

from .containers import Cells, Faces, Nodes
from .dynamics import D2Q9

F32, I32 = np.float32, np.int32

FLUX_METHODS = ("upwind", "lax_wendroff", "cc_upwind", "cc_lax_wendroff", "cc_alt_upwind")


def _unit_left_normal(p0: np.ndarray, p1: np.ndarray) -> np.ndarray:
    """Left unit normal of p0->p1 (reference ``utils/utils.py:162-173``)."""
    t = p1 - p0
    nrm = np.stack([-t[..., 1], t[..., 0]], axis=-1)
    return nrm / np.sqrt(nrm[..., 0] * nrm[..., 0] + nrm[..., 1] * nrm[..., 1])[..., None]


def _dot2(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]


def _norm2(a: np.ndarray) -> np.ndarray:
    return np.sqrt(a[..., 0] * a[..., 0] + a[..., 1] * a[..., 1])


class Mesher:
    """Mesh geometry and the ``to_env`` data contract (reference ``Mesher``)."""

    def __init__(self):
        self.points = None
        self.cells = None
        self.faces = None
        self.point_markers = None
        self.timings = {}

    # --- import -----------------------------------------------------------
    def import_meshpy(self, mesh):
        """Take ``points``, ``elements``, ``faces`` and ``point_markers`` from
        a meshpy-like object (``src/mesher.py:48-61``)."""
        self.points = np.array(mesh.points, dtype=np.float64)
        self.cells = np.array(mesh.elements, dtype=np.int32)
        self.faces = np.array(mesh.faces, dtype=np.int32)
        self.point_markers = np.array(mesh.point_markers, dtype=np.int32)
        self.enforce_ccw()
        return self

    @classmethod
    def from_raw(cls, raw):
        return cls().import_meshpy(raw)

    def enforce_ccw(self):
        """Swap vertices 1 and 2 of clockwise triangles (``src/mesher.py:63-78``)."""
        p = self.points[self.cells]
        area = 0.5 * ((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1])
                      - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
        neg = area < 0
        c = self.cells.copy()
        c[neg] = c[neg][:, [0, 2, 1]]
        self.cells = c

    # --- connectivity helpers ---------------------------------------------
    def _face_cells(self):
        """For each face, the cells listing it in cell order (at most 2)."""
        P = np.int64(self.points.shape[0])
        c = self.cells.astype(np.int64)
        a = c.ravel()
        b = np.roll(c, -1, axis=1).ravel()
        hkey = np.minimum(a, b) * P + np.maximum(a, b)
        hcell = np.repeat(np.arange(c.shape[0], dtype=np.int64), 3)
        order = np.argsort(hkey, kind="stable")
        hk, hc = hkey[order], hcell[order]
        f = self.faces.astype(np.int64)
        fkey = np.minimum(f[:, 0], f[:, 1]) * P + np.maximum(f[:, 0], f[:, 1])
        lo = np.searchsorted(hk, fkey, side="left")
        hi = np.searchsorted(hk, fkey, side="right")
        cnt = hi - lo
        if np.any(cnt > 2):
            raise ValueError("a face is shared by more than two cells")
        fc = -np.ones((f.shape[0], 2), dtype=np.int64)
        has0 = cnt > 0
        fc[has0, 0] = hc[lo[has0]]
        has1 = cnt > 1
        fc[has1, 1] = hc[lo[has1] + 1]
        return fc, cnt

    # --- geometry ---------------------------------------------------------
    def calc_mesh_properties(self, verbose: bool = False):
        """All geometry and connectivity (``src/mesher.py:319-383``)."""
        t0 = time.perf_counter()
        pts = self.points
        c = self.cells
        P = np.int64(pts.shape[0])
        p0, p1, p2 = pts[c[:, 0]], pts[c[:, 1]], pts[c[:, 2]]
        self.cell_centers = ((p0 + p1) + p2) / 3.0
        self.cell_areas = 0.5 * np.abs((p1[:, 0] - p0[:, 0]) * (p2[:, 1] - p0[:, 1])
                                       - (p2[:, 0] - p0[:, 0]) * (p1[:, 1] - p0[:, 1]))

        # boundary faces: left normal must point away from the owning cell
        fc, cnt = self._face_cells()
        faces = self.faces.copy()
        bnd = np.nonzero(cnt == 1)[0]
        q0, q1 = pts[faces[bnd, 0]], pts[faces[bnd, 1]]
        nrm = _unit_left_normal(q0, q1)
        to_c = self.cell_centers[fc[bnd, 0]] - (q0 + q1) / 2.0
        flip = ~(_dot2(nrm, to_c) < 0)
        faces[bnd[flip]] = faces[bnd[flip]][:, ::-1]
        self.faces = faces

        fp0, fp1 = pts[faces[:, 0]], pts[faces[:, 1]]
        self.face_centers = (fp0 + fp1) / 2.0
        self.face_normals = _unit_left_normal(fp0, fp1)
        self.face_lengths = _norm2(fp1 - fp0)

        # per-cell faces (c0,c1),(c1,c2),(c2,c0) and outward normals
        f64 = faces.astype(np.int64)
        fkey = np.minimum(f64[:, 0], f64[:, 1]) * P + np.maximum(f64[:, 0], f64[:, 1])
        forder = np.argsort(fkey, kind="stable")
        fks = fkey[forder]
        ca = c.astype(np.int64)
        cb = np.roll(ca, -1, axis=1)
        ckey = np.minimum(ca, cb) * P + np.maximum(ca, cb)
        pos = np.searchsorted(fks, ckey, side="right") - 1
        if np.any(pos < 0) or np.any(fks[np.clip(pos, 0, None)] != ckey):
            raise ValueError("a cell edge is missing from the face list")
        self.cell_face_indices = forder[pos].astype(np.int64)
        e0, e1 = pts[ca], pts[cb]
        enrm = _unit_left_normal(e0, e1)
        to_c = self.cell_centers[:, None, :] - (e0 + e1) / 2.0
        out = _dot2(enrm, to_c) < 0
        self.cell_face_normals = np.where(out[..., None], enrm, -enrm)
        dots = _dot2(self.cell_face_normals, self.face_normals[self.cell_face_indices])
        self.cell_face_normal_signs = np.sign(dots).astype(np.int32)

        # stencil norms (cell0->cell1 for interior, cell->face centre for boundary)
        v = np.zeros_like(self.face_normals)
        two = cnt == 2
        one = cnt == 1
        v[two] = self.cell_centers[fc[two, 1]] - self.cell_centers[fc[two, 0]]
        v[one] = self.face_centers[one] - self.cell_centers[fc[one, 0]]
        vn = _norm2(v)
        sn = np.where((vn > 0)[:, None], v / np.where(vn > 0, vn, 1.0)[:, None], v)
        fnu = self.face_normals / np.linalg.norm(self.face_normals, axis=1, keepdims=True)
        snu = sn / (np.linalg.norm(sn, axis=1, keepdims=True) + 1e-14)
        sflip = np.einsum("ij,ij->i", fnu, snu) < 0
        sn[sflip] *= -1
        self.stencil_norms = sn

        # face->cell slots and normal-projected distances
        mid = self.face_centers
        fci = fc.copy()
        d = -np.ones((faces.shape[0], 2))
        dcc = -np.ones((faces.shape[0], 2))
        b0 = (fc[:, 0] != -1) & (fc[:, 1] == -1)
        b1 = (fc[:, 0] == -1) & (fc[:, 1] != -1)
        for sel, slot in ((b0, 0), (b1, 1)):
            cc = self.cell_centers[fc[sel, slot]] - mid[sel]
            d[sel, slot] = _dot2(self.face_normals[sel], cc)
            dcc[sel, slot] = _dot2(sn[sel], cc)
        it = (fc[:, 0] != -1) & (fc[:, 1] != -1)
        v0 = self.cell_centers[fc[it, 0]] - mid[it]
        v1 = self.cell_centers[fc[it, 1]] - mid[it]
        n_it, s_it = self.face_normals[it], sn[it]
        d0, d1 = _dot2(n_it, v0), _dot2(n_it, v1)
        c0, c1 = _dot2(s_it, v0), _dot2(s_it, v1)
        keep = d0 < d1
        fci[it, 0] = np.where(keep, fc[it, 0], fc[it, 1])
        fci[it, 1] = np.where(keep, fc[it, 1], fc[it, 0])
        d[it, 0], d[it, 1] = np.where(keep, d0, d1), np.where(keep, d1, d0)
        dcc[it, 0], dcc[it, 1] = np.where(keep, c0, c1), np.where(keep, c1, c0)
        self.face_cell_indices = fci
        d, dcc = np.abs(d), np.abs(dcc)
        # mirror the ghost side
        m0, m1 = fci[:, 0] == -1, fci[:, 1] == -1
        d[m0, 0], d[m1, 1] = d[m0, 1], d[m1, 0]
        dcc[m0, 0], dcc[m1, 1] = dcc[m0, 1], dcc[m1, 0]
        self.face_cell_center_distances = d
        self.cc_stencil_dist = dcc

        # point -> cells (cell order), Euclidean distances, padded with -1
        pc_p = ca.ravel()
        pc_c = np.repeat(np.arange(c.shape[0], dtype=np.int64), 3)
        order = np.argsort(pc_p, kind="stable")
        pp, pcc = pc_p[order], pc_c[order]
        counts = np.bincount(pp, minlength=int(P))
        K = int(counts.max()) if counts.size else 1
        start = np.concatenate([[0], np.cumsum(counts)[:-1]])
        slot = np.arange(pp.shape[0]) - start[pp]
        pci = -np.ones((int(P), K), dtype=np.int64)
        pci[pp, slot] = pcc
        pcd = -np.ones((int(P), K))
        pcd[pp, slot] = _norm2(pts[pp] - self.cell_centers[pcc])
        self.point_cell_indices = pci
        self.point_cell_center_distances = pcd

        dots = np.clip(np.einsum("ij,ij->i", fnu, sn / np.linalg.norm(sn, axis=1, keepdims=True)), -1.0, 1.0)
        self.face_stencil_angles = np.arccos(dots)
        self.timings["calc_mesh_properties_s"] = time.perf_counter() - t0
        if verbose:
            print(f"mesh properties: {c.shape[0]} cells, {faces.shape[0]} faces "
                  f"in {self.timings['calc_mesh_properties_s']:.3f}s")
        return self

    # --- contract ---------------------------------------------------------
    def to_env(self, dynamics, flux_method: str = "upwind", dim_multiplier=1):
        """Build ``Cells``, ``Faces``, ``Nodes`` (``src/mesher.py:610-693``)."""
        if flux_method not in FLUX_METHODS:
            raise ValueError(f"Unsupported flux method: {flux_method}")
        N, F, P = self.cells.shape[0], self.faces.shape[0], self.points.shape[0]
        cells = Cells(N, dynamics)
        cells.face_indices = self.cell_face_indices.astype(I32)
        cells.face_normals = self.cell_face_normal_signs.astype(I32)
        # not part of the reference containers: centroids (for the locality
        # order of the device numbering) and areas (finite-volume mode, mass)
        cells.centroids = self.cell_centers.astype(F32)
        cells.areas = self.cell_areas.astype(F32)

        scheme = "lax_wendroff" if flux_method in ("lax_wendroff", "cc_lax_wendroff") else "upwind"
        faces = Faces(F, dynamics, flux_scheme=scheme)
        faces.L = self.face_lengths.astype(F32)[..., None] * dim_multiplier
        faces.nodes_index = self.faces.astype(I32)
        faces.stencil_cells_index = self.face_cell_indices.astype(I32)
        if flux_method in ("cc_upwind", "cc_lax_wendroff"):
            faces.stencil_variant = "cos"
            faces.n = self.stencil_norms.astype(F32)
            faces.alpha = self.face_stencil_angles.astype(F32)[..., None]
            faces.stencil_dists = self.cc_stencil_dist.astype(F32) * dim_multiplier
        else:
            faces.n = self.face_normals.astype(F32)
            faces.stencil_dists = self.face_cell_center_distances.astype(F32) * dim_multiplier
            if flux_method == "cc_alt_upwind":
                faces.stencil_variant = "ksi"
                faces.npq = self.stencil_norms.astype(F32)
        faces.L = faces.L.astype(F32)
        faces.stencil_dists = faces.stencil_dists.astype(F32)

        nodes = Nodes(P, dynamics)
        nodes.cells_index = self.point_cell_indices.astype(I32)
        cd = self.point_cell_center_distances.astype(F32)
        pos = cd > 0
        cd[pos] = (cd[pos] * dim_multiplier).astype(F32)
        nodes.cell_dists = cd
        nodes.type = np.zeros((P, 1), I32)
        return cells, faces, nodes

    def set_vel_node(self, nodes, marker: int, velocity):
        """Velocity nodes by point marker (``src/mesher.py:697-719``)."""
        velocity = np.asarray(velocity)
        assert velocity.shape == (nodes.dynamics.DIM,)
        sel = self.point_markers == marker
        t = np.array(nodes.type)
        t[sel] = 1
        nodes.type = t
        v = np.array(nodes.vel)
        v[sel] = velocity
        nodes.vel = v
        return nodes

    def set_rho_node(self, nodes, marker: int, rho: float):
        """Density nodes by point marker (``src/mesher.py:721-742``)."""
        assert rho > 0
        sel = self.point_markers == marker
        t = np.array(nodes.type)
        t[sel] = 2
        nodes.type = t
        r = np.array(nodes.rho)
        r[sel] = rho
        nodes.rho = r
        return nodes

    # --- output -----------------------------------------------------------
    def to_pickle(self, env, filename: str):
        """Checkpoint (src/mesher.py:600-603): ``filename.pkl`` holds the
        environment, with its current state, and this mesher."""
        import pickle
        with open(f"{filename}.pkl", "wb") as fh:
            pickle.dump((env, self), fh)

    @classmethod
    def from_pickle(cls, filename: str):
        """(env, mesher) from ``to_pickle`` (src/mesher.py:605-608); the
        environment continues from the saved state at its next step."""
        import pickle
        with open(f"{filename}.pkl", "rb") as fh:
            return pickle.load(fh)

    def to_vtk(self, env, filename: str, save_f: bool = False, save_feq: bool = False) -> str:
        """Legacy-ASCII VTK unstructured grid with cell ``Velocity`` (3-vector,
        z=0) and ``Density``, optionally ``pdf`` and ``feq`` (the fields the
        reference writes through pyvista, ``src/mesher.py:562-598``).  Returns
        the path written."""
        pts = np.hstack([self.points, np.zeros_like(self.points[:, :1])])
        N = self.cells.shape[0]
        vel = np.asarray(env.cells.vel, dtype=np.float64)
        rho = np.asarray(env.cells.rho, dtype=np.float64).reshape(N)
        buf = io.StringIO()
        buf.write("# vtk DataFile Version 3.0\nfvdbm\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        buf.write(f"POINTS {pts.shape[0]} double\n")
        np.savetxt(buf, pts, fmt="%.17g")
        buf.write(f"CELLS {N} {4 * N}\n")
        np.savetxt(buf, np.hstack([np.full((N, 1), 3), self.cells]), fmt="%d")
        buf.write(f"CELL_TYPES {N}\n")
        np.savetxt(buf, np.full((N, 1), 5), fmt="%d")
        buf.write(f"CELL_DATA {N}\nVECTORS Velocity double\n")
        np.savetxt(buf, np.hstack([vel, np.zeros((N, 1))]), fmt="%.9g")
        buf.write("SCALARS Density double 1\nLOOKUP_TABLE default\n")
        np.savetxt(buf, rho[:, None], fmt="%.9g")
        # pdf and feq are cell arrays of 9 (13) components: one FIELD block
        # holding each requested array, as VTK's legacy writer emits them
        extra = [(name, np.asarray(getattr(env.cells, arr), dtype=np.float64).reshape(N, -1))
                 for flag, name, arr in ((save_f, "pdf", "pdf"), (save_feq, "feq", "pdf_eq")) if flag]
        if extra:
            buf.write(f"FIELD FieldData {len(extra)}\n")
            for name, a in extra:
                buf.write(f"{name} {a.shape[1]} {N} double\n")
                np.savetxt(buf, a, fmt="%.9g")
        path = f"{filename}.vtk"
        with open(path, "w") as fh:
            fh.write(buf.getvalue())
        return path


def build_case(raw, dynamics: D2Q9, flux_method: str = "upwind", dim_multiplier=1):
    """Raw mesh -> (mesher, cells, faces, nodes) with no boundary types set."""
    m = Mesher().import_meshpy(SimpleNamespace(points=raw.points, elements=raw.elements,
                                               faces=raw.faces, point_markers=raw.point_markers))
    m.calc_mesh_properties()
    cells, faces, nodes = m.to_env(dynamics, flux_method, dim_multiplier)
    return m, cells, faces, nodes
