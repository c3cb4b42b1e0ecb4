"""Domain decomposition of one mesh over several ranks: which cells each rank
owns, which cells it must receive every step (its halo) and which owned cells
it sends to each peer.

A step reads, for each owned cell, its own pdf, the pdfs of the cells across
its faces (src/containers.py:191-278) and, for ghost faces, the boundary nodes
at the face's ends, whose values come from the pdfs of the nodes' stencil
cells (src/containers.py:339-404).  So the halo of a rank is those neighbour
and node-stencil cells that it does not own, plus the last cell and the last
face's cells where the reference's padded -1 indices wrap to them.  With the
halo received before the step, a rank updates its own cells with exactly the
arithmetic of the single-domain step: the partitioned result is bitwise the
single-domain one.  One exchange of 36 bytes per halo cell per step; no other
communication.
"""
from __future__ import annotations

import numpy as np


def partition_cells(cells, faces, n_parts: int) -> np.ndarray:
    """Owner rank of each cell: contiguous ranges, of near-equal size, of a
    locality order (Morton order of the centroids when the cells carry them,
    else the cell index order)."""
    n = int(np.asarray(cells.face_indices).shape[0])
    xy = getattr(cells, "centroids", None)
    if xy is not None:
        xy = np.asarray(xy, np.float64)
        lo, span = xy.min(0), max(float(np.ptp(xy[:, 0])), float(np.ptp(xy[:, 1])), 1e-30)
        q = np.clip(((xy - lo) / span * 65535.0).astype(np.int64), 0, 65535)

        def spread(v):
            v = v & 0xFFFF
            v = (v | (v << 8)) & 0x00FF00FF
            v = (v | (v << 4)) & 0x0F0F0F0F
            v = (v | (v << 2)) & 0x33333333
            return (v | (v << 1)) & 0x55555555
        order = np.argsort(spread(q[:, 0]) | (spread(q[:, 1]) << 1), kind="stable")
    else:
        order = np.arange(n)
    owner = np.empty(n, np.int32)
    bounds = np.linspace(0, n, n_parts + 1).round().astype(np.int64)
    for r in range(n_parts):
        owner[order[bounds[r]:bounds[r + 1]]] = r
    return owner


def needed_cells(cells, faces, nodes, owner: np.ndarray, rank: int) -> np.ndarray:
    """Cells whose pdfs rank `rank` reads in one step (owned ones included)."""
    fi = np.asarray(cells.face_indices, np.int64)
    fc = np.asarray(faces.stencil_cells_index, np.int64)
    fn = np.asarray(faces.nodes_index, np.int64)
    nc = np.asarray(nodes.cells_index, np.int64)
    nt = np.asarray(nodes.type).reshape(-1)
    N, F, P = fi.shape[0], fc.shape[0], nt.shape[0]
    own = np.flatnonzero(owner == rank)
    f_used = np.unique(np.where(fi[own] < 0, F - 1, fi[own]))  # -1 slots read the last face
    need = set(own.tolist())
    for c in fc[f_used].reshape(-1):
        if c >= 0:
            need.add(int(c))
    ghost = f_used[(fc[f_used, 0] < 0) | (fc[f_used, 1] < 0)]
    nd = np.unique(np.where(fn[ghost] < 0, P - 1, fn[ghost]).reshape(-1))
    nd = nd[nt[nd] != 0]  # frozen nodes read no cells
    for c in nc[nd].reshape(-1):
        need.add(int(c) if c >= 0 else N - 1)  # padded entries gather the last cell
    return np.array(sorted(need), np.int64)


class HaloPlan:
    """Per-rank exchange lists.  recv[q]: cells this rank receives from rank
    q; send[q]: owned cells it sends to rank q (in the order q expects)."""

    def __init__(self, cells, faces, nodes, owner: np.ndarray, rank: int):
        self.rank, self.n_parts = rank, int(owner.max()) + 1
        self.owned = np.flatnonzero(owner == rank)
        self.needed = needed_cells(cells, faces, nodes, owner, rank)
        halo = self.needed[owner[self.needed] != rank]
        self.recv = {q: halo[owner[halo] == q] for q in range(self.n_parts) if q != rank}
        self.send = {}
        for q in range(self.n_parts):
            if q == rank:
                continue
            other = needed_cells(cells, faces, nodes, owner, q)
            self.send[q] = other[owner[other] == rank]

    @property
    def halo_cells(self) -> int:
        return int(sum(v.size for v in self.recv.values()))


class SubDomain:
    """One rank's part of a partitioned mesh, as containers a handle can step
    on its own: its owned cells and its halo (the cells it reads and does not
    own), with every static array renumbered to local indices.

    Local cells are the owned cells, then the halo, in global order, except
    that the global last cell (which the reference's padded node entries
    gather) is moved to the end; likewise the global last face and last node.
    A halo cell's face to a cell outside the sub-domain becomes a ghost face,
    and a boundary node whose stencil is not all local becomes a frozen
    (type 0) node: both only feed halo cells, whose pdfs the exchange
    overwrites after every step, so owned cells are stepped with exactly the
    single-domain arithmetic.

    ``cells/faces/nodes`` are the containers; ``cell_g``/``face_g``/``node_g``
    map local to global indices; ``owned`` are local indices of the owned
    cells; ``recv[q]`` are local indices of the halo cells owned by rank q,
    in the order rank q sends them (``send_local[q]`` on rank q, in ascending
    global order); ``send_local[q]`` are local indices of the owned cells that
    rank q reads."""

    def __init__(self, cells, faces, nodes, owner: np.ndarray, rank: int):
        from .containers import Cells, Faces, Nodes, from_any
        c, f, n = from_any(cells, faces, nodes)
        dyn = c.dynamics
        plan = HaloPlan(c, f, n, owner, rank)
        fi = np.asarray(c.face_indices, np.int64)
        fc = np.asarray(f.stencil_cells_index, np.int64)
        fn = np.asarray(f.nodes_index, np.int64)
        nc = np.asarray(n.cells_index, np.int64)
        nt = np.asarray(n.type).reshape(-1)
        N, F, P = fi.shape[0], fc.shape[0], nt.shape[0]

        def order_last(ids, last):
            ids = np.asarray(ids, np.int64)
            if last in set(ids.tolist()):
                ids = np.concatenate([ids[ids != last], [last]])
            return ids

        halo = plan.needed[owner[plan.needed] != rank]
        cell_g = order_last(np.concatenate([plan.owned, halo]), N - 1)
        lc = -np.ones(N, np.int64)
        lc[cell_g] = np.arange(cell_g.size)
        # faces: every face of a local cell (padded slots read the last face)
        fl = fi[cell_g]
        face_g = np.unique(fl[fl >= 0])
        if (fl < 0).any():
            face_g = np.union1d(face_g, [F - 1])
        face_g = order_last(face_g, F - 1)
        lf = -np.ones(F, np.int64)
        lf[face_g] = np.arange(face_g.size)
        # nodes: every node of a local face (padded node slots read the last node)
        nl = fn[face_g]
        node_g = np.unique(nl[nl >= 0])
        if (nl < 0).any():
            node_g = np.union1d(node_g, [P - 1])
        node_g = order_last(node_g, P - 1)
        ln = -np.ones(P, np.int64)
        ln[node_g] = np.arange(node_g.size)

        Nl, Fl, Pl = cell_g.size, face_g.size, node_g.size
        cl = Cells(Nl, dyn)
        cl.pdf = np.asarray(c.pdf)[cell_g]
        cl.rho = np.asarray(c.rho)[cell_g]
        cl.vel = np.asarray(c.vel)[cell_g]
        cl.pdf_eq = np.asarray(c.pdf_eq)[cell_g]
        cl.face_indices = np.where(fl >= 0, lf[np.maximum(fl, 0)], -1).astype(np.int32)
        cl.face_normals = np.asarray(c.face_normals)[cell_g].astype(np.int32)
        for extra in ("centroids", "areas"):
            if getattr(c, extra, None) is not None:
                setattr(cl, extra, np.asarray(getattr(c, extra))[cell_g])
        flc = Faces(Fl, dyn, f.flux_scheme)
        flc.pdf = np.asarray(f.pdf)[face_g]
        sc = fc[face_g]
        flc.stencil_cells_index = np.where(sc >= 0, lc[np.maximum(sc, 0)], -1).astype(np.int32)
        flc.nodes_index = np.where(fn[face_g] >= 0, ln[np.maximum(fn[face_g], 0)], -1).astype(np.int32)
        flc.stencil_dists = np.asarray(f.stencil_dists)[face_g]
        flc.n = np.asarray(f.n)[face_g]
        flc.L = np.asarray(f.L)[face_g]
        flc.stencil_variant = f.stencil_variant
        if f.alpha is not None:
            flc.alpha = np.asarray(f.alpha)[face_g]
        if f.npq is not None:
            flc.npq = np.asarray(f.npq)[face_g]
        nlc = Nodes(Pl, dyn)
        nlc.pdf = np.asarray(n.pdf)[node_g]
        nlc.rho = np.asarray(n.rho)[node_g]
        nlc.vel = np.asarray(n.vel)[node_g]
        st = nc[node_g]
        local_st = np.where(st >= 0, lc[np.maximum(st, 0)], -1)
        complete = np.all((st < 0) | (local_st >= 0), axis=1)
        nlc.type = np.where(complete, nt[node_g], 0).reshape(Pl, 1).astype(np.int32)
        nlc.cells_index = np.where(st >= 0, local_st, -1).astype(np.int32)
        nlc.cell_dists = np.asarray(n.cell_dists)[node_g]
        self.cells, self.faces, self.nodes = cl, flc, nlc
        self.cell_g, self.face_g, self.node_g = cell_g, face_g, node_g
        self.owned = lc[plan.owned]
        self.recv = {q: lc[np.sort(g)] for q, g in plan.recv.items()}
        self.send_local = {q: lc[np.sort(g)] for q, g in plan.send.items()}
        self.plan = plan
