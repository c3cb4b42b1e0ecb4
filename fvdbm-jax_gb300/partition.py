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
