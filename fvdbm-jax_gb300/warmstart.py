"""Learned warm start: a message-passing network over the cells of a mesh
predicts the steady rho and u of a case from its geometry; the solver starts
from f = feq(rho, u) instead of the uniform state and still runs to its
residual threshold, which judges the result.  A case whose residual stalls is
restarted from the uniform state.

The reference has no counterpart (it always starts from feq(1, 0),
src/containers.py:24-30).  The network is trained on steady states that the
solver itself produces (``Batch.run_to_steady``), by the library's own CUDA
kernels (include/fvdbm_mpnn.h): bfloat16 weights, float32 activations and
accumulation, Adam on float32 master weights.  PyTorch only provides the
device memory and the stream.

Network (hidden 64, 4 message-passing layers):
    h0 = relu(x W0^T + b0)
    m_l = A_l h_{l-1};  h_l = h_{l-1} + relu([h_{l-1} | m_l] W_l^T + b_l)
    y = h_4 W_out^T + b_out
Layer l's messages come from one of two kinds of neighbourhood (``SCALES``):
"mesh", the mean over a cell's neighbours through interior faces, or a
coarse grid of g x g bins over the case, where the message is the mean over
the cell's bin (cell -> bin -> cell, two sparse stages).  The grid layers let
four layers see the whole domain: the steady velocity in a pore depends on
the flow paths through the whole sample, not only on the cells nearby.  Per-cell
features x: centroid (2), distance to the nearest wall, area, inlet and
outlet density; outputs: (rho - rho_out)/drho, u/drho (drho = rho_in - rho_out),
each standardised over the training set.
"""
from __future__ import annotations

import numpy as np

from . import _native as nat

HIDDEN, LAYERS, NFEAT, NOUT = 64, 4, 9, 3
# neighbourhood of each message-passing layer: mesh neighbours, then count-aware
# bins of 16 x 16, 4 x 4 and 1 x 1 (the whole sample)
SCALES = ("mesh", "c16", "c4", "c1")


# ----------------------------------------------------------------------------
# graph and features
SPMM_CHUNK = 64  # entries per chunk of a long row


def _chunks(indptr):
    """Chunks of at most SPMM_CHUNK entries inside each CSR row: entry
    offsets [nchunks+1] and each row's first chunk [rows+1]."""
    lens = np.diff(indptr).astype(np.int64)
    per = (lens + SPMM_CHUNK - 1) // SPMM_CHUNK
    cptr = np.concatenate([[0], np.cumsum(per)]).astype(np.int32)
    row = np.repeat(np.arange(lens.size), per)
    k = np.arange(int(cptr[-1])) - np.repeat(cptr[:-1].astype(np.int64), per)
    start = (indptr[:-1].astype(np.int64)[row] + k * SPMM_CHUNK)
    return np.concatenate([start, [int(indptr[-1])]]).astype(np.int32), cptr


def _stage(S):
    """One sparse stage of a layer's aggregation: the CSR of S and of S^T
    (row_ptr, col, wt, chunk_start, chunk_ptr), each row's entries in
    ascending column order, cut into chunks for the long rows."""
    S = S.tocsr().astype(np.float32)
    S.sort_indices()
    St = S.T.tocsr()
    St.sort_indices()

    def pack(M):
        ip = M.indptr.astype(np.int32)
        cs, cp = _chunks(ip)
        return (ip, M.indices.astype(np.int32), M.data.astype(np.float32), cs, cp)
    return {"rows": S.shape[0], "cols": S.shape[1], "M": pack(S), "Mt": pack(St)}


def mesh_mean(faces, n_cells: int):
    """Row-normalised adjacency through interior faces (a cell without
    neighbours gets a zero row)."""
    import scipy.sparse as sp
    fc = np.asarray(faces.stencil_cells_index, np.int64)
    inner = (fc[:, 0] >= 0) & (fc[:, 1] >= 0) & (fc[:, 0] != fc[:, 1])
    a, b = fc[inner, 0], fc[inner, 1]
    M = sp.coo_matrix((np.ones(2 * a.size), (np.concatenate([a, b]), np.concatenate([b, a]))),
                      shape=(n_cells, n_cells)).tocsr()
    M.data[:] = 1.0
    M.sum_duplicates()
    M.data[:] = 1.0
    deg = np.asarray(M.sum(1)).reshape(-1)
    return (sp.diags(np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)) @ M).tocsr()


def grid_mean(centers, g: int, counted: bool = False):
    """The two stages of a bin mean on a g x g grid over the cells' bounding
    box: P [bins, N] (mean of the bin's cells) and U [N, bins] (back to the
    cells).  counted: P sums the bin's cells, divided by the mean bin
    population, so that the message also says how full the bin is (the
    solid fraction of that part of the sample)."""
    import scipy.sparse as sp
    c = np.asarray(centers, np.float64)
    lo, hi = c.min(0), c.max(0)
    ij = np.clip(((c - lo) / np.maximum(hi - lo, 1e-30) * g).astype(np.int64), 0, g - 1)
    b = ij[:, 0] * g + ij[:, 1]
    n = c.shape[0]
    cnt = np.bincount(b, minlength=g * g).astype(np.float64)
    w = np.full(n, g * g / n) if counted else 1.0 / cnt[b]
    P = sp.csr_matrix((w, (b, np.arange(n))), shape=(g * g, n))
    U = sp.csr_matrix((np.ones(n), (np.arange(n), b)), shape=(n, g * g))
    return P, U


def aggregations(faces, centers, n_cells: int, scales=SCALES):
    """Per layer, the list of sparse stages whose product is A_l."""
    out = []
    for sc in scales:
        if sc == "mesh":
            out.append([_stage(mesh_mean(faces, n_cells))])
        else:  # "c<g>": count-aware bins
            counted = isinstance(sc, str) and sc.startswith("c")
            P, U = grid_mean(centers, int(sc[1:]) if counted else int(sc), counted)
            out.append([_stage(P), _stage(U)])
    return out


def wall_distance(mesher, faces, nodes):
    """Distance from each cell centroid to the nearest wall: the midpoints of
    boundary faces that are not open (both end nodes density nodes)."""
    from scipy.spatial import cKDTree
    fc = np.asarray(faces.stencil_cells_index)
    fn = np.asarray(faces.nodes_index)
    t = np.asarray(nodes.type).reshape(-1)
    bnd = (fc[:, 0] < 0) | (fc[:, 1] < 0)
    open_ = (t[fn[:, 0]] == 2) & (t[fn[:, 1]] == 2)
    wall = bnd & ~open_
    mid = np.asarray(mesher.face_centers, np.float64)[wall]
    cen = np.asarray(mesher.cell_centers, np.float64)
    if mid.shape[0] == 0:
        return np.full(cen.shape[0], 1.0)
    return cKDTree(mid).query(cen)[0]


class PotentialSystem:
    """The potential-flow estimate of one case as a linear problem: the cell
    Laplacian A phi = rhs (A symmetric positive definite on every part of the
    mesh that touches an open boundary, CSR float32) and the affine map from
    phi to its Green-Gauss gradient, grad phi = (Gx phi + g0x, Gy phi + g0y)."""

    def __init__(self, A, rhs, Gx, Gy, g0x, g0y):
        self.A, self.rhs, self.Gx, self.Gy, self.g0x, self.g0y = A, rhs, Gx, Gy, g0x, g0y
        self.n = A.shape[0]

    def gradient(self, phi):
        phi = np.asarray(phi, np.float64)
        return self.Gx @ phi + self.g0x, self.Gy @ phi + self.g0y


def potential_system(mesher, cells, faces, nodes, rho_in: float, rho_out: float):
    """The system of ``potential``: phi = (rho - rho_out)/(rho_in - rho_out)
    on open boundary faces (both end nodes density nodes), no flux through
    walls, face conductances L/(d0 + d1) (L/d0 to a boundary face).  Face
    values of phi: linear between the two cells, the boundary value on open
    faces, the owner's value on walls; the gradient is
    sum_k sign_k phi_f n_f L_f / A per cell.  None when the mesh has no open
    boundary."""
    import scipy.sparse as sp
    fc = np.asarray(faces.stencil_cells_index, np.int64)
    sd = np.asarray(faces.stencil_dists, np.float64)
    L = np.asarray(faces.L, np.float64).reshape(-1)
    fn = np.asarray(faces.nodes_index, np.int64)
    t = np.asarray(nodes.type).reshape(-1)
    nr = np.asarray(nodes.rho, np.float64).reshape(-1)
    ncell = np.asarray(mesher.cell_centers).shape[0]
    F = fc.shape[0]
    inner = (fc[:, 0] >= 0) & (fc[:, 1] >= 0)
    bnd = ~inner
    open_ = bnd & (t[fn[:, 0]] == 2) & (t[fn[:, 1]] == 2)
    if not open_.any():
        return None
    d = max(rho_in - rho_out, 1e-30)
    phib = np.zeros(F)
    phib[open_] = 0.5 * ((nr[fn[open_, 0]] - rho_out) + (nr[fn[open_, 1]] - rho_out)) / d
    w_in = L[inner] / np.maximum(sd[inner, 0] + sd[inner, 1], 1e-30)
    a, b = fc[inner, 0], fc[inner, 1]
    owner = np.where(fc[:, 0] >= 0, fc[:, 0], fc[:, 1])
    w_bd = L[open_] / np.maximum(sd[open_, 0], 1e-30)
    ob = owner[open_]
    diag = np.bincount(a, w_in, ncell) + np.bincount(b, w_in, ncell) + np.bincount(ob, w_bd, ncell)
    A = sp.coo_matrix((np.concatenate([-w_in, -w_in, diag]),
                       (np.concatenate([a, b, np.arange(ncell)]), np.concatenate([b, a, np.arange(ncell)]))),
                      shape=(ncell, ncell)).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    rhs = np.bincount(ob, w_bd * phib[open_], ncell)
    # face values pf = P phi + pf0
    fin = np.nonzero(inner)[0]
    d0, d1 = sd[inner, 0], sd[inner, 1]
    den = np.maximum(d0 + d1, 1e-30)
    wall = np.nonzero(bnd & ~open_)[0]
    P = sp.csr_matrix((np.concatenate([d1 / den, d0 / den, np.ones(wall.size)]),
                       (np.concatenate([fin, fin, wall]), np.concatenate([a, b, owner[wall]]))), shape=(F, ncell))
    pf0 = np.where(open_, phib, 0.0)
    # gradient rows: C[c, f] = sign * n * L / area over the cell's face slots
    n = np.asarray(faces.n, np.float64)
    cf = np.asarray(cells.face_indices, np.int64)
    cs = np.asarray(cells.face_normals, np.float64)
    area = np.asarray(mesher.cell_areas, np.float64).reshape(-1)
    ok = cf >= 0
    fi = np.where(ok, cf, 0)
    rows = np.repeat(np.arange(ncell), cf.shape[1])
    base = ((cs * ok) * L[fi] / area[:, None]).reshape(-1)
    fcol = fi.reshape(-1)
    Cx = sp.csr_matrix((base * n[fcol, 0], (rows, fcol)), shape=(ncell, F))
    Cy = sp.csr_matrix((base * n[fcol, 1], (rows, fcol)), shape=(ncell, F))
    return PotentialSystem(A, rhs, (Cx @ P).tocsr(), (Cy @ P).tocsr(), Cx @ pf0, Cy @ pf0)


def potential(mesher, cells, faces, nodes, rho_in: float, rho_out: float):
    """A potential-flow estimate of the flow pattern (``potential_system``),
    solved on the host by a sparse direct solver: phi and grad phi per cell
    (zeros when the mesh has no open boundary).  Its gradient points along
    the channels the steady flow takes.  ``solve_potentials`` solves the same
    systems on the GPU."""
    import scipy.sparse.linalg as spl
    ps = potential_system(mesher, cells, faces, nodes, rho_in, rho_out)
    if ps is None:
        z = np.zeros(np.asarray(mesher.cell_centers).shape[0])
        return z, z, z
    phi = spl.spsolve(ps.A.tocsc(), ps.rhs)
    gx, gy = ps.gradient(phi)
    return phi, gx, gy


def features(mesher, cells, faces, nodes, rho_in: float, rho_out: float, phi=None) -> np.ndarray:
    """Per cell: centroid, wall distance, area, inlet and outlet density, and
    the potential-flow estimate phi, grad phi (columns 6-8).  phi: False
    leaves those three columns zero (``sample(..., defer_potential=True)``)."""
    cen = np.asarray(mesher.cell_centers, np.float64)
    area = np.asarray(mesher.cell_areas, np.float64).reshape(-1)
    wd = wall_distance(mesher, faces, nodes)
    n = cen.shape[0]
    if phi is False:
        ph = gx = gy = np.zeros(n)
    else:
        ph, gx, gy = potential(mesher, cells, faces, nodes, rho_in, rho_out)
    return np.stack([cen[:, 0], cen[:, 1], wd, area, np.full(n, rho_in), np.full(n, rho_out), ph, -gx, -gy],
                    1).astype(np.float32)


def solve_potentials(samples, device: int = 0, rtol: float = 1e-6, max_iter: int = 50_000,
                     check_every: int = 100):
    """Fill the potential-flow columns of the samples built with
    ``defer_potential=True``: their systems are solved together on the GPU as
    one block-diagonal system (``fvdbm_pcg``: Jacobi-preconditioned
    conjugate gradients, float32 vectors, fixed-order dot products),
    then each gradient is formed on the host.  Returns (iterations, relative
    residual); a residual above rtol means that max_iter ran out first."""
    import ctypes as C

    import torch
    pend = [s for s in samples if getattr(s, "pending", None) is not None]
    if not pend:
        return 0, 0.0
    off, ip, ix, vals, rhs = 0, [np.zeros(1, np.int64)], [], [], []
    nnz = 0
    for s in pend:
        A = s.pending.A
        ip.append(A.indptr[1:].astype(np.int64) + nnz)
        ix.append(A.indices.astype(np.int64) + off)
        vals.append(A.data)
        rhs.append(s.pending.rhs)
        off += A.shape[0]
        nnz += A.nnz
    if off >= 2 ** 31 or nnz >= 2 ** 31:
        raise ValueError("potential systems too large for one solve (2^31 unknowns or entries)")
    dev = torch.device(f"cuda:{device}")
    t_ip = torch.from_numpy(np.concatenate(ip).astype(np.int32)).to(dev)
    t_ix = torch.from_numpy(np.concatenate(ix).astype(np.int32)).to(dev)
    t_v = torch.from_numpy(np.concatenate(vals).astype(np.float32)).to(dev)
    t_b = torch.from_numpy(np.concatenate(rhs).astype(np.float32)).to(dev)
    t_x = torch.zeros(off, dtype=torch.float32, device=dev)
    L = nat.lib()
    wb = int(L.fvdbm_pcg_work_bytes(off))
    work = torch.empty(wb, dtype=torch.uint8, device=dev)
    it, rel = C.c_int32(0), C.c_double(0.0)
    st = torch.cuda.current_stream(dev).cuda_stream
    rc = L.fvdbm_pcg(off, t_ip.data_ptr(), t_ix.data_ptr(), t_v.data_ptr(), t_b.data_ptr(), t_x.data_ptr(),
                     int(max_iter), float(rtol), int(check_every), work.data_ptr(), wb, st, C.byref(it), C.byref(rel))
    if rc != 0:
        raise nat.FvdbmError(f"fvdbm_pcg failed ({rc})")
    if not np.isfinite(rel.value):
        raise nat.FvdbmError("fvdbm_pcg: non-finite residual (matrix not positive definite?)")
    x = t_x.cpu().numpy().astype(np.float64)
    o = 0
    for s in pend:
        ps = s.pending
        phi = x[o:o + ps.n]
        o += ps.n
        gx, gy = ps.gradient(phi)
        s.x[:, 6] = phi
        s.x[:, 7] = -gx
        s.x[:, 8] = -gy
        s.pending = None
    return int(it.value), float(rel.value)


def targets(rho, vel, rho_in: float, rho_out: float) -> np.ndarray:
    d = rho_in - rho_out
    rho = np.asarray(rho, np.float64).reshape(-1)
    vel = np.asarray(vel, np.float64).reshape(-1, 2)
    return np.stack([(rho - rho_out) / d, vel[:, 0] / d, vel[:, 1] / d], 1).astype(np.float32)


def untarget(y, rho_in: float, rho_out: float):
    d = rho_in - rho_out
    y = np.asarray(y, np.float64)
    return (rho_out + d * y[:, 0]).astype(np.float32), (d * y[:, 1:3]).astype(np.float32)


class Sample:
    """One case for the network: features, per-layer aggregation stages and
    (for training) targets."""

    def __init__(self, x, aggs, t=None, pending=None):
        self.x = np.asarray(x, np.float32)
        self.aggs = aggs
        self.t = None if t is None else np.asarray(t, np.float32)
        self.n = self.x.shape[0]
        self.pending = pending  # PotentialSystem still to solve (solve_potentials)


def _cat_csr(mats, rows, cols):
    """Block-diagonal union of CSR matrices (row/column sizes per block),
    with their chunk tables."""
    ptr, col, wt, off_e, off_c = [np.zeros(1, np.int32)], [], [], 0, 0
    cst, cpt, off_k = [], [np.zeros(1, np.int32)], 0
    for (p, c, w, cs, cp), nc in zip(mats, cols):
        ptr.append(p[1:] + off_e)
        col.append(c + off_c)
        wt.append(w)
        cst.append(cs[:-1].astype(np.int64) + off_e)
        cpt.append(cp[1:].astype(np.int64) + off_k)
        off_e += int(p[-1])
        off_c += nc
        off_k += int(cp[-1])
    cst.append(np.array([off_e], np.int64))
    return (np.concatenate(ptr).astype(np.int32), np.concatenate(col).astype(np.int32), np.concatenate(wt),
            np.concatenate(cst).astype(np.int32), np.concatenate(cpt).astype(np.int32))


def _concat(samples):
    """Block-diagonal union of several samples' aggregation stages."""
    layers = []
    for l in range(len(samples[0].aggs)):
        stages = []
        for k in range(len(samples[0].aggs[l])):
            st = [s.aggs[l][k] for s in samples]
            rows, cols = [x["rows"] for x in st], [x["cols"] for x in st]
            stages.append({"rows": sum(rows), "cols": sum(cols), "M": _cat_csr([x["M"] for x in st], rows, cols),
                           "Mt": _cat_csr([x["Mt"] for x in st], cols, rows)})
        layers.append(stages)
    x = np.concatenate([s.x for s in samples])
    t = None if samples[0].t is None else np.concatenate([s.t for s in samples])
    return x, layers, t


# ----------------------------------------------------------------------------
class MPNN:
    """The warm-start network; parameters live on the GPU (float32 master,
    bfloat16 copy used by the kernels)."""

    def __init__(self, hidden: int = HIDDEN, layers: int = LAYERS, seed: int = 0, device: int = 0,
                 scales=SCALES):
        import torch
        if len(scales) != layers:
            raise ValueError("one neighbourhood scale per layer")
        self.hidden, self.layers, self.device, self.scales = hidden, layers, device, tuple(scales)
        self.shapes = [((hidden, NFEAT), (hidden,))] + [((hidden, 2 * hidden), (hidden,))] * layers + \
                      [((NOUT, hidden), (NOUT,))]
        self.offs = []
        o = 0
        for ws, bs in self.shapes:
            nw, nb = int(np.prod(ws)), int(np.prod(bs))
            self.offs.append((o, o + nw, o + nw + nb))
            o += nw + nb
        self.size = o
        rng = np.random.default_rng(seed)
        host = np.zeros(o, np.float32)
        for (ws, _), (a, b, c) in zip(self.shapes, self.offs):
            host[a:b] = (rng.standard_normal(int(np.prod(ws))) * np.sqrt(2.0 / ws[1])).astype(np.float32)
        self._dev = f"cuda:{device}"
        self.P = torch.from_numpy(host).to(self._dev)
        self.Pb = torch.zeros(o, dtype=torch.int16, device=self._dev)
        self.G = torch.zeros(o, dtype=torch.float32, device=self._dev)
        self.M = torch.zeros_like(self.G)
        self.V = torch.zeros_like(self.G)
        self.step_count = 0
        self.x_mu = np.zeros(NFEAT, np.float32)
        self.x_sd = np.ones(NFEAT, np.float32)
        self.t_mu = np.zeros(NOUT, np.float32)
        self.t_sd = np.ones(NOUT, np.float32)
        self._sync_bf16()

    # -- plumbing ------------------------------------------------------------
    def _stream(self):
        import torch
        return torch.cuda.current_stream(self.device).cuda_stream

    @staticmethod
    def _p(t):
        return 0 if t is None else int(t.data_ptr())

    def _w(self, l, buf=None):
        """Address of layer l's weights in buf (default: the bfloat16 copy)."""
        buf = self.Pb if buf is None else buf
        return self._p(buf) + buf.element_size() * self.offs[l][0]

    def _b(self, l, buf=None):
        """Address of layer l's bias in buf (default: the float32 master)."""
        buf = self.P if buf is None else buf
        return self._p(buf) + buf.element_size() * self.offs[l][1]

    def _sync_bf16(self):
        nat.check(nat.lib().fvdbm_mp_to_bf16(self._p(self.P), self._p(self.Pb), self.size, self._stream()))

    def get_params(self, rounded: bool = True):
        """[(W, b)] on the host; W rounded to bfloat16 as the kernels see it."""
        host = self.P.detach().cpu().numpy()
        out = []
        for (ws, bs), (a, b, c) in zip(self.shapes, self.offs):
            W = host[a:b].reshape(ws)
            if rounded:
                u = W.view(np.uint32).astype(np.uint64)
                W = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32).view(np.float32)
            out.append((W.copy(), host[b:c].copy()))
        return out

    def set_params(self, params):
        import torch
        host = np.zeros(self.size, np.float32)
        for (W, bb), (a, b, c) in zip(params, self.offs):
            host[a:b] = np.asarray(W, np.float32).reshape(-1)
            host[b:c] = np.asarray(bb, np.float32).reshape(-1)
        self.P.copy_(torch.from_numpy(host))
        self._sync_bf16()

    def grads(self):
        host = self.G.detach().cpu().numpy()
        return [(host[a:b].reshape(ws).copy(), host[b:c].copy()) for (ws, _), (a, b, c) in zip(self.shapes, self.offs)]

    # -- device batch ---------------------------------------------------------
    def _upload(self, samples, with_targets: bool, work=None):
        """The samples' inputs on the device (features, targets, aggregation
        stages) and the work buffers of one forward/backward pass.  ``work``
        (a dict from an earlier upload with at least as many cells and stage
        rows) lends its buffers, so that several minibatches share them."""
        import torch
        if any(getattr(s, "pending", None) is not None for s in samples):
            raise ValueError("a sample's potential-flow system is unsolved: call solve_potentials first")
        x, layers, t = _concat(samples)
        xn = (x - self.x_mu) / self.x_sd
        d = self._dev
        dev = lambda trip: [torch.from_numpy(np.ascontiguousarray(a)).to(d) for a in trip]
        H = self.hidden
        n = x.shape[0]

        def buf(rows, key, shape_rows):
            if work is not None and key in work and work[key].shape[0] >= shape_rows:
                return work[key][:shape_rows]
            return torch.empty((rows, H), device=d)
        g = {"n": n, "x": torch.from_numpy(np.ascontiguousarray(xn, np.float32)).to(d), "agg": []}
        for li, stages in enumerate(layers):
            ag = []
            for k, st in enumerate(stages):
                last = k == len(stages) - 1
                wk = None if work is None else work["agg"][li][k]
                nchM, nchMt = int(st["M"][4][-1]), int(st["Mt"][4][-1])
                ag.append({"rows": st["rows"], "cols": st["cols"], "M": dev(st["M"]), "Mt": dev(st["Mt"]),
                           # chunk partials of long rows (none when every row is one chunk)
                           "pM": torch.empty((nchM, H), device=d) if nchM > st["rows"] else None,
                           "pMt": torch.empty((nchMt, H), device=d) if nchMt > st["cols"] else None,
                           "nchM": nchM, "nchMt": nchMt,
                           # forward output of a stage before the last; its gradient
                           "tmp": None if last else (wk["tmp"][:st["rows"]] if wk is not None and wk["tmp"] is not None
                                                     and wk["tmp"].shape[0] >= st["rows"]
                                                     else torch.empty((st["rows"], H), device=d)),
                           "gtmp": None if k == 0 else (wk["gtmp"][:st["cols"]] if wk is not None and wk["gtmp"] is not None
                                                        and wk["gtmp"].shape[0] >= st["cols"]
                                                        else torch.empty((st["cols"], H), device=d))})
            g["agg"].append(ag)
        if with_targets:
            tn = (t - self.t_mu) / self.t_sd
            g["t"] = torch.from_numpy(np.ascontiguousarray(tn, np.float32)).to(d)
        if work is not None and work["n"] >= n:
            g["h"] = [a[:n] for a in work["h"]]
            g["z"] = [a[:n] for a in work["z"]]
            g["m"] = [a[:n] for a in work["m"]]
            g["y"] = work["y"][:n]
            for k in ("wscr", "dh", "dz", "dm", "dy", "mscr"):
                if work.get(k) is not None:
                    g[k] = work[k] if k in ("wscr", "mscr") else work[k][:n]
        else:
            g["h"] = [torch.empty((n, H), device=d) for _ in range(self.layers + 1)]
            g["z"] = [torch.empty((n, H), device=d) for _ in range(self.layers + 1)]
            g["m"] = [torch.empty((n, H), device=d) for _ in range(self.layers)]
            g["y"] = torch.empty((n, NOUT), device=d)
        return g

    def _spmm(self, M, rows, nch, partial, src, dst, accumulate):
        """dst (+)= M src over the CSR M: one thread per (row, feature), or in
        chunks when the matrix has rows longer than one chunk."""
        L, s, H, P = nat.lib(), self._stream(), self.hidden, self._p
        if partial is None:
            nat.check(L.fvdbm_mp_spmm(P(M[0]), P(M[1]), P(M[2]), rows, P(src), H, P(dst), int(accumulate), s))
        else:
            nat.check(L.fvdbm_mp_spmm_chunked(P(M[3]), P(M[4]), nch, P(M[1]), P(M[2]), rows, P(src), H, P(dst),
                                              int(accumulate), P(partial), s))

    def _forward(self, g):
        L, s, n, H = nat.lib(), self._stream(), g["n"], self.hidden
        P = self._p
        nat.check(L.fvdbm_mp_dense_fwd(P(g["x"]), NFEAT, 0, 0, n, self._w(0), self._b(0), H, 1, 0,
                                       P(g["z"][0]), P(g["h"][0]), s))
        for l in range(1, self.layers + 1):
            hp = g["h"][l - 1]
            src = hp
            for st in g["agg"][l - 1]:
                dst = st["tmp"] if st["tmp"] is not None else g["m"][l - 1]
                M = st["M"]
                self._spmm(M, st["rows"], st["nchM"], st["pM"], src, dst, 0)
                src = dst
            nat.check(L.fvdbm_mp_dense_fwd(P(hp), H, P(g["m"][l - 1]), H, n, self._w(l), self._b(l), H, 1, P(hp),
                                           P(g["z"][l]), P(g["h"][l]), s))
        lo = self.layers + 1
        nat.check(L.fvdbm_mp_dense_fwd(P(g["h"][-1]), H, 0, 0, n, self._w(lo), self._b(lo), NOUT, 0, 0, 0,
                                       P(g["y"]), s))

    def _ensure_work(self, g):
        """Backward work buffers of g (weight-gradient partials, dh, dz, dm, dy
        and the loss scratch), sized for its cells."""
        import torch
        L, n, H = nat.lib(), g["n"], self.hidden
        scratch_n = max(L.fvdbm_mp_wgrad_scratch(n, H, 2 * H), L.fvdbm_mp_wgrad_scratch(n, NOUT, H),
                        L.fvdbm_mp_wgrad_scratch(n, H, NFEAT))
        if g.get("wscr") is None or g["wscr"].numel() * 4 < scratch_n:
            g["wscr"] = torch.empty((scratch_n + 3) // 4, dtype=torch.float32, device=self._dev)
        if g.get("dh") is None or g["dh"].shape[0] < n:
            g["dh"] = torch.empty((n, H), device=self._dev)
            g["dz"] = torch.empty((n, H), device=self._dev)
            g["dm"] = torch.empty((n, H), device=self._dev)
        if g.get("dy") is None or g["dy"].shape[0] < n:
            g["dy"] = torch.empty((n, NOUT), device=self._dev)
            nb = L.fvdbm_mp_mse_scratch(n * NOUT)
            g["mscr"] = torch.empty((nb + 7) // 8, dtype=torch.float64, device=self._dev)

    def _backward(self, g, dy):
        L, s, n, H = nat.lib(), self._stream(), g["n"], self.hidden
        P = self._p
        self._ensure_work(g)
        ws, wsn = P(g["wscr"]), g["wscr"].numel() * 4
        lo = self.layers + 1
        G = self.G
        nat.check(L.fvdbm_mp_dense_bwd_weight(P(dy), n, NOUT, P(g["h"][-1]), H, 0, 0, self._w(lo, G), self._b(lo, G),
                                              ws, wsn, s))
        nat.check(L.fvdbm_mp_dense_bwd_data(P(dy), n, NOUT, self._w(lo), H, 0, P(g["dh"]), 0, 0, s))
        for l in range(self.layers, 0, -1):
            nat.check(L.fvdbm_mp_relu_bwd(P(g["dh"]), P(g["z"][l]), P(g["dz"]), n * H, s))
            nat.check(L.fvdbm_mp_dense_bwd_weight(P(g["dz"]), n, H, P(g["h"][l - 1]), H, P(g["m"][l - 1]), H,
                                                  self._w(l, G), self._b(l, G), ws, wsn, s))
            nat.check(L.fvdbm_mp_dense_bwd_data(P(g["dz"]), n, H, self._w(l), H, H, P(g["dh"]), 1, P(g["dm"]), s))
            grad = g["dm"]
            for k in range(len(g["agg"][l - 1]) - 1, -1, -1):
                st = g["agg"][l - 1][k]
                Mt = st["Mt"]
                if k == 0:  # back to the cells: accumulate into dh
                    self._spmm(Mt, st["cols"], st["nchMt"], st["pMt"], grad, g["dh"], 1)
                else:
                    self._spmm(Mt, st["cols"], st["nchMt"], st["pMt"], grad, st["gtmp"], 0)
                    grad = st["gtmp"]
        nat.check(L.fvdbm_mp_relu_bwd(P(g["dh"]), P(g["z"][0]), P(g["dz"]), n * H, s))
        nat.check(L.fvdbm_mp_dense_bwd_weight(P(g["dz"]), n, H, P(g["x"]), NFEAT, 0, 0, self._w(0, G), self._b(0, G),
                                              ws, wsn, s))

    def loss_and_grads(self, g):
        """Forward, mean squared error against g['t'] and backward into self.G."""
        import torch
        L, s, n = nat.lib(), self._stream(), g["n"]
        self._ensure_work(g)
        self._forward(g)
        nat.check(L.fvdbm_mp_mse(self._p(g["y"]), self._p(g["t"]), 0, n * NOUT, float(n * NOUT), self._p(g["dy"]),
                                 self._p(g["mscr"]), g["mscr"].numel() * 8, s))
        self._backward(g, g["dy"])
        return g["mscr"][0]

    # -- training and prediction ------------------------------------------
    def fit(self, samples, epochs: int = 1500, lr: float = 2e-3, lr_final: float = 1e-4, log_every: int = 100,
            b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8, batch_cells: int | None = None):
        """Adam over the samples (their graphs joined); the learning rate
        decays geometrically from lr to lr_final.  Full batch by default; with
        ``batch_cells`` the samples are split, in order, into minibatches of
        at most that many cells (a sample is never split), uploaded once and
        stepped in turn, one Adam step each, sharing one set of work buffers.
        Returns the loss history [(epoch, loss)], the loss of the epoch's last
        minibatch."""
        if any(getattr(s, "pending", None) is not None for s in samples):
            raise ValueError("a sample's potential-flow system is unsolved: call solve_potentials first")
        x = np.concatenate([s.x for s in samples])
        t = np.concatenate([s.t for s in samples])
        self.x_mu, self.x_sd = x.mean(0), np.maximum(x.std(0), 1e-12)
        self.t_mu, self.t_sd = t.mean(0), np.maximum(t.std(0), 1e-12)
        groups = [list(samples)]
        if batch_cells:
            groups, cur, cells = [], [], 0
            for smp in samples:
                if cur and cells + smp.n > batch_cells:
                    groups.append(cur)
                    cur, cells = [], 0
                cur.append(smp)
                cells += smp.n
            if cur:
                groups.append(cur)
        # the largest minibatch first: its work buffers serve every minibatch
        order = sorted(range(len(groups)), key=lambda i: -sum(s.n for s in groups[i]))
        gs = [None] * len(groups)
        for i in order:
            gs[i] = self._upload(groups[i], True, work=gs[order[0]])
            if i == order[0]:
                self._ensure_work(gs[i])
        L, s = nat.lib(), self._stream()
        hist = []
        steps = epochs * len(gs)
        for ep in range(epochs):
            for gi, g in enumerate(gs):
                loss = self.loss_and_grads(g)
                self.step_count += 1
                k = ep * len(gs) + gi
                rate = lr * (lr_final / lr) ** (k / max(steps - 1, 1))
                nat.check(L.fvdbm_mp_adam(self._p(self.P), self._p(self.M), self._p(self.V), self._p(self.Pb),
                                          self._p(self.G), self.size, rate, b1, b2, eps, self.step_count, s))
            if ep % log_every == 0 or ep == epochs - 1:
                hist.append((ep, float(loss.item())))
        return hist

    def evaluate(self, samples):
        g = self._upload(samples, True)
        return float(self.loss_and_grads(g).item())

    def predict(self, sample: Sample) -> np.ndarray:
        """Network output (in target units, not standardised) [N,3]."""
        g = self._upload([sample], False)
        self._forward(g)
        y = g["y"].detach().cpu().numpy()
        return y * self.t_sd + self.t_mu

    def predict_many(self, samples, batch_cells: int = 2_000_000):
        """Network outputs of several samples (target units) [N_i,3] each:
        the samples are joined into groups of at most ``batch_cells`` cells
        (a sample is never split), one forward pass per group, all groups on
        the work buffers of the largest."""
        groups, cur, cells = [], [], 0
        for smp in samples:
            if cur and cells + smp.n > batch_cells:
                groups.append(cur)
                cur, cells = [], 0
            cur.append(smp)
            cells += smp.n
        if cur:
            groups.append(cur)
        order = sorted(range(len(groups)), key=lambda i: -sum(s.n for s in groups[i]))
        outs = [None] * len(groups)
        work = None
        for i in order:
            g = self._upload(groups[i], False, work=work)
            if work is None:
                work = g
            self._forward(g)
            y = g["y"].detach().cpu().numpy()[:sum(s.n for s in groups[i])]
            outs[i] = np.split(y * self.t_sd + self.t_mu, np.cumsum([s.n for s in groups[i]])[:-1])
        return [y for grp in outs for y in grp]

    def save(self, path):
        np.savez(path, P=self.P.detach().cpu().numpy(), x_mu=self.x_mu, x_sd=self.x_sd, t_mu=self.t_mu,
                 t_sd=self.t_sd, hidden=self.hidden, layers=self.layers, scales=np.array([str(s) for s in self.scales]))

    @classmethod
    def load(cls, path, device: int = 0):
        import torch
        z = np.load(path)
        scales = tuple(s if (s == "mesh" or s.startswith("c")) else int(s) for s in z["scales"])
        net = cls(int(z["hidden"]), int(z["layers"]), device=device, scales=scales)
        net.P.copy_(torch.from_numpy(z["P"]))
        net._sync_bf16()
        for k in ("x_mu", "x_sd", "t_mu", "t_sd"):
            setattr(net, k, z[k])
        return net


# ----------------------------------------------------------------------------
# solver side
def sample(case, rho_in: float, rho_out: float, rho=None, vel=None, scales=SCALES,
           defer_potential: bool = False) -> Sample:
    """Sample of a case (dynamics, cells, faces, nodes, mesher); with the
    steady rho/vel it carries the training targets.  defer_potential: leave
    the potential-flow system unsolved (``solve_potentials`` solves many on
    the GPU at once); else it is solved here on the host."""
    dyn, c, f, n, m = case
    pend = None
    if defer_potential:
        x = features(m, c, f, n, rho_in, rho_out, phi=False)
        pend = potential_system(m, c, f, n, rho_in, rho_out)
    else:
        x = features(m, c, f, n, rho_in, rho_out)
    t = None if rho is None else targets(rho, vel, rho_in, rho_out)
    return Sample(x, aggregations(f, m.cell_centers, x.shape[0], scales), t, pending=pend)


def _case_arrays(case, rho_in: float, rho_out: float):
    """Host arrays of one case for the GPU feature kernels, index ranges
    checked (the kernels trust them)."""
    dyn, c, f, n, m = case
    cf = np.ascontiguousarray(np.asarray(c.face_indices), np.int32)
    cs = np.ascontiguousarray(np.asarray(c.face_normals), np.float32)
    fc = np.ascontiguousarray(np.asarray(f.stencil_cells_index), np.int32)
    fd = np.ascontiguousarray(np.asarray(f.stencil_dists), np.float32)
    fL = np.ascontiguousarray(np.asarray(f.L, np.float32).reshape(-1))
    fnrm = np.ascontiguousarray(np.asarray(f.n), np.float32)
    fno = np.asarray(f.nodes_index, np.int64)
    t = np.asarray(n.type).reshape(-1)
    nr = np.asarray(n.rho, np.float64).reshape(-1)
    cen = np.ascontiguousarray(np.asarray(m.cell_centers, np.float64))
    area = np.asarray(m.cell_areas, np.float64).reshape(-1)
    N, F = cen.shape[0], fc.shape[0]
    if cf.shape != (N, 3) or fc.shape != (F, 2) or fd.shape != (F, 2) or fL.shape != (F,) or fnrm.shape != (F, 2):
        raise ValueError("the GPU features take triangles (3 face slots per cell) with per-face stencils")
    if N and (cf.max() >= F or cf.min() < -1):
        raise ValueError("cell face index out of range")
    if F and (fc.max() >= N or fc.min() < -1):
        raise ValueError("face cell index out of range")
    inner = (fc[:, 0] >= 0) & (fc[:, 1] >= 0)
    bnd = ~inner
    open_ = bnd & (t[fno[:, 0]] == 2) & (t[fno[:, 1]] == 2)
    kind = np.where(inner, 0, np.where(open_, 2, 1)).astype(np.uint8)
    d = max(rho_in - rho_out, 1e-30)
    phib = np.zeros(F, np.float32)
    phib[open_] = (0.5 * ((nr[fno[open_, 0]] - rho_out) + (nr[fno[open_, 1]] - rho_out)) / d).astype(np.float32)
    wall = np.asarray(m.face_centers, np.float64)[bnd & ~open_]
    return {"N": N, "F": F, "cf": cf, "cs": cs, "fc": fc, "fd": fd, "fL": fL, "fn": fnrm, "kind": kind,
            "phib": phib, "cen": cen, "area": area.astype(np.float32), "wall": wall.astype(np.float32),
            "rho_in": rho_in, "rho_out": rho_out, "has_open": bool(open_.any())}


def predict_cases(net, cases, rho_in, rho_out, batch_cells: int = 2_000_000, rtol: float = 1e-6,
                  max_iter: int = 50_000):
    """The network's predictions (target units, [N_i, 3] each) for cases
    (dynamics, cells, faces, nodes, mesher), with every input built on the
    GPU: the features (wall distance, the potential-flow solve of all cases
    as one block-diagonal system, its gradient) and the aggregation stages
    (include/fvdbm_mpnn.h ``fvdbm_ws_*``), the same quantities as ``sample``
    builds on the host.  The network runs over groups of cases of at most
    ``batch_cells`` cells.  Returns (predictions, pcg iterations, pcg
    relative residual)."""
    import ctypes as C

    import torch
    if len(cases) != len(rho_in) or len(cases) != len(rho_out):
        raise ValueError("one inlet and one outlet density per case")
    if not cases:
        return [], 0, 0.0
    L, P = nat.lib(), MPNN._p
    dev = torch.device(net._dev)
    st = net._stream()
    chk = nat.check
    arr = [_case_arrays(cs, ri, ro) for cs, ri, ro in zip(cases, rho_in, rho_out)]
    up = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    D = []
    for a in arr:
        D.append({k: up(a[k]) for k in ("cf", "cs", "fc", "fd", "fL", "fn", "kind", "phib", "area")})
        D[-1]["cen"] = up(a["cen"])
        D[-1]["cx"] = up(a["cen"][:, 0].astype(np.float32))
        D[-1]["cy"] = up(a["cen"][:, 1].astype(np.float32))
        D[-1]["wx"] = up(a["wall"][:, 0].copy()) if a["wall"].shape[0] else None
        D[-1]["wy"] = up(a["wall"][:, 1].copy()) if a["wall"].shape[0] else None
    offs = np.concatenate([[0], np.cumsum([a["N"] for a in arr])]).astype(np.int64)
    ntot = int(offs[-1])
    if 4 * ntot >= 2 ** 31:
        raise ValueError("too many cells for one feature build")
    x = torch.empty((ntot, NFEAT), dtype=torch.float32, device=dev)
    acol = torch.empty(4 * ntot, dtype=torch.int32, device=dev)
    aval = torch.empty(4 * ntot, dtype=torch.float32, device=dev)
    rhs = torch.empty(ntot, dtype=torch.float32, device=dev)
    wd = torch.empty(ntot, dtype=torch.float32, device=dev)
    ngx = torch.empty(ntot, dtype=torch.float32, device=dev)
    ngy = torch.empty(ntot, dtype=torch.float32, device=dev)
    for a, d, o in zip(arr, D, offs[:-1]):
        n, o = a["N"], int(o)
        chk(L.fvdbm_ws_wall_distance(n, P(d["cx"]), P(d["cy"]), a["wall"].shape[0], P(d["wx"]), P(d["wy"]),
                                     P(wd[o:]), st))
        chk(L.fvdbm_ws_potential_rows(n, P(d["cf"]), P(d["fc"]), P(d["fd"]), P(d["fL"]), P(d["kind"]),
                                      P(d["phib"]), o, P(acol[4 * o:]), P(aval[4 * o:]), P(rhs[o:]), st))
    # the potential-flow systems of every case in one solve (fvdbm_pcg)
    ip = torch.arange(0, 4 * ntot + 1, 4, dtype=torch.int32, device=dev)
    phi = torch.zeros(ntot, dtype=torch.float32, device=dev)
    wb = int(L.fvdbm_pcg_work_bytes(ntot))
    work = torch.empty(wb, dtype=torch.uint8, device=dev)
    it, rel = C.c_int32(0), C.c_double(0.0)
    chk(L.fvdbm_pcg(ntot, P(ip), P(acol), P(aval), P(rhs), P(phi), int(max_iter), float(rtol), 100, P(work), wb,
                    st, C.byref(it), C.byref(rel)))
    if not np.isfinite(rel.value):
        raise nat.FvdbmError("fvdbm_pcg: non-finite residual")
    del work, acol, aval, rhs, ip
    for a, d, o in zip(arr, D, offs[:-1]):
        n, o = a["N"], int(o)
        chk(L.fvdbm_ws_potential_grad(n, P(d["cf"]), P(d["cs"]), P(d["fc"]), P(d["fd"]), P(d["fL"]), P(d["fn"]),
                                      P(d["kind"]), P(d["phib"]), P(phi[o:]), P(d["area"]), P(ngx[o:]),
                                      P(ngy[o:]), st))
        if not a["has_open"]:  # no open boundary: the host path's zeros
            phi[o:o + n].zero_()
            ngx[o:o + n].zero_()
            ngy[o:o + n].zero_()
        x[o:o + n, 0] = d["cx"]
        x[o:o + n, 1] = d["cy"]
        x[o:o + n, 3] = d["area"]
        x[o:o + n, 4] = float(np.float32(a["rho_in"]))
        x[o:o + n, 5] = float(np.float32(a["rho_out"]))
    x[:, 2] = wd
    x[:, 6] = phi
    x[:, 7] = ngx
    x[:, 8] = ngy
    xn = (x - torch.from_numpy(net.x_mu).to(dev)) / torch.from_numpy(net.x_sd).to(dev)
    del x
    # groups of cases for the network
    groups, cur, cells = [], [], 0
    for k, a in enumerate(arr):
        if cur and cells + a["N"] > batch_cells:
            groups.append(cur)
            cur, cells = [], 0
        cur.append(k)
        cells += a["N"]
    if cur:
        groups.append(cur)
    nmax = max(sum(arr[k]["N"] for k in g) for g in groups)
    H = net.hidden
    buf = {"h": [torch.empty((nmax, H), device=dev) for _ in range(net.layers + 1)],
           "z": [torch.empty((nmax, H), device=dev) for _ in range(net.layers + 1)],
           "m": [torch.empty((nmax, H), device=dev) for _ in range(net.layers)],
           "y": torch.empty((nmax, NOUT), device=dev)}
    preds = [None] * len(arr)
    for grp in groups:
        gofs = np.concatenate([[0], np.cumsum([arr[k]["N"] for k in grp])]).astype(np.int64)
        ng = int(gofs[-1])
        o0 = int(offs[grp[0]])
        agg = []
        for sc in net.scales:
            if sc == "mesh":
                col = torch.empty(3 * ng, dtype=torch.int32, device=dev)
                wt = torch.empty(3 * ng, dtype=torch.float32, device=dev)
                for k, go in zip(grp, gofs[:-1]):
                    chk(L.fvdbm_ws_mesh_mean(arr[k]["N"], P(D[k]["cf"]), P(D[k]["fc"]), int(go), P(col[3 * int(go):]),
                                             P(wt[3 * int(go):]), st))
                ipm = torch.arange(0, 3 * ng + 1, 3, dtype=torch.int32, device=dev)
                rows = torch.arange(0, ng + 1, dtype=torch.int32, device=dev)
                agg.append([{"rows": ng, "cols": ng, "M": (ipm, col, wt, ipm, rows), "nchM": ng, "pM": None,
                             "tmp": None}])
                continue
            counted = isinstance(sc, str) and sc.startswith("c")
            gg = int(sc[1:]) if counted else int(sc)
            nb = gg * gg
            bins = torch.empty(ng, dtype=torch.int32, device=dev)
            count = torch.zeros(nb * len(grp), dtype=torch.int32, device=dev)
            for j, (k, go) in enumerate(zip(grp, gofs[:-1])):
                cen = arr[k]["cen"]
                lo, hi = cen.min(0), cen.max(0)
                sp = np.maximum(hi - lo, 1e-30)
                chk(L.fvdbm_ws_bin_ids(arr[k]["N"], P(D[k]["cen"]), float(lo[0]), float(lo[1]), float(sp[0]),
                                       float(sp[1]), gg, P(bins[int(go):]), P(count[nb * j:]), st))
            cnt = count.cpu().numpy().astype(np.int64)
            ipp = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
            wbin = np.empty(nb * len(grp), np.float32)
            for j, k in enumerate(grp):
                c_ = cnt[nb * j:nb * (j + 1)]
                wbin[nb * j:nb * (j + 1)] = (np.full(nb, nb / arr[k]["N"]) if counted
                                             else 1.0 / np.maximum(c_, 1)).astype(np.float32)
            t_ip, t_w = up(ipp), up(wbin)
            pcol = torch.empty(ng, dtype=torch.int32, device=dev)
            pwt = torch.empty(ng, dtype=torch.float32, device=dev)
            ucol = torch.empty(ng, dtype=torch.int32, device=dev)
            for j, (k, go) in enumerate(zip(grp, gofs[:-1])):
                chk(L.fvdbm_ws_bin_rows(arr[k]["N"], nb, P(bins[int(go):]), P(t_ip[nb * j:]), P(t_w[nb * j:]),
                                        int(go), nb * j, P(pcol), P(pwt), P(ucol[int(go):]), st))
            cs_, cp_ = _chunks(ipp)
            nch = int(cp_[-1])
            rows_b = nb * len(grp)
            ipu = torch.arange(0, ng + 1, dtype=torch.int32, device=dev)
            ones = torch.ones(ng, dtype=torch.float32, device=dev)
            agg.append([{"rows": rows_b, "cols": ng, "M": (t_ip, pcol, pwt, up(cs_), up(cp_)), "nchM": nch,
                         "pM": torch.empty((nch, H), device=dev) if nch > rows_b else None,
                         "tmp": torch.empty((rows_b, H), device=dev)},
                        {"rows": ng, "cols": rows_b, "M": (ipu, ucol, ones, ipu, ipu), "nchM": ng, "pM": None,
                         "tmp": None}])
        g = {"n": ng, "x": xn[o0:o0 + ng], "agg": agg, "h": [a_[:ng] for a_ in buf["h"]],
             "z": [a_[:ng] for a_ in buf["z"]], "m": [a_[:ng] for a_ in buf["m"]], "y": buf["y"][:ng]}
        net._forward(g)
        y = g["y"].detach().cpu().numpy() * net.t_sd + net.t_mu
        for k, a0, a1 in zip(grp, gofs[:-1], gofs[1:]):
            preds[k] = y[int(a0):int(a1)]
    return preds, int(it.value), float(rel.value)


def macros(pdf):
    """rho, u of cell pdfs [N,9] (src/dynamics.py:35-47), for targets and checks."""
    from .dynamics import D2Q9
    pdf = np.asarray(pdf, np.float64)
    rho = pdf.sum(1)
    return rho, (pdf @ D2Q9.KSI.astype(np.float64)) / rho[:, None]


def run_cases(batch, threshold: float, check_every: int, cap: int, init=None, stall_checks: int = 100,
              stall_factor: float = 0.95, check_time: float = 0.0):
    """Steps a Batch to steady state with per-case retirement, like
    ``Batch.run_to_steady``, and with the warm-start fallback: when ``init`` =
    (rho [N], vel [N,2]) is given every case starts from feq(rho, u), and a
    case whose residual after ``stall_checks`` checks is not below
    ``stall_factor`` times its value ``stall_checks`` checks earlier restarts
    from the uniform state feq(1, 0).  ``check_time`` > 0 takes a case's
    residual only once it has advanced that much of its own time since its
    last check (whole chunks of ``check_every`` steps), as
    ``fvdbm_batch_run_to_steady_time`` does.  Returns per-case steps
    (including the steps before a restart), status (1 converged, 0 cap, 2
    non-finite, 3 frozen: residual exactly 0 before the threshold) and the
    restart flags."""
    S = batch.n_cases
    if init is not None:
        batch.set_cells_eq(*init)
    dts = np.array([float(d.delta_t) for d in batch.dynamics])
    window = np.full(S, check_every, np.int64)
    if check_time > 0:
        window = np.maximum(1, np.ceil(check_time / dts)).astype(np.int64)
    steps = np.zeros(S, np.int64)
    since = np.zeros(S, np.int64)
    status = np.zeros(S, np.int32)
    restarted = np.zeros(S, bool)
    active = np.ones(S, bool)
    hist = [[] for _ in range(S)]
    batch.set_active(active.astype(np.int32))
    batch.residual()
    while active.any():
        n = int(min(check_every, np.min(cap - steps[active])))
        batch.step(n)
        steps[active] += n
        since[active] += n
        take = active & ((since >= window) | (steps >= cap))
        if not take.any():
            continue
        r, _ = batch.residual(take)
        restart = []
        for s in np.flatnonzero(take):
            since[s] = 0
            hist[s].append(r[s])
            if np.isnan(r[s]):
                status[s], active[s] = 2, False
            elif r[s] == 0.0:  # exact float32 fixed point: converged if it was near the threshold
                near = len(hist[s]) > 1 and hist[s][-2] < 100.0 * threshold
                status[s], active[s] = (1 if near else 3), False
            elif r[s] < threshold:
                status[s], active[s] = 1, False
            elif steps[s] >= cap:
                active[s] = False
            elif (init is not None and not restarted[s] and len(hist[s]) > stall_checks
                  and r[s] > stall_factor * hist[s][-1 - stall_checks]):
                restart.append(s)
        for s in restart:
            from .dynamics import D2Q9
            nc = int(batch.cell_ptr[s + 1] - batch.cell_ptr[s])
            batch.set_case_pdf(s, np.tile(D2Q9.W.astype(np.float32), (nc, 1)))
            restarted[s] = True
            hist[s] = []
        batch.set_active(active.astype(np.int32))
        if restart:
            batch.residual()  # new snapshots after the restart (every case)
            since[:] = 0
    return steps, status, restarted
