"""Warm-start network inputs on the CPU: the potential-flow estimate is a
bounded harmonic interpolation between inlet (1) and outlet (0) whose
gradient points from the inlet (left) towards the outlet (right)."""
import numpy as np


def test_potential_flow_features():
    from fvdbm_jax_gb300 import cases
    from fvdbm_jax_gb300 import warmstart as WS
    case = cases.porous_square(12, 3000, 0.65, rho_in=1.03, rho_out=0.97, porosity=0.8, delta_t=1.0, seed=5,
                               mesher=True)
    dyn, c, f, n, m = case
    x = WS.features(m, c, f, n, 1.03, 0.97)
    assert x.shape == (np.shape(c.pdf)[0], WS.NFEAT)
    assert np.isfinite(x).all()
    phi, ux, uy = x[:, 6], x[:, 7], x[:, 8]
    assert phi.min() >= -1e-5 and phi.max() <= 1 + 1e-5
    cx = np.asarray(m.cell_centers)[:, 0]
    assert phi[cx < 0.1].mean() > 0.8 and phi[cx > 0.9].mean() < 0.2
    assert ux.mean() > 0 and abs(uy.mean()) < 0.2 * ux.mean()
    # deterministic: the same case gives the same inputs
    assert np.array_equal(x, WS.features(m, c, f, n, 1.03, 0.97))


def test_chunk_tables_cover_each_row_in_order():
    """The chunk tables of a sparse stage cut every row into consecutive
    pieces of at most SPMM_CHUNK entries, never crossing a row, and the
    block-diagonal join keeps them consistent."""
    import scipy.sparse as sp
    from fvdbm_jax_gb300.warmstart import SPMM_CHUNK, _cat_csr, _chunks, _stage
    lens = np.array([0, 1, SPMM_CHUNK, SPMM_CHUNK + 1, 3 * SPMM_CHUNK + 7, 5])
    ip = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    cs, cp = _chunks(ip)
    assert cp[0] == 0 and cs[0] == 0 and cs[-1] == ip[-1]
    for r in range(lens.size):
        pieces = [(cs[c], cs[c + 1]) for c in range(cp[r], cp[r + 1])]
        assert sum(b - a for a, b in pieces) == lens[r]
        assert all(0 < b - a <= SPMM_CHUNK for a, b in pieces)
        if pieces:
            assert pieces[0][0] == ip[r] and pieces[-1][1] == ip[r + 1]
    A = sp.random(40, 200, density=0.3, random_state=1, format="csr")
    B = sp.random(30, 50, density=0.5, random_state=2, format="csr")
    sa, sb = _stage(A), _stage(B)
    p, c, w, cst, cpt = _cat_csr([sa["M"], sb["M"]], [40, 30], [200, 50])
    assert cpt[-1] == int(sa["M"][4][-1]) + int(sb["M"][4][-1]) and cst[-1] == p[-1]
    want = sp.block_diag([A, B]).toarray()
    got = np.zeros_like(want)
    for r in range(70):
        for k in range(cpt[r], cpt[r + 1]):
            for e in range(cst[k], cst[k + 1]):
                got[r, c[e]] += w[e]
    assert np.allclose(got, want)


def test_potential_system_and_deferred_sample():
    """The potential-flow estimate as a linear problem: A is symmetric with
    a positive, dominant diagonal; the host solve satisfies it; the affine
    gradient map equals the Green-Gauss sum over face values written out
    directly; a deferred sample leaves the three columns for the GPU solve."""
    import scipy.sparse.linalg as spl
    from fvdbm_jax_gb300 import cases
    from fvdbm_jax_gb300 import warmstart as WS
    dyn, c, f, n, m = cases.porous_square(10, 2500, 0.65, rho_in=1.02, rho_out=0.98, porosity=0.8,
                                          delta_t=1.0, seed=9, mesher=True)
    ps = WS.potential_system(m, c, f, n, 1.02, 0.98)
    A = ps.A
    assert abs(A - A.T).max() == 0.0
    d = A.diagonal()
    off = np.asarray(abs(A).sum(1)).reshape(-1) - np.abs(d)
    assert np.all(d > 0) and np.all(d >= off - 1e-12 * d)
    phi = spl.spsolve(A.tocsc(), ps.rhs)
    assert np.abs(A @ phi - ps.rhs).max() <= 1e-10 * max(np.abs(ps.rhs).max(), 1.0)
    p2, gx, gy = WS.potential(m, c, f, n, 1.02, 0.98)
    assert np.allclose(p2, phi, rtol=0, atol=1e-12)
    # Green-Gauss written out: face values, then sum_k sign_k pf n L / area
    fc = np.asarray(f.stencil_cells_index, np.int64)
    sd = np.asarray(f.stencil_dists, np.float64)
    L = np.asarray(f.L, np.float64).reshape(-1)
    fn = np.asarray(f.nodes_index, np.int64)
    t = np.asarray(n.type).reshape(-1)
    nr = np.asarray(n.rho, np.float64).reshape(-1)
    inner = (fc[:, 0] >= 0) & (fc[:, 1] >= 0)
    open_ = ~inner & (t[fn[:, 0]] == 2) & (t[fn[:, 1]] == 2)
    owner = np.where(fc[:, 0] >= 0, fc[:, 0], fc[:, 1])
    pf = phi[owner].copy()
    a, b = fc[inner, 0], fc[inner, 1]
    pf[inner] = (phi[a] * sd[inner, 1] + phi[b] * sd[inner, 0]) / (sd[inner, 0] + sd[inner, 1])
    pf[open_] = 0.5 * ((nr[fn[open_, 0]] - 0.98) + (nr[fn[open_, 1]] - 0.98)) / 0.04
    cf = np.asarray(c.face_indices, np.int64)
    cs = np.asarray(c.face_normals, np.float64)
    nn = np.asarray(f.n, np.float64)
    g = (cs[:, :, None] * (pf[cf] * L[cf])[:, :, None] * nn[cf]).sum(1) / np.asarray(m.cell_areas).reshape(-1, 1)
    assert np.allclose(gx, g[:, 0], rtol=1e-10, atol=1e-12) and np.allclose(gy, g[:, 1], rtol=1e-10, atol=1e-12)
    s = WS.sample((dyn, c, f, n, m), 1.02, 0.98, defer_potential=True)
    assert s.pending is not None and s.pending.n == s.n
    assert not s.x[:, 6:].any()
    full = WS.sample((dyn, c, f, n, m), 1.02, 0.98)
    assert full.pending is None and np.array_equal(full.x[:, :6], s.x[:, :6])


def test_gpu_feature_inputs_match_the_host_system():
    """The host side of the GPU feature path (warmstart._case_arrays): face
    kinds and open-face potentials as the host potential system uses them,
    wall points as the host wall distance uses them, and index ranges
    checked before anything reaches a kernel."""
    import copy
    import pytest
    from fvdbm_jax_gb300 import cases
    from fvdbm_jax_gb300 import warmstart as WS
    case = cases.porous_square(10, 2500, 0.65, rho_in=1.02, rho_out=0.98, porosity=0.8, delta_t=1.0, seed=9,
                               mesher=True)
    dyn, c, f, n, m = case
    a = WS._case_arrays(case, 1.02, 0.98)
    fc = np.asarray(f.stencil_cells_index)
    assert np.array_equal(a["kind"] == 0, (fc[:, 0] >= 0) & (fc[:, 1] >= 0))
    ps = WS.potential_system(m, c, f, n, 1.02, 0.98)
    # rhs of the host system from the kinds and boundary values
    sd = np.asarray(f.stencil_dists, np.float64)
    L = np.asarray(f.L, np.float64).reshape(-1)
    op = a["kind"] == 2
    owner = np.where(fc[:, 0] >= 0, fc[:, 0], fc[:, 1])
    rhs = np.bincount(owner[op], L[op] / sd[op, 0] * a["phib"][op].astype(np.float64), a["N"])
    assert np.allclose(rhs, ps.rhs, rtol=1e-6, atol=1e-12)
    from scipy.spatial import cKDTree
    wd = cKDTree(a["wall"].astype(np.float64)).query(a["cen"])[0]
    assert np.allclose(wd, WS.wall_distance(m, f, n), rtol=1e-6, atol=1e-6)
    bad = copy.deepcopy(case)
    fi = np.array(bad[1].face_indices)
    fi[0, 0] = a["F"] + 5
    bad[1].face_indices = fi
    with pytest.raises(ValueError, match="out of range"):
        WS._case_arrays(bad, 1.02, 0.98)
