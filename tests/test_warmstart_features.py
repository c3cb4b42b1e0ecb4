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
