"""Host I/O through the C ABI: page-locked arrays, which the device reads and
writes directly over the host link, give the same bytes as pageable arrays,
which go through a staging copy.  After a single step the page-locked
rho/vel read-back runs beside the step on a second stream."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lattice", ["D2Q9", "D2Q13"])
def test_page_locked_and_pageable_io_agree(lattice):
    torch = pytest.importorskip("torch")
    from fvdbm_jax_gb300 import D2Q9, D2Q13, Environment, Mesher, meshgen
    from fvdbm_jax_gb300 import _native as nat
    m = Mesher().import_meshpy(meshgen.cavity(n=23, seed=2))
    m.calc_mesh_properties()
    dyn = (D2Q9 if lattice == "D2Q9" else D2Q13)(0.6, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, "upwind")
    n = m.set_vel_node(n, 3, (0.1, 0.0))
    N, Q = np.shape(c.pdf)
    assert N % 256 != 0  # a partial last block
    rng = np.random.default_rng(3)
    pdf = (np.asarray(c.pdf, np.float32) * (1.0 + 0.2 * rng.standard_normal((N, Q)))).astype(np.float32)
    L = nat.lib()
    out = {}
    for kind in ("pageable", "page-locked"):
        env = Environment(c, f, n)
        env.init()
        h = env.handle

        def buf(shape):
            a = np.zeros(shape, np.float32)
            return torch.from_numpy(a).pin_memory().numpy() if kind == "page-locked" else a

        src = buf((N, Q))
        src[...] = pdf
        nat.check(L.fvdbm_set_state(h, nat.fptr(src), None, None, None), h)
        src[...] = 0.0  # the call has read its input
        nat.check(L.fvdbm_step(h, 1), h)
        nat.check(L.fvdbm_step(h, 1), h)  # a single step: page-locked rho/vel are read beside it
        p, r, v = buf((N, Q)), buf((N,)), buf((N, 2))
        nat.check(L.fvdbm_get_cells(h, nat.fptr(p), None, None, None), h)
        nat.check(L.fvdbm_get_cells(h, None, nat.fptr(r), nat.fptr(v), None), h)
        r_only, v_only = buf((N,)), buf((N, 2))
        nat.check(L.fvdbm_get_cells(h, None, nat.fptr(r_only), None, None), h)
        nat.check(L.fvdbm_get_cells(h, None, None, nat.fptr(v_only), None), h)
        assert np.array_equal(r_only, r) and np.array_equal(v_only, v)
        out[kind] = (np.array(p), np.array(r), np.array(v))
        env.close()
    for a, b in zip(out["pageable"], out["page-locked"]):
        assert np.array_equal(a, b)
    assert np.isfinite(out["pageable"][1]).all() and np.abs(out["pageable"][2]).max() > 0
