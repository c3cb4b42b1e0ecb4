"""fvdbm_step_static_scratch (staged step with the face fluxes in a fixed
device array, no device allocation per call) against fvdbm_step on the same
mesh, called through the C ABI.  Results must be identical (tolerance 0, as
in every parity test here), on two calls in a row."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _channel(flux):
    from fvdbm_jax_gb300 import D2Q9, Mesher, meshgen
    m = Mesher().import_meshpy(meshgen.channel_cylinder())
    m.calc_mesh_properties()
    dyn = D2Q9(0.55, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, flux)
    for mk in (1, 3, 5):
        n = m.set_vel_node(n, mk, (0.0, 0.0))
    n = m.set_vel_node(n, 4, (0.0, 0.0))
    sel = m.point_markers == 4
    y = m.points[sel, 1]
    v = np.array(n.vel)
    v[sel, 0] = 4 * 0.1 * y * (0.41 - y) / 0.41 ** 2
    n.vel = v
    n = m.set_rho_node(n, 2, 1.0)
    return c, f, n


def _read(L, nat, h, N, P):
    out = {"pdf": np.empty((N, 9), np.float32), "rho": np.empty(N, np.float32),
           "vel": np.empty((N, 2), np.float32), "pdf_eq": np.empty((N, 9), np.float32),
           "npdf": np.empty((P, 9), np.float32), "nrho": np.empty(P, np.float32),
           "nvel": np.empty((P, 2), np.float32)}
    nat.check(L.fvdbm_get_cells(h, nat.fptr(out["pdf"]), nat.fptr(out["rho"]), nat.fptr(out["vel"]),
                                nat.fptr(out["pdf_eq"])), h)
    nat.check(L.fvdbm_get_nodes(h, nat.fptr(out["npdf"]), nat.fptr(out["nrho"]), nat.fptr(out["nvel"])), h)
    return out


@pytest.mark.parametrize("flux", ["upwind", "lax_wendroff"])
def test_static_scratch_matches_step(flux):
    from fvdbm_jax_gb300 import Environment
    from fvdbm_jax_gb300 import _native as nat
    L = nat.lib()
    c, f, n = _channel(flux)
    ref = Environment(c, f, n, kernel="staged")
    ref.init()
    new = Environment(c, f, n, kernel="staged")
    new.init()
    N, P = c.pdf.shape[0], n.pdf.shape[0]
    try:
        for call in range(2):
            nat.check(L.fvdbm_step(ref.handle, 5), ref.handle)
            nat.check(L.fvdbm_step_static_scratch(new.handle, 5), new.handle)
            a = _read(L, nat, ref.handle, N, P)
            b = _read(L, nat, new.handle, N, P)
            for k in a:
                assert np.array_equal(a[k], b[k], equal_nan=True), (call, k)
        assert np.abs(a["vel"]).max() > 1e-6  # the inlet drives a flow
    finally:
        ref.close()
        new.close()


def test_static_scratch_rejects_oversize_fused_and_batch():
    from fvdbm_jax_gb300 import D2Q9, Batch, Environment, Mesher, meshgen
    from fvdbm_jax_gb300 import _native as nat
    L = nat.lib()
    m = Mesher().import_meshpy(meshgen.cavity(230))
    m.calc_mesh_properties()
    c, f, n = m.to_env(D2Q9(0.6, 0.5 * float(m.face_lengths.min())), "upwind")
    assert f.n.shape[0] > 131072
    big = Environment(c, f, n, kernel="staged")
    big.init()
    fused = Environment(c, f, n, kernel="fused")
    fused.init()
    # a packed batch steps each case with its own 1/tau and dt and skips
    # retired cases: the single-mesh staged kernels would not
    ms = Mesher().import_meshpy(meshgen.cavity(12, seed=1))
    ms.calc_mesh_properties()
    cs, fs, ns = ms.to_env(D2Q9(0.6, 0.5 * float(ms.face_lengths.min())), "upwind")
    batch = Batch([(cs, fs, ns), (cs, fs, ns)])
    batch.init()
    try:
        assert L.fvdbm_step_static_scratch(big.handle, 1) == -1  # FVDBM_EINVAL
        assert b"at most 131072 padded faces" in L.fvdbm_last_error(big.handle)
        assert L.fvdbm_step_static_scratch(fused.handle, 1) == -1
        assert b"FVDBM_KERNEL_STAGED" in L.fvdbm_last_error(fused.handle)
        assert L.fvdbm_step_static_scratch(batch.handle, 1) == -1
        assert b"not a batch" in L.fvdbm_last_error(batch.handle)
        assert L.fvdbm_step_static_scratch(big.handle, -1) == -1
        assert L.fvdbm_step_static_scratch(None, 1) == -1
        nat.check(L.fvdbm_sync(big.handle), big.handle)
    finally:
        big.close()
        fused.close()
        batch.close()
