"""Failure detection without a GPU fault: the bounded wait that the step
kernels use (the single-launch step's node blocks wait for the blocks that
record the stencil macros) runs out on a flag that nothing sets, records
FVDBM_STATUS_WAIT_TIMEOUT in the device status word and returns; the
context stays usable, and a step run afterwards is still exact."""
import ctypes as C

import numpy as np
import pytest

import oracle_np as O

pytestmark = pytest.mark.gpu

STATUS_WAIT_TIMEOUT = 1


def test_bounded_wait_runs_out_reports_and_leaves_the_context_usable():
    from fvdbm_jax_gb300 import D2Q9, Environment, Mesher, meshgen
    from fvdbm_jax_gb300 import _native as nat
    L = nat.lib()
    st = C.c_int32(-1)
    nat.check(L.fvdbm_wait_selftest(0, 0, 1 << 16, C.byref(st)))
    assert st.value == STATUS_WAIT_TIMEOUT
    nat.check(L.fvdbm_wait_selftest(0, 1, 1 << 16, C.byref(st)))
    assert st.value == 0
    with pytest.raises(Exception):
        nat.check(L.fvdbm_wait_selftest(0, 0, 0, C.byref(st)))  # no iterations: refused on the host
    m = Mesher().import_meshpy(meshgen.cavity(n=9, seed=3))
    m.calc_mesh_properties()
    dyn = D2Q9(0.6, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, "upwind")
    n = m.set_vel_node(n, 3, (0.1, 0.0))
    geo = O.geo_from_containers(c, f, n)
    ref = O.state_from_containers(c, n)
    for _ in range(5):
        ref = O.step(geo, ref, dyn.inv_tau, dyn.dt32)
    env = Environment(c, f, n, kernel="fused_nodes")
    env.init()
    env.step(5)
    assert np.array_equal(np.asarray(env.cells.pdf).reshape(ref["cells_pdf"].shape), ref["cells_pdf"])
    env.close()
