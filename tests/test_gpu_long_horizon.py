"""Parity at the configurations' stated horizons, bit for bit against the C
oracle (the reference step restated in C, float32, no contraction):

* the channel with a cylinder (about 60k triangles, tau 0.55) for 20,000
  steps with the upwind and the Lax-Wendroff flux, as the configuration
  states (the reference's own channel run is ``env = env.step()`` in a loop,
  ``tests/flow_over_cyl.ipynb:258-259``);
* the 1M-triangle porous square for 300 steps in a regime in which the flow
  develops: finite-volume scaling of the flux sum by 1/area and
  dt = 0.25 * min edge (the reference's own scaling, no 1/area and
  dt = 0.5 * min edge, leaves 99 % of the cells unchanged in float32 over
  such a horizon).  The test asserts that the velocity field moves.

Every comparison uses ``np.array_equal``: a 1e-5 relative tolerance on rho
and u is met with zero difference."""
import numpy as np
import pytest

import goldens as G
import oracle_c as OC
import oracle_np as O

pytestmark = pytest.mark.gpu


def _porous_fv(steps_factor=0.25):
    from fvdbm_jax_gb300 import D2Q9, Mesher, meshgen
    m = Mesher().import_meshpy(meshgen.porous())
    m.calc_mesh_properties()
    dyn = D2Q9(0.6, steps_factor * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, "upwind")
    for mk in (1, 3, 5):
        n = m.set_vel_node(n, mk, (0.0, 0.0))
    n = m.set_rho_node(n, 4, 1.001)
    n = m.set_rho_node(n, 2, 1.0)
    return dyn, c, f, n


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
    return dyn, c, f, n


def _compare(env, ref):
    got = G.env_state(env)
    for k in ("cells_pdf", "cells_rho", "cells_vel", "cells_pdf_eq", "nodes_pdf", "nodes_rho", "nodes_vel"):
        assert np.array_equal(got[k].reshape(ref[k].shape), ref[k], equal_nan=True), k


@pytest.mark.parametrize("flux", ["upwind", "lax_wendroff"])
def test_channel_20000_steps_bitwise(flux):
    from fvdbm_jax_gb300 import Environment
    dyn, c, f, n = _channel(flux)
    assert c.pdf.shape[0] > 50_000
    geo, st = O.geo_from_containers(c, f, n), O.state_from_containers(c, n)
    pr = OC.Prepared(geo, dyn.inv_tau, dyn.dt32)
    mid = OC.step(geo, st, dyn.inv_tau, dyn.dt32, n_steps=10_000, prepared=pr)
    ref = OC.step(geo, mid, dyn.inv_tau, dyn.dt32, n_steps=10_000, prepared=pr)
    for kernel in ("auto", "fused_nodes", "persist", "staged"):
        env = Environment(c, f, n, kernel=kernel)
        env.init()
        env.step(10_000)
        _compare(env, mid)
        env.step(10_000)
        _compare(env, ref)
        env.close()
    # the inlet drives a flow that keeps changing between the two halves
    u0, u1 = mid["cells_vel"], ref["cells_vel"]
    assert np.all(np.isfinite(u1))
    assert np.abs(u1).max() > 5e-3
    assert np.abs(u1 - u0).max() > 1e-3


def test_porous_1m_evolving_regime_bitwise():
    from fvdbm_jax_gb300 import Environment
    dyn, c, f, n = _porous_fv()
    assert c.pdf.shape[0] > 900_000
    ia = (np.float32(1) / np.asarray(c.areas, np.float32)).reshape(-1)
    geo, st = O.geo_from_containers(c, f, n), O.state_from_containers(c, n)
    pr = OC.Prepared(geo, dyn.inv_tau, dyn.dt32, ia)
    ref = OC.step(geo, st, dyn.inv_tau, dyn.dt32, n_steps=300, inv_area=ia, prepared=pr)
    u = ref["cells_vel"]
    assert np.all(np.isfinite(u))
    moving = np.mean(np.abs(u).max(axis=1) > 1e-7)
    assert moving > 0.03, moving  # the flow develops from the inlet and outlet
    assert np.abs(u).max() > 1e-4
    for kernel in ("auto", "fused", "staged"):
        env = Environment(c, f, n, kernel=kernel, finite_volume=True)
        env.init()
        env.step(300)
        _compare(env, ref)
        env.close()
