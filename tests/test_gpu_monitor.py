"""FP64 convergence monitor (fvdbm_residual / fvdbm_run_to_steady) against the
same quantities computed here from the C oracle's float32 states."""
import numpy as np
import pytest

import oracle_c as OC
import oracle_np as ON

pytestmark = pytest.mark.gpu


def _cavity():
    from fvdbm_jax_gb300 import D2Q9, Mesher, meshgen
    m = Mesher().import_meshpy(meshgen.cavity(41))
    m.calc_mesh_properties()
    dyn = D2Q9(0.6, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, "upwind")
    for mk in (1, 2, 4):
        n = m.set_vel_node(n, mk, (0.0, 0.0))
    n = m.set_vel_node(n, 3, (0.1, 0.0))
    return dyn, c, f, n


def _macros(pdf):
    rho, u = ON.calc_macro(np.asarray(pdf, np.float32))
    return rho.reshape(-1).astype(np.float64), u.astype(np.float64)


def _res(u_prev, u_now, K, dt):
    return np.linalg.norm(u_now - u_prev) / (K * float(np.float32(dt)) * max(np.linalg.norm(u_prev), 1e-30))


def _advance(geo, st, pr, k):
    r = OC.step(geo, st, None, None, k, prepared=pr)
    return {"cells_pdf": r["cells_pdf"], "nodes_pdf": r["nodes_pdf"], "nodes_rho": r["nodes_rho"],
            "nodes_vel": r["nodes_vel"]}


def test_residual_and_mass_match_oracle():
    from fvdbm_jax_gb300 import Environment
    dyn, c, f, n = _cavity()
    geo, st = ON.geo_from_containers(c, f, n), ON.state_from_containers(c, n)
    pr = OC.Prepared(geo, dyn.inv_tau, dyn.dt32)
    area = np.asarray(c.areas, np.float32).reshape(-1).astype(np.float64)
    env = Environment(c, f, n)
    env.init()
    r0, m0 = env.residual()
    assert r0 == np.inf
    rho, u_prev = _macros(st["cells_pdf"])
    assert abs(m0 - np.sum(rho * area)) <= 1e-12 * abs(m0)
    for K in (1, 50, 200):
        env.step(K)
        st = _advance(geo, st, pr, K)
        r, m = env.residual()
        rho, u = _macros(st["cells_pdf"])
        assert abs(m - np.sum(rho * area)) <= 1e-12 * abs(m)
        want = _res(u_prev, u, K, dyn.delta_t)
        assert abs(r - want) <= 1e-10 * want, (K, r, want)
        u_prev = u
    # no step since the last call, and a state upload, both restart the measure
    assert env.residual()[0] == np.inf
    env.step(3)
    assert np.isfinite(env.residual()[0])
    env.cells.pdf = np.asarray(st["cells_pdf"])
    env.step(1)
    # a non-finite cell is reported as NaN
    bad = np.array(st["cells_pdf"], np.float32)
    bad[7, 3] = np.nan
    env.cells.pdf = bad
    env.residual()
    env.step(1)
    assert np.isnan(env.residual()[0])
    env.close()


def test_residual_bitwise_reproducible():
    from fvdbm_jax_gb300 import Environment
    dyn, c, f, n = _cavity()
    out = []
    for kernel in ("fused", "fused", "staged", "tile_split"):
        env = Environment(c, f, n, kernel=kernel)
        env.init()
        env.residual()
        seq = []
        for _ in range(3):
            env.step(40)
            seq.append(env.residual())
        out.append(seq)
        env.close()
    for seq in out[1:]:
        assert seq == out[0]


def test_run_to_steady_step_count():
    from fvdbm_jax_gb300 import Environment
    dyn, c, f, n = _cavity()
    geo, st = ON.geo_from_containers(c, f, n), ON.state_from_containers(c, n)
    pr = OC.Prepared(geo, dyn.inv_tau, dyn.dt32)
    thr, every = 2e-2, 500
    # oracle: residual every `every` steps until below thr
    _, u_prev = _macros(st["cells_pdf"])
    steps, want = 0, np.inf
    while steps < 40000:
        st = _advance(geo, st, pr, every)
        steps += every
        _, u = _macros(st["cells_pdf"])
        want = _res(u_prev, u, every, dyn.delta_t)
        u_prev = u
        if want < thr:
            break
    assert want < thr
    env = Environment(c, f, n)
    env.init()
    got_steps, got = env.run_to_steady(thr, every, 40000)
    assert got_steps == steps
    assert abs(got - want) <= 1e-10 * want
    assert np.array_equal(env.cells.pdf, st["cells_pdf"])
    env.close()
