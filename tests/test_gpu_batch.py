"""Packed batch (fvdbm_batch_*): every case of a batch evolves bit for bit as
it does alone (against its own Environment and the C oracle), retirement
leaves a case exactly at the state of its last active step, per-case
residuals agree with single-case ones, and the autotuner restores the state."""
import numpy as np
import pytest

import oracle_c as OC
import oracle_np as ON

pytestmark = pytest.mark.gpu


def _case(kind, flux, tau, dt_scale=0.5, seed=0):
    from fvdbm_jax_gb300 import D2Q9, Mesher, meshgen
    raw = {"cavity41": lambda: meshgen.cavity(41, seed=seed), "cavity25": lambda: meshgen.cavity(25, seed=seed),
           "porous": lambda: meshgen.porous(n_obstacles=12, n_target=6000, porosity=0.8, seed=seed)}[kind]()
    m = Mesher().import_meshpy(raw)
    m.calc_mesh_properties()
    dyn = D2Q9(tau, dt_scale * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, flux)
    if kind.startswith("cavity"):
        for mk in (1, 2, 4):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_vel_node(n, 3, (0.1, 0.0))
    else:
        for mk in (1, 3, 5):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_rho_node(n, 4, 1.05)
        n = m.set_rho_node(n, 2, 0.95)
    return dyn, c, f, n


def _cases(flux):
    return [_case("cavity41", flux, 0.6), _case("porous", flux, 0.65, 0.3, seed=1),
            _case("cavity25", flux, 0.52, 0.8, seed=2), _case("porous", flux, 0.7, 0.5, seed=3)]


def _alone(dyn, c, f, n, steps):
    from fvdbm_jax_gb300 import Environment
    env = Environment(c, f, n)
    env.init()
    env.step(steps)
    out = {"pdf": np.asarray(env.cells.pdf), "rho": np.asarray(env.cells.rho).reshape(-1),
           "vel": np.asarray(env.cells.vel), "node_pdf": np.asarray(env.nodes.pdf)}
    env.close()
    return out


@pytest.mark.parametrize("flux", ["upwind", "lax_wendroff"])
def test_batch_cases_match_alone_and_oracle(flux):
    from fvdbm_jax_gb300 import Batch
    cases = _cases(flux)
    b = Batch([(c, f, n) for _, c, f, n in cases])
    b.init()
    assert b.info()["kernel"] == 6
    b.step(150)
    st = b.state()
    for s, (dyn, c, f, n) in enumerate(cases):
        got = b.case_state(s, st)
        ref = _alone(dyn, c, f, n, 150)
        for k in ("pdf", "rho", "vel", "node_pdf"):
            assert np.array_equal(got[k], ref[k]), (s, k)
        geo, st0 = ON.geo_from_containers(c, f, n), ON.state_from_containers(c, n)
        orc = OC.step(geo, st0, dyn.inv_tau, dyn.dt32, 150)
        assert np.array_equal(got["pdf"], orc["cells_pdf"]), s
    b.close()


def test_batch_launch_shapes_agree():
    from fvdbm_jax_gb300 import Batch
    cases = _cases("upwind")
    b = Batch([(c, f, n) for _, c, f, n in cases])
    b.init()
    ref = None
    for blk, waves in ((256, 1), (128, 0), (128, 2), (256, 0)):
        b.init()
        b.config(blk, waves)
        b.step(64)
        pdf = b.state()["pdf"]
        if ref is None:
            ref = pdf
        assert np.array_equal(pdf, ref), (blk, waves)
    b.close()


def test_batch_retirement_and_residuals():
    from fvdbm_jax_gb300 import Batch, Environment
    cases = _cases("upwind")
    b = Batch([(c, f, n) for _, c, f, n in cases])
    b.init()
    caps = np.array([3000, 3000, 600, 3000])
    steps, res, status = b.run_to_steady(2e-2, 200, caps)
    # every case stopped: below the threshold, or at its cap
    for s in range(len(cases)):
        assert (status[s] == 1 and res[s] < 2e-2) or (status[s] == 0 and steps[s] == caps[s]), (s, steps, res)
    assert steps[2] <= 600
    assert len(set(steps.tolist())) > 1  # the cases retired at different times
    st = b.state()
    for s, (dyn, c, f, n) in enumerate(cases):
        ref = _alone(dyn, c, f, n, int(steps[s]))
        assert np.array_equal(b.case_state(s, st)["pdf"], ref["pdf"]), s
    # a retired case stays put while the others step
    b.set_active([1, 0, 0, 0])
    b.step(10)
    st2 = b.state()
    for s in (1, 2, 3):
        assert np.array_equal(b.case_state(s, st2)["pdf"], b.case_state(s, st)["pdf"]), s
    # per-case residuals agree with each case alone (summation order differs)
    b.set_active([1, 1, 1, 1])
    b.residual()
    b.step(40)
    r, m = b.residual()
    for s, (dyn, c, f, n) in enumerate(cases):
        env = Environment(c, f, n)
        env.init()
        env.cells.pdf = b.case_state(s, st2)["pdf"]
        env.nodes.pdf = b.case_state(s, st2)["node_pdf"]
        env.residual()
        env.step(40)
        r1, m1 = env.residual()
        env.close()
        assert abs(r[s] - r1) <= 1e-9 * r1 and abs(m[s] - m1) <= 1e-12 * m1, (s, r[s], r1, m[s], m1)
    b.close()


def test_batch_autotune_restores_state():
    from fvdbm_jax_gb300 import Batch
    cases = _cases("upwind")
    b = Batch([(c, f, n) for _, c, f, n in cases])
    b.init()
    b.step(20)
    before = b.state()
    rec = b.autotune(steps=32, use_cache=False)
    assert tuple(rec["best"]) in {(256, 1), (256, 0), (256, 2), (128, 1), (128, 0), (128, 2)}
    after = b.state()
    assert np.array_equal(before["pdf"], after["pdf"])
    assert np.array_equal(before["node_pdf"], after["node_pdf"])
    b.close()


def test_batch_rejects_mixed_schemes():
    from fvdbm_jax_gb300 import Batch
    a = _case("cavity25", "upwind", 0.6)
    c = _case("cavity25", "lax_wendroff", 0.6)
    b = Batch([a[1:], c[1:]])
    with pytest.raises(ValueError, match="parameters other than"):
        b.init()
