"""Convergence bookkeeping of the batch on the GPU: per-case residual windows
in each case's own time (fvdbm_batch_run_to_steady_time), residuals of a
subset of cases (fvdbm_batch_residual_cases), and the statuses frozen and
non-finite, plus FVDBM_ENONFINITE from a diverging single run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fv_cases():
    from fvdbm_jax_gb300 import cases as CS
    out = [CS.lid_cavity(17, CS.tau_from_re(100.0, rule="dbm"), fv_dt=1.0, seed=1),
           CS.lid_cavity(25, CS.tau_from_re(200.0, rule="dbm"), fv_dt=1.0, seed=2),
           CS.porous_square(8, 3000, CS.tau_from_re(100.0, rule="dbm"), porosity=0.8, fv_dt=1.0,
                            rho_in=1.05, rho_out=0.95, seed=3)]
    return out


def test_windows_in_case_time_and_residual_subset():
    from fvdbm_jax_gb300 import Batch, Environment
    cases = _fv_cases()
    every, T, thr = 100, 0.5, 1e-5
    b = Batch([(c, f, n) for _, c, f, n in cases], finite_volume=True)
    b.init()
    steps, res, status = b.run_to_steady(thr, every, 40_000, check_time=T)
    for s, (dyn, c, f, n) in enumerate(cases):
        window = int(np.ceil(max(1, int(np.ceil(T / float(dyn.delta_t)))) / every)) * every
        assert steps[s] % window == 0 or steps[s] == 40_000, (s, steps[s], window)
        assert status[s] in (0, 1, 3), status
        # the case alone, checked over the same window, stops at the same step
        env = Environment(c, f, n, finite_volume=True)
        env.init()
        k, r = env.run_to_steady(thr, window, 40_000)
        assert k == steps[s], (s, k, steps[s])
        if np.isfinite(r) and r > 0:
            assert abs(r - res[s]) <= 1e-9 * r  # same sums, other chunking
        env.close()
    # a residual of a subset renews only those snapshots
    b.set_active([1, 1, 1])
    b.residual()
    b.step(200)
    r1, _ = b.residual(take=[1, 0, 0])
    assert np.isfinite(r1[0]) and np.isnan(r1[1]) and np.isnan(r1[2])
    b.step(200)
    r2, _ = b.residual(take=[0, 1, 1])
    rall, _ = b.residual()
    # cases 1 and 2 measured over 400 steps in r2; case 0 over 200 steps in
    # rall, where cases 1 and 2 have taken no step since r2 (K = 0: infinite)
    assert np.isnan(r2[0]) and np.isfinite(r2[1]) and np.isfinite(r2[2])
    assert np.isfinite(rall[0]) and np.isinf(rall[1]) and np.isinf(rall[2])
    b.step(100)
    r3, _ = b.residual()
    assert np.all(np.isfinite(r3))
    b.close()


def test_frozen_and_nonfinite_statuses():
    from fvdbm_jax_gb300 import Batch, Environment
    from fvdbm_jax_gb300 import _native as nat
    from fvdbm_jax_gb300 import cases as CS
    dyn, c, f, n = CS.lid_cavity(13, 0.6, seed=4)
    rest = CS.lid_cavity(13, 0.6, lid=0.0, seed=5)  # nothing drives the flow: it never moves
    bad = CS.lid_cavity(13, 0.6, seed=6)
    b = Batch([(c, f, n), rest[1:], bad[1:]])
    b.init()
    pdf = np.array(b.state()["pdf"])
    lo, hi = int(b.cell_ptr[2]), int(b.cell_ptr[3])
    pdf[lo + 3, 2] = np.nan
    b._set_state(pdf, None, None, None)
    steps, res, status = b.run_to_steady(1e-30, 50, 400)
    assert status[1] == nat.CASE_FROZEN and res[1] == 0.0
    assert status[2] == nat.CASE_NONFINITE and np.isnan(res[2])
    assert status[0] == nat.CASE_CAPPED and steps[0] == 400
    b.close()
    env = Environment(*bad[1:])
    env.init()
    p = np.array(env.cells.pdf)
    p[5, 1] = np.inf
    env.cells.pdf = p
    with pytest.raises(nat.NonFiniteError):
        env.run_to_steady(1e-6, 20, 200)
    env.close()


def test_lattice_units_reach_the_threshold():
    """In lattice units (mesh spacing ~1, the reference's update, the
    notebooks' tau rule, dt = 0.5 min edge) cavities and a porous square
    converge below 1e-6: genuine convergence, not a frozen float32 state;
    each case alone stops at the same step."""
    from fvdbm_jax_gb300 import Batch, Environment
    from fvdbm_jax_gb300 import cases as CS
    cases = []
    for n_, re in ((21, 100.0), (31, 400.0)):
        sc = CS.cavity_lattice_scale(n_)
        cases.append(CS.lid_cavity(n_, CS.tau_from_re(re, length=sc), seed=n_, scale=sc))
    sp = CS.porous_lattice_scale(4000, 0.8)
    cases.append(CS.porous_square(10, 4000, CS.tau_from_re(200.0, length=sp), porosity=0.8, rho_in=1.05,
                                  rho_out=0.95, seed=5, scale=sp))
    every, T, thr, cap = 100, 100.0, 1e-6, 200_000
    b = Batch([(c, f, n) for _, c, f, n in cases])
    b.init()
    steps, res, status = b.run_to_steady(thr, every, cap, check_time=T)
    b.close()
    assert list(status) == [1, 1, 1], (status, res, steps)
    assert np.all((res > 0) & (res < thr)), res
    for s, (dyn, c, f, n) in enumerate(cases):
        window = int(np.ceil(max(1, int(np.ceil(T / float(dyn.delta_t)))) / every)) * every
        env = Environment(c, f, n)
        env.init()
        k, r = env.run_to_steady(thr, window, cap)
        env.close()
        assert k == steps[s] and 0 < r < thr, (s, k, steps[s], r)
