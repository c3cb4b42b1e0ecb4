"""The warm start's potential-flow estimate solved on the GPU
(``fvdbm_pcg``, Jacobi-preconditioned conjugate gradients, through
``warmstart.solve_potentials``): against the host's sparse direct solve of the
same systems, for several cases solved together as one block-diagonal
system, and bitwise reproducible."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    from fvdbm_jax_gb300 import cases as CS
    out = []
    for i, (k, nt) in enumerate(((20, 6000), (60, 15000), (120, 30000))):
        rin, rout = 1.01 + 0.01 * i, 0.99 - 0.01 * i
        out.append((CS.porous_square(k, nt, 0.003, rho_in=rin, rho_out=rout, porosity=0.8, fv_dt=1.0,
                                     seed=700 + i, mesher=True), rin, rout))
    return out


def test_gpu_potential_matches_host_solve():
    from fvdbm_jax_gb300 import warmstart as WS
    cs = _cases()
    host = [WS.sample(case, rin, rout) for case, rin, rout in cs]
    runs = []
    for _ in range(2):
        dev = [WS.sample(case, rin, rout, defer_potential=True) for case, rin, rout in cs]
        assert all(s.pending is not None for s in dev)
        it, rel = WS.solve_potentials(dev, rtol=1e-6)
        assert all(s.pending is None for s in dev)
        assert 0 < it < 50_000 and rel <= 1e-6, (it, rel)
        runs.append(dev)
    for h, d, d2 in zip(host, runs[0], runs[1]):
        assert np.array_equal(d.x, d2.x)  # bitwise reproducible
        assert np.array_equal(h.x[:, :6], d.x[:, :6])  # the other features are untouched
        phi_h, phi_d = h.x[:, 6].astype(np.float64), d.x[:, 6].astype(np.float64)
        assert np.abs(phi_d - phi_h).max() <= 2e-4, np.abs(phi_d - phi_h).max()
        g_h, g_d = h.x[:, 7:9].astype(np.float64), d.x[:, 7:9].astype(np.float64)
        assert np.abs(g_d - g_h).max() <= 2e-3 * np.abs(g_h).max(), (np.abs(g_d - g_h).max(), np.abs(g_h).max())


def test_unsolved_samples_are_refused():
    from fvdbm_jax_gb300 import warmstart as WS
    case, rin, rout = _cases()[0]
    s = WS.sample(case, rin, rout, defer_potential=True)
    net = WS.MPNN(seed=0)
    with pytest.raises(ValueError, match="solve_potentials"):
        net.fit([s], epochs=1)


def test_predict_many_equals_predict():
    from fvdbm_jax_gb300 import warmstart as WS
    cs = _cases()
    smp = [WS.sample(case, rin, rout, defer_potential=True) for case, rin, rout in cs]
    WS.solve_potentials(smp)
    net = WS.MPNN(seed=3)
    one = [net.predict(s) for s in smp]
    for bc in (10**9, 20_000):  # one group; several groups on shared buffers
        many = net.predict_many(smp, batch_cells=bc)
        assert len(many) == len(one)
        for a, b in zip(one, many):
            assert np.array_equal(a, b)


def test_predict_cases_on_the_gpu_matches_the_host_path():
    """Features and stages built on the GPU (warmstart.predict_cases) give the
    network the same inputs as the host path (sample + solve_potentials +
    predict_many): the same predictions up to the potential solve's rounding,
    and the same bits on a repeat."""
    from fvdbm_jax_gb300 import warmstart as WS
    cs = _cases()
    smp = [WS.sample(case, rin, rout, defer_potential=True) for case, rin, rout in cs]
    WS.solve_potentials(smp, rtol=1e-6)
    net = WS.MPNN(seed=5)
    x = np.concatenate([s.x for s in smp])
    net.x_mu, net.x_sd = x.mean(0), np.maximum(x.std(0), 1e-12)
    host = net.predict_many(smp)
    rin, rout = [c[1] for c in cs], [c[2] for c in cs]
    for bc in (10 ** 9, 20_000):
        gpu, it, rel = WS.predict_cases(net, [c[0] for c in cs], rin, rout, batch_cells=bc)
        again, _, _ = WS.predict_cases(net, [c[0] for c in cs], rin, rout, batch_cells=bc)
        assert rel <= 1e-6 and it > 0
        for h, g, g2 in zip(host, gpu, again):
            assert np.array_equal(g, g2)
            assert g.shape == h.shape
            scale = np.abs(h).max(0)
            assert np.all(np.abs(g - h).max(0) <= 1e-3 * scale + 1e-6), (np.abs(g - h).max(0), scale)
