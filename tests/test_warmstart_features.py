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
