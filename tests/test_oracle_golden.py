"""The numpy oracle against golden vectors produced by the reference's own
``Environment.step`` (see tests/golden/make_golden.py): bit-exact."""
import numpy as np
import pytest

import goldens as G
import oracle_np as O


@pytest.mark.parametrize("name", G.names())
def test_oracle_matches_reference_steps(name):
    g = G.load(name)
    geo = G.geo(g)
    st = G.state(g)
    inv_tau, dt = G.inv_tau_dt(g)
    steps = [int(s) for s in g["steps"]]
    with np.errstate(all="ignore"):
        for s in range(1, max(steps) + 1):
            st = O.step(geo, st, inv_tau, dt)
            if s in steps:
                ex = G.expected(g, s)
                for k, v in ex.items():
                    assert np.array_equal(st[k].reshape(v.shape), v, equal_nan=True), (name, s, k)


def test_oracle_rest_state_is_fixed_point_without_flow():
    """feq(1,0) everywhere with all-zero-velocity walls stays put (up to
    the float32 rounding of the collision term, which is exactly zero)."""
    g = G.load("cavity7_upwind")
    geo = G.geo(g)
    st = G.state(g)
    st["nodes_vel"] = np.zeros_like(st["nodes_vel"])
    inv_tau, dt = G.inv_tau_dt(g)
    out = O.step(geo, st, inv_tau, dt)
    assert np.allclose(out["cells_pdf"], st["cells_pdf"], rtol=0, atol=1e-7)
