"""CUDA path (through the C ABI) against the golden vectors produced by the
reference's own Environment.step: every recorded leaf bit for bit, for each
kernel family and cell numbering."""
import numpy as np
import pytest

import goldens as G

pytestmark = pytest.mark.gpu

NOT_FUSABLE = {"mixed_quadtri_upwind", "cavity7_cc_alt_upwind"}
D2Q13 = {"cavity7_d2q13_upwind", "channel_d2q13_lw"}  # staged and fused kernels


def _cases():
    out = []
    for name in G.names():
        if name in NOT_FUSABLE:
            kernels = ["staged", "auto"]
        elif name in D2Q13:
            kernels = ["staged", "fused", "auto"]
        else:
            kernels = ["one", "tile", "tile_split", "fused", "fused_nodes", "persist", "staged"]
        for k in kernels:
            for order in ("none", "rcm", "morton"):
                out.append((name, k, order))
    return out


def _centroids(g):
    pts, el = g["raw_points"], g["raw_elements"]
    return (pts[el[:, 0]] + pts[el[:, 1]] + pts[el[:, 2]]) / 3.0


@pytest.mark.parametrize("name,kernel,order", _cases())
def test_gpu_matches_reference(name, kernel, order):
    from fvdbm_jax_gb300 import Environment

    g = G.load(name)
    c, f, n = G.containers(g)
    if order == "morton":
        if "raw_points" not in g:
            pytest.skip("no coordinates for this case")
        c.centroids = _centroids(g).astype(np.float32)
    env = Environment(c, f, n, kernel=kernel, ordering=order)
    env.init()
    steps = [int(s) for s in g["steps"]]
    done = 0
    for s in steps:
        if s == 0:
            continue
        env = env.step(s - done)
        done = s
        got = G.env_state(env)
        ex = G.expected(g, s)
        for k, v in ex.items():
            assert np.array_equal(got[k].reshape(v.shape), v, equal_nan=True), (name, kernel, order, s, k)
    env.close()


def test_d2q13_rejected_by_d2q9_only_parts():
    """The single-launch and tile families, the batch, the monitor and the
    warm-start initialisation are D2Q9 only and say so; AUTO runs D2Q13 on
    the fused kernels."""
    from fvdbm_jax_gb300 import Batch, Environment
    g = G.load("cavity7_d2q13_upwind")
    c, f, n = G.containers(g)
    for kernel in ("fused_nodes", "tile", "one"):
        with pytest.raises(ValueError, match="D2Q13"):
            Environment(c, f, n, kernel=kernel).init()
    env = Environment(c, f, n)
    env.init()
    assert env.info()["kernel"] == 2
    from fvdbm_jax_gb300 import _native as nat
    with pytest.raises(nat.FvdbmError, match="D2Q9"):
        env.residual()
    env.close()
    with pytest.raises(ValueError, match="D2Q13"):
        Batch([(c, f, n)]).init()
