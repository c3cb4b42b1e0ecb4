"""Every kernel family from a random, far-from-equilibrium state against the
oracle, bit for bit.  Random pdfs give every product and sum of the step its
own rounding, so a kernel whose compiled code fused a product into a sum (one
rounding instead of two) or reordered a fold differs here within a step."""
import numpy as np
import pytest

import goldens as G
import oracle_np as O

pytestmark = pytest.mark.gpu

KERNELS = ("one", "tile", "tile_split", "fused", "fused_nodes", "staged")
KEYS = ("cells_pdf", "cells_rho", "cells_vel", "cells_pdf_eq", "faces_pdf", "nodes_pdf", "nodes_rho", "nodes_vel")


@pytest.mark.parametrize("flux", ["upwind", "lax_wendroff"])
def test_random_state_bitwise(flux):
    from fvdbm_jax_gb300 import D2Q9, Environment, Mesher, meshgen
    m = Mesher().import_meshpy(meshgen.cavity(n=17, seed=5))
    m.calc_mesh_properties()
    dyn = D2Q9(0.6, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, flux)
    for mk in (1, 2, 4):
        n = m.set_vel_node(n, mk, (0.0, 0.0))
    n = m.set_vel_node(n, 3, (0.1, 0.0))
    rng = np.random.default_rng(11)
    pdf = np.asarray(c.pdf, np.float32)
    c.pdf = (pdf * (1.0 + 0.3 * rng.standard_normal(pdf.shape))).astype(np.float32)
    geo = O.geo_from_containers(c, f, n)
    st = O.state_from_containers(c, n)
    ref = []
    for _ in range(3):
        st = O.step(geo, st, dyn.inv_tau, dyn.dt32)
        ref.append({k: np.array(st[k]) for k in KEYS if k in st})
    for kernel in KERNELS:
        env = Environment(c, f, n, kernel=kernel)
        env.init()
        for s in range(3):
            env = env.step()
            got = G.env_state(env)
            for k, v in ref[s].items():
                assert np.array_equal(got[k].reshape(v.shape), v, equal_nan=True), (flux, kernel, s + 1, k)
        env.close()
