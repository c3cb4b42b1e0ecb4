"""Every kernel family from a random, far-from-equilibrium state against the
oracle, bit for bit.  Random pdfs give every product and sum of the step its
own rounding, so a kernel whose compiled code fused a product into a sum (one
rounding instead of two) or reordered a fold differs here within a step.  A
second set plants NaN, +-inf, values near the float32 limits, subnormals and
signed zeros, which take the literal (non-finite) paths."""
import numpy as np
import pytest

import goldens as G
import oracle_np as O

pytestmark = pytest.mark.gpu

KERNELS = {"D2Q9": ("one", "tile", "tile_split", "fused", "fused_nodes", "persist", "staged"),
           "D2Q13": ("staged", "fused")}
KEYS = ("cells_pdf", "cells_rho", "cells_vel", "cells_pdf_eq", "faces_pdf", "nodes_pdf", "nodes_rho", "nodes_vel")
SPECIAL = np.array([np.nan, np.inf, -np.inf, 3.0e38, -3.0e38, 1.0e-40, -1.0e-40, 0.0, -0.0, 1.0e20, 1.0e-30],
                   np.float32)


def _run(lattice, flux, seed, special):
    from fvdbm_jax_gb300 import D2Q9, D2Q13, Environment, Mesher, meshgen
    m = Mesher().import_meshpy(meshgen.cavity(n=17, seed=seed))
    m.calc_mesh_properties()
    dyn = (D2Q9 if lattice == "D2Q9" else D2Q13)(0.6, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, flux)
    for mk in (1, 2, 4):
        n = m.set_vel_node(n, mk, (0.0, 0.0))
    n = m.set_vel_node(n, 3, (0.1, 0.0))
    rng = np.random.default_rng(seed + 6)
    pdf = np.asarray(c.pdf, np.float32)
    pdf = (pdf * (1.0 + 0.3 * rng.standard_normal(pdf.shape))).astype(np.float32)
    if special:
        pick = rng.random(pdf.shape) < 0.02
        pdf[pick] = SPECIAL[rng.integers(0, SPECIAL.size, int(pick.sum()))]
    c.pdf = pdf
    geo = O.geo_from_containers(c, f, n)
    st = O.state_from_containers(c, n)
    ref = []
    with np.errstate(all="ignore"):
        for _ in range(3):
            st = O.step(geo, st, dyn.inv_tau, dyn.dt32)
            ref.append({k: np.array(st[k]) for k in KEYS if k in st})
    if special:
        assert np.isnan(ref[-1]["cells_pdf"]).any() and np.isfinite(ref[-1]["cells_pdf"]).any()
    for kernel in KERNELS[lattice]:
        env = Environment(c, f, n, kernel=kernel)
        env.init()
        for s in range(3):
            env = env.step()
            got = G.env_state(env)
            for k, v in ref[s].items():
                assert np.array_equal(got[k].reshape(v.shape), v, equal_nan=True), (lattice, flux, kernel, s + 1, k)
        env.close()


@pytest.mark.parametrize("lattice", ["D2Q9", "D2Q13"])
@pytest.mark.parametrize("flux", ["upwind", "lax_wendroff"])
def test_random_state_bitwise(lattice, flux):
    _run(lattice, flux, seed=5, special=False)


@pytest.mark.parametrize("lattice", ["D2Q9", "D2Q13"])
@pytest.mark.parametrize("flux", ["upwind", "lax_wendroff"])
def test_non_finite_and_extreme_values_bitwise(lattice, flux):
    _run(lattice, flux, seed=6, special=True)
