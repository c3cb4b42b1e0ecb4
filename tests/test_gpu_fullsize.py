"""CUDA path against the C oracle at the configurations' full sizes (bit for
bit), plus run-to-run determinism and state round trips."""
import numpy as np
import pytest

import goldens as G
import oracle_c as OC

pytestmark = pytest.mark.gpu


def _case(raw, flux="upwind", tau=0.6, bc="cavity"):
    from fvdbm_jax_gb300 import D2Q9, Mesher
    m = Mesher().import_meshpy(raw)
    m.calc_mesh_properties()
    dyn = D2Q9(tau, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, flux)
    if bc == "cavity":
        for mk in (1, 2, 4):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_vel_node(n, 3, (0.1, 0.0))
    elif bc == "channel":
        for mk in (1, 3, 5):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_vel_node(n, 4, (0.0, 0.0))
        sel = m.point_markers == 4
        y = m.points[sel, 1]
        v = np.array(n.vel)
        v[sel, 0] = 4 * 0.1 * y * (0.41 - y) / 0.41 ** 2
        n.vel = v
        n = m.set_rho_node(n, 2, 1.0)
    else:  # porous
        for mk in (1, 3, 5):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_rho_node(n, 4, 1.001)
        n = m.set_rho_node(n, 2, 1.0)
    return m, dyn, c, f, n


def _oracle(c, f, n, dyn, steps):
    import oracle_np as O
    geo = O.geo_from_containers(c, f, n)
    st = O.state_from_containers(c, n)
    return OC.step(geo, st, dyn.inv_tau, dyn.dt32, n_steps=steps)


def _compare(env, ref, keys=("cells_pdf", "cells_rho", "cells_vel", "cells_pdf_eq", "faces_pdf",
                             "nodes_pdf", "nodes_rho", "nodes_vel")):
    got = G.env_state(env)
    for k in keys:
        assert np.array_equal(got[k].reshape(ref[k].shape), ref[k], equal_nan=True), k


def test_cavity_config_2000_steps_bitwise():
    from fvdbm_jax_gb300 import Environment, meshgen
    m, dyn, c, f, n = _case(meshgen.cavity())
    ref = _oracle(c, f, n, dyn, 2000)
    env = Environment(c, f, n)
    env.init()
    env.step(2000)
    _compare(env, ref)
    # the lid drives a flow: the result is not the rest state
    assert np.abs(ref["cells_vel"]).max() > 1e-3


@pytest.mark.parametrize("flux", ["upwind", "lax_wendroff"])
def test_channel_config_bitwise(flux):
    from fvdbm_jax_gb300 import Environment, meshgen
    m, dyn, c, f, n = _case(meshgen.channel_cylinder(), flux, tau=0.55, bc="channel")
    ref = _oracle(c, f, n, dyn, 100)
    for kernel in ("one", "tile", "tile_split", "fused", "fused_nodes", "staged"):
        env = Environment(c, f, n, kernel=kernel)
        env.init()
        env.step(100)
        _compare(env, ref)
        env.close()


def test_porous_1m_bitwise_and_deterministic():
    from fvdbm_jax_gb300 import Environment, meshgen
    m, dyn, c, f, n = _case(meshgen.porous(), bc="porous")
    assert c.pdf.shape[0] > 900_000
    ref = _oracle(c, f, n, dyn, 4)
    env = Environment(c, f, n, kernel="tile")
    env.init()
    assert env.info()["kernel"] == 3  # the tile kernel, several tiles per CTA
    env.step(4)
    _compare(env, ref)
    a = np.array(env.cells.pdf)
    env2 = Environment(c, f, n)
    env2.init()
    env2.step(4)
    assert np.array_equal(np.array(env2.cells.pdf), a)
    for kernel in ("one", "fused", "fused_nodes", "tile_split"):
        env3 = Environment(c, f, n, kernel=kernel)
        env3.init()
        env3.step(4)
        assert np.array_equal(np.array(env3.cells.pdf), a), kernel


@pytest.mark.parametrize("kernel", ["auto", "fused_nodes"])
def test_graph_and_eager_steps_agree(kernel):
    from fvdbm_jax_gb300 import Environment, meshgen
    m, dyn, c, f, n = _case(meshgen.cavity(n=21))
    e1 = Environment(c, f, n, kernel=kernel)
    e1.init()
    e1.step(70)            # 2 graph replays of 32 + 6 eager steps
    e2 = Environment(c, f, n, kernel=kernel)
    e2.init()
    for _ in range(70):
        e2.step()
    assert np.array_equal(np.array(e1.cells.pdf), np.array(e2.cells.pdf))
    assert np.array_equal(np.array(e1.nodes.pdf), np.array(e2.nodes.pdf))


@pytest.mark.parametrize("kernel", ["auto", "fused_nodes"])
def test_state_round_trip_and_midrun_write(kernel):
    from fvdbm_jax_gb300 import Environment, meshgen
    m, dyn, c, f, n = _case(meshgen.cavity(n=15))
    env = Environment(c, f, n, kernel=kernel)
    env.init()
    rng = np.random.default_rng(0)
    pdf = (np.array(c.pdf) * (1 + 0.01 * rng.uniform(-1, 1, c.pdf.shape))).astype(np.float32)
    env.cells.pdf = pdf
    assert np.array_equal(np.array(env.cells.pdf), pdf)
    # writing a velocity boundary value mid-run is seen by the next step
    env.step(3)
    v = np.array(env.nodes.vel)
    v[m.point_markers == 3, 0] = 0.05
    env.nodes.vel = v
    env.step(2)
    import oracle_np as O
    geo = O.geo_from_containers(c, f, n)
    st = {"cells_pdf": pdf, "nodes_pdf": np.array(n.pdf), "nodes_rho": np.array(n.rho),
          "nodes_vel": np.array(n.vel)}
    st = OC.step(geo, st, dyn.inv_tau, dyn.dt32, n_steps=3)
    st["nodes_vel"] = v
    st = OC.step(geo, st, dyn.inv_tau, dyn.dt32, n_steps=2)
    _compare(env, st)


@pytest.mark.parametrize("form", [5, 2])
@pytest.mark.parametrize("lattice,which", [("D2Q9", "c2"), ("D2Q9", "c4x2"), ("D2Q9", "c2x2"), ("D2Q13", "c2"),
                                           ("D2Q13", "c4x2"), ("D2Q13", "c2x2"), ("D2Q13", "c6x2")])
def test_known_divisor_division_exhaustive(lattice, which, form):
    """Every float32 dividend: the known-divisor division (five- and
    two-operation forms) equals IEEE x/y, for each lattice constant."""
    import ctypes as C
    from fvdbm_jax_gb300 import D2Q9, D2Q13
    from fvdbm_jax_gb300 import _native as nat
    y = float(getattr((D2Q9 if lattice == "D2Q9" else D2Q13)(0.6, 0.1), which))
    bad, ex = C.c_uint64(), C.c_uint32()
    nat.check(nat.lib().fvdbm_const_div_check_form(0, y, form, C.byref(bad), C.byref(ex)))
    x = np.array([ex.value], np.uint32).view(np.float32)[0]
    assert bad.value == 0, f"{bad.value} mismatches, first dividend {x!r} (bits {ex.value:#x})"


def test_known_divisor_division_verified_and_used():
    """The three lattice-constant divisors pass the exhaustive check of the
    two-operation form (every float32 dividend gives the IEEE quotient), so
    the kernels use that form."""
    from fvdbm_jax_gb300 import Environment, meshgen
    m, dyn, c, f, n = _case(meshgen.cavity(n=5))
    env = Environment(c, f, n)
    env.init()
    assert env.info()["const_division"] == 2


@pytest.mark.parametrize("kernel", ["auto", "fused"])
def test_checkpoint_resume_is_exact(kernel, tmp_path):
    from fvdbm_jax_gb300 import Environment, Mesher, meshgen
    m, dyn, c, f, n = _case(meshgen.cavity(n=21))
    ref = Environment(c, f, n, kernel=kernel)
    ref.init()
    ref.step(70)
    env = Environment(c, f, n, kernel=kernel)
    env.init()
    env.step(30)
    m.to_pickle(env, str(tmp_path / "ck"))
    env.close()
    env2, m2 = Mesher.from_pickle(str(tmp_path / "ck"))
    assert env2.handle is None
    env2.step(40)
    for a, b in ((ref.cells.pdf, env2.cells.pdf), (ref.cells.rho, env2.cells.rho), (ref.nodes.pdf, env2.nodes.pdf),
                 (ref.nodes.rho, env2.nodes.rho), (ref.faces.pdf, env2.faces.pdf)):
        assert np.array_equal(np.asarray(a), np.asarray(b))
