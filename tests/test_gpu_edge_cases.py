"""Edge cases of the mesh: an empty mesh (no cells, faces or nodes) steps and
reads back empty arrays, as the reference's jitted step does on empty leaves;
a single triangle (every face a ghost face, one padded 32-cell group) and a
strip of two triangles match the oracle bit for bit in every family."""
from types import SimpleNamespace

import numpy as np
import pytest

import goldens as G
import oracle_np as O

pytestmark = pytest.mark.gpu

FAMILIES = ("auto", "staged", "fused", "fused_nodes", "one", "tile", "tile_split")


def _empty():
    from fvdbm_jax_gb300.containers import Cells, Faces, Nodes
    from fvdbm_jax_gb300.dynamics import D2Q9
    dyn = D2Q9(0.6, 0.1)
    c = Cells(0, dyn)
    c.face_indices = np.zeros((0, 3), np.int32)
    c.face_normals = np.zeros((0, 3), np.int32)
    return c, Faces(0, dyn), Nodes(0, dyn)


@pytest.mark.parametrize("kernel", ["auto", "staged"])
def test_empty_mesh(kernel):
    from fvdbm_jax_gb300 import Environment
    c, f, n = _empty()
    env = Environment(c, f, n, kernel=kernel)
    env.init()
    env = env.step()
    env = env.step(40)  # past the captured-graph length
    got = G.env_state(env)
    for k, v in got.items():
        assert v.size == 0, k
    env.close()


def _small(points, elements, markers):
    from fvdbm_jax_gb300 import D2Q9, Mesher
    pts = np.asarray(points, np.float64)
    el = np.asarray(elements, np.int32)
    edges = sorted({tuple(sorted((int(t[k]), int(t[(k + 1) % 3])))) for t in el for k in range(3)})
    m = Mesher().import_meshpy(SimpleNamespace(points=pts, elements=el, faces=np.asarray(edges, np.int32),
                                               point_markers=np.asarray(markers, np.int32)))
    m.calc_mesh_properties()
    dyn = D2Q9(0.6, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, "upwind")
    n = m.set_vel_node(n, 1, (0.0, 0.0))
    n = m.set_vel_node(n, 3, (0.1, 0.02))
    rng = np.random.default_rng(1)
    pdf = np.asarray(c.pdf, np.float32)
    c.pdf = (pdf * (1.0 + 0.1 * rng.standard_normal(pdf.shape))).astype(np.float32)
    return dyn, c, f, n


@pytest.mark.parametrize("shape", ["one_triangle", "two_triangles"])
def test_tiny_meshes_bitwise(shape):
    from fvdbm_jax_gb300 import Environment
    if shape == "one_triangle":
        dyn, c, f, n = _small([[0, 0], [1, 0], [0.3, 0.8]], [[0, 1, 2]], [1, 3, 3])
    else:
        dyn, c, f, n = _small([[0, 0], [1, 0], [1, 1], [0, 1]], [[0, 1, 2], [0, 2, 3]], [1, 1, 3, 3])
    geo = O.geo_from_containers(c, f, n)
    st = O.state_from_containers(c, n)
    ref = []
    for _ in range(5):
        st = O.step(geo, st, dyn.inv_tau, dyn.dt32)
        ref.append({k: np.array(v) for k, v in st.items()})
    for kernel in FAMILIES:
        env = Environment(c, f, n, kernel=kernel)
        env.init()
        for s in range(5):
            env = env.step()
            got = G.env_state(env)
            for k, v in ref[s].items():
                assert np.array_equal(got[k].reshape(v.shape), v, equal_nan=True), (shape, kernel, s + 1, k)
        env.close()
