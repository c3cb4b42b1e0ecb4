"""Vectorised Mesher against the reference Mesher.to_env output recorded in
the golden vectors: integer arrays exact, float32 arrays within one ulp."""
from types import SimpleNamespace

import numpy as np
import pytest

import goldens as G
from fvdbm_jax_gb300.dynamics import D2Q9
from fvdbm_jax_gb300.mesher import Mesher
from fvdbm_jax_gb300 import meshgen


def _ulps(a, b):
    a = np.ascontiguousarray(a, dtype=np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, dtype=np.float32).view(np.int32).astype(np.int64)
    return int(np.max(np.abs(a - b))) if a.size else 0


MESHED = [n for n in G.names() if "raw_points" in np.load(f"{G.GOLDEN_DIR}/{n}.npz").files]


@pytest.mark.parametrize("name", MESHED)
def test_to_env_matches_reference(name):
    g = G.load(name)
    raw = SimpleNamespace(points=g["raw_points"], elements=g["raw_elements"],
                          faces=g["raw_faces"], point_markers=g["raw_point_markers"])
    m = Mesher().import_meshpy(raw)
    m.calc_mesh_properties()
    dm = float(g["dim_multiplier"])
    c, f, n = m.to_env(D2Q9(float(g["tau"]), float(g["delta_t"])), str(g["flux_method"]),
                       int(dm) if dm == int(dm) else dm)
    for k, arr in [("c_face_indices", c.face_indices), ("c_face_normals", c.face_normals),
                   ("f_stencil_cells_index", f.stencil_cells_index), ("f_nodes_index", f.nodes_index),
                   ("n_cells_index", n.cells_index)]:
        assert np.array_equal(arr, g[k]), k
    floats = [("f_stencil_dists", f.stencil_dists), ("f_n", f.n), ("f_L", f.L), ("n_cell_dists", n.cell_dists)]
    if f.alpha is not None:
        floats.append(("f_alpha", f.alpha))
    if f.npq is not None:
        floats.append(("f_npq", f.npq))
    for k, arr in floats:
        assert _ulps(np.asarray(arr).reshape(g[k].shape), g[k]) <= 1, k
    assert float(g["delta_t"]) == 0.5 * float(m.face_lengths.min())


def test_unknown_flux_method_raises():
    m = Mesher().import_meshpy(meshgen.cavity(n=5))
    m.calc_mesh_properties()
    with pytest.raises(ValueError):
        m.to_env(D2Q9(0.6, 0.01), "central")


def test_cavity_config_sizes():
    raw = meshgen.cavity()
    assert raw.elements.shape == (3200, 3)
    assert raw.faces.shape == (4880, 2)
    assert raw.points.shape == (1681, 2)


def test_pickle_round_trip_without_device(tmp_path):
    """Checkpoint files hold the containers and the mesher; no GPU needed
    until the environment steps."""
    import numpy as np
    from fvdbm_jax_gb300 import D2Q9, Environment, Mesher, meshgen
    m = Mesher().import_meshpy(meshgen.cavity(9))
    m.calc_mesh_properties()
    c, f, n = m.to_env(D2Q9(0.6, 0.01), "upwind")
    env = Environment(c, f, n)
    m.to_pickle(env, str(tmp_path / "ck"))
    env2, m2 = Mesher.from_pickle(str(tmp_path / "ck"))
    assert np.array_equal(np.asarray(env2.cells.pdf), np.asarray(c.pdf))
    assert np.array_equal(m2.points, m.points)
