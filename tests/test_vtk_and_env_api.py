"""Output and API surface around the step that needs no GPU:

* ``Mesher.to_vtk`` (reference ``src/mesher.py:562-598``, written there by
  pyvista): the legacy file is parsed back and every array checked, with
  and without the optional ``pdf`` / ``feq`` cell arrays;
* ``Environment.create`` / ``Environment.define`` (``src/environment.py:20-36``)
  build environments from sizes and from containers without touching a
  device."""
import numpy as np
import pytest
from types import SimpleNamespace


def _parse_vtk(path):
    """Legacy ASCII unstructured grid -> dict of sections and arrays."""
    tok = open(path).read().split("\n")
    assert tok[0].startswith("# vtk DataFile")
    assert tok[2] == "ASCII" and tok[3] == "DATASET UNSTRUCTURED_GRID"
    words = " ".join(tok[4:]).split()
    out, i = {"fields": {}}, 0

    def take(k, conv=float):
        nonlocal i
        v = [conv(w) for w in words[i:i + k]]
        i += k
        return v

    while i < len(words):
        w = words[i]
        if w == "POINTS":
            n = int(words[i + 1]); i += 3
            out["points"] = np.array(take(3 * n)).reshape(n, 3)
        elif w == "CELLS":
            n, size = int(words[i + 1]), int(words[i + 2]); i += 3
            out["cells"] = np.array(take(size, int)).reshape(n, -1)
        elif w == "CELL_TYPES":
            n = int(words[i + 1]); i += 2
            out["cell_types"] = np.array(take(n, int))
        elif w == "CELL_DATA":
            out["n_cell_data"] = int(words[i + 1]); i += 2
        elif w == "VECTORS":
            name = words[i + 1]; i += 3
            out[name] = np.array(take(3 * out["n_cell_data"])).reshape(-1, 3)
        elif w == "SCALARS":
            name, ncomp = words[i + 1], int(words[i + 3]); i += 4
            assert words[i] == "LOOKUP_TABLE"; i += 2
            out[name] = np.array(take(ncomp * out["n_cell_data"])).reshape(-1, ncomp)
        elif w == "FIELD":
            k = int(words[i + 2]); i += 3
            out["field_blocks"] = out.get("field_blocks", 0) + 1
            for _ in range(k):
                name, nc, nt = words[i], int(words[i + 1]), int(words[i + 2]); i += 4
                out["fields"][name] = np.array(take(nc * nt)).reshape(nt, nc)
        else:
            raise AssertionError(f"unexpected token {w!r}")
    return out


def _mesh():
    from fvdbm_jax_gb300 import D2Q9, Mesher, meshgen
    m = Mesher().import_meshpy(meshgen.cavity(n=7, seed=2))
    m.calc_mesh_properties()
    c, f, n = m.to_env(D2Q9(0.6, 0.5 * float(m.face_lengths.min())), "upwind")
    return m, c, f, n


def _fake_env(N, seed=0):
    rng = np.random.default_rng(seed)
    cells = SimpleNamespace(vel=rng.normal(size=(N, 2)).astype(np.float32),
                            rho=(1 + 0.01 * rng.normal(size=(N, 1))).astype(np.float32),
                            pdf=rng.random((N, 9)).astype(np.float32),
                            pdf_eq=rng.random((N, 9)).astype(np.float32))
    return SimpleNamespace(cells=cells)


@pytest.mark.parametrize("save_f,save_feq", [(False, False), (True, False), (False, True), (True, True)])
def test_to_vtk_round_trip(tmp_path, save_f, save_feq):
    m, c, f, n = _mesh()
    N = c.pdf.shape[0]
    env = _fake_env(N)
    path = m.to_vtk(env, str(tmp_path / "out"), save_f=save_f, save_feq=save_feq)
    assert path.endswith(".vtk")
    v = _parse_vtk(path)
    # geometry: points with z = 0, triangles (VTK type 5) over the mesher's cells
    assert np.array_equal(v["points"][:, :2], m.points) and not v["points"][:, 2].any()
    assert np.array_equal(v["cells"][:, 0], np.full(N, 3))
    assert np.array_equal(v["cells"][:, 1:], m.cells)
    assert np.array_equal(v["cell_types"], np.full(N, 5))
    # cell data: Velocity (u, v, 0) and Density, float32 values exactly
    assert v["n_cell_data"] == N
    assert np.array_equal(v["Velocity"][:, :2].astype(np.float32), env.cells.vel)
    assert not v["Velocity"][:, 2].any()
    assert np.array_equal(v["Density"].astype(np.float32), env.cells.rho.reshape(N, 1))
    want = {k: a for k, a, flag in (("pdf", env.cells.pdf, save_f), ("feq", env.cells.pdf_eq, save_feq)) if flag}
    assert set(v["fields"]) == set(want)
    for k, a in want.items():
        assert np.array_equal(v["fields"][k].astype(np.float32), a), k
    # every optional array sits in one FIELD block, as VTK's own writer puts it
    assert v.get("field_blocks", 0) == (1 if want else 0)


def test_environment_create_and_define():
    from fvdbm_jax_gb300 import D2Q9, Environment
    from fvdbm_jax_gb300.containers import Cells, Faces, Nodes
    dyn = D2Q9(0.6, 0.01)
    saved = Environment.dynamics
    try:
        Environment.dynamics = None
        with pytest.raises(ValueError):
            Environment.create(4, 5, 6)
        Environment.dynamics = dyn
        env = Environment.create(4, 5, 6)
        assert isinstance(env.cells, Cells) and isinstance(env.faces, Faces) and isinstance(env.nodes, Nodes)
        # every container starts at feq(1, 0) = W (src/containers.py:24-30)
        for cont, k in ((env.cells, 4), (env.faces, 5), (env.nodes, 6)):
            pdf = np.asarray(cont.pdf)
            assert pdf.shape == (k, 9)
            assert np.array_equal(pdf, np.tile(D2Q9.W.astype(np.float32), (k, 1)))
        assert env.handle is None  # nothing on a device before init()
    finally:
        Environment.dynamics = saved
    m, c, f, n = _mesh()
    env = Environment.define(c, f, n)
    assert isinstance(env, Environment) and env.handle is None
    assert np.array_equal(np.asarray(env.cells.face_indices), np.asarray(c.face_indices))
    assert np.array_equal(np.asarray(env.faces.n), np.asarray(f.n))
    assert np.array_equal(np.asarray(env.nodes.type), np.asarray(n.type))
    # define keeps the caller's containers untouched (it holds copies)
    assert env.cells is not c
