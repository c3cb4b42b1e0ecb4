"""Domain decomposition stepped by libfvdbm on one GPU: each rank's
sub-domain (owned cells plus a one-ring halo, ``partition.SubDomain``) is
its own handle; after every step each rank packs the owned rows its
neighbours read (``fvdbm_pack_cells`` into a device buffer) and the
neighbours unpack them over their halo rows (``fvdbm_unpack_cells``).  The
owned cells gathered from all ranks equal the single-domain step bit for bit,
for every kernel family that the mesh allows.  (One process drives all
handles in turn, so no kernel waits on another rank's kernel.)"""
import numpy as np
import pytest

import goldens as G

pytestmark = pytest.mark.gpu


def _run_partitioned(c, f, n, ws, steps, kernel):
    import torch
    from fvdbm_jax_gb300 import Environment
    from fvdbm_jax_gb300 import _native as nat
    from fvdbm_jax_gb300.partition import SubDomain, partition_cells
    L = nat.lib()
    owner = partition_cells(c, f, ws)
    subs = [SubDomain(c, f, n, owner, r) for r in range(ws)]
    envs = []
    for s in subs:
        e = Environment(s.cells, s.faces, s.nodes, kernel=kernel)
        e.init()
        envs.append(e)
    Q = 9
    bufs = {(r, q): torch.empty((max(len(loc), 1), Q), dtype=torch.float32, device="cuda")
            for r in range(ws) for q, loc in subs[r].send_local.items()}
    idx = {k: np.ascontiguousarray(v, np.int32) for k, v in
           [((r, q), loc) for r in range(ws) for q, loc in subs[r].send_local.items()]}
    ridx = {(r, q): np.ascontiguousarray(subs[q].recv[r], np.int32) for (r, q) in bufs}
    moved = 0
    for _ in range(steps):
        for e in envs:
            e.step(1)
        for (r, q), b in bufs.items():
            nat.check(L.fvdbm_pack_cells(envs[r].handle, nat.iptr(idx[r, q]), len(idx[r, q]), b.data_ptr()),
                      envs[r].handle)
        for e in envs:
            e.sync()
        for (r, q), b in bufs.items():
            assert len(ridx[r, q]) == len(idx[r, q])
            nat.check(L.fvdbm_unpack_cells(envs[q].handle, nat.iptr(ridx[r, q]), len(ridx[r, q]), b.data_ptr()),
                      envs[q].handle)
            moved += len(ridx[r, q])
        for e in envs:
            e.sync()
    N = c.pdf.shape[0]
    full = np.full((N, Q), np.nan, np.float32)
    for s, e in zip(subs, envs):
        pdf = np.asarray(e.cells.pdf)
        full[s.cell_g[s.owned]] = pdf[s.owned]
        e.close()
    return full, moved


def _single(c, f, n, steps, kernel):
    from fvdbm_jax_gb300 import Environment
    e = Environment(c, f, n, kernel=kernel)
    e.init()
    e.step(steps)
    out = np.array(e.cells.pdf)
    e.close()
    return out


@pytest.mark.parametrize("ws", [2, 3])
@pytest.mark.parametrize("name,kernels", [
    ("channel_upwind", ("auto", "fused_nodes", "staged")),
    ("channel_lw", ("auto", "fused_nodes", "staged")),
    ("mixed_quadtri_upwind", ("auto",)),
    ("porous_frozen_upwind", ("auto", "fused_nodes", "tile_split")),
    ("cavity7_lw_dm2", ("auto", "staged")),
])
def test_partitioned_handles_equal_single_domain(name, kernels, ws):
    g = G.load(name)
    c, f, n = G.containers(g)
    steps = 12
    for kernel in kernels:
        got, moved = _run_partitioned(c, f, n, ws, steps, kernel)
        want = _single(c, f, n, steps, kernel)
        assert np.array_equal(got, want, equal_nan=True), (name, ws, kernel)
        assert moved > 0  # a real exchange took place


def test_partitioned_channel_60k_fused_nodes():
    from fvdbm_jax_gb300 import D2Q9, Mesher, meshgen
    m = Mesher().import_meshpy(meshgen.channel_cylinder())
    m.calc_mesh_properties()
    dyn = D2Q9(0.55, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, "upwind")
    for mk in (1, 3, 5):
        n = m.set_vel_node(n, mk, (0.0, 0.0))
    n = m.set_vel_node(n, 4, (0.0, 0.0))
    sel = m.point_markers == 4
    y = m.points[sel, 1]
    v = np.array(n.vel)
    v[sel, 0] = 4 * 0.1 * y * (0.41 - y) / 0.41 ** 2
    n.vel = v
    n = m.set_rho_node(n, 2, 1.0)
    got, moved = _run_partitioned(c, f, n, 4, 50, "fused_nodes")
    want = _single(c, f, n, 50, "fused_nodes")
    assert np.array_equal(got, want)
    assert moved > 0 and np.abs(want[:, 1] - want[:, 3]).max() > 0  # the inlet drives a flow
