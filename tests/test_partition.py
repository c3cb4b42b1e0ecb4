"""Domain decomposition on CPU ranks (gloo): each rank owns a part of the
mesh, receives its halo every step and updates its own cells with the oracle
step; the gathered result is bitwise the single-domain result."""
import os
import socket

import numpy as np
import pytest

import goldens as G
import oracle_np as ON

CASES = ["channel_upwind", "channel_lw", "mixed_quadtri_upwind", "porous_frozen_upwind", "cavity7_lw_dm2"]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _case(name):
    if name == "cavity_morton":
        from fvdbm_jax_gb300 import cases as CS
        dyn, c, f, n = CS.lid_cavity(21, 0.6, "upwind")
        return c, f, n, np.float32(dyn.inv_tau), np.float32(dyn.dt32)
    g = G.load(name)
    c, f, n = G.containers(g)
    it, dt = G.inv_tau_dt(g)
    return c, f, n, it, dt


def _worker(rank, ws, port, name, steps, out):
    import torch
    import torch.distributed as dist
    from fvdbm_jax_gb300.partition import HaloPlan, partition_cells
    os.environ["MASTER_ADDR"], os.environ["MASTER_PORT"] = "127.0.0.1", str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        c, f, n, it, dt = _case(name)
        geo, st0 = ON.geo_from_containers(c, f, n), ON.state_from_containers(c, n)
        owner = partition_cells(c, f, ws)
        plan = HaloPlan(c, f, n, owner, rank)
        N = st0["cells_pdf"].shape[0]
        pdf = np.full((N, 9), np.nan, np.float32)
        pdf[plan.owned] = st0["cells_pdf"][plan.owned]
        st = dict(st0, cells_pdf=pdf)
        for _ in range(steps):
            reqs, bufs = [], {}
            for q, cells in plan.send.items():
                if cells.size:
                    reqs.append(dist.isend(torch.from_numpy(np.ascontiguousarray(st["cells_pdf"][cells])), q))
            for q, cells in plan.recv.items():
                if cells.size:
                    bufs[q] = torch.empty((cells.size, 9), dtype=torch.float32)
                    reqs.append(dist.irecv(bufs[q], q))
            for r in reqs:
                r.wait()
            for q, b in bufs.items():
                st["cells_pdf"][plan.recv[q]] = b.numpy()
            with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
                new = ON.step(geo, st, it, dt)
            keep = np.full((N, 9), np.nan, np.float32)  # only owned cells carry over
            keep[plan.owned] = new["cells_pdf"][plan.owned]
            st = {"cells_pdf": keep, "nodes_pdf": new["nodes_pdf"], "nodes_rho": new["nodes_rho"],
                  "nodes_vel": new["nodes_vel"]}
        part = torch.from_numpy(np.ascontiguousarray(st["cells_pdf"]))
        if rank == 0:
            full = st["cells_pdf"].copy()
            for q in range(1, ws):
                b = torch.empty((N, 9), dtype=torch.float32)
                dist.recv(b, q)
                own_q = np.flatnonzero(owner == q)
                full[own_q] = b.numpy()[own_q]
            np.save(out, full)
            np.save(out + ".halo.npy", np.array([plan.halo_cells, plan.owned.size]))
        else:
            dist.send(part, 0)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("ws", [2, 3])
@pytest.mark.parametrize("name", CASES + ["cavity_morton"])
def test_partitioned_step_is_bitwise_single_domain(name, ws, tmp_path):
    import torch.multiprocessing as mp
    steps = 12
    out = str(tmp_path / "full.npy")
    mp.spawn(_worker, args=(ws, _free_port(), name, steps, out), nprocs=ws, join=True)
    got = np.load(out)
    halo, owned = np.load(out + ".halo.npy")
    c, f, n, it, dt = _case(name)
    st = ON.state_from_containers(c, n)
    geo = ON.geo_from_containers(c, f, n)
    for _ in range(steps):
        st = ON.step(geo, st, it, dt)
    assert np.array_equal(got, st["cells_pdf"], equal_nan=True)
    assert halo > 0 and owned > 0  # a real exchange took place


@pytest.mark.parametrize("ws", [2, 3])
@pytest.mark.parametrize("name", CASES)
def test_subdomains_step_alone_with_halo_exchange(name, ws):
    """Each rank's SubDomain (owned cells + halo, renumbered, faces to the
    outside turned into ghosts) is stepped on its own by the oracle; the
    halo rows are exchanged after every step.  The owned cells equal the
    single-domain step bit for bit."""
    from fvdbm_jax_gb300.partition import SubDomain, partition_cells
    c, f, n, it, dt = _case(name)
    owner = partition_cells(c, f, ws)
    subs = [SubDomain(c, f, n, owner, r) for r in range(ws)]
    assert sum(s.owned.size for s in subs) == c.pdf.shape[0]
    geos = [ON.geo_from_containers(s.cells, s.faces, s.nodes) for s in subs]
    sts = [ON.state_from_containers(s.cells, s.nodes) for s in subs]
    geo, ref = ON.geo_from_containers(c, f, n), ON.state_from_containers(c, n)
    for _ in range(10):
        with np.errstate(all="ignore"):
            sts = [ON.step(geos[r], sts[r], it, dt) for r in range(ws)]
            ref = ON.step(geo, ref, it, dt)
        for r in range(ws):
            for q, loc in subs[r].send_local.items():
                sts[q]["cells_pdf"][subs[q].recv[r]] = sts[r]["cells_pdf"][loc]
    full = np.full_like(ref["cells_pdf"], np.nan)
    for s, st in zip(subs, sts):
        full[s.cell_g[s.owned]] = st["cells_pdf"][s.owned]
    assert np.array_equal(full, ref["cells_pdf"], equal_nan=True)
    assert all(s.cells.pdf.shape[0] < c.pdf.shape[0] for s in subs)  # real sub-meshes
