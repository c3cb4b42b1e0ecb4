"""Generate the golden vectors in this folder by running the reference's own,
unmodified ``src/mesher.py``, ``src/containers.py``, ``src/faces.py``,
``src/dynamics.py`` and ``src/environment.py`` (from a checkout of
MADALERAU/FVDBM-JAX) with the numpy stand-in for jax in ``refshim/``.

Usage (needs a checkout of the reference; its path is required):

    python tests/golden/make_golden.py <reference checkout> [--only name,name]

Each case writes ``<name>.npz`` holding the raw mesh, the containers the
reference's ``Mesher.to_env`` + boundary setters produced, the initial
dynamic state and the state after selected steps of ``Environment.step``.
"""
from __future__ import annotations

import contextlib
import io
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _setup(ref_path):
    sys.path[:0] = [os.path.join(HERE, "refshim"), ref_path, os.path.join(REPO, "fvdbm-jax_gb300")]


def _np(x):
    return np.array(np.asarray(x))


def _record(env, prefix, out):
    c, f, n = env.cells, env.faces, env.nodes
    out[prefix + "c_pdf"] = _np(c.pdf)
    out[prefix + "c_rho"] = _np(c.rho)
    out[prefix + "c_vel"] = _np(c.vel)
    out[prefix + "c_pdf_eq"] = _np(c.pdf_eq)
    out[prefix + "f_pdf"] = _np(f.pdf)
    out[prefix + "n_pdf"] = _np(n.pdf)
    out[prefix + "n_rho"] = _np(n.rho)
    out[prefix + "n_vel"] = _np(n.vel)


def _static(env, out):
    c, f, n = env.cells, env.faces, env.nodes
    out["c_face_indices"] = _np(c.face_indices)
    out["c_face_normals"] = _np(c.face_normals)
    out["f_stencil_cells_index"] = _np(f.stencil_cells_index)
    out["f_stencil_dists"] = _np(f.stencil_dists)
    out["f_nodes_index"] = _np(f.nodes_index)
    out["f_n"] = _np(f.n)
    out["f_L"] = _np(f.L)
    if hasattr(f, "alpha"):
        out["f_alpha"] = _np(f.alpha)
    if hasattr(f, "npq"):
        out["f_npq"] = _np(f.npq)
    out["n_type"] = _np(n.type)
    out["n_cells_index"] = _np(n.cells_index)
    out["n_cell_dists"] = _np(n.cell_dists)


def run_case(name, raw, flux_method, tau, bc, steps, record, dim_multiplier=1,
             perturb=None, seed=0, prebuilt=None, lattice="D2Q9"):
    if ONLY and name not in ONLY:
        return
    from src import dynamics
    from src.environment import Environment
    from src.mesher import Mesher

    out = {}
    t0 = time.time()
    if prebuilt is None:
        mesh = types.SimpleNamespace(points=raw.points, elements=raw.elements,
                                     faces=raw.faces, point_markers=raw.point_markers)
        me = Mesher()
        with contextlib.redirect_stdout(io.StringIO()):
            me.import_meshpy(mesh)
            me.calc_mesh_properties()
        dt = 0.5 * float(np.min(me.face_lengths))
        d = getattr(dynamics, lattice)(tau=tau, delta_t=dt)
        cells, faces, nodes = me.to_env(d, flux_method=flux_method, dim_multiplier=dim_multiplier)
        nodes = bc(me, nodes)
        out.update(raw_points=raw.points, raw_elements=raw.elements, raw_faces=raw.faces,
                   raw_point_markers=raw.point_markers)
    else:
        cells, faces, nodes, dt = prebuilt(tau)
        d = cells.dynamics
    if perturb is not None:
        cells, nodes = perturb(cells, nodes, np.random.default_rng(seed))
    env = Environment(cells, faces, nodes)
    env.init()
    _static(env, out)
    _record(env, "s0_", out)
    out["tau"] = np.float64(tau)
    out["delta_t"] = np.float64(dt)
    out["flux_method"] = np.array(flux_method)
    out["dim_multiplier"] = np.float64(dim_multiplier)
    out["lattice"] = np.int32(d.NUM_QUIVERS)
    out["steps"] = np.array(sorted(record), dtype=np.int32)
    for s in range(1, steps + 1):
        env = env.step()
        if s in record:
            _record(env, f"s{s}_", out)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: N={out['c_pdf' if 'c_pdf' in out else 's0_c_pdf'].shape[0]} "
          f"steps={steps} {time.time() - t0:.1f}s", flush=True)


def cavity_bc(lid=0.1):
    def bc(me, nodes):
        for mk in (1, 2, 4):
            nodes = me.set_vel_node(nodes, mk, np.asarray((0.0, 0.0)))
        return me.set_vel_node(nodes, 3, np.asarray((lid, 0.0)))
    return bc


def channel_bc(height, umax=0.1):
    def bc(me, nodes):
        for mk in (1, 3, 5):
            nodes = me.set_vel_node(nodes, mk, np.asarray((0.0, 0.0)))
        nodes = me.set_vel_node(nodes, 4, np.asarray((0.0, 0.0)))
        sel = me.point_markers == 4
        y = me.points[sel, 1]
        u = 4.0 * umax * y * (height - y) / height ** 2
        prof = np.stack([u, np.zeros_like(u)], axis=1)
        nodes.vel = nodes.vel.at[sel].set(prof)
        return me.set_rho_node(nodes, 2, 1.0)
    return bc


def porous_bc_frozen(me, nodes):
    """Inlet/outlet density nodes, wall velocity nodes, obstacle points left
    as type 0: their pdf stays frozen and feeds the obstacle ghosts."""
    for mk in (1, 3):
        nodes = me.set_vel_node(nodes, mk, np.asarray((0.0, 0.0)))
    nodes = me.set_rho_node(nodes, 4, 1.05)
    nodes = me.set_rho_node(nodes, 2, 0.95)
    return nodes


def perturb_pdf(scale=0.05):
    def p(cells, nodes, rng):
        cells.pdf = cells.pdf * (1.0 + scale * rng.uniform(-1, 1, size=np.shape(cells.pdf))).astype(np.float32)
        nodes.pdf = nodes.pdf * (1.0 + scale * rng.uniform(-1, 1, size=np.shape(nodes.pdf))).astype(np.float32)
        return cells, nodes
    return p


def mixed_quadtri(tau):
    """A 4x3 grid of unit-spaced quads, every other quad split into two
    triangles, built directly as containers (as the reference's
    ``tests/ldcFVDBM.ipynb`` builds a structured quad mesh).  Triangles have a
    padded 4th face slot (-1 index, -1 sign), which the reference's gather
    wraps to the last face."""
    import jax.numpy as jnp
    from src.containers import Cells, Faces, Nodes
    from src.dynamics import D2Q9

    nx, ny, h = 4, 3, 0.25
    P = (nx + 1) * (ny + 1)
    pts = np.array([[i * h, j * h] for j in range(ny + 1) for i in range(nx + 1)], dtype=np.float64)
    polys = []
    for j in range(ny):
        for i in range(nx):
            a = j * (nx + 1) + i
            b, c, dd = a + 1, a + nx + 2, a + nx + 1
            if (i + j) % 2:
                polys += [[a, b, c], [a, c, dd]]
            else:
                polys.append([a, b, c, dd])
    N = len(polys)
    edges = {}
    cell_faces, cell_signs = [], []
    fl = []
    for ci, poly in enumerate(polys):
        cf, cs = [], []
        cen = pts[poly].mean(axis=0)
        for k in range(len(poly)):
            p0, p1 = poly[k], poly[(k + 1) % len(poly)]
            key = (min(p0, p1), max(p0, p1))
            if key not in edges:
                edges[key] = len(fl)
                fl.append([p0, p1, []])
            fi = edges[key]
            fl[fi][2].append(ci)
            t2 = pts[p1] - pts[p0]
            en = np.array([-t2[1], t2[0]]) / np.hypot(*t2)
            mid = 0.5 * (pts[p0] + pts[p1])
            if np.dot(en, cen - mid) >= 0:
                en = -en
            cf.append(fi)
            cs.append(en)
        cell_faces.append(cf)
        cell_signs.append(cs)
    F = len(fl)
    K = max(len(c) for c in cell_faces)
    cen = np.array([pts[p].mean(axis=0) for p in polys])
    sci = -np.ones((F, 2), np.int32)
    sd = -np.ones((F, 2))
    nodes_index = np.zeros((F, 2), np.int32)
    normals = np.zeros((F, 2))
    lengths = np.zeros(F)
    for fi, (p0, p1, cl) in enumerate(fl):
        t = pts[p1] - pts[p0]
        n = np.array([-t[1], t[0]]) / np.hypot(*t)
        mid = 0.5 * (pts[p0] + pts[p1])
        if len(cl) == 1 and np.dot(n, cen[cl[0]] - mid) >= 0:
            p0, p1, n = p1, p0, -n
        nodes_index[fi] = (p0, p1)
        normals[fi] = n
        lengths[fi] = np.hypot(*t)
        ds = [np.dot(n, cen[c] - mid) for c in cl]
        if len(cl) == 2 and ds[0] > ds[1]:
            cl, ds = cl[::-1], ds[::-1]
        for s, (c, dv) in enumerate(zip(cl, ds)):
            sci[fi, s], sd[fi, s] = c, abs(dv)
        if len(cl) == 1:
            sd[fi, 1] = sd[fi, 0]
    fi_arr = -np.ones((N, K), np.int32)
    fs_arr = -np.ones((N, K), np.int32)
    for ci in range(N):
        fi_arr[ci, :len(cell_faces[ci])] = cell_faces[ci]
        fs_arr[ci, :len(cell_faces[ci])] = [int(np.sign(np.dot(en, normals[fi])))
                                           for fi, en in zip(cell_faces[ci], cell_signs[ci])]
    pc = [[] for _ in range(P)]
    for ci, poly in enumerate(polys):
        for p in poly:
            pc[p].append(ci)
    Kn = max(len(x) for x in pc)
    pci = -np.ones((P, Kn), np.int32)
    pcd = -np.ones((P, Kn))
    for p in range(P):
        for k, c in enumerate(pc[p]):
            pci[p, k] = c
            pcd[p, k] = np.hypot(*(pts[p] - cen[c]))

    dt = 0.5 * float(lengths.min())
    dyn = D2Q9(tau=tau, delta_t=dt)
    cells = Cells(N, dyn)
    cells.face_indices = jnp.array(fi_arr, dtype=jnp.int32)
    cells.face_normals = jnp.array(fs_arr, dtype=jnp.int32)
    faces = Faces(F, dyn)
    faces.n = jnp.array(normals, dtype=jnp.float64)
    faces.L = jnp.array(lengths, dtype=jnp.float64)[..., jnp.newaxis]
    faces.nodes_index = jnp.array(nodes_index, dtype=jnp.int32)
    faces.stencil_cells_index = jnp.array(sci, dtype=jnp.int32)
    faces.stencil_dists = jnp.array(sd, dtype=jnp.float64)
    nodes = Nodes(P, dyn)
    nodes.cells_index = jnp.array(pci, dtype=jnp.int32)
    nodes.cell_dists = jnp.array(pcd, dtype=jnp.float64)
    on_b = np.array([(x[0] in (0, nx * h)) or (x[1] in (0, ny * h)) for x in pts])
    lid = np.array([x[1] == ny * h and 0 < x[0] < nx * h for x in pts])
    t = np.zeros((P, 1), np.int32)
    t[on_b] = 1
    v = np.zeros((P, 2), np.float32)
    v[lid, 0] = 0.1
    nodes.type = jnp.array(t, dtype=jnp.int32)
    nodes.vel = jnp.array(v, dtype=jnp.float32)
    return cells, faces, nodes, dt


def main(ref_path):
    _setup(ref_path)
    import meshgen as mg

    c7 = mg.cavity(n=7, seed=1)
    run_case("cavity7_upwind", c7, "upwind", 0.6, cavity_bc(), 60, {1, 2, 60})
    run_case("cavity7_lw_dm2", c7, "lax_wendroff", 0.6, cavity_bc(), 40, {1, 40},
             dim_multiplier=2, perturb=perturb_pdf(), seed=11)
    run_case("cavity7_cc_upwind", c7, "cc_upwind", 0.7, cavity_bc(), 20, {1, 20})
    run_case("cavity7_cc_lax_wendroff", c7, "cc_lax_wendroff", 0.7, cavity_bc(), 20, {1, 20})
    run_case("cavity7_cc_alt_upwind", c7, "cc_alt_upwind", 0.7, cavity_bc(), 20, {1, 20})
    ch = mg.channel_cylinder(n_target=500, seed=2)
    run_case("channel_upwind", ch, "upwind", 0.55, channel_bc(0.41), 30, {1, 30})
    run_case("channel_lw", ch, "lax_wendroff", 0.55, channel_bc(0.41), 30, {1, 30},
             perturb=perturb_pdf(0.02), seed=5)
    po = mg.porous(n_obstacles=3, n_target=800, porosity=0.9, seed=4)
    run_case("porous_frozen_upwind", po, "upwind", 0.6, porous_bc_frozen, 30, {1, 30},
             perturb=perturb_pdf(0.02), seed=7)
    run_case("mixed_quadtri_upwind", None, "upwind", 0.65, None, 30, {1, 30},
             prebuilt=mixed_quadtri, perturb=perturb_pdf(0.03), seed=3)
    c41 = mg.cavity(n=41, seed=0)
    run_case("cavity41_upwind", c41, "upwind", 0.6, cavity_bc(), 3, {1, 3})
    # D2Q13 (src/dynamics.py:77-102): 13 velocities, third-order equilibrium
    run_case("cavity7_d2q13_upwind", c7, "upwind", 0.6, cavity_bc(), 40, {1, 40}, lattice="D2Q13")
    run_case("channel_d2q13_lw", ch, "lax_wendroff", 0.55, channel_bc(0.41), 30, {1, 30},
             perturb=perturb_pdf(0.02), seed=5, lattice="D2Q13")


ONLY = set()

if __name__ == "__main__":
    # make_golden.py <reference checkout> [--only name,name]: regenerate some cases
    args = sys.argv[1:]
    if "--only" in args:
        i = args.index("--only")
        ONLY.update(args[i + 1].split(","))
        del args[i:i + 2]
    if len(args) != 1 or not os.path.isdir(os.path.join(args[0], "src")):
        sys.exit("usage: make_golden.py <path of a MADALERAU/FVDBM-JAX checkout> [--only name,name]")
    main(args[0])
