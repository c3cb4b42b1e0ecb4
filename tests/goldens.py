"""Loading helpers for the golden vectors in ``tests/golden`` (produced by
``tests/golden/make_golden.py`` from the reference's own code)."""
from __future__ import annotations

import glob
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

SCHEMES = {
    "upwind": ("upwind", None),
    "lax_wendroff": ("lax_wendroff", None),
    "cc_upwind": ("upwind", "cos"),
    "cc_lax_wendroff": ("lax_wendroff", "cos"),
    "cc_alt_upwind": ("upwind", "ksi"),
}


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    return {k: z[k] for k in z.files}


def geo(g):
    scheme, variant = SCHEMES[str(g["flux_method"])]
    out = {
        "face_indices": g["c_face_indices"].astype(np.int32),
        "face_signs": g["c_face_normals"].astype(np.int32),
        "face_cells": g["f_stencil_cells_index"].astype(np.int32),
        "face_dists": g["f_stencil_dists"].astype(np.float32),
        "face_nodes": g["f_nodes_index"].astype(np.int32),
        "face_n": g["f_n"].astype(np.float32),
        "face_L": g["f_L"].astype(np.float32).reshape(-1, 1),
        "scheme": scheme,
        "variant": variant,
        "node_type": g["n_type"].astype(np.int32).reshape(-1, 1),
        "node_cells": g["n_cells_index"].astype(np.int32),
        "node_dists": g["n_cell_dists"].astype(np.float32),
    }
    if variant == "cos":
        out["face_alpha"] = g["f_alpha"].astype(np.float32).reshape(-1, 1)
    if variant == "ksi":
        out["face_npq"] = g["f_npq"].astype(np.float32).reshape(-1, 2)
    return out


def state(g, step=0):
    p = f"s{step}_"
    return {"cells_pdf": g[p + "c_pdf"], "nodes_pdf": g[p + "n_pdf"],
            "nodes_rho": g[p + "n_rho"].reshape(-1, 1), "nodes_vel": g[p + "n_vel"].reshape(-1, 2)}


def expected(g, step):
    p = f"s{step}_"
    return {"cells_pdf": g[p + "c_pdf"], "cells_rho": g[p + "c_rho"], "cells_vel": g[p + "c_vel"],
            "cells_pdf_eq": g[p + "c_pdf_eq"], "faces_pdf": g[p + "f_pdf"],
            "nodes_pdf": g[p + "n_pdf"], "nodes_rho": g[p + "n_rho"], "nodes_vel": g[p + "n_vel"]}


def lattice(g) -> int:
    """Velocities of a golden case's lattice (9 when not recorded)."""
    return int(g["lattice"]) if "lattice" in g else 9


def inv_tau_dt(g):
    tau = float(g["tau"])
    dt = float(g["delta_t"])
    return np.float32(1 / tau), np.float32(dt)


def containers(g):
    """Host containers (this package's) holding a golden case's reference
    containers and initial state."""
    from fvdbm_jax_gb300.containers import Cells, Faces, Nodes
    from fvdbm_jax_gb300.dynamics import D2Q9, D2Q13

    scheme, variant = SCHEMES[str(g["flux_method"])]
    lat = D2Q13 if lattice(g) == 13 else D2Q9
    dyn = lat(float(g["tau"]), float(g["delta_t"]))
    N, F, P = g["s0_c_pdf"].shape[0], g["s0_f_pdf"].shape[0], g["s0_n_pdf"].shape[0]
    c = Cells(N, dyn)
    c.face_indices = g["c_face_indices"].astype(np.int32)
    c.face_normals = g["c_face_normals"].astype(np.int32)
    c.pdf, c.rho, c.vel, c.pdf_eq = g["s0_c_pdf"], g["s0_c_rho"], g["s0_c_vel"], g["s0_c_pdf_eq"]
    f = Faces(F, dyn, scheme)
    f.pdf = g["s0_f_pdf"]
    f.stencil_cells_index = g["f_stencil_cells_index"].astype(np.int32)
    f.stencil_dists = g["f_stencil_dists"].astype(np.float32)
    f.nodes_index = g["f_nodes_index"].astype(np.int32)
    f.n = g["f_n"].astype(np.float32)
    f.L = g["f_L"].astype(np.float32).reshape(-1, 1)
    f.stencil_variant = variant
    if variant == "cos":
        f.alpha = g["f_alpha"].astype(np.float32).reshape(-1, 1)
    if variant == "ksi":
        f.npq = g["f_npq"].astype(np.float32).reshape(-1, 2)
    n = Nodes(P, dyn)
    n.pdf, n.rho, n.vel = g["s0_n_pdf"], g["s0_n_rho"], g["s0_n_vel"]
    n.type = g["n_type"].astype(np.int32).reshape(-1, 1)
    n.cells_index = g["n_cells_index"].astype(np.int32)
    n.cell_dists = g["n_cell_dists"].astype(np.float32)
    return c, f, n


def env_state(env):
    """The reference-visible state of an Environment as a flat dict."""
    return {"cells_pdf": np.array(env.cells.pdf), "cells_rho": np.array(env.cells.rho),
            "cells_vel": np.array(env.cells.vel), "cells_pdf_eq": np.array(env.cells.pdf_eq),
            "faces_pdf": np.array(env.faces.pdf), "nodes_pdf": np.array(env.nodes.pdf),
            "nodes_rho": np.array(env.nodes.rho), "nodes_vel": np.array(env.nodes.vel)}


def quad_grid(nx=12, ny=10, h=0.1, tau=0.6, lid=0.1, lattice=9, seed=0):
    """A structured grid of nx*ny square cells built directly as containers,
    as the reference's ``tests/ldcFVDBM.ipynb`` builds its quad meshes (its
    Mesher makes triangles only): four face slots per cell, every slot a face
    of its cell.  Reference conventions: slot 0 of a face is the cell on its
    -n side; a boundary face has its owner in slot 0, -1 in slot 1 and an
    outward n, with the ghost distance mirrored; face_normals is +1 where n
    points out of the cell; node stencils are the cells sharing the point at
    their centroid distance, padded with -1.  Lid-driven cavity: every
    boundary point is a velocity node, the lid's (corners excluded) moving
    at (lid, 0).  Cell pdfs start at W perturbed by 5 %."""
    from fvdbm_jax_gb300.containers import Cells, Faces, Nodes
    from fvdbm_jax_gb300.dynamics import D2Q9, D2Q13

    P = (nx + 1) * (ny + 1)
    pts = np.array([[i * h, j * h] for j in range(ny + 1) for i in range(nx + 1)], np.float64)
    polys = [[j * (nx + 1) + i, j * (nx + 1) + i + 1, (j + 1) * (nx + 1) + i + 1, (j + 1) * (nx + 1) + i]
             for j in range(ny) for i in range(nx)]
    N = len(polys)
    cen = np.array([pts[p].mean(axis=0) for p in polys])
    edges, fl, cell_faces = {}, [], []
    for ci, poly in enumerate(polys):
        cf = []
        for k in range(4):
            p0, p1 = poly[k], poly[(k + 1) % 4]
            key = (min(p0, p1), max(p0, p1))
            if key not in edges:
                edges[key] = len(fl)
                fl.append([p0, p1, []])
            fl[edges[key]][2].append(ci)
            cf.append(edges[key])
        cell_faces.append(cf)
    F = len(fl)
    dyn = (D2Q9 if lattice == 9 else D2Q13)(tau, 0.5 * h)
    fn, fL = np.zeros((F, 2)), np.zeros(F)
    sc, sd, fnodes = -np.ones((F, 2), np.int64), -np.ones((F, 2)), np.zeros((F, 2), np.int64)
    for fi, (p0, p1, cs) in enumerate(fl):
        t = pts[p1] - pts[p0]
        L = float(np.hypot(*t))
        n = np.array([-t[1], t[0]]) / L
        mid = 0.5 * (pts[p0] + pts[p1])
        c0 = cs[0]
        if len(cs) == 1:
            if np.dot(n, cen[c0] - mid) > 0:
                n = -n
            d = abs(np.dot(cen[c0] - mid, n))
            sc[fi], sd[fi] = [c0, -1], [d, d]
        else:
            c1 = cs[1]
            if np.dot(n, cen[c0] - mid) > 0:
                c0, c1 = c1, c0
            sc[fi] = [c0, c1]
            sd[fi] = [abs(np.dot(cen[c0] - mid, n)), abs(np.dot(cen[c1] - mid, n))]
        fn[fi], fL[fi], fnodes[fi] = n, L, [p0, p1]
    signs = [[1 if sc[f_, 0] == ci else -1 for f_ in cf] for ci, cf in enumerate(cell_faces)]
    c = Cells(N, dyn)
    c.face_indices = np.array(cell_faces, np.int32)
    c.face_normals = np.array(signs, np.int32)
    rng = np.random.default_rng(seed)
    pdf = np.asarray(c.pdf, np.float32)
    c.pdf = (pdf * (1.0 + 0.05 * rng.standard_normal(pdf.shape))).astype(np.float32)
    f = Faces(F, dyn, "upwind")
    f.stencil_cells_index = sc.astype(np.int32)
    f.stencil_dists = sd.astype(np.float32)
    f.nodes_index = fnodes.astype(np.int32)
    f.n = fn.astype(np.float32)
    f.L = fL.reshape(-1, 1).astype(np.float32)
    pc = [[] for _ in range(P)]
    for ci, poly in enumerate(polys):
        for p_ in poly:
            pc[p_].append(ci)
    cidx, cdist = -np.ones((P, 4), np.int32), -np.ones((P, 4), np.float32)
    for p_ in range(P):
        for k, ci in enumerate(pc[p_]):
            cidx[p_, k] = ci
            cdist[p_, k] = np.float32(np.hypot(*(pts[p_] - cen[ci])))
    ix, iy = np.arange(P) % (nx + 1), np.arange(P) // (nx + 1)
    boundary = (ix == 0) | (ix == nx) | (iy == 0) | (iy == ny)
    lidpts = (iy == ny) & (ix > 0) & (ix < nx)
    nd = Nodes(P, dyn)
    typ = np.zeros((P, 1), np.int32)
    typ[boundary] = 1
    nd.type = typ
    vel = np.zeros((P, 2), np.float32)
    vel[lidpts, 0] = lid
    nd.vel = vel
    nd.cells_index, nd.cell_dists = cidx, cdist
    return c, f, nd, dyn
