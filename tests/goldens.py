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
