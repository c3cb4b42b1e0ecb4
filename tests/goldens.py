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


def inv_tau_dt(g):
    tau = float(g["tau"])
    dt = float(g["delta_t"])
    return np.float32(1 / tau), np.float32(dt)
