"""ORACLE (test infrastructure only).  A vectorised numpy restatement of the
reference's FVDBM time step, used as the checker for the CUDA path.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import it; the product never does.

Parity status: pinned.  ``tests/golden/`` holds states produced by running the
reference's own ``src/containers.py``/``src/dynamics.py``/``src/environment.py``
(under a numpy stand-in for jax, see ``tests/golden/refshim``); this module
reproduces them bit for bit.

It consumes the reference's container layout (``Mesher.to_env`` output):

    geo["face_indices"]   [N,K] int32   Cells.face_indices
    geo["face_signs"]     [N,K] int32   Cells.face_normals
    geo["face_cells"]     [F,2] int32   Faces.stencil_cells_index
    geo["face_dists"]     [F,2] f32     Faces.stencil_dists
    geo["face_nodes"]     [F,2] int32   Faces.nodes_index
    geo["face_n"]         [F,2] f32     Faces.n
    geo["face_L"]         [F,1] f32     Faces.L
    geo["scheme"]         "upwind" | "lax_wendroff"
    geo["variant"]        None | "cos" (Faces.alpha) | "ksi" (Faces.npq)
    geo["node_type"]      [P,1] int32   Nodes.type
    geo["node_cells"]     [P,Kn] int32  Nodes.cells_index
    geo["node_dists"]     [P,Kn] f32    Nodes.cell_dists

and the dynamic state ``cells_pdf [N,9]``, ``nodes_pdf [P,9]``,
``nodes_rho [P,1]``, ``nodes_vel [P,2]``.

Arithmetic is float32 throughout, in the reference's operation order.  Sums
that the reference writes as ``jnp.sum``/``jnp.dot``/``jnp.mean`` are
sequential left folds (index 0 first), the order the golden vectors fix.
Negative gather indices wrap to the last row, as JAX indexing does.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32
KSI = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1],
                [1, 1], [-1, 1], [-1, -1], [1, -1]], dtype=np.int32)
KSI_F = KSI.astype(F32)
W = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36], dtype=F32)
C = F32(1) / np.sqrt(F32(3))
C2 = F32(C * C)
C4X2 = F32(F32(2) * F32(C2 * C2))
C2X2 = F32(F32(2) * C2)

# D2Q13 (src/dynamics.py:77-102): C = 1/sqrt(2); the powers of C as jax's
# integer_pow forms them (C**4 = (C*C)*(C*C), C**6 = (C*C)*((C*C)*(C*C)))
KSI13 = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1],
                  [2, 0], [0, 2], [-2, 0], [0, -2]], dtype=np.int32)
KSI13_F = KSI13.astype(F32)
W13 = np.array([3 / 8, 1 / 12, 1 / 12, 1 / 12, 1 / 12, 1 / 16, 1 / 16, 1 / 16, 1 / 16,
                1 / 96, 1 / 96, 1 / 96, 1 / 96], dtype=F32)
C13 = F32(1) / np.sqrt(F32(2))
C13_2 = F32(C13 * C13)
C13_4 = F32(C13_2 * C13_2)
C13_4X2 = F32(F32(2) * C13_4)
C13_2X2 = F32(F32(2) * C13_2)
C13_6X2 = F32(F32(2) * F32(C13_2 * C13_4))


def ksi(q: int) -> np.ndarray:
    """Lattice velocities (float32) of the 9- or 13-velocity lattice."""
    return KSI_F if q == 9 else KSI13_F


def _fold(x: np.ndarray, axis: int) -> np.ndarray:
    x = np.moveaxis(x, axis, 0)
    acc = x[0].copy()
    for i in range(1, x.shape[0]):
        acc = acc + x[i]
    return acc


def calc_macro(pdf: np.ndarray):
    """rho = sum_q f_q (``src/dynamics.py:35-37``); u = (KSI^T f)/rho
    (``:39-41``).  pdf [M,9] -> rho [M,1], vel [M,2]."""
    rho = _fold(pdf, 1)[:, None]
    K = ksi(pdf.shape[1])
    num = _fold(K.T[None, :, :] * pdf[:, None, :], 2)          # [M,2]
    return rho, num / rho


def calc_eq(rho: np.ndarray, vel: np.ndarray, q: int = 9) -> np.ndarray:
    """Equilibrium.  D2Q9 (``src/dynamics.py:70-74``): ``(W*rho)*(((1 +
    a/C^2) + a^2/(2C^4)) - u.u/(2C^2))``, a = KSI.u folded over x then y.
    D2Q13 (``:97-98``) adds ``+ a^3/(2C^6) - 3 a u.u/(2C^4)`` in that order,
    with a^3 = a*(a*a) as jax's integer_pow forms it."""
    a = _fold(ksi(q)[None, :, :] * vel[:, None, :], 2)         # [M,Q]
    uu = _fold(vel * vel, 1)[:, None]                          # [M,1]
    if q == 9:
        inner = ((1 + a / C2) + (a * a) / C4X2) - uu / C2X2
        return (W * rho) * inner
    a3 = a * (a * a)
    inner = ((((1 + a / C13_2) + (a * a) / C13_4X2) - uu / C13_2X2) + a3 / C13_6X2) - ((3 * a) * uu) / C13_4X2
    return (W13 * rho) * inner


def _idw(x: np.ndarray, w: np.ndarray, sumw: np.ndarray) -> np.ndarray:
    """weighted_avg (``utils/utils.py:34-45``): fold_k(x_k*w_k) / fold_k(w_k).
    x [P,K,D], w [P,K], sumw [P,1]."""
    return _fold(x * w[:, :, None], 1) / sumw


def node_pdfs(geo, cells_pdf, cells_eq, cells_rho, cells_vel, nodes_pdf, nodes_rho, nodes_vel):
    """``Nodes.calc_pdfs`` (``src/containers.py:339-404``): velocity nodes
    (type 1) take rho by IDW of cell rho; density nodes (type 2) take u by IDW
    of cell u; both set pdf = feq(rho, u) + IDW(f - feq) of their cells.
    IDW weights are 1/d with negative weights zeroed (``utils/utils.py:47-60``).
    Type-0 nodes keep their state."""
    idx = geo["node_cells"]
    d = geo["node_dists"]
    t = geo["node_type"]
    w = F32(1.0) / d
    w = np.where(w < 0, F32(0), w).astype(F32)
    sumw = _fold(w[:, :, None], 1)                             # [P,1]
    rho_ext = _idw(cells_rho[idx], w, sumw)                    # [P,1]
    vel_ext = _idw(cells_vel[idx], w, sumw)                    # [P,2]
    neq_k = np.where((idx == -1)[:, :, None], F32(0), cells_pdf[idx] - cells_eq[idx])
    neq = _idw(neq_k.astype(F32), w, sumw)                     # [P,9]

    q = cells_pdf.shape[1]
    rho = np.where(t == 1, rho_ext, nodes_rho).astype(F32)
    pdf = np.where(t == 1, calc_eq(rho, nodes_vel, q) + neq, nodes_pdf).astype(F32)
    vel = np.where(t == 2, vel_ext, nodes_vel).astype(F32)
    pdf = np.where(t == 2, calc_eq(rho, vel, q) + neq, pdf).astype(F32)
    return pdf, rho, vel


def face_fluxes(geo, cells_pdf, nodes_pdf, dt: F32) -> np.ndarray:
    """``Faces.calc_fluxes`` (``src/containers.py:191-278``) with the ghost of
    ``calc_ghost``/``extrap_pdf`` (``:280-287``, ``utils/utils.py:153-154``)
    and the cell-centre stencil multipliers (``src/faces.py:54-74,119-141``).
    ``dt`` is float32(delta_t), used by Lax-Wendroff."""
    sc = geo["face_cells"]
    d = geo["face_dists"]
    nd = geo["face_nodes"]
    n = geo["face_n"]
    L = geo["face_L"]
    s0, s1 = sc[:, 0], sc[:, 1]
    d0, d1 = d[:, 0:1], d[:, 1:2]
    m = (nodes_pdf[nd[:, 0]] + nodes_pdf[nd[:, 1]]) / F32(2)
    ghost_l = m + (m - cells_pdf[s1]) * (d0 / d1)
    ghost_r = m + (m - cells_pdf[s0]) * (d1 / d0)
    left = np.where((s0 == -1)[:, None], ghost_l, cells_pdf[s0])
    right = np.where((s1 == -1)[:, None], ghost_r, cells_pdf[s1])
    v = _fold(ksi(cells_pdf.shape[1])[None, :, :] * n[:, None, :], 2)  # [F,Q]
    if geo["scheme"] == "upwind":
        phi = np.where(v >= 0, left, right)
    elif geo["scheme"] == "lax_wendroff":
        D = d0 + d1
        interp = (d0 / D) - (v * dt) / (F32(2) * D)
        phi = left + (right - left) * interp
    else:
        raise ValueError(f"Unknown flux scheme: {geo['scheme']}")
    flux = (phi * v) * L
    variant = geo.get("variant")
    if variant == "cos":
        flux = flux * np.cos(geo["face_alpha"].astype(F32))
    elif variant == "ksi":
        npq = geo["face_npq"]
        num = _fold(KSI_F[None, 1:, :] * n[:, None, :], 2)
        den = _fold(KSI_F[None, 1:, :] * npq[:, None, :], 2)
        with np.errstate(divide="ignore", invalid="ignore"):
            ratio = np.concatenate([np.zeros_like(n[:, 0:1]), num / den], axis=1)
        flux = flux * ratio
    return flux.astype(F32)


def cell_update(geo, cells_pdf, cells_eq, fluxes, inv_tau: F32, dt: F32, inv_area=None) -> np.ndarray:
    """``Cells.calc_pdf`` (``src/containers.py:115-121``): f + dt*((1/tau)
    (feq - f) - sum_k sigma_k F_k), summed over the cell's faces in stored
    order.  No division by area (parity mode).  ``inv_area`` [N,1] switches
    on the finite-volume scaling ``sum_k sigma_k F_k * (1/A)``."""
    fi = geo["face_indices"]
    sg = geo["face_signs"].astype(F32)
    flux = _fold(fluxes[fi] * sg[:, :, None], 1)               # [N,9]
    if inv_area is not None:
        flux = flux * inv_area
    return (cells_pdf + dt * (inv_tau * (cells_eq - cells_pdf) - flux)).astype(F32)


def step(geo, state, inv_tau: F32, dt: F32, inv_area=None):
    """One ``Environment.step`` (``src/environment.py:55-65``).  Returns the
    new state dict; ``cells_rho/vel/pdf_eq`` and ``faces_pdf`` are those of
    the pre-update pdf, as the reference leaves them."""
    f = state["cells_pdf"]
    rho, vel = calc_macro(f)
    eq = calc_eq(rho, vel, f.shape[1])
    npdf, nrho, nvel = node_pdfs(geo, f, eq, rho, vel, state["nodes_pdf"],
                                 state["nodes_rho"], state["nodes_vel"])
    fl = face_fluxes(geo, f, npdf, dt)
    fnew = cell_update(geo, f, eq, fl, inv_tau, dt, inv_area)
    return {"cells_pdf": fnew, "cells_rho": rho, "cells_vel": vel, "cells_pdf_eq": eq,
            "nodes_pdf": npdf, "nodes_rho": nrho, "nodes_vel": nvel, "faces_pdf": fl}


def geo_from_containers(cells, faces, nodes) -> dict:
    """Reference-layout arrays from any container triple with the
    reference's attribute names."""
    g = {
        "face_indices": np.asarray(cells.face_indices, dtype=np.int32),
        "face_signs": np.asarray(cells.face_normals, dtype=np.int32),
        "face_cells": np.asarray(faces.stencil_cells_index, dtype=np.int32),
        "face_dists": np.asarray(faces.stencil_dists, dtype=F32),
        "face_nodes": np.asarray(faces.nodes_index, dtype=np.int32),
        "face_n": np.asarray(faces.n, dtype=F32),
        "face_L": np.asarray(faces.L, dtype=F32).reshape(-1, 1),
        "scheme": faces.flux_scheme,
        "variant": getattr(faces, "stencil_variant", None),
        "node_type": np.asarray(nodes.type, dtype=np.int32).reshape(-1, 1),
        "node_cells": np.asarray(nodes.cells_index, dtype=np.int32),
        "node_dists": np.asarray(nodes.cell_dists, dtype=F32),
    }
    cls = type(faces).__name__
    if g["variant"] is None and cls == "CCStencilFaces":
        g["variant"] = "cos"
    if g["variant"] is None and cls == "CCStencilKsiFaces":
        g["variant"] = "ksi"
    if g["variant"] == "cos":
        g["face_alpha"] = np.asarray(faces.alpha, dtype=F32).reshape(-1, 1)
    if g["variant"] == "ksi":
        g["face_npq"] = np.asarray(faces.npq, dtype=F32).reshape(-1, 2)
    return g


def state_from_containers(cells, nodes) -> dict:
    return {"cells_pdf": np.array(cells.pdf, dtype=F32),
            "nodes_pdf": np.array(nodes.pdf, dtype=F32),
            "nodes_rho": np.array(nodes.rho, dtype=F32).reshape(-1, 1),
            "nodes_vel": np.array(nodes.vel, dtype=F32).reshape(-1, 2)}
