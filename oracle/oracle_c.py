"""ORACLE (test infrastructure only): builds and binds ``fvdbm_oracle.c``,
the C restatement of the reference step (see that file's header).  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs use it.

``step(geo, state, inv_tau, dt, n_steps)`` takes the same ``geo``/``state``
dicts as ``oracle_np`` and returns the same result dict.  ``step64(geo,
state, tau, dt, n_steps)`` runs the same statements in float64 (the
``-DORACLE_F64`` build) and returns float64 arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fvdbm_oracle.c")
LIB = os.path.join(HERE, "_build", "libfvdbm_oracle.so")
LIB64 = os.path.join(HERE, "_build", "libfvdbm_oracle64.so")
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]

F32 = np.float32
_i32p = C.POINTER(C.c_int32)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)


class OracleMesh(C.Structure):
    _fields_ = [("N", C.c_int32), ("F", C.c_int32), ("P", C.c_int32), ("K", C.c_int32), ("Kn", C.c_int32),
                ("face_indices", _i32p), ("face_signs", _i32p), ("face_cells", _i32p),
                ("face_dists", _f32p), ("face_nodes", _i32p), ("face_n", _f32p), ("face_L", _f32p),
                ("face_scale", _f32p), ("node_type", _i32p), ("node_cells", _i32p),
                ("node_dists", _f32p), ("inv_area", _f32p),
                ("scheme", C.c_int32), ("variant", C.c_int32),
                ("inv_tau", C.c_float), ("dt", C.c_float), ("c2", C.c_float),
                ("c4x2", C.c_float), ("c2x2", C.c_float)]


class OracleMesh64(C.Structure):
    _fields_ = OracleMesh._fields_[:-5] + [("inv_tau", C.c_double), ("dt", C.c_double), ("c2", C.c_double),
                                           ("c4x2", C.c_double), ("c2x2", C.c_double)]


def _build_one(out, defines, force):
    if force or not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(SRC):
        cmd = ["gcc", *CFLAGS, *defines, SRC, "-o", out + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
        os.replace(out + ".tmp", out)
    return out


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    _build_one(LIB64, ["-DORACLE_F64"], force)
    return _build_one(LIB, [], force)


_L = None
_L64 = None


def lib():
    global _L
    if _L is None:
        L = C.CDLL(build())
        L.oracle_step.argtypes = [C.POINTER(OracleMesh), _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_int,
                                  _f32p, _f32p, _f32p, _f32p]
        L.oracle_max_threads.restype = C.c_int
        _L = L
    return _L


def lib64():
    global _L64
    if _L64 is None:
        build()
        L = C.CDLL(LIB64)
        L.oracle_step_f64.argtypes = [C.POINTER(OracleMesh64), _f64p, _f64p, _f64p, _f64p, C.c_int, C.c_int,
                                      _f64p, _f64p, _f64p, _f64p]
        _L64 = L
    return _L64


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def face_scale(geo):
    """Flux multipliers of the cell-centre stencil variants, float32
    (``src/faces.py:71-72,136-138``)."""
    v = geo.get("variant")
    if v == "cos":
        return 1, np.ascontiguousarray(np.cos(geo["face_alpha"].astype(F32)).reshape(-1), F32)
    if v == "ksi":
        ksi = np.array([[1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]], F32)
        n, npq = geo["face_n"], geo["face_npq"]
        num = ksi[None, :, 0] * n[:, None, 0] + ksi[None, :, 1] * n[:, None, 1]
        den = ksi[None, :, 0] * npq[:, None, 0] + ksi[None, :, 1] * npq[:, None, 1]
        with np.errstate(divide="ignore", invalid="ignore"):
            r = np.concatenate([np.zeros((n.shape[0], 1), F32), num / den], axis=1)
        return 2, np.ascontiguousarray(r, F32)
    return 0, None


class Prepared:
    """Contiguous arrays and the C struct for one mesh (kept alive together)."""

    def __init__(self, geo, inv_tau, dt, inv_area=None, f64=False):
        from oracle_np import C2, C4X2, C2X2
        if f64:  # inv_tau is 1/tau in double; lattice constants of C = 1/sqrt(3) in double
            c = 1.0 / np.sqrt(3.0)
            C2, C4X2, C2X2 = c * c, 2.0 * ((c * c) * (c * c)), 2.0 * (c * c)
        self.a = {
            "fi": np.ascontiguousarray(geo["face_indices"], np.int32),
            "fs": np.ascontiguousarray(geo["face_signs"], np.int32),
            "fc": np.ascontiguousarray(geo["face_cells"], np.int32),
            "fd": np.ascontiguousarray(geo["face_dists"], F32),
            "fnd": np.ascontiguousarray(geo["face_nodes"], np.int32),
            "fn": np.ascontiguousarray(geo["face_n"], F32),
            "fL": np.ascontiguousarray(np.asarray(geo["face_L"]).reshape(-1), F32),
            "nt": np.ascontiguousarray(np.asarray(geo["node_type"]).reshape(-1), np.int32),
            "nc": np.ascontiguousarray(geo["node_cells"], np.int32),
            "nd": np.ascontiguousarray(geo["node_dists"], F32),
            "ia": None if inv_area is None else np.ascontiguousarray(np.asarray(inv_area).reshape(-1), F32),
        }
        variant, scale = face_scale(geo)
        self.a["scale"] = scale
        a = self.a
        N, F, P = a["fi"].shape[0], a["fc"].shape[0], a["nt"].shape[0]
        self.N, self.F, self.P = N, F, P
        scheme = {"upwind": 0, "lax_wendroff": 1}[geo["scheme"]]
        self.m = (OracleMesh64 if f64 else OracleMesh)(N, F, P, a["fi"].shape[1], a["nc"].shape[1],
                            _p(a["fi"], _i32p), _p(a["fs"], _i32p), _p(a["fc"], _i32p), _p(a["fd"], _f32p),
                            _p(a["fnd"], _i32p), _p(a["fn"], _f32p), _p(a["fL"], _f32p),
                            _p(a["scale"], _f32p), _p(a["nt"], _i32p), _p(a["nc"], _i32p),
                            _p(a["nd"], _f32p), _p(a["ia"], _f32p), scheme, variant,
                            float(inv_tau), float(dt), float(C2), float(C4X2), float(C2X2))


def step(geo, state, inv_tau, dt, n_steps: int = 1, threads: int = 0, inv_area=None, prepared=None):
    pr = prepared or Prepared(geo, inv_tau, dt, inv_area)
    N, F, P = pr.N, pr.F, pr.P
    pdf = np.array(state["cells_pdf"], F32, order="C", copy=True)
    npdf = np.array(state["nodes_pdf"], F32, order="C", copy=True)
    nrho = np.array(np.asarray(state["nodes_rho"]).reshape(-1), F32, copy=True)
    nvel = np.array(state["nodes_vel"], F32, order="C", copy=True)
    rho, vel = np.empty(N, F32), np.empty((N, 2), F32)
    eq, fl = np.empty((N, 9), F32), np.empty((F, 9), F32)
    rc = lib().oracle_step(C.byref(pr.m), _p(pdf, _f32p), _p(npdf, _f32p), _p(nrho, _f32p), _p(nvel, _f32p),
                           int(n_steps), int(threads), _p(rho, _f32p), _p(vel, _f32p), _p(eq, _f32p),
                           _p(fl, _f32p))
    if rc != 0:
        raise MemoryError("oracle scratch allocation failed")
    return {"cells_pdf": pdf, "cells_rho": rho.reshape(N, 1), "cells_vel": vel, "cells_pdf_eq": eq,
            "faces_pdf": fl, "nodes_pdf": npdf, "nodes_rho": nrho.reshape(P, 1), "nodes_vel": nvel}


def step64(geo, state, tau, dt, n_steps: int = 1, threads: int = 0, inv_area=None, prepared=None):
    """``step`` in float64: 1/tau and dt taken in double, state promoted."""
    pr = prepared or Prepared(geo, 1.0 / float(tau), float(dt), inv_area, f64=True)
    N, F, P = pr.N, pr.F, pr.P
    D = np.float64
    pdf = np.array(state["cells_pdf"], D, order="C", copy=True)
    npdf = np.array(state["nodes_pdf"], D, order="C", copy=True)
    nrho = np.array(np.asarray(state["nodes_rho"]).reshape(-1), D, copy=True)
    nvel = np.array(state["nodes_vel"], D, order="C", copy=True)
    rho, vel = np.empty(N, D), np.empty((N, 2), D)
    eq, fl = np.empty((N, 9), D), np.empty((F, 9), D)
    rc = lib64().oracle_step_f64(C.byref(pr.m), _p(pdf, _f64p), _p(npdf, _f64p), _p(nrho, _f64p),
                                 _p(nvel, _f64p), int(n_steps), int(threads), _p(rho, _f64p), _p(vel, _f64p),
                                 _p(eq, _f64p), _p(fl, _f64p))
    if rc != 0:
        raise MemoryError("oracle scratch allocation failed")
    return {"cells_pdf": pdf, "cells_rho": rho.reshape(N, 1), "cells_vel": vel, "cells_pdf_eq": eq,
            "faces_pdf": fl, "nodes_pdf": npdf, "nodes_rho": nrho.reshape(P, 1), "nodes_vel": nvel}
