"""``Batch``: many independent FVDBM cases stepped together on one GPU.

The reference steps one ``Environment`` at a time.  A ``Batch`` joins the
cases' meshes into one device mesh (``fvdbm_batch_create``): every step is one
boundary-node launch and one cell launch for all cases, each case with its own
``tau`` and ``delta_t``; cases retire independently once their residual falls
below a threshold (or at a per-case step cap), after which their cells are
skipped.  Each case evolves bit for bit as it would in its own
``Environment``.

    b = Batch([(cells, faces, nodes), ...])    # containers from Mesher.to_env
    b.init()
    b.autotune()                               # launch shape for this size bucket
    steps, res, status = b.run_to_steady(1e-6, check_every=100, max_steps=200_000)
    st = b.case_state(3)                       # that case's pdf / rho / vel / nodes
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import time

import numpy as np

from . import _native as nat
from .containers import from_any
from .environment import pack

F32, I32 = np.float32, np.int32

# launch shapes the autotuner tries: (threads per block, L2 prefetch waves)
CANDIDATES = ((256, 1), (256, 0), (256, 2), (128, 1), (128, 0), (128, 2))
_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")


def size_bucket(n_cells: int, n_cases: int, scheme: str) -> str:
    """Key of the autotuner's decision: the total and the mean case size,
    each rounded to a power of two, and the flux scheme."""
    tot = int(round(math.log2(max(n_cells, 1))))
    per = int(round(math.log2(max(n_cells // max(n_cases, 1), 1))))
    return f"{scheme}|cells2^{tot}|case2^{per}"


class Batch:
    def __init__(self, cases, *, ordering: str = "auto", device: int = 0, finite_volume: bool = False):
        self.cases = [from_any(c, f, n) for (c, f, n) in cases]
        if not self.cases:
            raise ValueError("a batch needs at least one case")
        self.ordering, self.device = ordering, device
        self.finite_volume = finite_volume
        self._h = None
        self.config_used = None

    # ------------------------------------------------------------------
    def init(self):
        L = nat.lib()
        packs = [pack(c, f, n, ordering=self.ordering, kernel="fused", device=self.device,
                      finite_volume=self.finite_volume) for (c, f, n) in self.cases]
        S = len(packs)
        meshes = (nat.Mesh * S)(*[p[0] for p in packs])
        params = (nat.Params * S)(*[p[1] for p in packs])
        self.close()
        h = C.c_void_p()
        rc = L.fvdbm_batch_create(meshes, params, S, C.byref(h))
        if rc != 0:
            msg = L.fvdbm_last_error(None)
            msg = msg.decode() if msg else ""
            if rc == -1:
                raise ValueError(msg)
            raise nat.FvdbmError(f"fvdbm_batch_create failed ({rc}): {msg}")
        self._h = h
        dims = np.array([p[3] for p in packs], np.int64)
        self.cell_ptr = np.concatenate([[0], np.cumsum(dims[:, 0])])
        self.face_ptr = np.concatenate([[0], np.cumsum(dims[:, 1])])
        self.node_ptr = np.concatenate([[0], np.cumsum(dims[:, 2])])
        self.dynamics = [p[4] for p in packs]
        self.scheme = self.cases[0][1].flux_scheme
        # initial state: every case's dynamic leaves
        pdf = np.concatenate([np.asarray(c.pdf, F32) for c, _, _ in self.cases])
        npdf = np.concatenate([np.asarray(n.pdf, F32) for _, _, n in self.cases])
        nrho = np.concatenate([np.asarray(n.rho, F32).reshape(-1) for _, _, n in self.cases])
        nvel = np.concatenate([np.asarray(n.vel, F32).reshape(-1, 2) for _, _, n in self.cases])
        self._set_state(pdf, npdf, nrho, nvel)
        return self

    def _set_state(self, pdf, npdf, nrho, nvel):
        arrs = [None if a is None else np.ascontiguousarray(a, F32) for a in (pdf, npdf, nrho, nvel)]
        nat.check(nat.lib().fvdbm_set_state(self._h, *[nat.fptr(a) for a in arrs]), self._h)

    @property
    def n_cases(self) -> int:
        return len(self.cases)

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        inf = nat.Info()
        nat.check(nat.lib().fvdbm_get_info(self._h, C.byref(inf)), self._h)
        return {k: getattr(inf, k) for k, _ in nat.Info._fields_}

    # ------------------------------------------------------------------
    def step(self, n_steps: int = 1):
        nat.check(nat.lib().fvdbm_step(self._h, int(n_steps)), self._h)
        return self

    def sync(self):
        nat.check(nat.lib().fvdbm_sync(self._h), self._h)
        return self

    def residual(self, take=None):
        """Per-case (res_u, mass) in double (``fvdbm_batch_residual``); with
        ``take`` (a mask over the cases) only those cases are measured and
        re-snapshotted (``fvdbm_batch_residual_cases``), the others read NaN."""
        S = self.n_cases
        r, m = np.full(S, np.nan), np.full(S, np.nan)
        if take is None:
            nat.check(nat.lib().fvdbm_batch_residual(self._h, r.ctypes.data_as(C.POINTER(C.c_double)),
                                                     m.ctypes.data_as(C.POINTER(C.c_double))), self._h)
        else:
            t = np.ascontiguousarray(np.asarray(take, np.int32).reshape(S))
            nat.check(nat.lib().fvdbm_batch_residual_cases(self._h, nat.iptr(t),
                                                           r.ctypes.data_as(C.POINTER(C.c_double)),
                                                           m.ctypes.data_as(C.POINTER(C.c_double))), self._h)
        return r, m

    def set_cells_eq(self, rho, vel):
        """Every cell's pdf = feq(rho, u) (union arrays rho [N], vel [N,2])."""
        r = np.ascontiguousarray(np.asarray(rho, F32).reshape(-1))
        v = np.ascontiguousarray(np.asarray(vel, F32).reshape(-1, 2))
        nat.check(nat.lib().fvdbm_set_cells_eq(self._h, nat.fptr(r), nat.fptr(v)), self._h)

    def set_case_pdf(self, s: int, pdf):
        """Replace case s's cell pdfs (the other cases keep their state)."""
        st = self.state()
        c0, c1 = int(self.cell_ptr[s]), int(self.cell_ptr[s + 1])
        st["pdf"][c0:c1] = np.asarray(pdf, F32).reshape(c1 - c0, 9)
        self._set_state(st["pdf"], None, None, None)

    def set_active(self, active):
        a = np.ascontiguousarray(np.asarray(active, np.int32).reshape(self.n_cases))
        nat.check(nat.lib().fvdbm_batch_set_active(self._h, nat.iptr(a)), self._h)

    def run_to_steady(self, threshold: float = 1e-6, check_every: int = 100, max_steps=1_000_000,
                      check_time: float = 0.0):
        """Step until every case's residual is below ``threshold`` (or NaN,
        or its step cap).  Returns per-case (steps, res_u, status) with status
        1 = converged (below the threshold, or an exact float32 fixed point
        reached from a residual below 100 x threshold), 0 = step cap, 2 =
        non-finite, 3 = frozen (residual exactly 0 far from convergence),
        4 = stalled (no new residual minimum in 50 checks).  ``check_time`` > 0
        takes each case's residual over a window of at least that much of its
        own time (``fvdbm_batch_run_to_steady_time``)."""
        S = self.n_cases
        cap = np.ascontiguousarray(np.broadcast_to(np.asarray(max_steps, np.int64), (S,)))
        steps, res, status = np.empty(S, np.int64), np.empty(S, np.float64), np.empty(S, np.int32)
        nat.check(nat.lib().fvdbm_batch_run_to_steady_time(
            self._h, float(threshold), int(check_every), float(check_time), cap.ctypes.data_as(C.POINTER(C.c_int64)),
            steps.ctypes.data_as(C.POINTER(C.c_int64)), res.ctypes.data_as(C.POINTER(C.c_double)),
            nat.iptr(status)), self._h)
        return steps, res, status

    # ------------------------------------------------------------------
    def state(self) -> dict:
        """Union read-back (cases in order), as ``Environment`` exposes it."""
        L = nat.lib()
        N, P = int(self.cell_ptr[-1]), int(self.node_ptr[-1])
        out = {"pdf": np.empty((N, 9), F32), "rho": np.empty(N, F32), "vel": np.empty((N, 2), F32),
               "pdf_eq": np.empty((N, 9), F32), "node_pdf": np.empty((P, 9), F32),
               "node_rho": np.empty(P, F32), "node_vel": np.empty((P, 2), F32)}
        nat.check(L.fvdbm_get_cells(self._h, nat.fptr(out["pdf"]), nat.fptr(out["rho"]), nat.fptr(out["vel"]),
                                    nat.fptr(out["pdf_eq"])), self._h)
        nat.check(L.fvdbm_get_nodes(self._h, nat.fptr(out["node_pdf"]), nat.fptr(out["node_rho"]),
                                    nat.fptr(out["node_vel"])), self._h)
        return out

    def case_state(self, s: int, state: dict | None = None) -> dict:
        st = state if state is not None else self.state()
        c0, c1 = int(self.cell_ptr[s]), int(self.cell_ptr[s + 1])
        n0, n1 = int(self.node_ptr[s]), int(self.node_ptr[s + 1])
        return {k: (v[n0:n1] if k.startswith("node_") else v[c0:c1]) for k, v in st.items()}

    # ------------------------------------------------------------------
    def config(self, block: int, prefetch_waves: int):
        nat.check(nat.lib().fvdbm_batch_config(self._h, int(block), int(prefetch_waves)), self._h)
        self.config_used = (int(block), int(prefetch_waves))

    def autotune(self, steps: int = 64, candidates=CANDIDATES, use_cache: bool = True) -> dict:
        """Pick the cell kernel's launch shape for this batch's size bucket by
        timing each candidate for ``steps`` steps (the state is saved and
        restored around the trials).  Decisions are cached per GPU model and
        size bucket."""
        key = f"{_device_name(self.device)}|{size_bucket(int(self.cell_ptr[-1]), self.n_cases, self.scheme)}"
        cache = _load_cache() if use_cache else {}
        if key in cache:
            b, w = cache[key]["best"]
            self.config(b, w)
            return cache[key]
        st = self.state()
        times = {}
        for b, w in candidates:
            self.config(b, w)
            self.step(steps // 2).sync()  # warm (graph capture)
            t0 = time.perf_counter()
            self.step(steps).sync()
            times[f"{b}x{w}"] = (time.perf_counter() - t0) / steps
        best = min(times, key=times.get)
        b, w = (int(x) for x in best.split("x"))
        self.config(b, w)
        self._set_state(st["pdf"], st["node_pdf"], st["node_rho"], st["node_vel"])
        rec = {"best": [b, w], "sec_per_step": times}
        if use_cache:
            cache[key] = rec
            _save_cache(cache)
        return rec

    def close(self):
        if getattr(self, "_h", None) is not None:
            nat.lib().fvdbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _device_name(device: int) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return f"cuda:{device}"


def _load_cache() -> dict:
    try:
        with open(_CACHE) as fh:
            return json.load(fh)
    except Exception:
        return {}


def _save_cache(cache: dict):
    try:
        os.makedirs(os.path.dirname(_CACHE), exist_ok=True)
        with open(_CACHE + ".tmp", "w") as fh:
            json.dump(cache, fh, indent=1)
        os.replace(_CACHE + ".tmp", _CACHE)
    except OSError:
        pass
