"""Ready-made cases (mesh + containers + boundary values) for tests, benches
and studies: the lid-driven cavity, the porous square and the mixed suite of
many such cases that a ``Batch`` steps together.

Each function returns ``(dynamics, cells, faces, nodes)`` as ``Mesher.to_env``
and the boundary setters (``src/mesher.py:610-742``) leave them.
"""
from __future__ import annotations

import numpy as np

from . import meshgen
from .dynamics import D2Q9
from .mesher import Mesher

LID_U = 0.1  # lid speed of the cavities; also the velocity scale of Re


def tau_from_re(re: float, u: float = LID_U, length: float = 1.0) -> float:
    """tau = 3 U L / Re + 1/2, the convention of the reference's notebooks."""
    return 3.0 * u * length / re + 0.5


def _mesher(raw):
    m = Mesher().import_meshpy(raw)
    m.calc_mesh_properties()
    return m


def lid_cavity(n: int = 41, tau: float = 0.6, flux: str = "upwind", dt_scale: float = 0.5,
               lid: float = LID_U, seed: int = 0, mesher: bool = False):
    """Unit square from an n x n jittered grid; lid (marker 3) moving at
    ``lid``, other walls at rest; dt = dt_scale * min edge."""
    m = _mesher(meshgen.cavity(n, seed=seed))
    dyn = D2Q9(tau, dt_scale * float(m.face_lengths.min()))
    c, f, nd = m.to_env(dyn, flux)
    for mk in (1, 2, 4):
        nd = m.set_vel_node(nd, mk, (0.0, 0.0))
    nd = m.set_vel_node(nd, 3, (lid, 0.0))
    return (dyn, c, f, nd, m) if mesher else (dyn, c, f, nd)


def porous_square(n_obstacles: int = 400, n_target: int = 1_000_000, tau: float = 0.6,
                  rho_in: float = 1.001, rho_out: float = 1.0, porosity: float = 0.70,
                  flux: str = "upwind", dt_scale: float = 0.5, delta_t: float | None = None,
                  seed: int = 0, mesher: bool = False):
    """Porous unit square: inlet density rho_in (left, marker 4), outlet
    rho_out (right, marker 2), no-slip walls and obstacles.  dt is ``delta_t``
    when given, else dt_scale * min edge.  When the obstacles do not fit with
    the default clearance, the clearance is reduced."""
    raw = None
    for gap in (2.5, 1.5, 1.0, 0.5):
        try:
            raw = meshgen.porous(n_obstacles=n_obstacles, n_target=n_target, porosity=porosity, seed=seed,
                                 gap_cells=gap)
            break
        except RuntimeError:
            continue
    if raw is None:
        raise RuntimeError("could not place the obstacles")
    m = _mesher(raw)
    dt = delta_t if delta_t is not None else dt_scale * float(m.face_lengths.min())
    dyn = D2Q9(tau, dt)
    c, f, nd = m.to_env(dyn, flux)
    for mk in (1, 3, 5):
        nd = m.set_vel_node(nd, mk, (0.0, 0.0))
    nd = m.set_rho_node(nd, 4, rho_in)
    nd = m.set_rho_node(nd, 2, rho_out)
    return (dyn, c, f, nd, m) if mesher else (dyn, c, f, nd)


def _make(spec):
    if spec["kind"] == "cavity":
        return lid_cavity(spec["grid"], spec["tau"], spec["flux"], seed=spec["seed"])
    return porous_square(spec["obstacles"], spec["n_target"], spec["tau"], porosity=spec["porosity"],
                         flux=spec["flux"], seed=spec["seed"])


def partition_cases(costs, n_parts: int):
    """Greedy longest-processing-time split of independent cases over
    n_parts ranks: cases in decreasing cost, each to the currently lightest
    rank.  Returns one ascending list of case indices per rank."""
    costs = np.asarray(costs, np.float64)
    load = np.zeros(n_parts)
    parts = [[] for _ in range(n_parts)]
    for i in np.argsort(-costs, kind="stable"):
        r = int(np.argmin(load))
        parts[r].append(int(i))
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def batch_suite(seed: int = 0, n_cavity: int = 128, n_porous: int = 128, flux: str = "upwind",
                cavity_cells=(2_000, 60_000), porous_cells=(10_000, 120_000), obstacles=(20, 200),
                re=(50.0, 400.0), porosity: float = 0.8, workers: int = 0, rank: int = 0, n_ranks: int = 1):
    """Independent cases of uneven size and Reynolds number: cavities with
    N uniform in ``cavity_cells`` (grid n from N = 2(n-1)^2) and porous squares
    with N uniform in ``porous_cells`` and an obstacle count uniform in
    ``obstacles``; Re uniform in ``re`` sets tau (``tau_from_re``).  Returns a
    list of (dynamics, cells, faces, nodes) and one description per case.
    ``workers`` > 0 meshes the cases in that many spawned processes (call it
    before any GPU work of the calling process).  With n_ranks > 1 only this
    rank's share (``partition_cases`` over the target cell counts) is meshed
    and returned."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_cavity):
        N = rng.uniform(*cavity_cells)
        r = float(rng.uniform(*re))
        specs.append({"kind": "cavity", "grid": int(round(np.sqrt(N / 2.0))) + 1, "re": r,
                      "tau": tau_from_re(r), "flux": flux, "seed": seed * 100_003 + i})
    for i in range(n_porous):
        N = int(rng.uniform(*porous_cells))
        k = int(rng.integers(obstacles[0], obstacles[1] + 1))
        r = float(rng.uniform(*re))
        specs.append({"kind": "porous", "obstacles": k, "n_target": N, "re": r, "tau": tau_from_re(r),
                      "porosity": porosity, "flux": flux, "seed": seed * 100_003 + n_cavity + i})
    if n_ranks > 1:
        target = [2.0 * (s["grid"] - 1) ** 2 if s["kind"] == "cavity" else s["n_target"] for s in specs]
        specs = [specs[i] for i in partition_cases(target, n_ranks)[rank]]
    if workers > 0:
        import concurrent.futures as cf
        import multiprocessing as mp
        with cf.ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
            cases = list(ex.map(_make, specs, chunksize=2))
    else:
        cases = [_make(s) for s in specs]
    desc = []
    for s, cs in zip(specs, cases):
        d = {k: v for k, v in s.items() if k in ("kind", "grid", "obstacles", "re", "tau")}
        d["cells"] = int(cs[1].pdf.shape[0])
        desc.append(d)
    return cases, desc
