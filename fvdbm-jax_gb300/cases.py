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


def tau_from_re(re: float, u: float = LID_U, length: float = 1.0, rule: str = "notebook") -> float:
    """tau from the Reynolds number.  ``notebook``: tau = 3 U L / Re + 1/2,
    the lattice-Boltzmann convention of the reference's notebooks
    (tests/flow_over_cyl.ipynb:216).  ``dbm``: tau = 3 U L / Re, the
    viscosity nu = c_s^2 tau of the discrete Boltzmann equation that the
    finite-volume scaled update integrates (no streaming correction)."""
    if rule == "dbm":
        return 3.0 * u * length / re
    return 3.0 * u * length / re + 0.5


def _mesher(raw, scale: float = 1.0):
    """Mesher of a raw mesh whose coordinates are multiplied by ``scale``."""
    if scale != 1.0:
        raw.points = np.asarray(raw.points, np.float64) * float(scale)
    m = Mesher().import_meshpy(raw)
    m.calc_mesh_properties()
    return m


def cavity_lattice_scale(n: int) -> float:
    """Scale that puts the n x n cavity grid at spacing 1 (lattice units: the
    domain side is n - 1)."""
    return float(n - 1)


def porous_lattice_scale(n_target: int, porosity: float) -> float:
    """Scale that puts the porous square's mesh spacing (``meshgen.porous``)
    at about 1 (lattice units: the domain side is the scale)."""
    return float(1.0 / np.sqrt(4.0 * porosity / (np.sqrt(3.0) * n_target)))


def fv_stable_dt(m, factor: float = 1.0) -> float:
    """Time step of the finite-volume scaled update (flux sum / area):
    factor * min over cells of area / perimeter.  With |xi| <= sqrt(2) the
    explicit upwind update stays stable for factor up to about 2 on these
    meshes (measured: 2.1 stable, 2.6 diverged); 1.0 keeps a margin."""
    per = np.asarray(m.face_lengths, np.float64)[np.asarray(m.cell_face_indices)].sum(axis=1)
    return float(factor * np.min(np.asarray(m.cell_areas, np.float64) / per))


def _dt(m, dt_scale, delta_t, fv_dt, tau=None):
    """delta_t when given; else fv_stable_dt(m, fv_dt), at most tau (the
    explicit relaxation then moves at most the whole way to equilibrium);
    else dt_scale * min edge."""
    if delta_t is not None:
        return delta_t
    if fv_dt is not None:
        dt = fv_stable_dt(m, fv_dt)
        return min(dt, tau) if tau is not None else dt
    return dt_scale * float(m.face_lengths.min())


def lid_cavity(n: int = 41, tau: float = 0.6, flux: str = "upwind", dt_scale: float = 0.5,
               lid: float = LID_U, seed: int = 0, mesher: bool = False, fv_dt: float | None = None,
               scale: float = 1.0):
    """Unit square from an n x n jittered grid (side ``scale``); lid (marker
    3) moving at ``lid``, other walls at rest; dt = dt_scale * min edge, or
    ``fv_stable_dt(m, fv_dt)`` when fv_dt is given (finite-volume mode)."""
    m = _mesher(meshgen.cavity(n, seed=seed), scale)
    dyn = D2Q9(tau, _dt(m, dt_scale, None, fv_dt, tau))
    c, f, nd = m.to_env(dyn, flux)
    for mk in (1, 2, 4):
        nd = m.set_vel_node(nd, mk, (0.0, 0.0))
    nd = m.set_vel_node(nd, 3, (lid, 0.0))
    return (dyn, c, f, nd, m) if mesher else (dyn, c, f, nd)


def porous_square(n_obstacles: int = 400, n_target: int = 1_000_000, tau: float = 0.6,
                  rho_in: float = 1.001, rho_out: float = 1.0, porosity: float = 0.70,
                  flux: str = "upwind", dt_scale: float = 0.5, delta_t: float | None = None,
                  seed: int = 0, mesher: bool = False, fv_dt: float | None = None, scale: float = 1.0):
    """Porous unit square (side ``scale``): inlet density rho_in (left, marker 4), outlet
    rho_out (right, marker 2), no-slip walls and obstacles.  dt is ``delta_t``
    when given, else ``fv_stable_dt(m, fv_dt)`` when fv_dt is given, else
    dt_scale * min edge.  When the obstacles do not fit with the default
    clearance, the clearance is reduced."""
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
    m = _mesher(raw, scale)
    dyn = D2Q9(tau, _dt(m, dt_scale, delta_t, fv_dt, tau))
    c, f, nd = m.to_env(dyn, flux)
    for mk in (1, 3, 5):
        nd = m.set_vel_node(nd, mk, (0.0, 0.0))
    nd = m.set_rho_node(nd, 4, rho_in)
    nd = m.set_rho_node(nd, 2, rho_out)
    return (dyn, c, f, nd, m) if mesher else (dyn, c, f, nd)


def _make(spec):
    fv = spec.get("fv_dt")
    sc = spec.get("scale", 1.0)
    if spec["kind"] == "cavity":
        return lid_cavity(spec["grid"], spec["tau"], spec["flux"], seed=spec["seed"], fv_dt=fv, scale=sc)
    return porous_square(spec["obstacles"], spec["n_target"], spec["tau"], porosity=spec["porosity"],
                         flux=spec["flux"], seed=spec["seed"], fv_dt=fv,
                         rho_in=spec.get("rho_in", 1.001), rho_out=spec.get("rho_out", 1.0), scale=sc)


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
                re=(50.0, 400.0), porosity: float = 0.8, workers: int = 0, rank: int = 0, n_ranks: int = 1,
                fv_dt: float | None = None, rho_in: float = 1.001, rho_out: float = 1.0,
                tau_rule: str = "notebook", units: str = "unit"):
    """Independent cases of uneven size and Reynolds number: cavities with
    N uniform in ``cavity_cells`` (grid n from N = 2(n-1)^2) and porous squares
    with N uniform in ``porous_cells`` and an obstacle count uniform in
    ``obstacles``; Re uniform in ``re`` sets tau (``tau_from_re``).  Returns a
    list of (dynamics, cells, faces, nodes) and one description per case.
    ``workers`` > 0 meshes the cases in that many spawned processes (call it
    before any GPU work of the calling process).  With n_ranks > 1 only this
    rank's share (``partition_cases`` over the target cell counts) is meshed
    and returned.  ``fv_dt`` sets every case's dt to ``fv_stable_dt(m,
    fv_dt)`` (for finite-volume mode, at most tau); ``rho_in``/``rho_out``
    are the porous cases' inlet and outlet densities; ``tau_rule`` is the
    Re -> tau rule of ``tau_from_re``.  ``units``: "unit" meshes every case
    on the unit square (Re with L = 1); "lattice" scales each case so that its
    mesh spacing is about 1 (``cavity_lattice_scale``,
    ``porous_lattice_scale``) and takes L = the scaled side, the units the
    reference's notebooks use (tau = 3 U L / Re + 1/2 with L in cells)."""
    if units not in ("unit", "lattice"):
        raise ValueError("units must be 'unit' or 'lattice'")
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_cavity):
        N = rng.uniform(*cavity_cells)
        r = float(rng.uniform(*re))
        g = int(round(np.sqrt(N / 2.0))) + 1
        sc = cavity_lattice_scale(g) if units == "lattice" else 1.0
        specs.append({"kind": "cavity", "grid": g, "re": r, "scale": sc,
                      "tau": tau_from_re(r, length=sc, rule=tau_rule), "flux": flux, "seed": seed * 100_003 + i,
                      "fv_dt": fv_dt})
    for i in range(n_porous):
        N = int(rng.uniform(*porous_cells))
        k = int(rng.integers(obstacles[0], obstacles[1] + 1))
        r = float(rng.uniform(*re))
        sc = porous_lattice_scale(N, porosity) if units == "lattice" else 1.0
        specs.append({"kind": "porous", "obstacles": k, "n_target": N, "re": r, "scale": sc,
                      "tau": tau_from_re(r, length=sc, rule=tau_rule),
                      "porosity": porosity, "flux": flux, "seed": seed * 100_003 + n_cavity + i,
                      "fv_dt": fv_dt, "rho_in": rho_in, "rho_out": rho_out})
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
        d = {k: v for k, v in s.items() if k in ("kind", "grid", "obstacles", "re", "tau", "scale")}
        d["cells"] = int(cs[1].pdf.shape[0])
        d["dt"] = float(cs[0].delta_t)
        desc.append(d)
    return cases, desc
