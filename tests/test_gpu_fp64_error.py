"""Float32 rounding error of the step, per configuration: the GPU path (which
equals the reference's float32 step bit for bit) against the float64 oracle
(the same statements in double) after the stated steps.  The bounds are the
measured errors with headroom; set FVDBM_REPORT=<file> to write the figures
as JSON."""
import json
import os

import numpy as np
import pytest

import oracle_c as OC
import oracle_np as ON

pytestmark = pytest.mark.gpu

_REPORT = {}


def _case(raw, flux, tau, bc):
    from fvdbm_jax_gb300 import D2Q9, Mesher
    m = Mesher().import_meshpy(raw)
    m.calc_mesh_properties()
    dyn = D2Q9(tau, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, flux)
    if bc == "cavity":
        for mk in (1, 2, 4):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_vel_node(n, 3, (0.1, 0.0))
    elif bc == "channel":
        for mk in (1, 3, 5):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_vel_node(n, 4, (0.0, 0.0))
        sel = m.point_markers == 4
        y = m.points[sel, 1]
        v = np.array(n.vel)
        v[sel, 0] = 4 * 0.1 * y * (0.41 - y) / 0.41 ** 2
        n.vel = v
        n = m.set_rho_node(n, 2, 1.0)
    else:
        for mk in (1, 3, 5):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_rho_node(n, 4, 1.001)
        n = m.set_rho_node(n, 2, 1.0)
    return dyn, c, f, n


def _macros64(pdf):
    pdf = np.asarray(pdf, np.float64)
    rho = pdf.sum(1)
    u = (pdf @ ON.KSI.astype(np.float64)) / rho[:, None]
    return rho, u


CASES = {
    # name: (mesh, flux, tau, bc, steps, rho bound, u bound relative to max|u|)
    "cavity_upwind": ("cavity", "upwind", 0.6, "cavity", 2000, 5e-5, 3e-3),
    "channel_upwind": ("channel", "upwind", 0.55, "channel", 2000, 1.5e-4, 1.5e-2),
    "channel_lax_wendroff": ("channel", "lax_wendroff", 0.55, "channel", 2000, 1.5e-4, 2e-2),
    "porous1m_upwind": ("porous", "upwind", 0.6, "porous", 20, 1e-7, 1.01),
}


@pytest.mark.parametrize("name", list(CASES))
def test_fp32_vs_fp64(name):
    from fvdbm_jax_gb300 import Environment, meshgen
    mesh, flux, tau, bc, steps, rb, ub = CASES[name]
    raw = {"cavity": lambda: meshgen.cavity(41), "channel": meshgen.channel_cylinder,
           "porous": meshgen.porous}[mesh]()
    dyn, c, f, n = _case(raw, flux, tau, bc)
    env = Environment(c, f, n)
    env.init()
    env.step(steps)
    got = np.asarray(env.cells.pdf)
    env.close()
    geo, st = ON.geo_from_containers(c, f, n), ON.state_from_containers(c, n)
    ref = OC.step64(geo, st, tau, dyn.delta_t, steps)["cells_pdf"]
    r32, u32 = _macros64(got)
    r64, u64 = _macros64(ref)
    rho_err = float(np.abs(r32 - r64).max() / np.abs(r64).max())
    umax = float(np.abs(u64).max())
    u_err = float(np.abs(u32 - u64).max() / max(umax, 1e-30))
    pdf_err = float(np.abs(got - ref).max() / np.abs(ref).max())
    _REPORT[name] = {"cells": int(got.shape[0]), "steps": steps, "rho_max_rel_err": rho_err,
                     "u_max_err_over_max_u": u_err, "max_u": umax, "pdf_max_rel_err": pdf_err}
    if os.environ.get("FVDBM_REPORT"):
        with open(os.environ["FVDBM_REPORT"], "w") as fh:
            json.dump(_REPORT, fh, indent=1)
    assert rho_err < rb and u_err < ub, _REPORT[name]
