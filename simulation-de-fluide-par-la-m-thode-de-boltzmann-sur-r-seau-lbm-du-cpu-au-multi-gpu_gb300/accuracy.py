"""Accuracy of the 16-bit storage forms against the FP64 form of the same step.

The FP64 form is itself bit-exact with the reference's double-precision v0 solver, so it is the
reference solution here. Both runs start from the same state and take the same steps; the
velocity error is the relative L2 norm over fluid cells,

    e_u = sqrt(sum (ux - ux64)^2 + (uy - uy64)^2) / sqrt(sum ux64^2 + uy64^2),

and the mass drift of a run is (M(t) - M(0)) / M(0), M = sum over fluid cells of rho, reduced in
FP64 on the device (lbm_total_mass).
"""
from __future__ import annotations

import numpy as np


def run_form(pkg, nx, ny, mask, tau, fx, fy, steps, precision, init=(1.0, 0.0, 0.0),
             state=None, variant=-1, u_in=None):
    """Runs one form; returns (ux, uy, mass0, mass1) with ux, uy as float64 arrays."""
    with pkg.Solver(nx, ny, tau, fx, fy, mask, precision=precision) as s:
        if variant >= 0:
            s.set_variant(variant)
        if u_in is not None:
            s.set_inflow_outflow(u_in)
        if state is None:
            s.init_equilibrium(*init)
        else:
            s.set_populations(state.astype(s.dtype))
        m0 = s.total_mass()
        s.run(steps)
        m1 = s.total_mass()
        _, ux, uy = s.macroscopic()
    return ux.astype(np.float64), uy.astype(np.float64), m0, m1


def compare_forms(pkg, nx, ny, mask, tau, fx, fy, steps, form, init=(1.0, 0.0, 0.0),
                  state=None, u_in=None, reference=None):
    """Velocity L2 error and mass drift of `form` against the FP64 form. `reference` may pass
    a previous FP64 run_form result to reuse it."""
    fluid = np.asarray(mask).reshape(-1) == 0
    ref = reference or run_form(pkg, nx, ny, mask, tau, fx, fy, steps, "fp64", init, state,
                                u_in=u_in)
    got = run_form(pkg, nx, ny, mask, tau, fx, fy, steps, form, init, state, u_in=u_in)
    dx = got[0][fluid] - ref[0][fluid]
    dy = got[1][fluid] - ref[1][fluid]
    norm = np.sqrt(np.sum(ref[0][fluid] ** 2 + ref[1][fluid] ** 2))
    err = float(np.sqrt(np.sum(dx * dx + dy * dy)) / norm) if norm > 0 else float("nan")
    return {
        "form": form, "steps": steps, "velocity_l2": err,
        "mass_drift": (got[3] - got[2]) / got[2],
        "mass_drift_fp64": (ref[3] - ref[2]) / ref[2],
        "u_max_fp64": float(np.max(np.hypot(ref[0][fluid], ref[1][fluid]))),
    }, ref
