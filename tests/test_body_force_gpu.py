"""Momentum-exchange body force (lbm_set_body / lbm_body_force) against the CPU restatement in
the oracle (oracle.body_force, computed from the v0 post-streaming populations)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY, D = 160, 64, 14.0


def _case(pkg):
    walls = pkg.make_channel(NX, NY)
    disc = pkg.make_cylinder(NX, NY, 48.0, 33.0, D).astype(bool) & (walls == 0)
    return (walls | disc).astype(np.uint8), disc.astype(np.uint8)


@pytest.mark.parametrize("precision,real", [("fp32", "f32"), ("fp64", "f64"), ("fp16", "f32")])
def test_body_force_matches_oracle(gpu_lib, orc, precision, real):
    solid, disc = _case(gpu_lib)
    with gpu_lib.Solver(NX, NY, 0.56, 2e-6, 0.0, solid, precision=precision) as s:
        s.init_equilibrium(1.0, 0.04, 0.0)
        s.run(700)
        s.set_body(disc)
        fx, fy = s.body_force()
        st = s.populations()
        s.set_body(None)
        ax, ay = s.body_force()  # every solid cell: disc + walls
    wx, wy = orc.body_force(NX, NY, solid, disc, st)
    assert fx > 0.0  # drag along the flow
    assert fx == pytest.approx(wx, rel=1e-9, abs=1e-12)
    assert fy == pytest.approx(wy, rel=1e-9, abs=1e-12)
    vx, vy = orc.body_force(NX, NY, solid, solid, st)
    assert ax == pytest.approx(vx, rel=1e-9, abs=1e-12)
    assert ay == pytest.approx(vy, rel=1e-9, abs=1e-12)


def test_body_force_open_domain(gpu_lib, orc):
    solid, disc = _case(gpu_lib)
    with gpu_lib.Solver(NX, NY, 0.6, 0.0, 0.0, solid, precision="fp64") as s:
        s.set_inflow_outflow(0.05)
        s.init_equilibrium(1.0, 0.05, 0.0)
        s.run(300)
        s.set_body(disc)
        fx, fy = s.body_force()
        st = s.populations()
    wx, wy = orc.body_force(NX, NY, solid, disc, st, open_x=True)
    assert fx == pytest.approx(wx, rel=1e-9, abs=1e-12)
    assert fy == pytest.approx(wy, rel=1e-9, abs=1e-12)


def test_body_must_be_solid(gpu_lib):
    solid, disc = _case(gpu_lib)
    bad = disc.copy()
    bad[NY // 2 * NX + 5] = 1  # a fluid cell
    with gpu_lib.Solver(NX, NY, 0.6, 0.0, 0.0, solid) as s:
        with pytest.raises(ValueError):
            s.set_body(bad)
