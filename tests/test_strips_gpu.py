"""Strip engine (lbm_strips_*): the lattice cut into horizontal strips with ghost rows and a
device halo exchange, as the reference's multi-rank solver (src/v4_mpi_cuda) with every strip
on one GPU. Mirrors the reference's tests/test_v4_vs_v0.cpp: the result must be bit-for-bit the
undivided solver's (itself bit-exact with v0 in FP32 / FP64) for any number of strips."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY = 203, 61


def _geometry(pkg):
    m = pkg.make_channel(NX, NY)
    m = m | pkg.make_cylinder(NX, NY, 60.0, 29.5, 15.0)  # crosses strip boundaries
    m = pkg.geometry.add_block(m, NX, 120, 131, 8, 25)
    return m.astype(np.uint8)


def _layout(ny, strips):
    base, extra = divmod(ny, strips)
    n = [base + (1 if k < extra else 0) for k in range(strips)]
    y0 = [k * base + (k if k < extra else extra) for k in range(strips)]
    return y0, n


@pytest.mark.parametrize("strips", [1, 2, 3, 4, 7])
@pytest.mark.parametrize("precision,real", [("fp32", "f32"), ("fp64", "f64"), ("fp16", "f32")])
def test_strips_equal_whole_lattice(gpu_lib, orc, strips, precision, real):
    mask = _geometry(gpu_lib)
    s0 = orc.seeded_state(99, 1e-3, NX, NY, mask, real)
    with gpu_lib.Solver(NX, NY, 0.57, 3e-6, -1e-6, mask, precision=precision) as a, \
            gpu_lib.Strips(NX, NY, 0.57, 3e-6, -1e-6, mask, strips, precision=precision) as b:
        y0, n = b.layout()
        assert (list(y0), list(n)) == _layout(NY, strips)
        a.set_populations(s0)
        b.set_populations(s0)
        assert np.array_equal(a.populations(), b.populations())
        a.run(137)
        b.run(137)  # graph replays of 16 steps and single steps
        assert np.array_equal(a.populations(), b.populations())
        for x, y in zip(a.macroscopic(), b.macroscopic()):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("strips", [2, 5])
def test_strips_open_domain(gpu_lib, strips):
    mask = _geometry(gpu_lib)
    with gpu_lib.Solver(NX, NY, 0.6, 0.0, 0.0, mask, precision="fp32") as a, \
            gpu_lib.Strips(NX, NY, 0.6, 0.0, 0.0, mask, strips, precision="fp32") as b:
        for s in (a, b):
            s.set_inflow_outflow(0.04)
            s.init_equilibrium(1.0, 0.04, 0.0)
            s.run(90)
        assert np.array_equal(a.populations(), b.populations())


def test_strips_match_reference_golden(gpu_lib):
    """The 53 x 31 block workload through 3 strips equals the reference v0's output."""
    from conftest import golden_cases, initial_state, load_golden
    case, g = golden_cases()["c1_block"], load_golden("c1_block")
    with gpu_lib.Strips(case["nx"], case["ny"], case["tau_f32"], case["fx"], case["fy"], g["mask"], 3) as s:
        s0, init = initial_state(case, g, "f32", None)
        if s0 is None:
            s.init_equilibrium(*init)
        else:
            s.set_populations(s0)
        s.run(case["steps"])
        assert np.array_equal(s.populations(), g["s_f32"])


def test_strips_need_two_rows_each(gpu_lib):
    mask = np.zeros(32 * 9, np.uint8)
    with pytest.raises(ValueError):
        gpu_lib.Strips(32, 9, 0.6, 0.0, 0.0, mask, 5)


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
@pytest.mark.parametrize("open_x", [False, True])
def test_wide_16bit_strips(gpu_lib, orc, precision, open_x):
    """Rows of at least 2048 cells with 16-bit storage take 2048-cell tiles (four passes per
    strip); 2100 cells leave a partial last tile. Same bits as the whole-lattice solver."""
    nx, ny = 2100, 40
    mask = gpu_lib.make_channel(nx, ny) | gpu_lib.make_cylinder(nx, ny, 2060.0, 20.5, 11.0)
    s0 = orc.seeded_state(7, 1e-3, nx, ny, mask, "f32")
    with gpu_lib.Solver(nx, ny, 0.58, 2e-6, 0.0, mask, precision=precision) as a, \
            gpu_lib.Strips(nx, ny, 0.58, 2e-6, 0.0, mask, 3, precision=precision) as b:
        for s in (a, b):
            if open_x:
                s.set_inflow_outflow(0.03)
                s.init_equilibrium(1.0, 0.03, 0.0)
            else:
                s.set_populations(s0)
            s.run(70)
        assert np.array_equal(a.populations(), b.populations())
