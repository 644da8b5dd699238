"""Parity of the CUDA path with the reference, through the C ABI (GPU).

The plain FP32 / FP64 forms must reproduce the reference's v0 bit for bit (numeric equality, as
the reference's own tests compare, tests/test_v3_vs_v0.cu:51-57): populations (all 9 planes, v0
layout), rho, ux, uy. Golden vectors come from the reference's own solvers
(tests/golden/make_golden.py); the oracle is used on the device side only as the checker.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, initial_state, load_golden

pytestmark = pytest.mark.gpu

CASES = sorted(golden_cases())
PREC = {"f32": "fp32", "f64": "fp64"}


def run_case(pkg, case, g, real, launch=None, orc=None):
    nx, ny, mask = case["nx"], case["ny"], g["mask"]
    s = pkg.Solver(nx, ny, case[f"tau_{real}"], case["fx"], case["fy"], mask, precision=PREC[real])
    if launch:
        s.set_launch(*launch)
    if case.get("open_x"):
        s.set_inflow_outflow(case["u_in"])
    s0, init = initial_state(case, g, real, orc)
    if s0 is None:
        s.init_equilibrium(*init)
    else:
        s.set_populations(s0)
    s.run(case["steps"])
    return s


@pytest.mark.parametrize("real", ["f32", "f64"])
@pytest.mark.parametrize("name", CASES)
def test_step_bit_exact_with_reference(gpu_lib, name, real):
    case = golden_cases()[name]
    g = load_golden(name)
    with run_case(gpu_lib, case, g, real) as s:
        pops = s.populations()
        rho, ux, uy = s.macroscopic()
        mass = s.total_mass()
        # probe == gathered state at a few fluid cells (populations_at, solver_v3.cu:234-249)
        fluid = np.flatnonzero(g["mask"] == 0)
        for c in fluid[:: max(1, len(fluid) // 7)]:
            y, x = divmod(int(c), case["nx"])
            assert np.array_equal(s.populations_at(x, y), pops[c * 9:(c + 1) * 9])
    want = g[f"s_{real}"]
    bad = np.flatnonzero(pops != want)
    assert bad.size == 0, (f"{bad.size} of {want.size} populations differ; first at cell "
                           f"{bad[0] // 9} dir {bad[0] % 9}: {pops[bad[0]]!r} vs {want[bad[0]]!r}")
    for k, a in (("rho", rho), ("ux", ux), ("uy", uy)):
        assert np.array_equal(a, g[f"{k}_{real}"]), f"{k} differs"
    # mass: same sum, different order (FP64 accumulation both sides)
    assert mass == pytest.approx(float(g[f"mass_{real}"]), rel=1e-12, abs=1e-9)


@pytest.mark.parametrize("launch", [(32, 1), (64, 3), (128, 0), (256, 7), (256, 0)])
def test_result_independent_of_launch_shape(gpu_lib, launch):
    case = golden_cases()["odd_width_disc"]
    g = load_golden("odd_width_disc")
    with run_case(gpu_lib, case, g, "f32", launch=launch) as s:
        assert np.array_equal(s.populations(), g["s_f32"])


@pytest.mark.parametrize("real", ["f32", "f64"])
def test_init_equilibrium_matches_oracle(gpu_lib, orc, real):
    nx, ny = 61, 19
    mask = gpu_lib.geometry.add_disc(gpu_lib.make_channel(nx, ny), nx, ny, 20.0, 9.0, 7.0)
    with gpu_lib.Solver(nx, ny, 0.7, 1e-5, 0.0, mask, precision=PREC[real]) as s:
        s.init_equilibrium(1.01, 0.03, -0.02)
        got = s.populations()
    want = orc.init_equilibrium(nx, ny, mask, 1.01, 0.03, -0.02, real)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("real", ["f32", "f64"])
def test_set_get_populations_round_trip(gpu_lib, orc, real):
    nx, ny = 70, 33
    mask = gpu_lib.geometry.add_disc(gpu_lib.make_channel(nx, ny), nx, ny, 30.0, 16.0, 9.0)
    s0 = orc.seeded_state(99, 1e-3, nx, ny, mask, real)
    with gpu_lib.Solver(nx, ny, 0.6, 0.0, 0.0, mask, precision=PREC[real]) as s:
        s.set_populations(s0)
        assert np.array_equal(s.populations(), s0)
        # zero steps leaves the state unchanged
        s.run(0)
        assert np.array_equal(s.populations(), s0)


def test_all_solid_and_single_cell_grids(gpu_lib):
    with gpu_lib.Solver(37, 5, 0.8, 1e-5, 0.0, np.ones(37 * 5, np.uint8)) as s:
        s.init_equilibrium(1.0, 0.01, 0.0)
        s.run(10)
        assert not s.populations().any()
        rho, ux, uy = s.macroscopic()
        assert not rho.any() and not ux.any() and not uy.any()
        assert s.total_mass() == 0.0


def test_errors_follow_reference(gpu_lib):
    mask = gpu_lib.make_channel(8, 6)
    with pytest.raises(ValueError):
        gpu_lib.Solver(8, 6, 0.5, 0.0, 0.0, mask)
    with pytest.raises(ValueError):
        gpu_lib.Solver(8, 5, 0.8, 0.0, 0.0, mask)
    with gpu_lib.Solver(8, 6, 0.8, 0.0, 0.0, mask) as s:
        with pytest.raises(ValueError):
            s.step(-1)
        with pytest.raises(ValueError):
            s.populations_at(8, 0)
        with pytest.raises(ValueError):
            s.set_populations(np.zeros(3, np.float32))
    with gpu_lib.Solver(2, 6, 0.8, 0.0, 0.0, gpu_lib.make_channel(2, 6)) as s:
        with pytest.raises(ValueError):
            s.set_inflow_outflow(0.05)  # open boundaries need nx >= 3


def test_divergence_is_detected(gpu_lib):
    """A state driven unstable (tau near 1/2, large velocity) is reported as non-finite."""
    nx, ny = 64, 32
    with gpu_lib.Solver(nx, ny, 0.5000001, 0.0, 0.0, np.zeros(nx * ny, np.uint8)) as s:
        s.init_equilibrium(1.0, 0.0, 0.0)
        assert s.check_finite()
        st = s.populations()
        st[::9] = np.float32(3e38)  # rest population near the float maximum
        st[1::9] = np.float32(3e38)
        s.set_populations(st)
        s.run(3)
        assert not s.check_finite()


VARIANTS = list(range(23))


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("real", ["f32", "f64"])
@pytest.mark.parametrize("name", ["c1_block", "cylinder_open", "periodic_scatter", "odd_width_disc",
                                  "tiny_1x5", "tiny_2x4", "open_seeded"])
def test_every_kernel_variant_bit_exact(gpu_lib, name, real, variant):
    """Every step-kernel variant (direct, register-prefetch, warp-specialised bulk-copy ring)
    reproduces the reference's populations bit for bit."""
    case = golden_cases()[name]
    g = load_golden(name)
    nx, ny, mask = case["nx"], case["ny"], g["mask"]
    with gpu_lib.Solver(nx, ny, case[f"tau_{real}"], case["fx"], case["fy"], mask,
                        precision=PREC[real]) as s:
        s.set_variant(variant)
        if case.get("open_x"):
            s.set_inflow_outflow(case["u_in"])
        s0, init = initial_state(case, g, real, None)
        if s0 is None:
            s.init_equilibrium(*init)
        else:
            s.set_populations(s0)
        s.run(case["steps"])
        assert np.array_equal(s.populations(), g[f"s_{real}"])
