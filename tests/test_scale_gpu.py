"""At-scale parity of the walled-channel workload (GPU).

Walled channel, periodic in x, tau 0.6, F = (1e-6, 0), f_i - w_i from the seeded SplitMix64
perturbation in [-1e-4, 1e-4]. The SHA-256 digests in tests/golden/hashes.json were computed
from the reference's own v1 solver (bitwise identical to v0) on the same inputs; negative zeros
are mapped to +0 before hashing (numeric equality). Grid 2048^2 runs the full 1000 steps in FP32
and FP64; 4096^2 and 8192^2 run fewer steps (their reference runs take minutes on the CPU).
Size-independent checks (mass conservation, launch-shape independence) cover the full sizes.
"""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import large_hashes

pytestmark = pytest.mark.gpu

PREC = {"f32": "fp32", "f64": "fp64"}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a + a.dtype.type(0)).tobytes()).hexdigest()


@pytest.mark.parametrize("name", sorted(large_hashes()))
def test_channel_at_scale_matches_reference_digest(gpu_lib, orc, name):
    h = large_hashes()[name]
    nx, ny, real = h["nx"], h["ny"], h["real"]
    mask = gpu_lib.make_channel(nx, ny)
    s0 = orc.seeded_state(h["seed"], h["amp"], nx, ny, mask, real)
    assert digest(s0) == h["s0"], "seeded initial state differs from the reference run's"
    with gpu_lib.Solver(nx, ny, h["tau"], h["fx"], h["fy"], mask, precision=PREC[real]) as s:
        s.set_populations(s0)
        del s0
        s.run(h["steps"])
        rho, ux, uy = s.macroscopic()
        assert digest(rho) == h["rho"]
        assert digest(ux) == h["ux"]
        assert digest(uy) == h["uy"]
        del rho, ux, uy
        assert digest(s.populations()) == h["s"]
        assert s.total_mass() == pytest.approx(h["mass"], rel=1e-13)


@pytest.mark.parametrize("n", [4096, 8192])
def test_mass_conserved_at_scale(gpu_lib, orc, n):
    mask = gpu_lib.make_channel(n, n)
    s0 = orc.seeded_state(5, 1e-4, n, n, mask, "f32")
    with gpu_lib.Solver(n, n, 0.6, 1e-6, 0.0, mask) as s:
        s.set_populations(s0)
        del s0
        m0 = s.total_mass()
        s.run(200)
        m1 = s.total_mass()
        assert s.check_finite()
    assert abs(m1 - m0) / m0 < 1e-6


def test_launch_shapes_agree_at_scale(gpu_lib, orc):
    n = 2048
    mask = gpu_lib.make_channel(n, n)
    s0 = orc.seeded_state(11, 1e-4, n, n, mask, "f32")
    digests = set()
    for launch in [(256, 0), (128, 152), (64, 1000)]:
        with gpu_lib.Solver(n, n, 0.6, 1e-6, 0.0, mask) as s:
            s.set_launch(*launch)
            s.set_populations(s0)
            s.run(50)
            digests.add(digest(s.populations()))
    assert len(digests) == 1


def _wake_hashes():
    import json
    from pathlib import Path
    return json.loads((Path(__file__).resolve().parent / "golden" / "wake_hashes.json").read_text())


@pytest.mark.parametrize("real", ["f32", "f64"])
def test_cylinder_wake_matches_reference_digest(gpu_lib, real):
    """The cylinder-wake workload (walled 1024 x 256, disc D = 32 at (256, 129), tau 0.548,
    calibrated force, start u = (0.05, 0)) after 200k steps: plain FP32 and FP64 equal the
    reference v1 (bitwise v0) run, digests in tests/golden/wake_hashes.json."""
    h = _wake_hashes()[f"wake_{real}"]
    solid, _ = gpu_lib.wake.geometry()
    assert hashlib.sha256(solid.tobytes()).hexdigest() == h["mask_sha"]
    with gpu_lib.Solver(h["nx"], h["ny"], h["tau"], h["fx"], h["fy"], solid,
                        precision=PREC[real]) as s:
        s.init_equilibrium(*h["init"])
        s.run(h["steps"])
        rho, ux, uy = s.macroscopic()
        assert digest(rho) == h["rho"]
        assert digest(ux) == h["ux"]
        assert digest(uy) == h["uy"]
        assert digest(s.populations()) == h["s"]
        assert s.total_mass() == pytest.approx(h["mass"], rel=1e-12)
