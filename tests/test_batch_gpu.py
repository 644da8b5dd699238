"""Batched ensemble (GPU): uneven closed channels stepped by one persistent launch per step.

Workload shape: seeded channels nx ~ U[64, 1024], ny ~ U[32, 512], 1-4 discs of radius 4-24
clear of the walls, tau ~ U[0.52, 1.0], fx ~ U[1e-6, 1e-5], seeded initial perturbation.
Checks: 8 sampled instances bit-exact against the oracle's port of the reference v1 solver (itself
pinned bit for bit to the reference v0); batched == one launch per instance, every launch shape;
the autotuner leaves the state unchanged; the FP16-storage batch stays close to FP32. The
benchmark's own ensemble (256 instances, seed 7, 5000 steps from rest, autotuned launch) is
checked on 8 seeded sampled instances against the reference's own v1 solver where it was built
(else the oracle's port).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COUNT, STEPS = 24, 300


@pytest.fixture(scope="module")
def specs(gpu_lib):
    return gpu_lib.workloads.ensemble_specs(COUNT, seed=11)


def _fill(b, specs, orc, real="f32"):
    for k, s in enumerate(specs):
        b.set_populations(k, orc.seeded_state(s["seed"], 1e-4, s["nx"], s["ny"], s["mask"], real))


def test_sampled_instances_bit_exact(gpu_lib, orc, specs):
    with gpu_lib.Batch(specs, precision="fp32") as b:
        _fill(b, specs, orc)
        b.run(STEPS)
        picks = np.linspace(0, COUNT - 1, 8).astype(int)
        for k in picks:
            s = specs[k]
            nx, ny, m = s["nx"], s["ny"], s["mask"]
            r = orc.s_to_r(nx, ny, m, orc.seeded_state(s["seed"], 1e-4, nx, ny, m))
            orc.pull_run(nx, ny, m, float(np.float32(s["tau"])), s["fx"], 0.0, r, STEPS)
            want = orc.r_to_s(nx, ny, m, r)
            assert np.array_equal(b.populations(k), want), f"instance {k} ({nx}x{ny})"


@pytest.mark.parametrize("launch", [(0, 256, 0), (1, 256, 152), (2, 128, 0), (4, 64, 300), (2, 256, 152)])
def test_batched_equals_separate_launches(gpu_lib, orc, specs, launch):
    with gpu_lib.Batch(specs) as a, gpu_lib.Batch(specs) as b:
        _fill(a, specs, orc)
        _fill(b, specs, orc)
        a.set_launch(*launch)
        a.run(130)  # graph replays (64 steps each) and a direct remainder
        b.run_separate(130)
        for k in range(COUNT):
            assert np.array_equal(a.populations(k), b.populations(k)), f"instance {k}"


def test_autotune_keeps_state(gpu_lib, orc, specs, tmp_path):
    cache = tmp_path / "tune.txt"
    with gpu_lib.Batch(specs) as b:
        _fill(b, specs, orc)
        b.run(10)
        before = [b.populations(k) for k in (0, COUNT - 1)]
        report = b.autotune(cache)
        assert report.startswith("tuned")
        after = [b.populations(k) for k in (0, COUNT - 1)]
        assert all(np.array_equal(x, y) for x, y in zip(before, after))
        assert b.autotune(cache).startswith("cached")


def test_fp16_batch_close_to_fp32(gpu_lib, orc, specs):
    sub = specs[:6]
    with gpu_lib.Batch(sub, precision="fp32") as a, gpu_lib.Batch(sub, precision="fp16") as h:
        _fill(a, sub, orc)
        _fill(h, sub, orc)
        a.run(200)
        h.run(200)
        for k in range(len(sub)):
            x, y = a.populations(k), h.populations(k)
            assert np.linalg.norm(x - y) / np.linalg.norm(x) < 5e-3
        for k in range(len(sub)):
            assert abs(h.total_mass(k) - a.total_mass(k)) / a.total_mass(k) < 1e-5


def test_fp16_batched_equals_separate_launches(gpu_lib, orc, specs):
    """The 16-bit forms round stochastically with keys from the step counter: graph replays,
    direct launches and per-instance launches give the same bits."""
    sub = specs[:8]
    with gpu_lib.Batch(sub, precision="fp16") as a, gpu_lib.Batch(sub, precision="fp16") as b:
        _fill(a, sub, orc)
        _fill(b, sub, orc)
        a.run(130)
        b.run_separate(130)
        for k in range(len(sub)):
            assert np.array_equal(a.populations(k), b.populations(k)), f"instance {k}"


def test_fp16_autotune_keeps_trajectory(gpu_lib, orc, specs, tmp_path):
    """Autotuning restores the state and the step counter: the run continues as if untouched."""
    sub = specs[:8]
    with gpu_lib.Batch(sub, precision="fp16") as a, gpu_lib.Batch(sub, precision="fp16") as b:
        _fill(a, sub, orc)
        _fill(b, sub, orc)
        a.run(10)
        a.autotune(tmp_path / "tune16.txt")
        a.run(70)
        b.run(80)
        for k in range(len(sub)):
            assert np.array_equal(a.populations(k), b.populations(k)), f"instance {k}"


@pytest.mark.parametrize("shape", [(8, 2, 2), (4, 2, 4), (4, 1, 4), (2, 2, 2)])
@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_ring_tile_shapes_equal_separate_launches(gpu_lib, orc, specs, shape, precision):
    sub = specs[:12]
    with gpu_lib.Batch(sub, precision=precision) as a, gpu_lib.Batch(sub, precision=precision) as b:
        _fill(a, sub, orc)
        _fill(b, sub, orc)
        a.set_tiles(*shape)
        a.run(70)
        b.run_separate(70)
        for k in range(len(sub)):
            assert np.array_equal(a.populations(k), b.populations(k)), f"instance {k}"


def _odd_specs(gpu_lib):
    """Instances narrower than one strip (a tile spans up to 8 rows), widths just off the strip
    and tile widths (tiles straddle two rows), a few solid cells next to the periodic x edges."""
    widths = [3, 5, 17, 31, 33, 63, 64, 65, 129, 200, 300, 513, 700, 1030]
    heights = [5, 9, 6, 12, 40, 7, 33, 11, 20, 8, 13, 6, 9, 5]
    rng = np.random.default_rng(5)
    out = []
    for k, (nx, ny) in enumerate(zip(widths, heights)):
        mask = gpu_lib.make_channel(nx, ny).reshape(ny, nx).copy()
        if ny > 4:
            mask[ny // 2, 0] = 1
            mask[ny // 2 + 1, nx - 1] = 1
            mask[1 + rng.integers(ny - 2), rng.integers(nx)] = 1
        out.append({"nx": nx, "ny": ny, "mask": mask.reshape(-1).astype(np.uint8),
                    "tau": 0.55 + 0.03 * k, "fx": 2e-6 * (1 + k % 3), "fy": 0.0, "seed": 900 + k})
    return out


@pytest.mark.parametrize("shape", [(8, 2, 2), (4, 2, 4), (4, 1, 4), (2, 2, 2)])
@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_odd_widths_multi_row_tiles(gpu_lib, orc, shape, precision):
    sub = _odd_specs(gpu_lib)
    real = "f32"
    with gpu_lib.Batch(sub, precision=precision) as a, gpu_lib.Batch(sub, precision=precision) as b:
        _fill(a, sub, orc, real)
        _fill(b, sub, orc, real)
        a.set_tiles(*shape)
        a.run(70)
        b.run_separate(70)
        for k in range(len(sub)):
            assert np.array_equal(a.populations(k), b.populations(k)), f"instance {k} ({sub[k]['nx']}x{sub[k]['ny']})"


def test_odd_widths_bit_exact(gpu_lib, orc):
    sub = _odd_specs(gpu_lib)
    with gpu_lib.Batch(sub, precision="fp32") as b:
        _fill(b, sub, orc)
        b.run(60)
        for k, s in enumerate(sub):
            nx, ny, m = s["nx"], s["ny"], s["mask"]
            r = orc.s_to_r(nx, ny, m, orc.seeded_state(s["seed"], 1e-4, nx, ny, m))
            orc.pull_run(nx, ny, m, float(np.float32(s["tau"])), s["fx"], 0.0, r, 60)
            assert np.array_equal(b.populations(k), orc.r_to_s(nx, ny, m, r)), f"instance {k} ({nx}x{ny})"


def test_benchmark_ensemble_sampled_instances_bit_exact(gpu_lib, orc):
    """The batched benchmark's workload as timed by bench.py: 256 channels of seed 7, rest
    start, the autotuned launch, 5000 steps; 8 instances picked by seed."""
    specs = gpu_lib.workloads.ensemble_specs(256, seed=7)
    picks = sorted({int(v * 256) for v in gpu_lib.workloads.uniform01(2024, 8)})
    steps = 5000
    with gpu_lib.Batch(specs, precision="fp32") as b:
        b.init_equilibrium(1.0, 0.0, 0.0)
        b.autotune()
        b.run(steps)
        got = {k: b.populations(k) for k in picks}
    ref = orc.Reference("f32") if orc.Reference.available("f32") else None
    for k in picks:
        s = specs[k]
        nx, ny, m = s["nx"], s["ny"], s["mask"]
        tau = float(np.float32(s["tau"]))
        if ref is not None:
            want = ref.run("v1", nx, ny, m, tau, s["fx"], 0.0, steps, init=(1.0, 0.0, 0.0))["s"]
        else:
            r = orc.s_to_r(nx, ny, m, orc.init_equilibrium(nx, ny, m, 1.0, 0.0, 0.0))
            orc.pull_run(nx, ny, m, tau, s["fx"], 0.0, r, steps)
            want = orc.r_to_s(nx, ny, m, r)
        assert np.array_equal(got[k], want), f"instance {k} ({nx}x{ny})"
