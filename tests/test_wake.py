"""Cylinder wake: the Strouhal estimator on synthetic series (CPU) and the wake itself on the
GPU (FP32 against FP16, against the expected range at Re 100)."""
from __future__ import annotations

import numpy as np
import pytest


def _series(period, amp=0.05, noise=0.0, n=4000, every=50, seed=0):
    t = np.arange(1, n + 1) * float(every)
    y = amp * np.sin(2 * np.pi * t / period) + 0.01
    if noise:
        y = y + noise * np.random.default_rng(seed).normal(size=n)
    return {"t": t, "lift": y, "drag": np.full(n, 0.1), "u_bulk": 0.05, "d": 32.0}


@pytest.mark.parametrize("period,noise", [(2861.9, 0.0), (2861.9, 0.01), (1500.0, 0.005), (6400.0, 0.0)])
def test_strouhal_of_a_sine(pkg, period, noise):
    r = pkg.wake.strouhal(_series(period, noise=noise))
    assert r["st"] == pytest.approx(32.0 / period / 0.05, rel=2e-3)
    assert r["drag_mean"] == pytest.approx(0.1)


def test_wake_force_formula(pkg):
    nu = (0.548 - 0.5) / 3.0
    assert pkg.wake.wake_force() == pytest.approx(12 * nu * 0.05 / 254 ** 2)
    solid, disc = pkg.wake.geometry()
    assert disc.sum() > 700 and np.all(solid[disc == 1] == 1)


# Noise streams of the 16-bit runs: step-counter offsets fixed before the stochastic rounding
# took its current form (they were the streams of the first bistability measurement).
WAKE_STREAMS = (0, 7, 1001, 50000)


@pytest.mark.gpu
def test_wake_fp16_tracks_fp32(gpu_lib):
    """The confined wake has two shedding states: St ~ 0.225, where FP32 and FP64 stay (also
    under seeded perturbations), and St ~ 0.26, which the 16-bit forms' rounding noise reaches on
    some noise streams and not others (FP16: 4 to 6 of 12 streams stay in the first state,
    depending on the rounding scheme). So FP16 must reproduce the FP32 shedding (St within 2 %,
    mean drag within 3 %) on at least one of four fixed streams, and stay finite on all."""
    a = gpu_lib.wake.lift_series(gpu_lib, "fp32", steps=200_000, every=50)
    ra = gpu_lib.wake.strouhal(a)
    assert a["finite"]
    assert a["u_bulk"] == pytest.approx(0.05, rel=0.03)
    assert 0.20 < ra["st"] < 0.25
    hits = []
    for off in WAKE_STREAMS:
        b = gpu_lib.wake.lift_series(gpu_lib, "fp16", steps=200_000, every=50, noise_offset=off)
        rb = gpu_lib.wake.strouhal(b)
        print(f"\nwake fp32 {ra}\nwake fp16 stream {off} {rb}")
        assert b["finite"]
        hits.append(abs(rb["st"] / ra["st"] - 1) < 0.02 and abs(rb["drag_mean"] / ra["drag_mean"] - 1) < 0.03)
    assert any(hits)


def _probe_dir(tmp_path, period, steps=160_000, every=50, amp=0.03, d=40, u=0.05, phase=0.3):
    step = np.arange(every, steps + 1, every)
    uy = amp * np.sin(2 * np.pi * step / period + phase) + 0.001
    lines = ["step,ux,uy,rho"] + [f"{s},0.05,{float(v)!r},1.0" for s, v in zip(step, uy)]
    (tmp_path / "probe.csv").write_text("\n".join(lines) + "\n")
    (tmp_path / "meta.json").write_text(
        f'{{"version": "b200", "case": "cylinder", "nx": 1000, "ny": 320, "tau": 0.56, '
        f'"u_in": {u}, "re": 100, "diameter": {d}, "steps": {steps}, "real": "float"}}')
    return tmp_path


@pytest.mark.parametrize("period", [4428.0, 3000.0, 5123.7])
def test_probe_strouhal_of_a_sine(pkg, tmp_path, period):
    r = pkg.wake.probe_strouhal(_probe_dir(tmp_path, period), start=0.55)
    assert r["st_fft"] == pytest.approx(40 / period / 0.05, rel=2e-3)
    assert r["st_zero_crossing"] == pytest.approx(40 / period / 0.05, rel=2e-3)
    assert r["window_start"] == 88000


def test_probe_strouhal_agrees_with_reference_script(pkg, orc, tmp_path):
    """The restated analysis against the reference's own scripts/strouhal.py on the same
    probe file (CPU; needs the reference tree)."""
    import subprocess
    import sys

    script = orc.REFERENCE_DIR / "scripts" / "strouhal.py"
    if not script.exists():
        pytest.skip("reference scripts/strouhal.py not present")
    d = _probe_dir(tmp_path, 4431.3)
    r = subprocess.run([sys.executable, str(script), str(d), "--from", "0.55", "--csv",
                        str(tmp_path / "st.csv")], capture_output=True, text=True)
    row = (tmp_path / "st.csv").read_text().splitlines()[1].split(",")
    head = (tmp_path / "st.csv").read_text().splitlines()[0].split(",")
    ref = dict(zip(head, row))
    got = pkg.wake.probe_strouhal(d, start=0.55)
    assert f"{got['st_fft']:.4f}" == ref["st_fft"], r.stdout
    assert f"{got['st_zero_crossing']:.4f}" == ref["st_zero_crossing"]
    assert got["periods"] == int(ref["periods"])
    assert f"{got['uy_amplitude']:.5f}" == ref["uy_amplitude"]
