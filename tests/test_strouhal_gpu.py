"""The reference's Strouhal known answer, reproduced on the GB300 (GPU).

The reference's open-BC cylinder case (1000 x 320 grid, D = 40 at (5 D, ny/2 + 1), Re 100,
inlet u = 0.05, tau 0.56, 160k steps, u probe 3 D behind the disc every 50 steps; reference
src/common/driver.hpp:167-251, README.md:141-153,191-193) runs through this library's
command-line driver in FP32, which is bit-exact with the reference's float solvers, and its
probe.csv is analysed as the reference's scripts/strouhal.py does with --from 0.55. The
reference publishes St = 0.1807 (FFT) and 0.1805 (zero crossings) over 15 periods with a u_y
amplitude of 0.03232, identical for its v1, v3 and v4 (results/strouhal.csv:2-4); the run here
must give the same four-decimal values.
"""
from __future__ import annotations

import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_strouhal_known_answer(gpu_lib, tmp_path):
    exe = gpu_lib.LIB_PATH.parent / "lbm_b200"
    out = tmp_path / "cyl"
    r = subprocess.run([str(exe), "--case", "cylinder", "--nx", "1000", "--ny", "320",
                        "--diameter", "40", "--re", "100", "--umax", "0.05", "--steps", "160000",
                        "--out", str(out)], capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stderr
    st = gpu_lib.wake.probe_strouhal(out, start=0.55)
    print(st)
    assert st["real"] == "float" and st["window_start"] == 88000
    assert f"{st['st_fft']:.4f}" == "0.1807"
    assert f"{st['st_zero_crossing']:.4f}" == "0.1805"
    assert st["periods"] == 15
    assert f"{st['uy_amplitude']:.5f}" == "0.03232"
