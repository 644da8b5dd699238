"""The command-line driver lbm_b200 (reference CLI and BENCH line format).

CPU: argument validation follows the reference's parser (src/common/params.cpp:8-44).
GPU: --bench prints one parseable "BENCH {json}" line per repetition with the keys the
reference's bench/run_bench.py reads; the Poiseuille run writes .npy fields equal to the
library's moment pass; the cylinder run writes probe.csv and meta.json.
"""
from __future__ import annotations

import json
import subprocess

import numpy as np
import pytest

RUN_BENCH_KEYS = {"version", "rep", "nx", "ny", "steps", "warmup", "threads", "time_s", "mlups",
                  "real", "compiler", "flags", "build_type", "gpu", "gpu_driver_cuda",
                  "cuda_runtime", "cuda_compiled", "ecc", "block", "variant"}


@pytest.fixture(scope="module")
def exe(pkg):
    pkg.build()
    return pkg.LIB_PATH.parent / "lbm_b200"


@pytest.mark.parametrize("args, msg", [
    (["--tau", "0.5"], "tau must be > 0.5"),
    (["--ny", "2"], "grid too small"),
    (["--reps", "0"], "need warmup >= 0 and reps >= 1"),
    (["--diameter", "1"], "invalid cylinder parameters"),
    (["--frobnicate", "1"], "unknown option --frobnicate"),
    (["--nx"], "missing value for --nx"),
])
def test_cli_validation(exe, args, msg):
    r = subprocess.run([str(exe), *args], capture_output=True, text=True)
    assert r.returncode == 1 and msg in r.stderr


def test_cli_unknown_case(exe):
    r = subprocess.run([str(exe), "--case", "wing"], capture_output=True, text=True)
    assert r.returncode == 1 and "unknown case" in r.stderr


@pytest.mark.gpu
def test_bench_lines(exe):
    r = subprocess.run([str(exe), "--bench", "--nx", "256", "--ny", "66", "--steps", "200",
                        "--warmup", "10", "--reps", "3"], capture_output=True, text=True, check=True)
    recs = [json.loads(l[len("BENCH "):]) for l in r.stdout.splitlines() if l.startswith("BENCH ")]
    assert len(recs) == 3
    for k, rec in enumerate(recs):
        assert RUN_BENCH_KEYS <= set(rec)
        assert rec["rep"] == k and rec["mlups"] > 0 and rec["real"] == "float"


@pytest.mark.gpu
def test_poiseuille_fields(exe, pkg, tmp_path):
    out = tmp_path / "p"
    subprocess.run([str(exe), "--nx", "48", "--ny", "22", "--steps", "300", "--out", str(out)],
                   capture_output=True, text=True, check=True)
    h = 20
    force = pkg.poiseuille_force(h, 0.9, 0.05)
    with pkg.Solver(48, 22, np.float32(0.9), force, 0.0, pkg.make_channel(48, 22)) as s:
        s.init_equilibrium(1.0, 0.0, 0.0)
        s.run(300)
        rho, ux, uy = s.macroscopic()
    assert np.array_equal(np.load(out / "rho.npy").reshape(-1), rho)
    assert np.array_equal(np.load(out / "ux.npy").reshape(-1), ux)
    assert np.load(out / "solid.npy").shape == (22, 48)
    meta = json.loads((out / "meta.json").read_text())
    assert meta["steps"] == 300 and meta["real"] == "float"


@pytest.mark.gpu
def test_cylinder_probe(exe, tmp_path):
    out = tmp_path / "c"
    subprocess.run([str(exe), "--case", "cylinder", "--nx", "200", "--ny", "64", "--diameter", "10",
                    "--re", "50", "--steps", "400", "--probe-every", "50", "--frame-every", "200",
                    "--out", str(out)], capture_output=True, text=True, check=True)
    lines = (out / "probe.csv").read_text().splitlines()
    assert lines[0] == "step,ux,uy,rho" and len(lines) == 1 + 400 // 50
    assert (out / "frames" / "vort_0000400.npy").exists()
    meta = json.loads((out / "meta.json").read_text())
    assert meta["case"] == "cylinder" and meta["probe_x"] == 80
