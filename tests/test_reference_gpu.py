"""The reference's own GPU code and its own v3 test programs, run on the GB300 (GPU).

1. Drop-in. The reference's v3 test programs, unmodified:
     tests/test_v3_vs_v0.cu     bitwise v3 == v0 on the 53x31 obstacle case (:20-68),
     tests/test_poiseuille_v3.cu  Poiseuille checks A/B/C (tests/poiseuille_check.hpp:128-158),
     tests/test_cylinder_v3.cu  open inflow/outflow cylinder, bitwise against v0,
   built with lbm::SolverV3 = lbm::SolverB200 (tests/dropin/solver_v3.hpp, the binding a
   maintainer adds) and linked against the library (oracle/Makefile `consumers`), in float and
   double. Each must exit 0, print ALL PASSED and no FAIL line. The programs loop over the
   reference's three kernel variants (LBM_V3_VARIANT), which the drop-in ignores.
2. The reference's own kernel. SolverV3 (src/v3_cuda_opt/solver_v3.cu, unmodified, built for
   sm_103a with the reference's --fmad=false) runs on the golden cases through
   oracle/ref_v3_shim.cu: it reproduces the golden vectors (the reference's v0), as the
   library does, and at 2048^2 x 1000 steps its populations hash to the reference v1 digest in
   tests/golden/hashes.json, as the library's do (tests/test_scale_gpu.py).

Needs the reference tree or the copy oracle/Makefile staged into oracle/_ref/tree (skipped,
with that reason, without either).
"""
from __future__ import annotations

import hashlib
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import golden_cases, initial_state, large_hashes, load_golden

pytestmark = pytest.mark.gpu

PROGRAMS = ["v3_vs_v0", "poiseuille", "cylinder"]


@pytest.fixture(scope="module")
def ref_tree(orc):
    if orc.reference_tree() is None:
        pytest.skip("neither the reference tree nor its staged copy (oracle/_ref/tree) is present")
    return orc.reference_tree()


@pytest.fixture(scope="module")
def consumers(gpu_lib, orc, ref_tree):
    orc.build(ref=True)
    orc.build_consumers(Path(gpu_lib.__file__).resolve().parent / "lib")
    return orc.REF_DIR


@pytest.mark.parametrize("real", ["f32", "f64"])
@pytest.mark.parametrize("program", PROGRAMS)
def test_reference_program_passes_on_dropin(consumers, program, real):
    exe = consumers / f"dropin_{program}_{real}"
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "ALL PASSED" in r.stdout
    assert "[FAIL]" not in r.stdout
    assert r.stdout.count("[PASS]") >= 3


@pytest.fixture(scope="module")
def ref_v3(orc, ref_tree):
    orc.build(ref=True, gpu=True)
    return {real: orc.ReferenceV3(real) for real in ("f32", "f64")}


PREC = {"f32": "fp32", "f64": "fp64"}


@pytest.mark.parametrize("real", ["f32", "f64"])
@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_reference_kernel_matches_golden_and_library(gpu_lib, orc, ref_v3, name, real):
    case = golden_cases()[name]
    g = load_golden(name)
    nx, ny, mask = case["nx"], case["ny"], g["mask"]
    s0, init = initial_state(case, g, real, orc)
    kw = dict(open_x=bool(case.get("open_x")), u_in=case.get("u_in", 0.0))
    if s0 is None:
        kw["init"] = init
    else:
        kw["s0"] = s0
    want = g[f"s_{real}"]
    ref = ref_v3[real].run(nx, ny, mask, case[f"tau_{real}"], case["fx"], case["fy"],
                           case["steps"], **kw)
    assert np.array_equal(ref["s"], want), "the reference's v3 kernel differs from its v0"
    for k in ("rho", "ux", "uy"):
        assert np.array_equal(ref[k], g[f"{k}_{real}"])
    with gpu_lib.Solver(nx, ny, case[f"tau_{real}"], case["fx"], case["fy"], mask,
                        precision=PREC[real]) as s:
        if kw["open_x"]:
            s.set_inflow_outflow(kw["u_in"])
        if s0 is None:
            s.init_equilibrium(*init)
        else:
            s.set_populations(s0)
        s.run(case["steps"])
        assert np.array_equal(s.populations(), ref["s"])


def _digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a + a.dtype.type(0)).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["channel_2048_f32", "channel_2048_f64"])
def test_reference_kernel_at_scale_matches_digest(gpu_lib, orc, ref_v3, name):
    h = large_hashes()[name]
    nx, ny, real = h["nx"], h["ny"], h["real"]
    mask = gpu_lib.make_channel(nx, ny)
    s0 = orc.seeded_state(h["seed"], h["amp"], nx, ny, mask, real)
    secs, info, out = ref_v3[real].bench(nx, ny, mask, h["tau"], h["fx"], h["fy"], s0,
                                         h["steps"], warmup=0, reps=1, state_out=True)
    assert "soa_pull_opt" in info and secs[0] > 0
    assert _digest(out) == h["s"]
