"""The C-ABI library builds, loads and exports every entry point of include/*.h (CPU only:
no compute calls). Also compiles the header-only C++ wrapper and the host build of the
collision header against the oracle."""
from __future__ import annotations

import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(lbm_[a-z0-9_]+)\s*\(",
                            text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("lbm_create", "lbm_destroy", "lbm_step", "lbm_macroscopic", "lbm_total_mass",
                 "lbm_get_populations", "lbm_set_populations", "lbm_populations_at"):
        assert must in names


def test_library_exports_every_declared_symbol(pkg):
    pkg.build()
    lib = pkg.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_library_fails_cleanly_without_gpu(pkg):
    """Without a usable GPU the ABI reports LBM_ERR_CUDA instead of crashing; argument errors
    are reported before any CUDA call."""
    import ctypes as C
    import numpy as np
    import torch
    lib = pkg.lib()
    h = C.c_void_p()
    m = np.zeros(16, np.uint8)
    assert lib.lbm_create(4, 4, C.c_void_p(m.ctypes.data), 0.5, 0.0, 0.0, 0, C.byref(h)) == pkg.ERR_INVALID_ARG
    assert lib.lbm_create(0, 4, C.c_void_p(m.ctypes.data), 0.8, 0.0, 0.0, 0, C.byref(h)) == pkg.ERR_INVALID_ARG
    assert lib.lbm_create(4, 4, None, 0.8, 0.0, 0.0, 0, C.byref(h)) == pkg.ERR_INVALID_ARG
    assert lib.lbm_create(4, 4, C.c_void_p(m.ctypes.data), 0.8, 0.0, 0.0, 7, C.byref(h)) == pkg.ERR_INVALID_ARG
    if not torch.cuda.is_available():
        assert lib.lbm_create(4, 4, C.c_void_p(m.ctypes.data), 0.8, 0.0, 0.0, 0, C.byref(h)) == pkg.ERR_CUDA
    assert lib.lbm_destroy(None) == pkg.OK


def test_python_solver_validates_like_reference(pkg):
    import numpy as np
    with pytest.raises(ValueError):
        pkg.Solver(4, 4, 0.8, 0.0, 0.0, np.zeros(15, np.uint8))  # mask size mismatch
    with pytest.raises(ValueError):
        pkg.Solver(4, 4, 0.5, 0.0, 0.0, np.zeros(16, np.uint8))  # tau <= 0.5


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host compiler")
def test_collision_algebra_on_host(tmp_path, orc):
    """collide.h compiled for the host: the simplified exact collision equals the literal v0
    collision on random states (float and double), value for value."""
    src = ROOT / "tests" / "cpp" / "collide_algebra_test.cpp"
    exe = tmp_path / "collide_algebra_test"
    pkgdir = next(ROOT.glob("simulation-de-fluide-*_gb300"))
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(pkgdir / "csrc"),
                    str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "200000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host compiler")
def test_fastdiv_on_host(tmp_path):
    """csrc/fastdiv.h (the tile decoders' division by invariant integers) equals integer
    division on edge and random dividends for divisors 1..4096 and large ones."""
    src = ROOT / "tests" / "cpp" / "fastdiv_test.cpp"
    exe = tmp_path / "fastdiv_test"
    pkgdir = next(ROOT.glob("simulation-de-fluide-*_gb300"))
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(pkgdir / "csrc"), str(src), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host compiler")
def test_cpp_wrapper_compiles(tmp_path):
    """include/lbm_b200.hpp (the SolverV3 drop-in) compiles standalone against the C header."""
    src = tmp_path / "w.cpp"
    src.write_text('#define LBM_B200_STANDALONE\n#include "lbm_b200.hpp"\n'
                   'int main(){ lbm::Mask m(64, 0); try { lbm::SolverB200 s(8, 8, 0.8f, 0.f, 0.f, m);'
                   ' s.init_equilibrium(1.f, 0.f, 0.f); s.run(2); auto p = s.populations();'
                   ' std::vector<lbm::real> r,u,v; s.macroscopic(r,u,v); (void)s.total_mass();'
                   ' lbm::real o[9]; s.populations_at(1,1,o); (void)s.timed_run(1);'
                   ' (void)s.bench_info(); return (int)p.size() == 0; } catch (...) { return 0; } }\n')
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"), str(src)],
                   check=True)
