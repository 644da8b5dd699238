"""Drop-in check: the reference's own templated consumers compile against lbm::SolverB200.

Compiles (syntax and template instantiation, no GPU needed) a translation unit that
instantiates, with lbm::SolverB200 in place of lbm::SolverV3:
  - poiseuille::run_all<Solver>   (reference tests/poiseuille_check.hpp:128-158)
  - cylinder_case::run<Solver>    (reference tests/cylinder_case.hpp:33-41)
  - lbm::run_driver<Solver>       (reference src/common/driver.hpp:255-300)
in float and double. Needs the reference tree or its staged copy (skipped without either). The
GPU test tests/test_reference_gpu.py builds and runs the reference's own v3 test programs
against the library.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle  # noqa: E402  (test infrastructure: locates the reference tree)

REF = oracle.reference_tree()

TU = r'''
#include "lbm_b200.hpp"
#include "cylinder_case.hpp"
#include "driver.hpp"
#include "poiseuille_check.hpp"

int main(int argc, char** argv) {
  int rc = poiseuille::run_all<lbm::SolverB200>("b200");
  const std::vector<lbm::real> g = cylinder_case::run<lbm::SolverB200>();
  rc |= g.empty();
  return rc | lbm::run_driver<lbm::SolverB200>(argc, argv, "b200");
}
'''


@pytest.mark.skipif(REF is None or shutil.which("g++") is None,
                    reason="reference tree or g++ not available")
@pytest.mark.parametrize("double", [False, True])
def test_reference_consumers_compile_against_wrapper(tmp_path, double, orc):
    orc.build(ref=True)  # generates oracle/_ref/build_info.hpp used by driver.hpp
    src = tmp_path / "dropin.cpp"
    src.write_text(TU)
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"),
           "-I", str(REF / "src" / "common"), "-I", str(REF / "tests"),
           "-I", str(ROOT / "oracle" / "_ref"), str(src)]
    if double:
        cmd.insert(2, "-DLBM_REAL_DOUBLE")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
