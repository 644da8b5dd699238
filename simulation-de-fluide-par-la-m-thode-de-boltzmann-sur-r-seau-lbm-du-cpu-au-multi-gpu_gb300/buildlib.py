"""Builds the CUDA library lib/liblbm_b200.so for sm_103a, in-tree.

Every .cu file under csrc/ is one translation unit, compiled in parallel with nvcc, then linked
with -shared. Flags:
  -gencode arch=compute_103a,code=sm_103a  the only target (GB300);
  --fmad=false                            no multiply-add contraction (the exact forms also use
                                          explicit round-to-nearest intrinsics);
  -Xcompiler -ffp-contract=off            same for host code (per-launch constants);
  -lineinfo                               source correlation for ncu.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "lib"
LIB = OUT_DIR / "liblbm_b200.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise FileNotFoundError("nvcc not found")


# Translation units whose plain-operator arithmetic may be contracted into FMA: their exact
# parts use explicit round-to-nearest intrinsics, which are never contracted.
FMAD_TRUE = {"adjoint.cu"}


def common_flags(src: Path | None = None) -> list[str]:
    fmad = "--fmad=true" if src is not None and src.name in FMAD_TRUE else "--fmad=false"
    return ARCH + [
        "-O3", "-std=c++17", "-lineinfo", fmad, "-Xcompiler", "-fPIC",
        "-Xcompiler", "-ffp-contract=off", "-I", str(CSRC), "-I", str(ROOT / "include"),
    ]


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


DRIVER = PKG / "driver" / "lbm_b200_main.cpp"
EXES = {"lbm_b200": [], "lbm_b200_double": ["-DLBM_REAL_DOUBLE"]}


def _stale(objs: list[Path]) -> bool:
    if not LIB.exists() or any(not (OUT_DIR / e).exists() for e in EXES):
        return True
    t = min([LIB.stat().st_mtime] + [(OUT_DIR / e).stat().st_mtime for e in EXES])
    deps = list(CSRC.glob("*")) + list((ROOT / "include").glob("*")) + [DRIVER, Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build_driver() -> None:
    """The command-line driver (float and double builds), linked against the library."""
    cxx = os.environ.get("CXX", "g++")
    for exe, defs in EXES.items():
        cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", *defs, "-I", str(ROOT / "include"),
               str(DRIVER), "-L", str(OUT_DIR), "-llbm_b200", "-Wl,-rpath,$ORIGIN",
               "-o", str(OUT_DIR / exe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stderr}")


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    objs = [OUT_DIR / (src.stem + ".o") for src in sources()]
    if not force and not ptxas_info and not _stale(objs):
        return LIB
    cc = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src: Path, obj: Path):
        cmd = [cc, *common_flags(src), *extra, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=min(len(objs), os.cpu_count() or 4)) as ex:
        logs = list(ex.map(compile_one, sources(), objs))
    if verbose or ptxas_info:
        for src, log in zip(sources(), logs):
            print(f"== {src.name}\n{log}", file=sys.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver()
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv, force=True)
    print(LIB)
