"""Register budgets of the default step kernels, from ptxas's report (CPU only, needs nvcc).

Each form's default kernel is sized for a number of resident blocks per SM (what hides the
latency of its collision). A block's warps are spread over the SM's 4 sub-partitions, each with
16,384 registers, and registers are allocated per warp in units of 8 per thread; a kernel that
outgrows its budget silently loses a block per SM (the FP64 ring at 98 registers keeps one
block where two fit its shared memory). This test compiles the library's translation units with
the library's own flags plus -Xptxas -v and checks, for every default kernel: no spill stores,
and ceil(warps per SM / 4) * round8(registers) * 32 <= 16,384.
"""

import re
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "simulation-de-fluide-par-la-m-thode-de-boltzmann-sur-r-seau-lbm-du-cpu-au-multi-gpu_gb300"

# (translation unit, kernel name with its template arguments as the demangler prints them,
# without namespaces and casts; warps per block; resident blocks per SM)
DEFAULTS = [
    ("solver.cu", "ring_step_kernel<float, ExactPhys<ExactF32>, 0, 8, 2, 2, 1>", 9, 3),
    ("solver.cu", "ring_step_kernel<__half, FastPhys, 0, 8, 4, 2, 2>", 9, 2),
    ("solver.cu", "ring_step_kernel<__nv_bfloat16, FastPhys, 0, 8, 4, 2, 2>", 9, 2),
    ("batch.cu", "batch_ring_kernel<float, ExactPhys<ExactF32>, 4, 2, 4>", 6, 4),
    ("batch.cu", "batch_ring_kernel<__half, FastPhys, 4, 2, 4>", 6, 4),
    # FP64 ring shapes at the most blocks per SM the autotuner tries (batch_ring_tune_blocks)
    ("batch.cu", "batch_ring_kernel<double, ExactPhys<ExactF64>, 8, 2, 2>", 9, 2),
    ("batch.cu", "batch_ring_kernel<double, ExactPhys<ExactF64>, 4, 2, 4>", 5, 4),
    ("batch.cu", "batch_ring_kernel<double, ExactPhys<ExactF64>, 4, 1, 4>", 5, 4),
    ("batch.cu", "batch_ring_kernel<double, ExactPhys<ExactF64>, 2, 2, 4>", 3, 6),
    ("adjoint.cu", "adj_forward_kernel<ExactF32, 2, 3, 3>", 9, 3),
    ("adjoint.cu", "adj_backward_kernel<float, 1, 3, 3>", 9, 3),
]


def short_name(demangled):
    """'void lbm_b200::k<float, (bool)0, (int)8>(args)' -> 'k<float, 0, 8>'."""
    n = demangled.split("(", 1)[0] if not demangled.startswith("void ") else demangled[5:]
    n = re.sub(r"\((?:int|bool)\)", "", n)
    n = n.replace("lbm_b200::", "").replace("<unnamed>::", "").replace("(anonymous namespace)::", "")
    depth, out = 0, []
    for ch in n:  # cut the parameter list after the template arguments
        if ch == "(" and depth == 0:
            break
        depth += ch == "<"
        depth -= ch == ">"
        out.append(ch)
    return "".join(out).strip()


def ptxas_report(unit, flags, nvcc, filt, out_dir):
    src = PKG / "csrc" / unit
    cmd = [nvcc, *flags(src), "-Xptxas", "-v", "-c", str(src), "-o", str(Path(out_dir) / (unit + ".o"))]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    kernels, name, spill = {}, None, None
    for line in r.stderr.splitlines():
        m = re.search(r"Compiling entry function '(\S+)'", line)
        if m:
            name = short_name(subprocess.run([filt, m.group(1)], capture_output=True, text=True).stdout.strip())
            spill = None
            continue
        m = re.search(r"(\d+) bytes spill stores", line)
        if m and name:
            spill = int(m.group(1))
        m = re.search(r"Used (\d+) registers", line)
        if m and name:
            kernels[name] = (int(m.group(1)), spill or 0)
    return kernels


@pytest.fixture(scope="module")
def reports():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    filt = shutil.which("cu++filt") or "/usr/local/cuda/bin/cu++filt"
    if not Path(nvcc).exists() or not Path(filt).exists():
        pytest.skip("nvcc / cu++filt not available")
    sys.path.insert(0, str(PKG))
    import buildlib  # the library's own compile flags (per-file --fmad)
    units = sorted({u for u, *_ in DEFAULTS})
    with tempfile.TemporaryDirectory() as d, ThreadPoolExecutor(len(units)) as ex:
        futs = {u: ex.submit(ptxas_report, u, buildlib.common_flags, nvcc, filt, d) for u in units}
        return {u: f.result() for u, f in futs.items()}


@pytest.mark.parametrize("unit,pattern,warps,blocks", DEFAULTS)
def test_default_kernel_fits_its_register_budget(reports, unit, pattern, warps, blocks):
    assert pattern in reports[unit], f"kernel {pattern} not compiled in {unit}"
    regs, spill = reports[unit][pattern]
    assert spill == 0, f"{pattern}: {spill} bytes of spill stores"
    per_warp = (regs + 7) // 8 * 8 * 32
    per_subpartition = -(-warps * blocks // 4)
    assert per_subpartition * per_warp <= 16384, (
        f"{pattern}: {regs} registers leave room for fewer than {blocks} blocks of {warps} warps per SM")
