"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on the CPU."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def pkg():
    return entry.package()


@pytest.fixture(scope="session")
def orc():
    o = entry.oracle_module()
    if not o.LIB.exists():
        o.build()
    o.lib()
    return o


@pytest.fixture(scope="session")
def gpu_lib(pkg):
    """The CUDA library, built if needed; the GPU must be usable."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test without a GPU")
    pkg.build()
    pkg.lib()
    return pkg


def golden_cases():
    return json.loads((GOLDEN / "cases.json").read_text())


def load_golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def large_hashes():
    return json.loads((GOLDEN / "hashes.json").read_text())


def real_dtype(real):
    return np.float32 if real == "f32" else np.float64


def initial_state(case, g, real, orc):
    """(s0, init) for a golden case: the stored seeded state, or the equilibrium tuple."""
    if f"s0_{real}" in g:
        return g[f"s0_{real}"], None
    init = [case["u_in"] if v == "u_in" else v for v in case["init"]]
    return None, tuple(init)
