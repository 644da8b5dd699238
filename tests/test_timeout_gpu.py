"""The failure path of the step kernels' bounded waits, made to run out on purpose (GPU).

A ring step kernel's consumer warps wait for each staged tile. lbm_test_set_consumer_wait_limit
shortens their first wait to a few non-blocking polls, so that it runs out although the data
arrives: the kernel sets its error flag, lets every copy it issued land and finishes without
computing the rest of its tiles (every wait still ends). The test then checks the host side of
the failure (solver.cu lbm_synchronize / check_step_flag): lbm_run returns LBM_ERR_TIMEOUT,
lbm_last_error names it, the flag is cleared (the next synchronising call is clean), and after
the state is set again a normal run reproduces the reference's golden vectors bit for bit.
No wait that never completes and no GPU fault is involved.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, initial_state, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("variant", [12, 17, 20])
@pytest.mark.parametrize("real", ["f32", "f64"])
def test_wait_that_runs_out_reports_timeout_and_recovers(gpu_lib, orc, variant, real):
    pkg = gpu_lib
    lib = pkg.lib()
    name = "ref_obstacle"
    case = golden_cases()[name]
    g = load_golden(name)
    nx, ny = case["nx"], case["ny"]
    s0, init = initial_state(case, g, real, orc)
    prec = {"f32": "fp32", "f64": "fp64"}[real]

    def reset(s):
        if s0 is None:
            s.init_equilibrium(*init)
        else:
            s.set_populations(s0)

    with pkg.Solver(nx, ny, case[f"tau_{real}"], case["fx"], case["fy"], g["mask"],
                    precision=prec) as s:
        s.set_variant(variant)
        reset(s)
        assert lib.lbm_test_set_consumer_wait_limit(1) == pkg.OK
        try:
            rc = lib.lbm_run(s.handle, 20)
        finally:
            assert lib.lbm_test_set_consumer_wait_limit(0) == pkg.OK
        assert rc == pkg.ERR_TIMEOUT
        assert "gave up waiting" in lib.lbm_last_error(s.handle).decode()
        assert lib.lbm_synchronize(s.handle) == pkg.OK  # the flag was cleared
        reset(s)
        s.run(case["steps"])
        pops = s.populations()
    assert np.array_equal(pops, g[f"s_{real}"])
