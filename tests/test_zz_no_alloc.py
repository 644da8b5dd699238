"""lbm_total_mass_noalloc: the mass reduction for callers that cannot let the library allocate.

Such callers (a host that owns all device memory through its own pool, a loop that cannot take
the synchronisation of cudaMalloc/cudaFree) pass every buffer themselves: here the test, as the
caller, provides the byte mask and the one-double output in device memory (allocated by torch
on the caller's side) and the population state is the solver's own, reached through
lbm_state_view. The entry point is called through the C ABI, twice in a row on the same state
and once more after further steps, and each result is checked against lbm_total_mass within
the relative tolerance the other mass checks use (1e-12: the two reductions add the same values
in different orders). The device's free memory (cudaMemGetInfo) is the same before and after
every call that follows the first, which loads the library's kernels and its static scratch.
The file is named to be collected last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-12


def _noalloc(lib, state, precision, nx, ny, pitch, plane, solid_dev, out_dev):
    f = lib.lbm_total_mass_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
    f.restype = C.c_int
    err = C.create_string_buffer(256)
    rc = f(state, precision, nx, ny, pitch, plane, solid_dev, out_dev, None, err, 256)
    return rc, err.value.decode()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_noalloc_mass_matches_total_mass(gpu_lib, orc, precision):
    import torch

    pkg = gpu_lib
    lib = pkg.lib()
    nx, ny = 301, 97
    mask = pkg.geometry.add_disc(pkg.make_channel(nx, ny), nx, ny, 80.0, 45.0, 21.0)
    real = "f32" if precision == "fp32" else "f64"
    s0 = orc.seeded_state(4242, 1e-3, nx, ny, mask, real)
    solid_dev = torch.from_numpy(mask.copy()).cuda()
    out_dev = torch.zeros(1, dtype=torch.float64, device="cuda")
    with pkg.Solver(nx, ny, 0.7, 2e-6, 0.0, mask, precision=precision) as s:
        s.set_populations(s0)
        s.run(25)
        for call in range(2):  # two calls in a row on the same state
            want = s.total_mass()
            state, plane, pitch = C.c_void_p(), C.c_longlong(), C.c_int()
            assert lib.lbm_state_view(s.handle, C.byref(state), C.byref(plane), C.byref(pitch)) == 0
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            rc, msg = _noalloc(lib, state, pkg.PRECISIONS[precision], nx, ny, pitch.value,
                               plane.value, C.c_void_p(solid_dev.data_ptr()),
                               C.c_void_p(out_dev.data_ptr()))
            assert rc == 0, msg
            torch.cuda.synchronize()
            if call > 0:
                assert torch.cuda.mem_get_info()[0] == free_before
            assert out_dev.item() == pytest.approx(want, rel=REL)
        s.run(40)  # the scratch keeps the last call's rows; a new state must not see them
        want = s.total_mass()
        assert lib.lbm_state_view(s.handle, C.byref(state), C.byref(plane), C.byref(pitch)) == 0
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc, msg = _noalloc(lib, state, pkg.PRECISIONS[precision], nx, ny, pitch.value,
                           plane.value, C.c_void_p(solid_dev.data_ptr()),
                           C.c_void_p(out_dev.data_ptr()))
        assert rc == 0, msg
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before
        assert out_dev.item() == pytest.approx(want, rel=REL)


def test_noalloc_rejects_too_many_rows(gpu_lib):
    lib = gpu_lib.lib()
    rows = 16385  # one more than LBM_NOALLOC_MAX_ROWS
    rc, msg = _noalloc(lib, C.c_void_p(16), 0, 8, rows, 8, 8 * rows, C.c_void_p(16),
                       C.c_void_p(16))
    assert rc == gpu_lib.ERR_INVALID_ARG and "LBM_NOALLOC_MAX_ROWS" in msg
