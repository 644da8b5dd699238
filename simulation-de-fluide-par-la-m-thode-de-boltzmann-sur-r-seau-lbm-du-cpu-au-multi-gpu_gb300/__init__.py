"""GB300 (sm_103a) D2Q9 lattice-Boltzmann hot path: Python binding of the C ABI.

`Solver` mirrors the member set of the reference's GPU solver lbm::SolverV3
(src/v3_cuda_opt/solver_v3.hpp:27-57): construct from grid, tau, force and solid mask; then
init_equilibrium / set_inflow_outflow / step / run / timed_run / macroscopic / total_mass /
populations / populations_at / threads / bench_info / nx / ny / solid. Errors follow the
reference: invalid arguments raise ValueError (std::invalid_argument there), CUDA failures raise
RuntimeError (the reference aborts).

The binding loads lib/liblbm_b200.so (built by buildlib.py). There is no CPU fallback: without
the library, or without a GPU, constructing a Solver raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import accuracy, geometry, wake, workloads  # noqa: F401  (re-exported)
from .geometry import make_channel, make_cylinder, poiseuille_force  # noqa: F401

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib" / "liblbm_b200.so"

FP32, FP64, FP16_STORE, BF16_STORE = 0, 1, 2, 3
PRECISIONS = {"fp32": FP32, "fp64": FP64, "fp16": FP16_STORE, "fp16_store": FP16_STORE,
              "bf16": BF16_STORE, "bf16_store": BF16_STORE}
HOST_DTYPE = {FP32: np.float32, FP64: np.float64, FP16_STORE: np.float32, BF16_STORE: np.float32}

OK, ERR_INVALID_ARG, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_DIVERGED, ERR_UNSUPPORTED, ERR_TIMEOUT = range(7)

_lib = None


def build(**kw) -> Path:
    """Compiles the CUDA library (see buildlib.py)."""
    import importlib
    return importlib.import_module(f"{__name__}.buildlib").build(**kw)


def lib() -> C.CDLL:
    """The loaded C library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"CUDA library missing: {LIB_PATH} (run build())")
        L = C.CDLL(str(LIB_PATH))
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        sig = {
            "lbm_version": ([], C.c_char_p),
            "lbm_create": ([i, i, vp, d, d, d, i, C.POINTER(vp)], i),
            "lbm_destroy": ([vp], i),
            "lbm_last_error": ([vp], C.c_char_p),
            "lbm_set_stream": ([vp, vp], i),
            "lbm_set_inflow_outflow": ([vp, d], i),
            "lbm_init_equilibrium": ([vp, d, d, d], i),
            "lbm_set_populations": ([vp, vp], i),
            "lbm_step": ([vp, i], i),
            "lbm_run": ([vp, i], i),
            "lbm_timed_run": ([vp, i, C.POINTER(d)], i),
            "lbm_synchronize": ([vp], i),
            "lbm_get_populations": ([vp, vp], i),
            "lbm_macroscopic": ([vp, vp, vp, vp], i),
            "lbm_total_mass": ([vp, C.POINTER(d)], i),
            "lbm_populations_at": ([vp, i, i, vp], i),
            "lbm_check_finite": ([vp, C.POINTER(i)], i),
            "lbm_device_info": ([vp, C.c_char_p, C.c_size_t], i),
            "lbm_get_shape": ([vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)], i),
            "lbm_set_launch": ([vp, i, i], i),
            "lbm_set_variant": ([vp, i], i),
            "lbm_set_body": ([vp, vp], i),
            "lbm_strips_create": ([i, i, vp, d, d, d, i, i, C.POINTER(vp)], i),
            "lbm_strips_destroy": ([vp], i),
            "lbm_strips_last_error": ([vp], C.c_char_p),
            "lbm_strips_layout": ([vp, vp, vp], i),
            "lbm_strips_set_inflow_outflow": ([vp, d], i),
            "lbm_strips_init_equilibrium": ([vp, d, d, d], i),
            "lbm_strips_set_populations": ([vp, vp], i),
            "lbm_strips_get_populations": ([vp, vp], i),
            "lbm_strips_macroscopic": ([vp, vp, vp, vp], i),
            "lbm_strips_step": ([vp, i], i),
            "lbm_strips_timed_run": ([vp, i, C.POINTER(d)], i),
            "lbm_body_force": ([vp, C.POINTER(d), C.POINTER(d)], i),
            "lbm_state_view": ([vp, C.POINTER(vp), C.POINTER(C.c_longlong), C.POINTER(i)], i),
            "lbm_test_set_consumer_wait_limit": ([C.c_uint], i),
            "lbm_adj_create": ([i, i, vp, d, d, d, i, i, i, C.POINTER(vp)], i),
            "lbm_adj_destroy": ([vp], i),
            "lbm_adj_last_error": ([vp], C.c_char_p),
            "lbm_adj_set_params": ([vp, d, d, d], i),
            "lbm_adj_set_alpha": ([vp, vp], i),
            "lbm_adj_forward": ([vp, vp, i, i, vp], i),
            "lbm_adj_backward": ([vp, vp, vp, vp, vp], i),
            "lbm_adj_get_populations": ([vp, i, vp], i),
            "lbm_adj_step_times": ([vp, C.POINTER(d), C.POINTER(d)], i),
            "lbm_kernel_launches": ([vp, C.POINTER(C.c_longlong)], i),
            "lbm_adj_set_tiles": ([vp, i, i], i),
            "lbm_adj_get_tiles": ([vp, C.POINTER(i), C.POINTER(i)], i),
            "lbm_batch_create": ([i, vp, vp, vp, vp, vp, vp, i, C.POINTER(vp)], i),
            "lbm_batch_destroy": ([vp], i),
            "lbm_batch_last_error": ([vp], C.c_char_p),
            "lbm_batch_init_equilibrium": ([vp, d, d, d], i),
            "lbm_batch_set_populations": ([vp, i, vp], i),
            "lbm_batch_get_populations": ([vp, i, vp], i),
            "lbm_batch_total_mass": ([vp, i, C.POINTER(d)], i),
            "lbm_batch_run": ([vp, i], i),
            "lbm_batch_timed_run": ([vp, i, C.POINTER(d)], i),
            "lbm_batch_run_separate": ([vp, i, C.POINTER(d)], i),
            "lbm_batch_set_launch": ([vp, i, i, i], i),
            "lbm_batch_set_tiles": ([vp, i, i, i], i),
            "lbm_batch_autotune": ([vp, C.c_char_p, C.c_char_p, C.c_size_t], i),
            "lbm_batch_info": ([vp, C.POINTER(i), C.POINTER(C.c_longlong), C.POINTER(i)], i),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class LbmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"lbm error {code}: {msg}")
        self.code = code


def _raise(code: int, msg: str):
    if code == ERR_INVALID_ARG:
        raise ValueError(msg or "invalid argument")
    raise LbmError(code, msg)


class Solver:
    """D2Q9 BGK + Guo + halfway bounce-back solver on one GPU (drop-in for lbm::SolverV3).

    precision: "fp32" / "fp64" (bit-exact with the reference's v0 in float / double),
    "fp16" / "bf16" (16-bit storage of 2^15 g_i with stochastic rounding, FP32 arithmetic).
    Host arrays use the reference's v0 layout and the solver's host dtype (float32, or float64
    for "fp64").
    """

    def __init__(self, nx: int, ny: int, tau: float, force_x: float, force_y: float, solid,
                 precision="fp32"):
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self.dtype = HOST_DTYPE[self.precision]
        self._solid = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
        if self._solid.size != nx * ny:
            raise ValueError("solid mask size does not match the grid")
        self._nx, self._ny = int(nx), int(ny)
        self.tau, self.fx, self.fy = float(tau), float(force_x), float(force_y)
        self._h = C.c_void_p()
        rc = lib().lbm_create(self._nx, self._ny, _ptr(self._solid), self.tau, self.fx, self.fy,
                              self.precision, C.byref(self._h))
        if rc != OK:
            _raise(rc, "lbm_create failed (tau must be > 0.5, nx, ny >= 1)")

    # -- lifetime ----------------------------------------------------------------------------
    def close(self):
        if self._h:
            lib().lbm_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc != OK:
            _raise(rc, (lib().lbm_last_error(self._h) or b"").decode())

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # -- SolverV3 member set ------------------------------------------------------------------
    def init_equilibrium(self, rho0: float, ux0: float, uy0: float):
        self._check(lib().lbm_init_equilibrium(self._h, rho0, ux0, uy0))

    def set_inflow_outflow(self, u_in: float):
        self._check(lib().lbm_set_inflow_outflow(self._h, u_in))

    def set_populations(self, s):
        s = np.ascontiguousarray(s, dtype=self.dtype).reshape(-1)
        if s.size != self._nx * self._ny * 9:
            raise ValueError("populations must hold nx*ny*9 values")
        self._check(lib().lbm_set_populations(self._h, _ptr(s)))

    def step(self, steps: int = 1):
        self._check(lib().lbm_step(self._h, steps))

    def run(self, steps: int):
        self._check(lib().lbm_run(self._h, steps))

    def timed_run(self, steps: int) -> float:
        t = C.c_double(0.0)
        self._check(lib().lbm_timed_run(self._h, steps, C.byref(t)))
        return t.value

    def synchronize(self):
        self._check(lib().lbm_synchronize(self._h))

    def macroscopic(self, out=None):
        n = self._nx * self._ny
        rho, ux, uy = out if out is not None else (np.empty(n, self.dtype) for _ in range(3))
        self._check(lib().lbm_macroscopic(self._h, _ptr(rho), _ptr(ux), _ptr(uy)))
        return rho, ux, uy

    def total_mass(self) -> float:
        m = C.c_double(0.0)
        self._check(lib().lbm_total_mass(self._h, C.byref(m)))
        return m.value

    def populations(self, out=None) -> np.ndarray:
        out = np.empty(self._nx * self._ny * 9, self.dtype) if out is None else out
        self._check(lib().lbm_get_populations(self._h, _ptr(out)))
        return out

    def populations_at(self, x: int, y: int) -> np.ndarray:
        out = np.empty(9, self.dtype)
        self._check(lib().lbm_populations_at(self._h, x, y, _ptr(out)))
        return out

    def check_finite(self) -> bool:
        f = C.c_int(0)
        self._check(lib().lbm_check_finite(self._h, C.byref(f)))
        return bool(f.value)

    def threads(self) -> int:
        return 0

    def kernel_launches(self) -> int:
        """Kernels enqueued for time steps so far (step launches and step-counter updates)."""
        n = C.c_longlong(0)
        self._check(lib().lbm_kernel_launches(self._h, C.byref(n)))
        return n.value

    def bench_info(self) -> str:
        buf = C.create_string_buffer(1024)
        self._check(lib().lbm_device_info(self._h, buf, 1024))
        return buf.value.decode()

    def set_launch(self, block_threads: int, grid_blocks: int = 0):
        self._check(lib().lbm_set_launch(self._h, block_threads, grid_blocks))

    def set_variant(self, variant: int):
        self._check(lib().lbm_set_variant(self._h, variant))

    def set_body(self, body=None):
        """Cells whose momentum-exchange force body_force() sums (a subset of the solid cells;
        None: every solid cell)."""
        if body is None:
            self._check(lib().lbm_set_body(self._h, None))
            return
        b = np.ascontiguousarray(body, dtype=np.uint8).reshape(-1)
        if b.size != self._nx * self._ny:
            raise ValueError("body must hold nx*ny values")
        self._body = b
        self._check(lib().lbm_set_body(self._h, _ptr(b)))

    def body_force(self):
        """(F_x, F_y) on the body by momentum exchange, FP64, lattice units."""
        fx, fy = C.c_double(), C.c_double()
        self._check(lib().lbm_body_force(self._h, C.byref(fx), C.byref(fy)))
        return fx.value, fy.value

    def set_stream(self, stream_handle: int):
        self._check(lib().lbm_set_stream(self._h, C.c_void_p(stream_handle)))

    def nx(self) -> int:
        return self._nx

    def ny(self) -> int:
        return self._ny

    def solid(self) -> np.ndarray:
        return self._solid


class Adjoint:
    """Forward/backward pair of the adjoint (C ABI lbm_adj_*): gradients of
    J = mean over the last `window` states of the mean u_x over fluid cells, with respect to tau,
    the body force and a per-cell Brinkman drag field alpha (F_tot = F - alpha rho u). A batch of
    instances shares geometry, tau and force and has one alpha field each. Closed domains."""

    def __init__(self, nx, ny, tau, fx, fy, solid, precision="fp64", batch=1,
                 checkpoint_every=100):
        self.nx, self.ny, self.batch = int(nx), int(ny), int(batch)
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self.dtype = HOST_DTYPE[self.precision]
        self._solid = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
        self._h = C.c_void_p()
        rc = lib().lbm_adj_create(self.nx, self.ny, _ptr(self._solid), tau, fx, fy, self.precision,
                                  self.batch, checkpoint_every, C.byref(self._h))
        if rc != OK:
            _raise(rc, "lbm_adj_create failed")

    def _check(self, rc):
        if rc != OK:
            _raise(rc, (lib().lbm_adj_last_error(self._h) or b"").decode())

    def close(self):
        if self._h:
            lib().lbm_adj_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_params(self, tau, fx, fy):
        self._check(lib().lbm_adj_set_params(self._h, tau, fx, fy))

    def set_alpha(self, alpha):
        """alpha: (batch, nx*ny) or (nx*ny,) for batch 1, or None for alpha = 0."""
        if alpha is None:
            self._check(lib().lbm_adj_set_alpha(self._h, None))
            return
        self._alpha = np.ascontiguousarray(alpha, dtype=np.float64).reshape(-1)
        if self._alpha.size != self.batch * self.nx * self.ny:
            raise ValueError("alpha must hold batch * nx * ny values")
        self._check(lib().lbm_adj_set_alpha(self._h, _ptr(self._alpha)))

    def forward(self, steps, window, s0=None) -> np.ndarray:
        J = np.zeros(self.batch, np.float64)
        if s0 is not None:
            s0 = np.ascontiguousarray(s0, dtype=self.dtype).reshape(-1)
            if s0.size != self.batch * self.nx * self.ny * 9:
                raise ValueError("s0 must hold batch * nx * ny * 9 values")
        self._check(lib().lbm_adj_forward(self._h, None if s0 is None else _ptr(s0), steps,
                                          window, _ptr(J)))
        return J

    def backward(self, want_alpha=True):
        """Returns dict(tau, fx, fy: arrays of batch values, alpha: (batch, nx*ny) or None)."""
        b = self.batch
        dt, dfx, dfy = (np.zeros(b) for _ in range(3))
        da = np.zeros(b * self.nx * self.ny) if want_alpha else None
        self._check(lib().lbm_adj_backward(self._h, _ptr(dt), _ptr(dfx), _ptr(dfy),
                                           None if da is None else _ptr(da)))
        return {"tau": dt, "fx": dfx, "fy": dfy,
                "alpha": None if da is None else da.reshape(b, -1)}

    def populations(self, instance=0) -> np.ndarray:
        out = np.empty(self.nx * self.ny * 9, self.dtype)
        self._check(lib().lbm_adj_get_populations(self._h, instance, _ptr(out)))
        return out

    def step_times(self):
        f, b = C.c_double(), C.c_double()
        self._check(lib().lbm_adj_step_times(self._h, C.byref(f), C.byref(b)))
        return f.value, b.value

    def set_tiles(self, forward_cells=0, backward_cells=0):
        """Cells per consumer lane of the forward / backward kernels: 1 (256-cell tiles), 2
        (512-cell tiles, FP32 only) or 0 (automatic). Results do not depend on it."""
        self._check(lib().lbm_adj_set_tiles(self._h, forward_cells, backward_cells))

    def tiles(self):
        f, b = C.c_int(), C.c_int()
        self._check(lib().lbm_adj_get_tiles(self._h, C.byref(f), C.byref(b)))
        return f.value, b.value


class Batch:
    """Ensemble of independent closed channels of uneven sizes stepped by one persistent launch
    per time step (C ABI lbm_batch_*). specs: list of dict(nx, ny, mask, tau, fx[, fy])."""

    def __init__(self, specs, precision="fp32"):
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self.dtype = HOST_DTYPE[self.precision]
        self.specs = specs
        n = len(specs)
        self._nx = np.array([s["nx"] for s in specs], np.int32)
        self._ny = np.array([s["ny"] for s in specs], np.int32)
        self._masks = [np.ascontiguousarray(s["mask"], np.uint8).reshape(-1) for s in specs]
        ptrs = (C.c_void_p * n)(*[m.ctypes.data for m in self._masks])
        self._tau = np.array([s["tau"] for s in specs], np.float64)
        self._fx = np.array([s["fx"] for s in specs], np.float64)
        self._fy = np.array([s.get("fy", 0.0) for s in specs], np.float64)
        self._h = C.c_void_p()
        rc = lib().lbm_batch_create(n, _ptr(self._nx), _ptr(self._ny), C.cast(ptrs, C.c_void_p),
                                    _ptr(self._tau), _ptr(self._fx), _ptr(self._fy),
                                    self.precision, C.byref(self._h))
        if rc != OK:
            _raise(rc, "lbm_batch_create failed")

    def _check(self, rc):
        if rc != OK:
            _raise(rc, (lib().lbm_batch_last_error(self._h) or b"").decode())

    def close(self):
        if self._h:
            lib().lbm_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.specs)

    def init_equilibrium(self, rho0, ux0, uy0):
        self._check(lib().lbm_batch_init_equilibrium(self._h, rho0, ux0, uy0))

    def set_populations(self, k, s):
        s = np.ascontiguousarray(s, dtype=self.dtype).reshape(-1)
        if s.size != int(self._nx[k]) * int(self._ny[k]) * 9:
            raise ValueError("populations must hold nx*ny*9 values")
        self._check(lib().lbm_batch_set_populations(self._h, k, _ptr(s)))

    def populations(self, k) -> np.ndarray:
        out = np.empty(int(self._nx[k]) * int(self._ny[k]) * 9, self.dtype)
        self._check(lib().lbm_batch_get_populations(self._h, k, _ptr(out)))
        return out

    def total_mass(self, k) -> float:
        m = C.c_double()
        self._check(lib().lbm_batch_total_mass(self._h, k, C.byref(m)))
        return m.value

    def run(self, steps):
        self._check(lib().lbm_batch_run(self._h, steps))

    def timed_run(self, steps) -> float:
        t = C.c_double()
        self._check(lib().lbm_batch_timed_run(self._h, steps, C.byref(t)))
        return t.value

    def run_separate(self, steps) -> float:
        t = C.c_double()
        self._check(lib().lbm_batch_run_separate(self._h, steps, C.byref(t)))
        return t.value

    def set_launch(self, cells_per_thread=0, block_threads=256, grid_blocks=0):
        self._check(lib().lbm_batch_set_launch(self._h, cells_per_thread, block_threads, grid_blocks))

    def set_tiles(self, consumer_warps=None, passes=None, stages=None):
        """Ring-kernel tile shape (and selects the ring kernel): 8x2, 4x2, 4x1 or 2x2 with 2 or
        4 ring stages. Arguments left out take the library's default for this precision, the
        shape used without a call: 4x2 with 4 stages, and 8x2 with 2 stages for FP64."""
        w, c, s = (8, 2, 2) if self.precision == PRECISIONS["fp64"] else (4, 2, 4)
        self._check(lib().lbm_batch_set_tiles(
            self._h, w if consumer_warps is None else consumer_warps,
            c if passes is None else passes, s if stages is None else stages))

    def autotune(self, cache_path=None) -> str:
        buf = C.create_string_buffer(4096)
        self._check(lib().lbm_batch_autotune(self._h, None if cache_path is None else str(cache_path).encode(),
                                             buf, 4096))
        return buf.value.decode()

    def info(self):
        n, cells, items = C.c_int(), C.c_longlong(), C.c_int()
        self._check(lib().lbm_batch_info(self._h, C.byref(n), C.byref(cells), C.byref(items)))
        return {"count": n.value, "cells": cells.value, "chunks": items.value}


class Strips:
    """The lattice as horizontal strips with ghost rows and a device halo exchange (C ABI
    lbm_strips_*): the reference's multi-rank solver (src/v4_mpi_cuda) with every strip on one
    GPU. Same results as Solver on the whole lattice, for any number of strips."""

    def __init__(self, nx, ny, tau, fx, fy, solid, strips, precision="fp32"):
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self.dtype = HOST_DTYPE[self.precision]
        self._nx, self._ny, self.strips = int(nx), int(ny), int(strips)
        self._solid = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
        if self._solid.size != self._nx * self._ny:
            raise ValueError("solid must hold nx*ny values")
        self._h = C.c_void_p()
        rc = lib().lbm_strips_create(self._nx, self._ny, _ptr(self._solid), tau, fx, fy,
                                     self.precision, self.strips, C.byref(self._h))
        if rc != OK:
            _raise(rc, "lbm_strips_create failed")

    def _check(self, rc):
        if rc != OK:
            _raise(rc, (lib().lbm_strips_last_error(self._h) or b"").decode())

    def close(self):
        if self._h:
            lib().lbm_strips_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def layout(self):
        y0 = np.zeros(self.strips, np.int32)
        n = np.zeros(self.strips, np.int32)
        self._check(lib().lbm_strips_layout(self._h, _ptr(y0), _ptr(n)))
        return y0, n

    def set_inflow_outflow(self, u_in):
        self._check(lib().lbm_strips_set_inflow_outflow(self._h, u_in))

    def init_equilibrium(self, rho0, ux0, uy0):
        self._check(lib().lbm_strips_init_equilibrium(self._h, rho0, ux0, uy0))

    def set_populations(self, s):
        s = np.ascontiguousarray(s, dtype=self.dtype).reshape(-1)
        if s.size != self._nx * self._ny * 9:
            raise ValueError("populations must hold nx*ny*9 values")
        self._check(lib().lbm_strips_set_populations(self._h, _ptr(s)))

    def populations(self):
        out = np.empty(self._nx * self._ny * 9, self.dtype)
        self._check(lib().lbm_strips_get_populations(self._h, _ptr(out)))
        return out

    def macroscopic(self):
        n = self._nx * self._ny
        rho, ux, uy = (np.empty(n, self.dtype) for _ in range(3))
        self._check(lib().lbm_strips_macroscopic(self._h, _ptr(rho), _ptr(ux), _ptr(uy)))
        return rho, ux, uy

    def run(self, steps):
        self._check(lib().lbm_strips_step(self._h, steps))

    def timed_run(self, steps) -> float:
        t = C.c_double()
        self._check(lib().lbm_strips_timed_run(self._h, steps, C.byref(t)))
        return t.value


def version() -> str:
    return lib().lbm_version().decode()
