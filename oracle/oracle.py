"""ctypes binding of the CPU oracle (oracle/lbm_oracle.c) and, where it was built, of the
reference's own v0/v1 solvers (oracle/_ref/libref_{f32,f64}.so, see oracle/Makefile).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg, always as the checker or as the timed CPU port of the reference. The product
(the CUDA library and its Python binding) never imports this module.

Layouts: "S" is the reference v0 state, post-streaming populations in array-of-structures order
s[(y*nx + x)*9 + i]; "R" is the pull state, post-collision populations in structure-of-arrays
planes r[i*nx*ny + y*nx + x].
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_DIR = HERE / "_ref"
# The reference tree: $LBM_REFERENCE_DIR, default /root/reference. Where it is absent (a
# machine that received only this repository), oracle/Makefile builds from the copy that
# `make stage` left in oracle/_ref/tree.
REFERENCE_DIR = Path(os.environ.get("LBM_REFERENCE_DIR", "/root/reference"))
STAGED_TREE = REF_DIR / "tree"

_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def reference_tree() -> Path | None:
    """The reference tree the Makefile reads (the original, else the staged copy), or None."""
    for t in (REFERENCE_DIR, STAGED_TREE):
        if (t / "src" / "v0_cpu" / "solver_v0.cpp").exists():
            return t
    return None


def _make(*targets: str, env: dict | None = None) -> None:
    subprocess.run(["make", "-s", "-C", str(HERE), f"-j{os.cpu_count() or 4}", *targets],
                   check=True, env=env)


def build(ref: bool = False, gpu: bool = False) -> None:
    """Compiles the oracle with gcc (flags as oracle/Makefile); with ref=True, also the
    reference's own CPU solvers into oracle/_ref (from the reference tree, staging a copy of
    its files into oracle/_ref/tree when the original is present), and with gpu=True the
    reference's own GPU solver v3 (needs nvcc)."""
    LIB.parent.mkdir(exist_ok=True)
    src = HERE / "lbm_oracle.c"
    stale = not LIB.exists() or any(p.stat().st_mtime > LIB.stat().st_mtime
                                     for p in (src, HERE / "lbm_oracle_impl.h"))
    if stale:
        tmp = LIB.with_suffix(".so.tmp")
        subprocess.run([os.environ.get("CC", "gcc"), "-std=c11", "-O3", "-ffp-contract=off",
                        "-fno-trapping-math", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp),
                        str(src)], check=True)
        os.replace(tmp, LIB)
    if ref and reference_tree() is not None:
        targets = ["ref"] + (["ref-gpu"] if gpu else [])
        if (REFERENCE_DIR / "src").exists():
            targets.insert(0, "stage")
        _make(*targets)


def build_consumers(lib_dir: Path) -> None:
    """Builds the reference's own v3 test programs against the library in lib_dir
    (oracle/Makefile `consumers`)."""
    _make("consumers", env={**os.environ, "LBM_LIB": str(lib_dir)})


def _dtype(real: str):
    return {"f32": np.float32, "f64": np.float64}[real]


class _Lib:
    def __init__(self, path: Path):
        self.lib = C.CDLL(str(path))
        L = self.lib
        L.oracle_seeded_uniform.restype = C.c_double
        L.oracle_seeded_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_double]
        L.oracle_seeded_fill.restype = None
        L.oracle_seeded_fill.argtypes = [C.c_uint64, C.c_double, C.c_uint64,
                                         np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")]
        L.oracle_max_threads.restype = C.c_int
        for real in ("f32", "f64"):
            t = C.c_float if real == "f32" else C.c_double
            p = np.ctypeslib.ndpointer(_dtype(real), flags="C_CONTIGUOUS")
            fn = lambda name: getattr(L, f"{name}_{real}")  # noqa: E731
            fn("oracle_equilibrium_state").argtypes = [t, t, t, p]
            fn("oracle_init_equilibrium").argtypes = [C.c_int, C.c_int, _u8p, t, t, t, p]
            fn("oracle_v0_run").restype = C.c_int
            fn("oracle_v0_run").argtypes = [C.c_int, C.c_int, _u8p, t, t, t, C.c_int, t, p,
                                            C.c_int]
            fn("oracle_macroscopic").argtypes = [C.c_int, C.c_int, _u8p, t, t, p, p, p, p]
            fn("oracle_total_mass").restype = C.c_double
            fn("oracle_total_mass").argtypes = [C.c_int, C.c_int, _u8p, p]
            fn("oracle_r_to_s").argtypes = [C.c_int, C.c_int, _u8p, C.c_int, t, p, p]
            fn("oracle_s_to_r").argtypes = [C.c_int, C.c_int, _u8p, C.c_int, p, p]
            fn("oracle_pull_run").restype = C.c_int
            fn("oracle_pull_run").argtypes = [C.c_int, C.c_int, _u8p, t, t, t, C.c_int, t, p,
                                              C.c_int, C.c_int]
            fn("oracle_pull_steps").restype = C.c_int
            fn("oracle_pull_steps").argtypes = [C.c_int, C.c_int, _u8p, t, t, t, C.c_int, t, p, p,
                                                C.c_int, C.c_int]
            fn("oracle_first_touch").argtypes = [C.c_int, C.c_int, p]
            fn("oracle_seeded_state").argtypes = [C.c_uint64, C.c_double, C.c_int, C.c_int,
                                                  _u8p, p]


_lib: _Lib | None = None


def lib() -> _Lib:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = _Lib(LIB)
    return _lib


def _f(name: str, real: str):
    return getattr(lib().lib, f"{name}_{real}")


def _mask(solid) -> np.ndarray:
    return np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)


# --------------------------------------------------------------------------------------------
# Oracle API (own restatement)
# --------------------------------------------------------------------------------------------
def seeded_uniform(seed: int, count: int, amp: float) -> np.ndarray:
    out = np.empty(count, np.float64)
    lib().lib.oracle_seeded_fill(seed, amp, count, out)
    return out


def seeded_state(seed, amp, nx, ny, solid, real="f32") -> np.ndarray:
    s = np.empty(nx * ny * 9, _dtype(real))
    _f("oracle_seeded_state", real)(seed, amp, nx, ny, _mask(solid), s)
    return s


def equilibrium_state(rho0, ux0, uy0, real="f32") -> np.ndarray:
    eq = np.empty(9, _dtype(real))
    _f("oracle_equilibrium_state", real)(rho0, ux0, uy0, eq)
    return eq


def init_equilibrium(nx, ny, solid, rho0, ux0, uy0, real="f32") -> np.ndarray:
    s = np.empty(nx * ny * 9, _dtype(real))
    _f("oracle_init_equilibrium", real)(nx, ny, _mask(solid), rho0, ux0, uy0, s)
    return s


def v0_run(nx, ny, solid, tau, fx, fy, s, steps, open_x=False, u_in=0.0, real="f32"):
    """Sequential push solver (reference v0 restated); returns the new S."""
    s = np.array(s, dtype=_dtype(real), copy=True).reshape(-1)
    rc = _f("oracle_v0_run", real)(nx, ny, _mask(solid), tau, fx, fy, int(open_x), u_in, s, steps)
    if rc != 0:
        raise MemoryError("oracle_v0_run: allocation failed")
    return s


def pull_run(nx, ny, solid, tau, fx, fy, r, steps, open_x=False, u_in=0.0, real="f32",
             threads=0):
    """OpenMP pull solver (reference v1 restated) on the R state, in place; returns r."""
    rc = _f("oracle_pull_run", real)(nx, ny, _mask(solid), tau, fx, fy, int(open_x), u_in, r,
                                     steps, threads)
    if rc != 0:
        raise MemoryError("oracle_pull_run: allocation failed")
    return r


class PullBuffers:
    """Two SoA buffers for timed pull runs (no allocation inside the timed region)."""

    def __init__(self, nx, ny, solid, r0, real="f32"):
        self.nx, self.ny, self.real = nx, ny, real
        self.solid = _mask(solid)
        self.a = np.empty(nx * ny * 9, _dtype(real))
        self.b = np.empty_like(self.a)
        _f("oracle_first_touch", real)(nx, ny, self.a)
        _f("oracle_first_touch", real)(nx, ny, self.b)
        self.a[:] = r0

    def run(self, tau, fx, fy, steps, open_x=False, u_in=0.0, threads=0):
        which = _f("oracle_pull_steps", self.real)(self.nx, self.ny, self.solid, tau, fx, fy,
                                                   int(open_x), u_in, self.a, self.b, steps,
                                                   threads)
        if which:
            self.a, self.b = self.b, self.a
        return self.a


def s_to_r(nx, ny, solid, s, open_x=False, real="f32") -> np.ndarray:
    r = np.empty(nx * ny * 9, _dtype(real))
    _f("oracle_s_to_r", real)(nx, ny, _mask(solid), int(open_x),
                              np.ascontiguousarray(s, _dtype(real)).reshape(-1), r)
    return r


def r_to_s(nx, ny, solid, r, open_x=False, u_in=0.0, real="f32") -> np.ndarray:
    s = np.empty(nx * ny * 9, _dtype(real))
    _f("oracle_r_to_s", real)(nx, ny, _mask(solid), int(open_x), u_in,
                              np.ascontiguousarray(r, _dtype(real)).reshape(-1), s)
    return s


def macroscopic(nx, ny, solid, fx, fy, s, real="f32"):
    dt = _dtype(real)
    rho, ux, uy = (np.empty(nx * ny, dt) for _ in range(3))
    _f("oracle_macroscopic", real)(nx, ny, _mask(solid), fx, fy,
                                   np.ascontiguousarray(s, dt).reshape(-1), rho, ux, uy)
    return rho, ux, uy


def total_mass(nx, ny, solid, s, real="f32") -> float:
    return _f("oracle_total_mass", real)(nx, ny, _mask(solid),
                                         np.ascontiguousarray(s, _dtype(real)).reshape(-1))


CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])
OPP = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6])
W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)


def body_force(nx, ny, solid, body, s, open_x=False):
    """Momentum-exchange force on `body` from a v0 post-streaming state S, in FP64 (numpy).

    Halfway bounce-back on stationary walls: a fluid cell x whose neighbour x + c_i is a body
    cell sends f*_i(x) (post-collision) into the wall and receives it back as S_opp(i)(x), so the
    link carries 2 c_i f*_i(x) = 2 c_i (S_opp(i)(x) + w_i) in the shifted variables. Written from
    the method (the reference computes no force); the solver's device sum is checked against it.
    Links leaving an open x boundary carry nothing."""
    solid = np.asarray(solid, bool).reshape(ny, nx)
    body = np.asarray(body, bool).reshape(ny, nx)
    st = np.asarray(s, np.float64).reshape(ny, nx, 9)
    fx = fy = 0.0
    ys, xs = np.mgrid[0:ny, 0:nx]
    fluid = ~solid
    for i in range(1, 9):
        xn, yn = xs + CX[i], (ys + CY[i]) % ny
        inside = (xn >= 0) & (xn < nx) if open_x else np.ones_like(fluid)
        xn = xn % nx
        link = fluid & inside & body[yn, xn]
        f = st[..., OPP[i]][link] + W[i]
        fx += 2.0 * CX[i] * f.sum()
        fy += 2.0 * CY[i] * f.sum()
    return fx, fy


def max_threads() -> int:
    return lib().lib.oracle_max_threads()


# --------------------------------------------------------------------------------------------
# The reference itself (only where oracle/_ref was built from the reference tree)
# --------------------------------------------------------------------------------------------
class Reference:
    """The reference's own SolverV0 / SolverV1, compiled from its unmodified sources."""

    def __init__(self, real="f32"):
        path = REF_DIR / f"libref_{real}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        self.real = real
        self.dt = _dtype(real)
        self.lib = C.CDLL(str(path))
        t = C.c_float if real == "f32" else C.c_double
        p = np.ctypeslib.ndpointer(self.dt, flags="C_CONTIGUOUS")
        dp = C.POINTER(C.c_double)
        common = [C.c_int, C.c_int, _u8p, t, t, t, C.c_int, t, C.c_int, t, t, t, p, C.c_int,
                  p, p, p, dp]
        self.lib.ref_v0_run.argtypes = common
        self.lib.ref_v0_run.restype = C.c_int
        self.lib.ref_v1_run.argtypes = common + [C.c_int]
        self.lib.ref_v1_run.restype = C.c_int
        assert self.lib.ref_real_size() == np.dtype(self.dt).itemsize

        for name in ("ref_v0_bench", "ref_v1_bench"):
            fn = getattr(self.lib, name)
            fn.restype = C.c_int
            fn.argtypes = [C.c_int, C.c_int, _u8p, t, t, t, p, C.c_int, C.c_int, C.c_int] + (
                [C.c_int] if name == "ref_v1_bench" else []) + [dp]

    @staticmethod
    def available(real="f32") -> bool:
        return (REF_DIR / f"libref_{real}.so").exists()

    def bench(self, version, nx, ny, solid, tau, fx, fy, s0, steps, *, warmup=1, reps=1,
              threads=0):
        """Seconds of each of `reps` timed runs of `steps` steps of v0 or v1 (threads: OpenMP
        threads of v1, 0 = all) from the post-streaming state s0, after `warmup` steps."""
        sec = (C.c_double * reps)()
        s = np.ascontiguousarray(s0, self.dt).reshape(-1)
        args = [nx, ny, _mask(solid), tau, fx, fy, s, warmup, steps, reps]
        if version == "v0":
            rc = self.lib.ref_v0_bench(*args, sec)
        else:
            rc = self.lib.ref_v1_bench(*args, threads, sec)
        if rc != 0:
            raise ValueError("the reference solver rejected its arguments")
        return list(sec)

    def run(self, version, nx, ny, solid, tau, fx, fy, steps, *, s0=None, init=(1.0, 0.0, 0.0),
            open_x=False, u_in=0.0, threads=0):
        """Runs v0 or v1; returns dict(s, rho, ux, uy, mass). s0 (v0 layout) overrides init."""
        n = nx * ny
        s = np.zeros(n * 9, self.dt) if s0 is None else np.array(s0, self.dt, copy=True)
        rho, ux, uy = (np.empty(n, self.dt) for _ in range(3))
        mass = C.c_double(0.0)
        args = [nx, ny, _mask(solid), tau, fx, fy, int(open_x), u_in, int(s0 is None),
                init[0], init[1], init[2], s, steps, rho, ux, uy, C.byref(mass)]
        if version == "v0":
            rc = self.lib.ref_v0_run(*args)
        else:
            rc = self.lib.ref_v1_run(*args, threads)
        if rc != 0:
            raise ValueError("the reference solver rejected its arguments")
        return {"s": s, "rho": rho, "ux": ux, "uy": uy, "mass": mass.value}


class ReferenceV3:
    """The reference's own GPU solver SolverV3 (src/v3_cuda_opt/solver_v3.cu, compiled from the
    unmodified source for sm_103a with --fmad=false by oracle/Makefile `ref-gpu`), run through
    oracle/ref_v3_shim.cu. Needs a GPU; aborts the process on a CUDA error, as the reference
    does."""

    def __init__(self, real="f32"):
        path = REF_DIR / f"libref_v3_{real}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        self.real = real
        self.dt = _dtype(real)
        self.lib = C.CDLL(str(path))
        t = C.c_float if real == "f32" else C.c_double
        p = np.ctypeslib.ndpointer(self.dt, flags="C_CONTIGUOUS")
        dp = C.POINTER(C.c_double)
        self.lib.ref_v3_run.argtypes = [C.c_int, C.c_int, _u8p, t, t, t, C.c_int, t, C.c_int, t,
                                        t, t, p, C.c_int, p, p, p, dp, C.c_char_p]
        self.lib.ref_v3_run.restype = C.c_int
        self.lib.ref_v3_bench.argtypes = [C.c_int, C.c_int, _u8p, t, t, t, p, C.c_int, C.c_int,
                                          C.c_int, dp, C.c_void_p, C.c_char_p, C.c_size_t,
                                          C.c_char_p]
        self.lib.ref_v3_bench.restype = C.c_int
        assert self.lib.ref_v3_real_size() == np.dtype(self.dt).itemsize

    @staticmethod
    def available(real="f32") -> bool:
        return (REF_DIR / f"libref_v3_{real}.so").exists()

    def run(self, nx, ny, solid, tau, fx, fy, steps, *, s0=None, init=(1.0, 0.0, 0.0),
            open_x=False, u_in=0.0, variant=None):
        """Same contract as Reference.run; variant: soa_push, soa_pull or soa_pull_opt (the
        reference's default)."""
        n = nx * ny
        s = np.zeros(n * 9, self.dt) if s0 is None else np.array(s0, self.dt, copy=True)
        rho, ux, uy = (np.empty(n, self.dt) for _ in range(3))
        mass = C.c_double(0.0)
        rc = self.lib.ref_v3_run(nx, ny, _mask(solid), tau, fx, fy, int(open_x), u_in,
                                 int(s0 is None), init[0], init[1], init[2], s, steps, rho, ux,
                                 uy, C.byref(mass), None if variant is None else variant.encode())
        if rc != 0:
            raise ValueError("the reference solver rejected its arguments")
        return {"s": s, "rho": rho, "ux": ux, "uy": uy, "mass": mass.value}

    def bench(self, nx, ny, solid, tau, fx, fy, s0, steps, *, warmup=10, reps=1,
              state_out=False, variant=None):
        """(seconds of each timed_run(steps), bench_info, final populations or None) after
        `warmup` steps from the post-streaming state s0."""
        sec = (C.c_double * reps)()
        out = np.empty(nx * ny * 9, self.dt) if state_out else None
        info = C.create_string_buffer(1024)
        rc = self.lib.ref_v3_bench(nx, ny, _mask(solid), tau, fx, fy,
                                   np.ascontiguousarray(s0, self.dt).reshape(-1), warmup, steps,
                                   reps, sec, None if out is None else out.ctypes.data, info,
                                   1024, None if variant is None else variant.encode())
        if rc != 0:
            raise ValueError("the reference solver rejected its arguments")
        return list(sec), info.value.decode(), out
