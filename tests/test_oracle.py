"""The oracle is pinned against the reference's own solvers (CPU only).

Golden vectors in tests/golden/ were produced by the reference's v0 and v1 sources compiled
unmodified (tests/golden/make_golden.py, which checked v0 == v1 on every case). These tests
check, bit for bit, that the oracle's v0 restatement (push, AoS) and its v1 restatement (pull,
SoA, OpenMP) reproduce them, and, where the reference tree was built here (oracle/_ref), compare
with the live reference on extra random cases.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, initial_state, load_golden, real_dtype

CASES = sorted(golden_cases())
REALS = ("f32", "f64")


def _run_oracle_v0(orc, case, g, real):
    nx, ny, mask = case["nx"], case["ny"], g["mask"]
    s0, init = initial_state(case, g, real, orc)
    if s0 is None:
        s0 = orc.init_equilibrium(nx, ny, mask, *init, real=real)
    return orc.v0_run(nx, ny, mask, case[f"tau_{real}"], case["fx"], case["fy"], s0,
                      case["steps"], open_x=bool(case.get("open_x")), u_in=case.get("u_in", 0.0),
                      real=real)


def _numeric_equal(a, b):
    return a.shape == b.shape and bool(np.all(a == b))


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("name", CASES)
def test_oracle_v0_matches_reference(orc, name, real):
    case = golden_cases()[name]
    g = load_golden(name)
    s = _run_oracle_v0(orc, case, g, real)
    assert _numeric_equal(s, g[f"s_{real}"]), "populations differ from the reference v0"
    rho, ux, uy = orc.macroscopic(case["nx"], case["ny"], g["mask"], case["fx"], case["fy"], s, real)
    for k, a in (("rho", rho), ("ux", ux), ("uy", uy)):
        assert _numeric_equal(a, g[f"{k}_{real}"]), f"{k} differs from the reference"
    assert orc.total_mass(case["nx"], case["ny"], g["mask"], s, real) == g[f"mass_{real}"]


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("name", CASES)
def test_oracle_pull_matches_reference(orc, name, real):
    case = golden_cases()[name]
    g = load_golden(name)
    nx, ny, mask = case["nx"], case["ny"], g["mask"]
    open_x, u_in = bool(case.get("open_x")), case.get("u_in", 0.0)
    s0, init = initial_state(case, g, real, orc)
    if s0 is None:
        s0 = orc.init_equilibrium(nx, ny, mask, *init, real=real)
    r = orc.s_to_r(nx, ny, mask, s0, open_x=open_x, real=real)
    orc.pull_run(nx, ny, mask, case[f"tau_{real}"], case["fx"], case["fy"], r, case["steps"],
                 open_x=open_x, u_in=u_in, real=real, threads=3)
    s = orc.r_to_s(nx, ny, mask, r, open_x=open_x, u_in=u_in, real=real)
    assert _numeric_equal(s, g[f"s_{real}"])


def splitmix_numpy(seed: int, count: int, amp: float) -> np.ndarray:
    """Independent numpy restatement of the counter-based SplitMix64 stream."""
    k = np.arange(1, count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    return -amp + 2.0 * amp * u


def test_seeded_generator(orc):
    a = orc.seeded_uniform(20240917, 10000, 1e-4)
    b = splitmix_numpy(20240917, 10000, 1e-4)
    assert np.array_equal(a, b)
    assert a.min() >= -1e-4 and a.max() < 1e-4
    # SplitMix64 reference values (Vigna's splitmix64.c, state 0): 0xE220A8397B1DCDAF first.
    first = splitmix_numpy(0, 1, 0.5)[0]
    assert first == -0.5 + (0xE220A8397B1DCDAF >> 11) * 2.0 ** -53


def test_package_generator_matches_oracle(pkg, orc):
    """bench.py draws its synthetic states from the package's generator (chunked, for 8192^2
    grids); it is the oracle's stream value for value, across chunk boundaries too."""
    import numpy as np
    mask = pkg.make_channel(300, 77)
    for real, dt in (("f32", np.float32), ("f64", np.float64)):
        assert np.array_equal(pkg.workloads.seeded_state(20240917, 1e-4, 300, 77, mask, dt),
                              orc.seeded_state(20240917, 1e-4, 300, 77, mask, real))
    n = (1 << 24) // 9 + 5  # cells whose 9 n values span two generator chunks
    mask = np.zeros(n, np.uint8)
    mask[::7] = 1
    assert np.array_equal(pkg.workloads.seeded_state(3, 0.5, n, 1, mask, np.float32),
                          orc.seeded_state(3, 0.5, n, 1, mask, "f32"))


@pytest.mark.parametrize("name", [n for n in CASES if "seeded" in golden_cases()[n]])
def test_golden_seeded_state(orc, name):
    case = golden_cases()[name]
    if case.get("open_x"):
        pytest.skip("open-domain states are made consistent with the inflow/outflow rules")
    g = load_golden(name)
    seed, amp = case["seeded"]
    for real in REALS:
        s0 = orc.seeded_state(seed, amp, case["nx"], case["ny"], g["mask"], real)
        assert np.array_equal(s0, g[f"s0_{real}"])


def test_geometry_matches_reference_masks(pkg):
    g = load_golden("cylinder_open")
    assert np.array_equal(pkg.make_cylinder(120, 48, 30.0, 25.0, 10.0), g["mask"])
    c = load_golden("channel_seeded")
    assert np.array_equal(pkg.make_channel(64, 40), c["mask"])
    blk = load_golden("c1_block")["mask"]
    assert np.array_equal(pkg.geometry.add_block(pkg.make_channel(53, 31), 53, 10, 18, 8, 15), blk)


def test_poiseuille_force_rounding(pkg, orc):
    import ctypes as C
    if not orc.Reference.available("f32"):
        pytest.skip("reference not built here")
    lib = C.CDLL(str(orc.REF_DIR / "libref_f32.so"))
    lib.ref_poiseuille_force.restype = C.c_float
    lib.ref_poiseuille_force.argtypes = [C.c_int, C.c_float, C.c_float]
    for h, tau, u in ((32, 0.5 + 3 ** 0.5 / 4, 0.05), (16, 1.0, 0.05), (64, 0.6, 0.1)):
        assert np.float32(lib.ref_poiseuille_force(h, tau, u)) == pkg.poiseuille_force(h, tau, u)


@pytest.mark.parametrize("real", REALS)
def test_oracle_matches_live_reference_random(orc, real):
    """Random masks, forces and states against the reference built from its sources."""
    if not orc.Reference.available(real):
        pytest.skip("reference not built here (oracle/_ref)")
    ref = orc.Reference(real)
    rng = np.random.default_rng(7)
    for trial in range(6):
        nx, ny = int(rng.integers(3, 40)), int(rng.integers(3, 30))
        mask = (rng.random(nx * ny) < 0.15).astype(np.uint8)
        tau = float(real_dtype(real)(rng.uniform(0.52, 1.5)))
        fx, fy = float(rng.uniform(-1e-4, 1e-4)), float(rng.uniform(-1e-4, 1e-4))
        s0 = orc.seeded_state(100 + trial, 1e-3, nx, ny, mask, real)
        steps = int(rng.integers(1, 60))
        want = ref.run("v0", nx, ny, mask, tau, fx, fy, steps, s0=s0)
        got = orc.v0_run(nx, ny, mask, tau, fx, fy, s0, steps, real=real)
        assert np.array_equal(got, want["s"]), f"trial {trial}"
