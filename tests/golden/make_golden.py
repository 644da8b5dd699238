"""Generates the golden vectors in tests/golden/ from the reference's OWN solvers.

Needs the reference tree and its CPU solvers compiled by oracle/Makefile (`make -C oracle ref`,
done by this script). Run from the repository root:

    python tests/golden/make_golden.py            # small cases (.npz) and large-case hashes
    python tests/golden/make_golden.py --small    # small cases only
    python tests/golden/make_golden.py --wake     # cylinder-wake digests only (minutes)

For every case both reference solvers run, v0 (sequential, push) and v1 (OpenMP, pull), and the
script checks that they agree bit for bit before writing anything. States injected with a seeded
perturbation use the SplitMix64 stream of oracle/lbm_oracle.c (oracle_seeded_state): v0 receives
it as is, v1 receives its preimage by streaming, so the v0 == v1 check also pins that preimage.

Small cases are stored whole (inputs and outputs, float and double). The at-scale channel
cases (2048^2 x 1000 steps, 4096^2, 8192^2) are stored as SHA-256 digests of the outputs, with
negative zeros mapped to +0 first (the reference's own tests compare with `!=`, which treats
-0 and +0 as equal). The cylinder-wake workload (walled channel 1024 x 256 with a disc of
diameter 32 at (256, 129), tau 0.548, calibrated body force, uniform start u = (0.05, 0),
200k steps) is stored the same way in wake_hashes.json, float and double.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent
SEED = 20240917
AMP = 1e-4


def _ref_mask_lib():
    import ctypes as C
    lib = C.CDLL(str(oracle.REF_DIR / "libref_f64.so"))
    u8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
    lib.ref_make_channel.argtypes = [C.c_int, C.c_int, u8]
    lib.ref_make_cylinder.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, u8]
    return lib


def ref_channel(nx, ny):
    m = np.zeros(nx * ny, np.uint8)
    _ref_mask_lib().ref_make_channel(nx, ny, m)
    return m


def ref_cylinder(nx, ny, xc, yc, d):
    m = np.zeros(nx * ny, np.uint8)
    _ref_mask_lib().ref_make_cylinder(nx, ny, xc, yc, d, m)
    return m


def block(mask, nx, xs, ys):
    m = mask.reshape(-1, nx).copy()
    m[ys[0]:ys[1], xs[0]:xs[1]] = 1
    return m.reshape(-1)


def random_solids(nx, ny, frac, seed):
    u = oracle.seeded_uniform(seed, nx * ny, 1.0)  # in [-1, 1)
    return (u < -1.0 + 2.0 * frac).astype(np.uint8)


def small_cases():
    """name -> dict(nx, ny, mask, tau, fx, fy, steps, init | seeded, open_x, u_in)."""
    cases = {}
    # BASELINE workload 1: walls + solid rectangle x in [10,17], y in [8,14] (inclusive), S0 = 0.
    nx, ny = 53, 31
    cases["c1_block"] = dict(nx=nx, ny=ny, mask=block(ref_channel(nx, ny), nx, (10, 18), (8, 15)),
                             tau=0.8, fx=1e-5, fy=2e-6, steps=500, init=(1.0, 0.0, 0.0))
    # The reference's own cross-version case (tests/test_v3_vs_v0.cu:20-39).
    cases["ref_obstacle"] = dict(nx=nx, ny=ny,
                                 mask=block(ref_channel(nx, ny), nx, (12, 16), (10, 17)),
                                 tau=0.8, fx=1e-5, fy=2e-6, steps=500, init=(1.0, 0.02, 0.01))
    # The reference's open-boundary cylinder case (tests/cylinder_case.hpp:16-31).
    kd, ku, kre = 10, 0.05, 20.0
    cases["cylinder_open"] = dict(nx=120, ny=48, mask=ref_cylinder(120, 48, 3.0 * kd, 48 // 2 + 1, kd),
                                  tau=("cyl_tau", ku, kd, kre), fx=0.0, fy=0.0, steps=1000,
                                  init=(1.0, "u_in", 0.0), open_x=True, u_in=ku)
    # BASELINE workload 2 at a small size: walled channel, seeded perturbation.
    cases["channel_seeded"] = dict(nx=64, ny=40, mask=ref_channel(64, 40), tau=0.6, fx=1e-6,
                                   fy=0.0, steps=200, seeded=(SEED, AMP))
    # Fully periodic (no walls), scattered solids, seeded state: exercises the y wrap.
    cases["periodic_scatter"] = dict(nx=45, ny=23, mask=random_solids(45, 23, 0.12, SEED + 1),
                                     tau=0.7, fx=2e-5, fy=-1e-5, steps=100, seeded=(SEED + 2, AMP))
    # Odd widths around the 4- and 32-cell vector widths, channel + disc.
    cases["odd_width_disc"] = dict(nx=133, ny=37,
                                   mask=(ref_channel(133, 37) | ref_cylinder(133, 37, 40.0, 19.0, 9.0)),
                                   tau=0.55, fx=3e-6, fy=0.0, steps=150, seeded=(SEED + 3, AMP))
    # Degenerate widths: every x neighbour wraps onto the cell itself (nx=1) or the other (nx=2).
    cases["tiny_1x5"] = dict(nx=1, ny=5, mask=ref_channel(1, 5), tau=0.9, fx=1e-5, fy=0.0,
                             steps=50, seeded=(SEED + 4, AMP))
    cases["tiny_2x4"] = dict(nx=2, ny=4, mask=np.zeros(8, np.uint8), tau=0.9, fx=1e-5, fy=3e-6,
                             steps=50, seeded=(SEED + 5, AMP))
    # Open domain with a seeded state on top of the inlet equilibrium, odd width.
    cases["open_seeded"] = dict(nx=77, ny=33, mask=ref_cylinder(77, 33, 20.0, 17.0, 8.0),
                                tau=0.6, fx=0.0, fy=0.0, steps=300, seeded=(SEED + 6, AMP),
                                open_x=True, u_in=0.04)
    return cases


def resolve_tau(tau, real):
    dt = np.float32 if real == "f32" else np.float64
    if isinstance(tau, tuple):  # tests/cylinder_case.hpp:25: real(0.5 + 3.0 * double(kU) * kD / kRe)
        _, ku, kd, kre = tau
        return float(dt(0.5 + 3.0 * float(dt(ku)) * kd / kre))
    return float(dt(tau))


def open_consistent(s0, case, real):
    """Perturbation on top of the inlet equilibrium, then the open-x rules of the reference
    applied to it (src/common/boundary.hpp:37-48): a post-streaming state of an open domain has
    the inlet populations (i = 1, 5, 8 at x = 0) equal to the inlet equilibrium and the outlet
    populations (i = 3, 6, 7 at x = nx - 1) equal to those of x = nx - 2. Push (v0) and pull
    (v1) schemes agree only on states that satisfy this."""
    dt = np.float32 if real == "f32" else np.float64
    nx, ny = case["nx"], case["ny"]
    mask = case["mask"].reshape(ny, nx)
    eq = oracle.equilibrium_state(1.0, case["u_in"], 0.0, real)
    s = s0.reshape(ny, nx, 9).copy()
    s = np.where((mask == 0)[:, :, None], s + eq[None, None, :], dt(0)).astype(dt)
    for y in range(ny):
        if not mask[y, 0]:
            s[y, 0, [1, 5, 8]] = eq[[1, 5, 8]]
        if not mask[y, nx - 1]:
            s[y, nx - 1, [3, 6, 7]] = s[y, nx - 2, [3, 6, 7]]
    return s.reshape(-1)


def initial_state(case, real):
    """Returns (s0 or None, init tuple)."""
    dt = np.float32 if real == "f32" else np.float64
    if "seeded" in case:
        seed, amp = case["seeded"]
        s0 = oracle.seeded_state(seed, amp, case["nx"], case["ny"], case["mask"], real)
        if case.get("open_x"):
            s0 = open_consistent(s0, case, real)
        return s0, None
    init = tuple(case["u_in"] if v == "u_in" else v for v in case["init"])
    return None, init


def run_ref(case, real, version, threads=0):
    ref = oracle.Reference(real)
    s0, init = initial_state(case, real)
    kw = dict(open_x=bool(case.get("open_x")), u_in=case.get("u_in", 0.0), threads=threads)
    if s0 is not None:
        kw["s0"] = s0
    else:
        kw["init"] = init
    return ref.run(version, case["nx"], case["ny"], case["mask"], resolve_tau(case["tau"], real),
                   case["fx"], case["fy"], case["steps"], **kw), s0


def canon(a: np.ndarray) -> np.ndarray:
    """-0 -> +0 (numeric equality, as the reference's tests compare)."""
    return np.ascontiguousarray(a + a.dtype.type(0))


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(canon(a).tobytes()).hexdigest()


def same(a, b) -> bool:
    return bool(np.array_equal(a, b))


def make_small():
    meta = {}
    for name, case in small_cases().items():
        arrays = {"mask": case["mask"]}
        for real in ("f32", "f64"):
            r0, s0 = run_ref(case, real, "v0")
            r1, _ = run_ref(case, real, "v1", threads=3)
            for k in ("s", "rho", "ux", "uy"):
                if not same(r0[k], r1[k]):
                    raise SystemExit(f"{name}/{real}: reference v0 and v1 differ on {k}")
            for k in ("s", "rho", "ux", "uy"):
                arrays[f"{k}_{real}"] = r0[k]
            arrays[f"mass_{real}"] = np.float64(r0["mass"])
            if s0 is not None:
                arrays[f"s0_{real}"] = s0
        params = {k: v for k, v in case.items() if k != "mask"}
        params["tau_f32"] = resolve_tau(case["tau"], "f32")
        params["tau_f64"] = resolve_tau(case["tau"], "f64")
        if isinstance(params["tau"], tuple):
            params["tau"] = list(params["tau"])
        meta[name] = params
        np.savez_compressed(OUT / f"{name}.npz", **arrays)
        print(f"{name}: {case['nx']}x{case['ny']} x {case['steps']} steps  v0 == v1 (f32, f64)")
    (OUT / "cases.json").write_text(json.dumps(meta, indent=1, default=list) + "\n")


def large_cases():
    # BASELINE workload 2: walled channel, tau 0.6, F = (1e-6, 0), seeded perturbation.
    return [
        dict(name="channel_2048_f32", nx=2048, ny=2048, real="f32", steps=1000),
        dict(name="channel_2048_f64", nx=2048, ny=2048, real="f64", steps=1000),
        dict(name="channel_4096_f32_s100", nx=4096, ny=4096, real="f32", steps=100),
        dict(name="channel_8192_f32_s20", nx=8192, ny=8192, real="f32", steps=20),
    ]


def make_large(only=None):
    path = OUT / "hashes.json"
    out = json.loads(path.read_text()) if path.exists() else {}
    threads = os.cpu_count() or 4
    for c in large_cases():
        if only and c["name"] not in only:
            continue
        nx, ny, real = c["nx"], c["ny"], c["real"]
        mask = ref_channel(nx, ny)
        case = dict(nx=nx, ny=ny, mask=mask, tau=0.6, fx=1e-6, fy=0.0, steps=c["steps"],
                    seeded=(SEED, AMP))
        t0 = time.time()
        r, s0 = run_ref(case, real, "v1", threads=threads)
        dt = time.time() - t0
        out[c["name"]] = {
            "nx": nx, "ny": ny, "real": real, "steps": c["steps"], "tau": 0.6, "fx": 1e-6,
            "fy": 0.0, "seed": SEED, "amp": AMP, "mask": "channel",
            "s0": digest(s0), "s": digest(r["s"]), "rho": digest(r["rho"]),
            "ux": digest(r["ux"]), "uy": digest(r["uy"]), "mass": r["mass"],
            "generator": "reference v1 (src/v1_omp/solver_v1.cpp), %d threads" % threads,
        }
        print(f"{c['name']}: reference v1 {dt:.1f} s, "
              f"{nx * ny * c['steps'] / dt / 1e6:.0f} MLUPS")
        path.write_text(json.dumps(out, indent=1) + "\n")


# The cylinder-wake workload's body force, calibrated once for a bulk velocity of 0.05 (the
# library's wake.WAKE_FORCE; repeated here so that this script needs only the reference).
WAKE_FORCE = 6.784303312490499e-07


def make_wake(steps=200_000):
    """Reference v1 digests of the cylinder-wake workload after `steps` steps."""
    path = OUT / "wake_hashes.json"
    out = {}
    threads = os.cpu_count() or 4
    nx, ny = 1024, 256
    mask = (ref_channel(nx, ny) | ref_cylinder(nx, ny, 256.0, 129.0, 32.0)).astype(np.uint8)
    for real in ("f32", "f64"):
        case = dict(nx=nx, ny=ny, mask=mask, tau=0.548, fx=WAKE_FORCE, fy=0.0, steps=steps,
                    init=(1.0, 0.05, 0.0))
        t0 = time.time()
        r, _ = run_ref(case, real, "v1", threads=threads)
        dt = time.time() - t0
        out[f"wake_{real}"] = {
            "nx": nx, "ny": ny, "real": real, "steps": steps, "tau": 0.548, "fx": WAKE_FORCE,
            "fy": 0.0, "init": [1.0, 0.05, 0.0], "mask": "channel | cylinder(256, 129, D 32)",
            "mask_sha": hashlib.sha256(mask.tobytes()).hexdigest(),
            "s": digest(r["s"]), "rho": digest(r["rho"]), "ux": digest(r["ux"]),
            "uy": digest(r["uy"]), "mass": r["mass"],
            "generator": "reference v1 (src/v1_omp/solver_v1.cpp), %d threads" % threads,
        }
        print(f"wake_{real}: reference v1 {dt:.1f} s, {nx * ny * steps / dt / 1e6:.0f} MLUPS")
        path.write_text(json.dumps(out, indent=1) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--small", action="store_true")
    ap.add_argument("--large", nargs="*", default=None)
    ap.add_argument("--wake", action="store_true")
    args = ap.parse_args()
    oracle.build(ref=True)
    if args.wake:
        make_wake()
        return
    if args.large is None:
        make_small()
    if not args.small:
        make_large(args.large or None)


if __name__ == "__main__":
    main()
