#!/usr/bin/env python3
"""Benchmark of the D2Q9 pull stream-collide hot path on GB300.

Workload (the reference's at-scale channel workload at the size its HBM target is quoted on):
walled channel 4096 x 4096, periodic in x, tau 0.6, body force (1e-6, 0), populations
f_i - w_i initialised from the seeded SplitMix64 perturbation in [-1e-4, 1e-4], plain FP32
(bit-exact with the reference's v0). One bench step = one lattice time step over the whole grid
(one launch of the fused step kernel). MLUPS = nx * ny * steps / time / 1e6, solid cells
included (reference src/common/driver.hpp:120).

  value     device-resident state, K steps timed with CUDA events on the solver's stream,
            barrier + synchronize on both sides, max over ranks; the K steps are timed as
            `reps` consecutive repetitions (median and standard deviation reported, clocks
            sampled per repetition), value = all K steps / their summed time.
  e2e       the same metric through the public C ABI with host buffers: each e2e step is one
            user job, upload of the initial state from pinned host memory (9 N floats), 1000
            lattice steps, download of rho/ux/uy (3 N floats), all inside the timed region.
  roofline  HBM-bound: algorithmic bytes per cell update 2 * 9 * sizeof(float) = 72 B; achieved
            = 72 B * N / (average step-kernel duration); peak = measured copy bandwidth
            (MEASURED_PEAKS.json hbm_gbs); traffic = ncu DRAM bytes per launch (profiles/).
  forms     the reference's own GPU kernel (src/v3_cuda_opt/solver_v3.cu, unmodified, built
            for sm_103a) timed on the same GPU, grid and seeded state, FP32 and FP64;
            the other forms on the same grid: FP64 (144 B/cell), FP16 and BF16 storage (36 B);
            the 16-bit forms' velocity error and mass drift against FP64 (cylinder wake);
            the adjoint's forward and backward step times (512 x 128 channel, batch of 32
            seeded alpha fields);
            the batched ensemble (256 uneven channels, 5000 steps) against one launch per
            instance;
            the plain method at every at-scale grid (2048^2, 4096^2, 8192^2; FP32 and FP64);
            the cylinder wake at Re 100 in every form (Strouhal number, lift, drag, velocity
            error of the mean flow and mass drift against FP64, 200k steps);
            the reference's Strouhal known answer (open-BC cylinder 1000 x 320, D = 40, Re 100,
            160k steps, reference results/strouhal.csv:2-4).
  cpu_baseline  the reference's own OpenMP solver v1 (src/v1_omp/solver_v1.cpp, compiled from
            the unmodified source on the GPU host) on all host cores, kind "reference"; the
            oracle's port of it (kind "port") where the reference could not be built.

--impl reference: the reference's CPU implementation of the path (its v1 solver as above, or
the oracle's port) on all host cores, same metric and workload, rank 0 only.

Inputs are larger than L2 (604 MB per population buffer vs 129 MB), so no L2 flush is needed.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "MLUPS & % of 72B/cell HBM roofline, 1 GB300: plain vs fp16-store vs adjoint"
SEED, AMP = 20240917, 1e-4
TAU, FX, FY = 0.6, 1e-6, 0.0
BYTES_PER_CELL = {"fp32": 72, "fp64": 144, "fp16": 36, "bf16": 36}
HBM_FALLBACK_GBS = 6800.0
E2E_LATTICE_STEPS = 1000


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return HBM_FALLBACK_GBS, "fallback"


def profiled_traffic(precision: str, n: int):
    """DRAM bytes per step launch from the committed ncu summary, scaled to this grid."""
    f = ROOT / "profiles" / f"pull_step_{precision}_traffic.txt"
    if not f.exists():
        return None
    vals = {}
    for line in f.read_text().splitlines():
        if ":" in line and not line.startswith("#"):
            k, v = line.split(":", 1)
            vals[k.strip()] = v.strip()
    try:
        per_cell = float(vals["dram_bytes_per_cell"])
    except (KeyError, ValueError):
        return None
    return per_cell * n * n


class ClockSampler:
    """nvidia-smi SM clock and throttle-reason samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None
        self.window = (0.0, 0.0)

    def start(self):
        self._t = threading.Thread(target=self._loop, daemon=True)
        self._t.start()

    def _loop(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                row = [c.strip() for c in out.stdout.strip().split(",")]
                if len(row) >= 8:
                    self.samples.append((time.time(), row))
            except Exception:
                pass
            self._stop.wait(0.1)

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        t0, t1 = self.window
        inside = [r for t, r in self.samples if t0 <= t <= t1]
        if not inside and self.samples:  # very short timed region: nearest samples
            mid = 0.5 * (t0 + t1)
            inside = [min(self.samples, key=lambda s: abs(s[0] - mid))[1]]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[0]) for r in inside if num(r[0]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in inside for k in range(4) if r[4 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": num(inside[0][1]), "reasons": reasons, "samples": len(inside),
                "power_w_median": statistics.median([num(r[2]) for r in inside if num(r[2])] or [0])}


class NvmlClocks:
    """SM clock, power and throttle reasons read through NVML (libnvidia-ml.so.1, ctypes) in a
    background thread about every half millisecond, so that timed regions of a few milliseconds
    still get samples; each sample is stamped with time.perf_counter(). Falls back to the
    nvidia-smi sampler where NVML cannot be loaded. Reading only: no setting is changed."""

    # clocks-event reason bits (nvml.h nvmlClocksEventReason*)
    REASONS = ((0x4, "sw_power_cap"), (0x8, "hw_slowdown"), (0x20, "sw_thermal_slowdown"),
               (0x40, "hw_thermal_slowdown"))

    def __init__(self, local: int):
        import ctypes as C
        self.C = C
        self.samples = []  # (t, sm_mhz, power_w, reasons bitmask)
        self._stop = threading.Event()
        self._t = None
        self.ok = False
        try:
            self.nvml = C.CDLL("libnvidia-ml.so.1")
            if self.nvml.nvmlInit_v2() != 0:
                return
            self.dev = C.c_void_p()
            got = False
            try:
                import torch
                pr = torch.cuda.get_device_properties(local)
                bus = f"{pr.pci_domain_id:04x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
                got = self.nvml.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), C.byref(self.dev)) == 0
            except Exception:
                got = False
            if not got and self.nvml.nvmlDeviceGetHandleByIndex_v2(local, C.byref(self.dev)) != 0:
                return
            self._reasons = getattr(self.nvml, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                self.nvml.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = C.c_uint()
            self.max_mhz = (float(mx.value) if self.nvml.nvmlDeviceGetMaxClockInfo(
                self.dev, 1, C.byref(mx)) == 0 else None)
            self.ok = self._sample() is not None
        except OSError:
            self.ok = False

    def _sample(self):
        C = self.C
        mhz, mw, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        if self.nvml.nvmlDeviceGetClockInfo(self.dev, 1, C.byref(mhz)) != 0:
            return None
        self.nvml.nvmlDeviceGetPowerUsage(self.dev, C.byref(mw))
        self._reasons(self.dev, C.byref(rs))
        return (time.perf_counter(), float(mhz.value), mw.value / 1000.0, int(rs.value))

    def start(self):
        self._t = threading.Thread(target=self._loop, daemon=True)
        self._t.start()

    def _loop(self):
        while not self._stop.is_set():
            r = self._sample()
            if r is not None:
                self.samples.append(r)
            time.sleep(0.0005)

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self, t0: float, t1: float):
        """Clocks over the perf_counter window [t0, t1] (nearest sample if none fell inside)."""
        inside = [r for r in self.samples if t0 <= r[0] <= t1]
        if not inside and self.samples:
            mid = 0.5 * (t0 + t1)
            inside = [min(self.samples, key=lambda r: abs(r[0] - mid))]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["unavailable"],
                    "samples": 0}
        bits = 0
        for r in inside:
            bits |= r[3]
        return {"sm_mhz": statistics.median(r[1] for r in inside), "sm_max_mhz": self.max_mhz,
                "reasons": sorted(n for b, n in self.REASONS if bits & b),
                "samples": len(inside), "source": "nvml",
                "power_w_median": round(statistics.median(r[2] for r in inside), 1)}


def clock_sampler(local: int):
    """NVML sampler, or the nvidia-smi one where NVML is not available."""
    s = NvmlClocks(local)
    return s if s.ok else ClockSampler(local)


def clocks_summary(sampler, t0: float, t1: float, wall0: float):
    """Summary over a perf_counter window, for either sampler (the nvidia-smi one stamps
    samples with time.time(); wall0 = time.time() - time.perf_counter() converts)."""
    if isinstance(sampler, NvmlClocks):
        return sampler.summary(t0, t1)
    sampler.window = (t0 + wall0, t1 + wall0)
    return sampler.summary()


def dist_setup(n_gpus: int, backend: str = "nccl"):
    """Rank, local rank, world size and the process group (None for one process). Each rank
    runs an independent replica of the workload; the group only carries the barrier and the
    max-over-ranks of the timed region."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return rank, local, world, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(x: float, dist) -> float:
    if dist is None:
        return x
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def channel_state(n: int, precision_real: str):
    """The at-scale workload's walled channel and its seeded perturbation (the package's
    synthetic-input generator; the oracle is not used outside the CPU-baseline leg)."""
    import __graft_entry__ as entry
    pkg = entry.package()
    mask = pkg.make_channel(n, n)
    dtype = np.float64 if precision_real == "f64" else np.float32
    s0 = pkg.workloads.seeded_state(SEED, AMP, n, n, mask, dtype)
    return pkg, mask, s0


def time_form(pkg, mask, s0, n, precision, steps, warmup):
    """Device-resident MLUPS of one form (CUDA events on the solver's stream)."""
    with pkg.Solver(n, n, TAU, FX, FY, mask, precision=precision) as s:
        s.set_populations(s0)
        s.run(warmup)
        t = s.timed_run(steps)
    return n * n * steps / t / 1e6, t


def rep_stats(cells: int, steps: int, secs: list[float]) -> dict:
    """MLUPS of each repetition, their median and sample standard deviation."""
    ml = [cells * steps / t / 1e6 for t in secs]
    return {"reps": len(ml), "steps_each": steps, "mlups": [round(v, 1) for v in ml],
            "median": round(statistics.median(ml), 1),
            "std": round(statistics.stdev(ml), 1) if len(ml) > 1 else 0.0}


def time_form_reps(pkg, mask, s0, n, precision, steps, warmup, reps, sampler=None):
    """Like time_form, `reps` timed runs of `steps` steps each on one solver; returns
    (repetition statistics, clocks over the timed runs)."""
    with pkg.Solver(n, n, TAU, FX, FY, mask, precision=precision) as s:
        s.set_populations(s0)
        s.run(warmup)
        t0 = time.perf_counter()
        secs = [s.timed_run(steps) for _ in range(reps)]
        t1 = time.perf_counter()
    st = rep_stats(n * n, steps, secs)
    if sampler is not None:
        st["clocks"] = clocks_summary(sampler, t0, t1, time.time() - time.perf_counter())
    return st


def channel_mask(nx: int, ny: int) -> np.ndarray:
    m = np.zeros(nx * ny, np.uint8)
    m[:nx] = 1
    m[-nx:] = 1
    return m


def cpu_baseline(orc, n: int, budget_s: float = 8.0):
    """The reference's own OpenMP solver v1 (all host threads) where it was built on this host
    (oracle/_ref, kind "reference"), else the oracle's port of it (kind "port"); bounded sample:
    the full grid, as many steps as fit in about budget_s seconds (at most 50). Also the
    reference's sequential v0 on one core (a bounded 1024^2 sample)."""
    threads = os.cpu_count() or 1
    mask = channel_mask(n, n)
    s0 = orc.seeded_state(SEED, AMP, n, n, mask)
    if orc.Reference.available("f32"):
        ref = orc.Reference("f32")
        kind, what = "reference", ("reference v1 (src/v1_omp/solver_v1.cpp, unmodified, built "
                                   "on this host with -O3 -ffp-contract=off -fno-trapping-math)")
        rows = 256  # per-cell cost from a probe on a strip of the grid
        pm = channel_mask(n, rows)
        one = ref.bench("v1", n, rows, pm, TAU, FX, FY, orc.seeded_state(SEED, AMP, n, rows, pm),
                        2, warmup=1, reps=1, threads=threads)[0] / (2 * n * rows)
        steps = int(max(1, min(50, budget_s / max(one * n * n, 1e-9))))
        dt = ref.bench("v1", n, n, mask, TAU, FX, FY, s0, steps, warmup=1, reps=1,
                       threads=threads)[0]
        m0 = 1024
        mask0 = channel_mask(m0, m0)
        s00 = orc.seeded_state(SEED, AMP, m0, m0, mask0)
        one0 = ref.bench("v0", m0, m0, mask0, TAU, FX, FY, s00, 1, warmup=0, reps=1)[0]
        k0 = int(max(1, min(20, 3.0 / max(one0, 1e-6))))
        t0v = ref.bench("v0", m0, m0, mask0, TAU, FX, FY, s00, k0, warmup=0, reps=1)[0]
        v0_what = "reference v0 (src/v0_cpu/solver_v0.cpp, unmodified, built on this host)"
    else:
        kind, what = "port", "oracle pull port of reference v1 (src/v1_omp/solver_v1.cpp)"
        bufs = orc.PullBuffers(n, n, mask, orc.s_to_r(n, n, mask, s0))
        t0 = time.perf_counter()
        bufs.run(TAU, FX, FY, 1, threads=threads)
        one = time.perf_counter() - t0
        steps = int(max(1, min(50, budget_s / max(one, 1e-6))))
        t0 = time.perf_counter()
        bufs.run(TAU, FX, FY, steps, threads=threads)
        dt = time.perf_counter() - t0
        del bufs
        m0 = 1024
        mask0 = channel_mask(m0, m0)
        s00 = orc.seeded_state(SEED, AMP, m0, m0, mask0)
        t0 = time.perf_counter()
        orc.v0_run(m0, m0, mask0, TAU, FX, FY, s00, 1)
        one0 = time.perf_counter() - t0
        k0 = int(max(1, min(20, 3.0 / max(one0, 1e-6))))
        t0 = time.perf_counter()
        orc.v0_run(m0, m0, mask0, TAU, FX, FY, s00, k0)
        t0v = time.perf_counter() - t0
        v0_what = "oracle restatement of reference v0 (src/v0_cpu/solver_v0.cpp)"
    return {"value": round(n * n * steps / dt / 1e6, 2), "unit": "MLUPS", "cores": threads,
            "kind": kind,
            "sample": f"{n}x{n} walled channel, {steps} steps after 1 warm-up step, FP32, "
                      f"{what}, {threads} OpenMP threads",
            "v0_single_core": {"value": round(m0 * m0 * k0 / t0v / 1e6, 2), "unit": "MLUPS",
                               "cores": 1, "kind": kind,
                               "sample": f"{m0}x{m0} walled channel, {k0} steps, FP32, {v0_what}"}}


def reference_v3_report(orc, pkg, n, peak, sampler, reps=5):
    """The reference's own GPU solver (SolverV3, src/v3_cuda_opt/solver_v3.cu, unmodified,
    built for sm_103a with the reference's -O3 --fmad=false; default kernel
    step_kernel<true,true,false>, block 32x8, one launch per step on the legacy stream) on the
    headline grid and seeded state, timed by its own timed_run (CUDA events), beside the
    library's default kernel timed the same way: `reps` repetitions of 1000 (FP32) / 100 (FP64)
    steps after 20 warm-up steps."""
    out = {}
    for real, prec, steps in (("f32", "fp32", 1000), ("f64", "fp64", 100)):
        if not orc.ReferenceV3.available(real):
            out[prec] = {"unavailable": "oracle/_ref/libref_v3 not built (no reference tree or "
                                        "staged copy on this host, or no nvcc)"}
            continue
        try:
            mask = pkg.make_channel(n, n)
            s0 = pkg.workloads.seeded_state(SEED, AMP, n, n, mask,
                                            np.float64 if real == "f64" else np.float32)
            t0 = time.perf_counter()
            secs, info, _ = orc.ReferenceV3(real).bench(n, n, mask, TAU, FX, FY, s0, steps,
                                                        warmup=20, reps=reps)
            t1 = time.perf_counter()
            ref = rep_stats(n * n, steps, secs)
            ref["clocks"] = clocks_summary(sampler, t0, t1, time.time() - time.perf_counter())
            ref["hbm_frac"] = round(BYTES_PER_CELL[prec] * ref["median"] * 1e6 / 1e9 / peak, 4)
            ref["kernel"] = "step_kernel<true,true,false> (soa_pull_opt), 32x8 blocks"
            ref["bench_info"] = json.loads("{" + info + "}")
            ours = time_form_reps(pkg, mask, s0, n, prec, steps, 20, reps, sampler)
            ours["hbm_frac"] = round(BYTES_PER_CELL[prec] * ours["median"] * 1e6 / 1e9 / peak, 4)
            del s0
            out[prec] = {"reference_v3": ref, "ours": ours,
                         "ours_over_reference": round(ours["median"] / ref["median"], 3)}
        except Exception as e:
            out[prec] = {"error": str(e)[:200]}
    out["workload"] = (f"walled channel {n}x{n}, tau {TAU}, F=({FX},0), seeded state, same GPU; "
                       "ours = the library's default kernel (lbm_timed_run)")
    return out


def strouhal_report(pkg, tmp: Path):
    """The reference's Strouhal known answer: its open-BC cylinder case (1000 x 320, D = 40,
    Re 100, inlet u = 0.05, tau 0.56, 160k steps, probe 3 D behind the disc every 50 steps;
    reference src/common/driver.hpp:167-251) run through this library's command-line driver
    (FP32, bit-exact with the reference), probe.csv analysed as the reference's
    scripts/strouhal.py does with --from 0.55 (README.md:191-193). Published:
    St = 0.1807 (FFT) / 0.1805 (zero crossings), 15 periods, u_y amplitude 0.03232
    (results/strouhal.csv:2-4)."""
    exe = pkg.LIB_PATH.parent / "lbm_b200"
    out = tmp / "strouhal_kat"
    t0 = time.perf_counter()
    r = subprocess.run([str(exe), "--case", "cylinder", "--nx", "1000", "--ny", "320",
                        "--diameter", "40", "--re", "100", "--umax", "0.05", "--steps", "160000",
                        "--out", str(out)], capture_output=True, text=True)
    wall = time.perf_counter() - t0
    if r.returncode != 0:
        return {"error": (r.stderr or r.stdout)[-300:]}
    res = pkg.wake.probe_strouhal(out, start=0.55)
    res = {k: (round(v, 5) if isinstance(v, float) else v) for k, v in res.items()}
    res.update({"published_st_fft": 0.1807, "published_st_zero_crossing": 0.1805,
                "published_periods": 15, "published_uy_amplitude": 0.03232,
                "wall_s": round(wall, 2),
                "workload": "open-BC cylinder 1000x320, D=40, Re 100, u_in 0.05, 160k steps, "
                            "FP32, driver lbm_b200 --case cylinder, window from 0.55"})
    return res


def accuracy_report(pkg):
    """Velocity L2 error and mass drift of the 16-bit forms against the FP64 form on the
    cylinder-wake geometry (1024 x 256, disc D = 32, tau 0.548, uniform start u = (0.05, 0),
    F = (1.5e-7, 0)) after 4000 steps."""
    nx, ny, tau, fx, steps, init = 1024, 256, 0.548, 1.5e-7, 4000, (1.0, 0.05, 0.0)
    mask = pkg.workloads.cylinder_wake(nx, ny)
    out, ref = {}, None
    for form in ("fp16", "bf16"):
        r, ref = pkg.accuracy.compare_forms(pkg, nx, ny, mask, tau, fx, 0.0, steps, form,
                                            init=init, reference=ref)
        out[form] = {k: (float(f"{v:.4g}") if isinstance(v, float) else v) for k, v in r.items()
                     if k != "form"}
    out["workload"] = (f"cylinder wake {nx}x{ny}, disc D=32 at (256,129), tau {tau}, "
                       f"F=({fx},0), start u=(0.05,0), {steps} steps, stochastic rounding")
    return out


def scale_report(pkg, peak):
    """The plain method at every grid of the at-scale workload (walled channel, tau 0.6,
    F = (1e-6, 0), seeded perturbation in [-1e-4, 1e-4]): 2048^2, 4096^2, 8192^2 in FP32 and
    FP16 storage (1000 steps each) and FP64 (1000, 1000 and 200 steps: FP64-ALU-bound, 25 ms
    per step at 8192^2), device-resident MLUPS and the fraction of the 72 / 36 / 144 B per cell
    roofline."""
    out = {}
    for prec, real, steps in (("fp32", "f32", (1000, 1000, 1000)), ("fp16", "f32", (1000, 1000, 1000)),
                              ("fp64", "f64", (1000, 1000, 200))):
        out[prec] = {}
        for n, k in zip((2048, 4096, 8192), steps):
            try:
                mask = pkg.make_channel(n, n)
                s0 = pkg.workloads.seeded_state(SEED, AMP, n, n, mask, np.float64 if real == "f64" else np.float32)
                ml, _ = time_form(pkg, mask, s0, n, prec, k, 10)
                del s0
                gbs = BYTES_PER_CELL[prec] * ml * 1e6 / 1e9
                out[prec][str(n)] = {"mlups": round(ml, 1), "achieved_gbs": round(gbs, 1),
                                     "hbm_frac": round(gbs / peak, 4), "steps": k}
            except Exception as e:
                out[prec][str(n)] = {"error": str(e)[:200]}
    return out


def wake_report(pkg):
    """Cylinder wake at Re 100 (1024 x 256, disc D = 32, tau 0.548, calibrated body force, start
    u = (0.05, 0)), 200k steps in every form: Strouhal number from the lift on the disc
    (momentum exchange on the device, sampled every 50 steps), lift rms and mean drag over the
    second half; against the FP64 run: the velocity L2 error of the mean flow (u averaged over
    the second half, sampled every 500 steps: the shedding phase drifts between forms, so the
    instantaneous fields decorrelate) and of the final field, and each run's mass drift.
    The 16-bit forms also report St over four noise streams (step-counter offsets 0, 7, 1001,
    50000): the wake has two shedding states and their rounding noise picks one per stream."""
    out, runs = {}, {}
    for prec in ("fp64", "fp32", "fp16", "bf16"):
        try:
            t0 = time.perf_counter()
            s = pkg.wake.lift_series(pkg, prec, steps=200_000, every=50, mean_every=500)
            r = pkg.wake.strouhal(s)
            runs[prec] = s
            out[prec] = {"st": round(r["st"], 5), "lift_rms": round(r["lift_rms"], 6),
                         "drag_mean": round(r["drag_mean"], 6), "u_bulk": round(s["u_bulk"], 6),
                         "mass_drift": float(f"{(s['mass1'] - s['mass0']) / s['mass0']:.4g}"),
                         "finite": bool(s["finite"]), "wall_s": round(time.perf_counter() - t0, 2)}
        except Exception as e:
            out[prec] = {"error": str(e)[:200]}
    if "st" in out.get("fp64", {}):
        ref = runs["fp64"]
        for prec in ("fp32", "fp16", "bf16"):
            if "st" in out.get(prec, {}):
                got = runs[prec]
                out[prec]["st_rel_diff_vs_fp64"] = round(out[prec]["st"] / out["fp64"]["st"] - 1.0, 5)
                out[prec]["velocity_l2_mean_flow"] = float(f"{pkg.wake.velocity_l2(got, ref, 'mean'):.4g}")
                out[prec]["velocity_l2_final"] = float(f"{pkg.wake.velocity_l2(got, ref, 'end'):.4g}")
    for prec in ("fp16", "bf16"):
        if "st" not in out.get(prec, {}):
            continue
        try:
            sts = [out[prec]["st"]] + [round(pkg.wake.strouhal(pkg.wake.lift_series(
                pkg, prec, steps=200_000, every=50, noise_offset=off))["st"], 5) for off in (7, 1001, 50000)]
            st32 = out.get("fp32", {}).get("st")
            out[prec]["streams"] = {"offsets": [0, 7, 1001, 50000], "st": sts,
                                    "within_2pct_of_fp32": (sum(1 for x in sts if abs(x / st32 - 1) < 0.02)
                                                            if st32 else None)}
        except Exception as e:
            out[prec]["streams"] = {"error": str(e)[:200]}
    out["workload"] = ("cylinder wake 1024x256, disc D=32 at (256,129), tau 0.548, Re 100, "
                       f"F=({pkg.wake.WAKE_FORCE:.4g},0) calibrated for u_bulk 0.05, 200k steps, "
                       "lift sampled every 50 steps")
    return out


def batch_report(pkg, peak, autotune=True, steps=5000):
    """Batched ensemble: 256 uneven closed channels (nx ~ U[64,1024], ny ~ U[32,512], 1-4 discs,
    tau ~ U[0.52,1], fx ~ U[1e-6,1e-5], seed 7), autotuned, 5000 steps as CUDA graphs of one
    persistent launch per step, against the same instances stepped one launch per instance
    (64 steps)."""
    specs = pkg.workloads.ensemble_specs(256, seed=7)
    cells = sum(s["nx"] * s["ny"] for s in specs)
    out = {"instances": len(specs), "cells": cells, "steps": steps}
    for prec in ("fp32", "fp16"):
        try:
            with pkg.Batch(specs, precision=prec) as b:
                b.init_equilibrium(1.0, 0.0, 0.0)
                tune = b.autotune() if autotune else "default: ring 4x2 stages=4 (not tuned)"
                b.run(64)
                tb = b.timed_run(steps)
                ts = b.run_separate(64)
            ml = cells * steps / tb / 1e6
            out[prec] = {"batched_mlups": round(ml, 1),
                         "separate_mlups": round(cells * 64 / ts / 1e6, 1),
                         "hbm_frac": round(BYTES_PER_CELL[prec] * ml * 1e6 / 1e9 / peak, 4),
                         "autotune": tune.split(" | ")[0]}
        except Exception as e:
            out[prec] = {"error": str(e)[:200]}
    return out


def adjoint_report(pkg, peak):
    """Adjoint form on its workload (512 x 128 channel, Brinkman fields, J = mean u_x over the
    last 100 of 2000 steps, checkpoints every 100 steps), a batch of 32 distinct seeded alpha
    fields (seeds 1234 ... 1265): forward and backward step times (recomputation included) and
    their ratio, FP32 and FP64."""
    nx, ny, tau, fx, steps, window, batch = 512, 128, 0.6, 5e-6, 2000, 100, 32
    mask = pkg.workloads.adjoint_channel(nx, ny)
    fields = pkg.workloads.brinkman_batch(nx, ny, batch, mask, seed=1234)
    out, grads = {}, {}
    for prec in ("fp32", "fp64"):
        try:
            with pkg.Adjoint(nx, ny, tau, fx, 0.0, mask, precision=prec, batch=batch,
                             checkpoint_every=100) as a:
                a.set_alpha(fields)
                a.forward(steps, window)
                grads[prec] = a.backward()
                f, b = a.step_times()
            cells = nx * ny * batch
            out[prec] = {"forward_step_us": round(f * 1e6, 2), "backward_step_us": round(b * 1e6, 2),
                         "backward_over_forward": round(b / f, 3),
                         "forward_mlups": round(cells / f / 1e6, 1),
                         "backward_mlups": round(cells / b / 1e6, 1)}
        except Exception as e:
            out[prec] = {"error": str(e)[:200]}
    if len(grads) == 2:  # the FP32 adjoint against the FP64 one, over the 32 instances
        g32, g64 = grads["fp32"], grads["fp64"]
        rel = lambda a, b: float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b))))
        a32, a64 = np.asarray(g32["alpha"]), np.asarray(g64["alpha"])
        big = np.abs(a64) > 1e-3 * np.max(np.abs(a64))
        out["fp32_vs_fp64_max_rel"] = {"fx": float(f"{rel(g32['fx'], g64['fx']):.3g}"),
                                       "tau": float(f"{rel(g32['tau'], g64['tau']):.3g}"),
                                       "alpha": float(f"{float(np.max(np.abs(a32 - a64)[big] / np.abs(a64)[big])):.3g}")}
    out["workload"] = (f"channel {nx}x{ny}, tau {tau}, F=({fx},0), {batch} distinct seeded "
                       f"Brinkman alpha fields in [0,0.1], {steps} steps, J window {window}, K=100")
    return out


def run_ours(args):
    import torch

    import __graft_entry__ as entry
    rank, local, world, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    pkg = entry.package()
    pkg.build()
    n = args.nx
    warmup = max(args.warmup, 3)
    prec = args.precision
    _, mask, s0 = channel_state(n, "f32")
    s_head = s0.astype(np.float64) if prec == "fp64" else s0

    solver = pkg.Solver(n, n, TAU, FX, FY, mask, precision=prec)
    if args.variant >= 0:
        solver.set_variant(args.variant)
    stream = torch.cuda.Stream()  # the solver's stream; the timed region's events go on it
    solver.set_stream(stream.cuda_stream)
    solver.set_populations(s_head)
    solver.run(warmup)
    sampler = clock_sampler(local)
    sampler.start()
    wall0 = time.time() - time.perf_counter()
    time.sleep(0.05)
    # One continuous timed region of K steps on the solver's own stream, split into `reps`
    # consecutive repetitions by CUDA events recorded between them (no synchronisation inside
    # the region); value = K steps / (last event - first event).
    reps = max(1, min(args.reps, args.steps))
    sizes = [args.steps // reps + (1 if k < args.steps % reps else 0) for k in range(reps)]
    events = [torch.cuda.Event(enable_timing=True) for _ in range(reps + 1)]
    barrier(dist)
    torch.cuda.synchronize()
    solver.synchronize()
    k_before = solver.kernel_launches()
    host = [time.perf_counter()]
    events[0].record(stream)
    for k, ev in zip(sizes, events[1:]):
        solver.step(k)
        ev.record(stream)
    for ev in events[1:]:
        ev.synchronize()
        host.append(time.perf_counter())
    solver.synchronize()
    launches = solver.kernel_launches() - k_before
    torch.cuda.synchronize()
    barrier(dist)
    rep_secs = [events[k].elapsed_time(events[k + 1]) * 1e-3 for k in range(reps)]
    secs = max_over_ranks(events[0].elapsed_time(events[-1]) * 1e-3, dist)
    info = solver.bench_info()
    solver.close()
    rep_ml = [n * n * k / t / 1e6 for k, t in zip(sizes, rep_secs)]
    windows = [(host[0] if k == 0 else host[k], host[k + 1]) for k in range(reps)]
    repetitions = {"reps": reps, "steps_each": sizes, "mlups": [round(v, 1) for v in rep_ml],
                   "median": round(statistics.median(rep_ml), 1),
                   "std": round(statistics.stdev(rep_ml), 1) if reps > 1 else 0.0,
                   "timing": "one region, CUDA events between repetitions",
                   "clocks": [clocks_summary(sampler, a, b, wall0) for a, b in windows]}
    head_clocks = clocks_summary(sampler, host[0], host[-1], wall0)

    cells = n * n
    value = cells * args.steps * world / secs / 1e6
    step_s = secs / args.steps
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_CELL[prec] * cells / step_s / 1e9
    traffic = profiled_traffic(prec, n)

    # e2e through the public API: pinned host input, 1000 steps, host output.
    e2e = None
    if args.e2e_jobs > 0:
        tdt = torch.float64 if prec == "fp64" else torch.float32
        pin = torch.empty(s0.size, dtype=tdt).pin_memory()
        pin.numpy()[:] = s_head
        outs = [torch.empty(cells, dtype=tdt).pin_memory() for _ in range(3)]
        with pkg.Solver(n, n, TAU, FX, FY, mask, precision=prec) as s:
            # One untimed job first: the first large upload and the step graph's capture are
            # one-time costs of a solver, not of a job.
            s.set_populations(pin.numpy())
            s.run(E2E_LATTICE_STEPS)
            s.macroscopic([o.numpy() for o in outs])
            barrier(dist)
            torch.cuda.synchronize()
            phase = [0.0, 0.0, 0.0]  # upload, lattice steps, moments + download (each call synchronises)
            t0 = time.perf_counter()
            for _ in range(args.e2e_jobs):
                ta = time.perf_counter()
                s.set_populations(pin.numpy())
                tb = time.perf_counter()
                s.run(E2E_LATTICE_STEPS)
                tc = time.perf_counter()
                s.macroscopic([o.numpy() for o in outs])
                td = time.perf_counter()
                phase[0] += tb - ta
                phase[1] += tc - tb
                phase[2] += td - tc
            torch.cuda.synchronize()
            barrier(dist)
            dt = max_over_ranks(time.perf_counter() - t0, dist)
        e2e = {"value": cells * E2E_LATTICE_STEPS * args.e2e_jobs * world / dt / 1e6,
               "unit": "MLUPS", "h2d_bytes_per_step": int(s_head.nbytes),
               "d2h_bytes_per_step": int(3 * cells * s_head.itemsize),
               "lattice_steps_per_e2e_step": E2E_LATTICE_STEPS, "e2e_steps": args.e2e_jobs,
               "api": "lbm_set_populations + lbm_run(1000) + lbm_macroscopic (C ABI)",
               "phase_ms_per_step": {"upload": round(1e3 * phase[0] / args.e2e_jobs, 2),
                                     "lattice_steps": round(1e3 * phase[1] / args.e2e_jobs, 2),
                                     "download": round(1e3 * phase[2] / args.e2e_jobs, 2)}}

    forms = {}
    if args.forms and rank == 0:
        del s_head
        for fp, steps in (("fp32", 1000), ("fp16", 1000), ("bf16", 1000), ("fp64", 50)):
            try:
                st = s0.astype(np.float64) if fp == "fp64" else s0
                r = time_form_reps(pkg, mask, st, n, fp, steps, 20, 5, sampler)
                del st
                gbs = BYTES_PER_CELL[fp] * r["median"] * 1e6 / 1e9
                forms[fp] = {"mlups": r["median"], "mlups_std": r["std"], "reps": r["reps"],
                             "bytes_per_cell": BYTES_PER_CELL[fp], "achieved_gbs": round(gbs, 1),
                             "hbm_frac": round(gbs / peak, 4), "steps": steps,
                             "clocks": r["clocks"]}
            except Exception as e:  # a form that fails is reported, not hidden
                forms[fp] = {"error": str(e)[:200]}
        if "mlups" in forms.get("fp16", {}) and "mlups" in forms.get("fp32", {}):
            forms["fp16_over_fp32"] = round(forms["fp16"]["mlups"] / forms["fp32"]["mlups"], 3)
        if args.reference_gpu:
            orc = entry.oracle_module()  # the reference's own kernel, timed as a baseline
            forms["reference_v3"] = reference_v3_report(orc, pkg, n, peak, sampler)
        if args.accuracy:
            forms["accuracy_vs_fp64"] = accuracy_report(pkg)
        if args.adjoint:
            forms["adjoint"] = adjoint_report(pkg, peak)
        if args.batch:
            forms["batch"] = batch_report(pkg, peak, args.batch_autotune, args.batch_steps)
        if args.scale:
            forms["scale"] = scale_report(pkg, peak)
        if args.wake:
            forms["cylinder_wake"] = wake_report(pkg)
        if args.strouhal:
            import tempfile
            with tempfile.TemporaryDirectory() as tmp:
                forms["strouhal_kat"] = strouhal_report(pkg, Path(tmp))
    sampler.stop()

    cpu = None
    if rank == 0 and args.cpu_baseline:
        orc = entry.oracle_module()  # the CPU-baseline leg is the oracle's one use here
        if not orc.LIB.exists():
            orc.build()
        cpu = cpu_baseline(orc, n)

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": warmup, "ms_per_step": round(step_s * 1e3, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "fp64": "f64", "fp16": "f32 (f16 storage)",
                  "bf16": "f32 (bf16 storage)"}[prec],
        "data": "synthetic: seeded SplitMix64 perturbation of f_i - w_i in [-1e-4, 1e-4]",
        "config": {"workload": f"walled channel {n}x{n}, periodic x, tau 0.6, F=(1e-6,0), "
                               + ("plain FP32 pull stream-collide (bit-exact with reference v0)"
                                  if prec == "fp32" else f"{prec} form of the pull stream-collide"),
                   "nx": n, "ny": n, "form": prec, "variant": args.variant,
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (population buffer 604 MB > 129 MB), no flush"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": BYTES_PER_CELL[prec] * cells},
        "clocks": head_clocks,
        "repetitions": repetitions,
        "gpu_launches": launches,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "forms": forms or None,
        "device": json.loads("{" + info + "}"),
    }
    print(json.dumps(line), flush=True)


def run_reference(args):
    """The reference's CPU path on the host cores, rank 0 only: its own OpenMP solver v1
    (src/v1_omp/solver_v1.cpp, unmodified, built on this host; kind "reference"), else the
    oracle's port of it (kind "port"). Each bench step is one lattice step; the grid keeps all
    4096 columns but its rows are bounded so that warm-up + timed steps stay within about two
    minutes."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import __graft_entry__ as entry
    orc = entry.oracle_module()
    if not orc.LIB.exists():
        orc.build()
    n = args.nx
    threads = os.cpu_count() or 1
    warmup = max(args.warmup, 3)
    use_ref = orc.Reference.available("f32")
    ref = orc.Reference("f32") if use_ref else None

    def timed(rows, steps, warm):
        m = channel_mask(n, rows)
        s0 = orc.seeded_state(SEED, AMP, n, rows, m)
        if use_ref:
            return ref.bench("v1", n, rows, m, TAU, FX, FY, s0, steps, warmup=warm, reps=1,
                             threads=threads)[0]
        bufs = orc.PullBuffers(n, rows, m, orc.s_to_r(n, rows, m, s0))
        bufs.run(TAU, FX, FY, warm, threads=threads)
        t0 = time.perf_counter()
        bufs.run(TAU, FX, FY, steps, threads=threads)
        return time.perf_counter() - t0

    probe_rows = 256
    per_cell = timed(probe_rows, 2, 1) / (2 * n * probe_rows)
    rows, budget = n, 120.0
    while rows > 1024 and per_cell * n * rows * (args.steps + warmup) > budget:
        rows //= 2
    dt = timed(rows, args.steps, warmup)
    value = n * rows * args.steps / dt / 1e6
    kind = "reference" if use_ref else "port"
    what = ("reference v1 (src/v1_omp/solver_v1.cpp, unmodified, built on this host with -O3 "
            "-ffp-contract=off -fno-trapping-math)" if use_ref else
            "oracle pull port of reference v1 (src/v1_omp/solver_v1.cpp)")
    sample = (f"{n}x{rows} walled channel (full {n}x{n} rows bounded to fit ~2 min), "
              f"{args.steps} timed lattice steps after {warmup}, FP32, {what}, "
              f"{threads} OpenMP threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": "MLUPS",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"walled channel {n}x{n}, periodic x, tau 0.6, F=(1e-6,0), "
                               "plain FP32 pull stream-collide (bit-exact with reference v0)",
                   "nx": n, "ny": rows},
        "cpu_baseline": {"value": round(value, 2), "unit": "MLUPS", "cores": threads,
                         "kind": kind, "sample": sample},
        "e2e": {"value": round(value, 2), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_gpu_only(args):
    """Only the reference's own GPU kernel on the headline grid and seeded state (`--warmup`
    steps, then one timed_run of `--steps` steps): the command its ncu profile is taken with."""
    import __graft_entry__ as entry
    pkg = entry.package()
    orc = entry.oracle_module()
    n = args.nx
    real = "f64" if args.precision == "fp64" else "f32"
    mask = pkg.make_channel(n, n)
    s0 = pkg.workloads.seeded_state(SEED, AMP, n, n, mask, np.float64 if real == "f64" else np.float32)
    secs, info, _ = orc.ReferenceV3(real).bench(n, n, mask, TAU, FX, FY, s0, args.steps,
                                                warmup=args.warmup, reps=1)
    print(json.dumps({"impl": "reference_v3_gpu", "nx": n, "ny": n, "real": real,
                      "steps": args.steps, "mlups": round(n * n * args.steps / secs[0] / 1e6, 1),
                      "bench_info": info}), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__,
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=100)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nx", type=int, default=4096)
    ap.add_argument("--e2e-jobs", type=int, default=5)
    ap.add_argument("--no-forms", dest="forms", action="store_false")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--precision", choices=["fp32", "fp64", "fp16", "bf16"], default="fp32",
                    help="form of the headline (timed) run; the default is the reference's FP32")
    ap.add_argument("--variant", type=int, default=-1,
                    help="step-kernel variant of the headline run (-1: automatic choice)")
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false",
                    help="skip the 16-bit forms' accuracy runs against FP64")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false",
                    help="skip the adjoint form")
    ap.add_argument("--no-batch", dest="batch", action="store_false",
                    help="skip the batched ensemble form")
    ap.add_argument("--no-batch-autotune", dest="batch_autotune", action="store_false",
                    help="batched ensemble with the library's default launch (profiling)")
    ap.add_argument("--batch-steps", type=int, default=5000,
                    help="timed steps of the batched ensemble (the workload's 5000; fewer for profiling)")
    ap.add_argument("--no-scale", dest="scale", action="store_false",
                    help="skip the 2048^2 / 4096^2 / 8192^2 FP32 and FP64 scale report")
    ap.add_argument("--no-wake", dest="wake", action="store_false",
                    help="skip the cylinder-wake comparison of the forms")
    ap.add_argument("--no-strouhal", dest="strouhal", action="store_false",
                    help="skip the reference's Strouhal known-answer run (open-BC cylinder)")
    ap.add_argument("--no-reference-gpu", dest="reference_gpu", action="store_false",
                    help="skip timing the reference's own GPU kernel")
    ap.add_argument("--reps", type=int, default=5,
                    help="repetitions the K timed steps of the headline are split into")
    ap.add_argument("--profile-reference-gpu", action="store_true",
                    help="run only the reference's own GPU kernel (for its ncu profile)")
    args = ap.parse_args()
    if args.steps < 1:
        ap.error("--steps must be >= 1")
    if args.profile_reference_gpu:
        run_reference_gpu_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
