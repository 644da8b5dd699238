"""Seeded synthetic inputs of the benchmark workloads (no dataset is involved).

All randomness comes from a counter-based SplitMix64 stream (Steele, Lea and Flood 2014):
element k of the stream of `seed` is the SplitMix64 finaliser of seed + (k + 1) * golden gamma,
mapped to [0, 1) through its top 53 bits. The same stream generates the seeded initial states
(oracle/lbm_oracle.c), so every workload is reproducible from its seed alone.
"""
from __future__ import annotations

import numpy as np

from .geometry import make_channel, make_cylinder

_GAMMA = np.uint64(0x9E3779B97F4A7C15)


def uniform01(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """count values of the seed's stream in [0, 1), starting at element `offset`."""
    k = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + k * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def seeded_state(seed: int, amp: float, nx: int, ny: int, solid, dtype=np.float32) -> np.ndarray:
    """f_i - w_i = U(-amp, amp) per population on fluid cells, 0 on solid cells, v0 layout
    (generated in chunks, so that 8192^2 grids need no multi-GB temporaries)."""
    n = nx * ny * 9
    s = np.empty(n, dtype)
    chunk = 1 << 24
    for k0 in range(0, n, chunk):
        k1 = min(n, k0 + chunk)
        s[k0:k1] = (-amp + 2.0 * amp * uniform01(seed, k1 - k0, offset=k0)).astype(dtype)
    s.reshape(-1, 9)[np.asarray(solid).reshape(-1) != 0] = 0
    return s


def brinkman_field(nx: int, ny: int, seed: int, n_gauss: int = 16, wmin: float = 8.0,
                   wmax: float = 32.0, alpha_max: float = 0.1) -> np.ndarray:
    """Smooth random drag field: a sum of n_gauss Gaussians (centres uniform in the domain,
    widths uniform in [wmin, wmax] cells, amplitudes uniform in [0.5, 1]; x distances periodic),
    scaled linearly onto [0, alpha_max]. Row-major nx * ny doubles."""
    u = uniform01(seed, 4 * n_gauss).reshape(n_gauss, 4)
    y, x = np.mgrid[0:ny, 0:nx].astype(np.float64)
    g = np.zeros((ny, nx))
    for cx, cy, w, a in u:
        cx, cy, w, a = cx * nx, cy * ny, wmin + (wmax - wmin) * w, 0.5 + 0.5 * a
        dx = np.abs(x - cx)
        dx = np.minimum(dx, nx - dx)
        g += a * np.exp(-(dx * dx + (y - cy) ** 2) / (2.0 * w * w))
    g = (g - g.min()) / (g.max() - g.min())
    return (alpha_max * g).reshape(-1)


def brinkman_batch(nx: int, ny: int, count: int, solid, seed: int) -> np.ndarray:
    """`count` distinct drag fields (brinkman_field of seeds seed, seed + 1, ...), zero on solid
    cells: a (count, nx * ny) array, the adjoint workload's batch of alpha fields."""
    fluid = np.asarray(solid).reshape(-1) == 0
    out = np.stack([brinkman_field(nx, ny, seed + k) for k in range(count)])
    out[:, ~fluid] = 0.0
    return out


def adjoint_channel(nx: int = 512, ny: int = 128):
    """The adjoint workload's geometry: walled channel, periodic in x (tau 0.6, F = (5e-6, 0))."""
    return make_channel(nx, ny)


def cylinder_wake(nx: int = 1024, ny: int = 256, d: float = 32.0, xc: float = 256.0,
                  yc: float = 129.0) -> np.ndarray:
    """Walled channel with a staircase disc of diameter d at (xc, yc) (off-centre by one cell)."""
    return (make_channel(nx, ny) | make_cylinder(nx, ny, xc, yc, d)).astype(np.uint8)


def ensemble_specs(count: int = 256, seed: int = 7) -> list[dict]:
    """Uneven channels of the batched workload: nx ~ U[64, 1024], ny ~ U[32, 512], 1-4 discs of
    radius 4-24 cells clear of the walls, tau ~ U[0.52, 1.0], fx ~ U[1e-6, 1e-5]."""
    specs = []
    u = uniform01(seed, count * 32).reshape(count, 32)
    for k in range(count):
        r = u[k]
        nx = 64 + int(r[0] * (1024 - 64 + 1))
        ny = 32 + int(r[1] * (512 - 32 + 1))
        mask = make_channel(nx, ny).reshape(ny, nx)
        ndisc = 1 + int(r[2] * 4)
        for j in range(ndisc):
            rad = 4.0 + r[3 + 4 * j] * 20.0
            rad = min(rad, (ny - 2) / 2.0 - 2.0)
            cx = r[4 + 4 * j] * nx
            lo, hi = 1.0 + rad + 1.0, ny - 2.0 - rad - 1.0
            cy = lo + r[5 + 4 * j] * max(hi - lo, 0.0)
            mask |= make_cylinder(nx, ny, cx, cy, 2.0 * rad).reshape(ny, nx)
        specs.append({"nx": nx, "ny": ny, "mask": mask.reshape(-1).astype(np.uint8),
                      "tau": 0.52 + r[20] * 0.48, "fx": 1e-6 + r[21] * 9e-6, "fy": 0.0,
                      "seed": seed * 1000003 + k})
    return specs
