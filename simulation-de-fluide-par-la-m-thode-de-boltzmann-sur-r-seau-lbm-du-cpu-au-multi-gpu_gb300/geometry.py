"""Solid masks and channel helpers, restating the reference's geometry module
(src/common/geometry.hpp:11-31, src/common/geometry.cpp:5-23) for Python callers.

A mask is a row-major uint8 array of nx*ny cells, solid[y*nx + x] = 1 for a solid cell.
"""
from __future__ import annotations

import numpy as np


def make_channel(nx: int, ny: int) -> np.ndarray:
    """Plane channel: solid rows y = 0 and y = ny - 1, periodic in x (geometry.cpp:5-12).
    With halfway bounce-back the channel height is H = ny - 2."""
    m = np.zeros((ny, nx), np.uint8)
    m[0, :] = 1
    m[ny - 1, :] = 1
    return m.reshape(-1)


def make_cylinder(nx: int, ny: int, xc: float, yc: float, d: float) -> np.ndarray:
    """Staircase disc of diameter d centred at (xc, yc): a cell is solid when its centre lies
    in the disc, dx*dx + dy*dy <= D*D/4 in double precision (geometry.cpp:14-23)."""
    y, x = np.mgrid[0:ny, 0:nx]
    dx = x.astype(np.float64) - xc
    dy = y.astype(np.float64) - yc
    return ((dx * dx + dy * dy) <= 0.25 * d * d).astype(np.uint8).reshape(-1)


def add_disc(mask: np.ndarray, nx: int, ny: int, xc: float, yc: float, d: float) -> np.ndarray:
    """Returns mask with the disc of make_cylinder added (logical or)."""
    return (mask.reshape(-1) | make_cylinder(nx, ny, xc, yc, d)).astype(np.uint8)


def add_block(mask: np.ndarray, nx: int, x0: int, x1: int, y0: int, y1: int) -> np.ndarray:
    """Returns mask with the cells x0 <= x < x1, y0 <= y < y1 made solid."""
    m = mask.reshape(-1, nx).copy()
    m[y0:y1, x0:x1] = 1
    return m.reshape(-1)


def viscosity(tau: float, dtype=np.float32):
    """nu = (tau - 1/2) / 3 in the solver precision (d2q9.hpp:30)."""
    t = dtype(tau)
    return dtype(dtype(t - dtype(0.5)) / dtype(3))


def poiseuille_force(h: int, tau: float, u_max: float, dtype=np.float32):
    """Body force of a Poiseuille profile of peak velocity u_max in a channel of height h,
    F = 8 nu u_max / h^2, evaluated in the solver precision in the reference's order
    (geometry.hpp:24-26)."""
    nu = viscosity(tau, dtype)
    hh = dtype(dtype(h) * dtype(h))
    return dtype(dtype(dtype(dtype(8) * nu) * dtype(u_max)) / hh)


def poiseuille_velocity(s: float, h: int, nu: float, force: float) -> float:
    """Analytic Poiseuille velocity at distance s from the effective wall (geometry.hpp:28-31)."""
    return force / (2.0 * nu) * s * (h - s)
