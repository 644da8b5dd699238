"""Adjoint forward/backward pair (GPU).

Workload: walled channel 512 x 128, periodic in x, tau 0.6, F = (5e-6, 0), Brinkman drag field
alpha in [0, 0.1] from the seeded sum of 16 Gaussians of width 8-32 cells; J = mean u_x over
the fluid cells averaged over the last 100 of 2000 steps; checkpoints every 100 steps.
Checks: alpha = 0 reproduces the plain method bit for bit; the gradient with respect to fx, tau
and 16 seeded alpha cells agrees with central finite differences (relative step 1e-3) of the
FP64 forward to 1e-4 relative; the FP32 adjoint agrees with the FP64 adjoint; a batch of alpha
fields gives each instance's single-run gradient; a backward step costs at most 3x a forward
step (recomputation included).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY, TAU, FX = 512, 128, 0.6, 5e-6
STEPS, WINDOW, K = 2000, 100, 100
FD_REL = 1e-3


@pytest.fixture(scope="module")
def setup(gpu_lib):
    pkg = gpu_lib
    mask = pkg.workloads.adjoint_channel(NX, NY)
    alpha = pkg.workloads.brinkman_field(NX, NY, seed=1234)
    alpha[mask != 0] = 0.0
    fluid = np.flatnonzero((mask == 0) & (alpha > 0.01))
    u = pkg.workloads.uniform01(4321, 16)
    cells = fluid[(u * len(fluid)).astype(int)]
    return pkg, mask, alpha, cells


@pytest.fixture(scope="module")
def adjoint64(setup):
    pkg, mask, alpha, cells = setup
    with pkg.Adjoint(NX, NY, TAU, FX, 0.0, mask, precision="fp64", checkpoint_every=K) as a:
        a.set_alpha(alpha)
        J = a.forward(STEPS, WINDOW)[0]
        g = a.backward()
        times = a.step_times()
    return J, g, times


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_zero_alpha_is_plain_method(setup, orc, precision):
    pkg, mask, _, _ = setup
    real = "f32" if precision == "fp32" else "f64"
    s0 = orc.seeded_state(77, 1e-4, NX, NY, mask, real)
    with pkg.Adjoint(NX, NY, TAU, FX, 0.0, mask, precision=precision, checkpoint_every=50) as a:
        a.forward(150, 1, s0=s0)
        got = a.populations(0)
    with pkg.Solver(NX, NY, TAU, FX, 0.0, mask, precision=precision) as s:
        s.set_populations(s0)
        s.run(150)
        want = s.populations()
    assert np.array_equal(got, want)


def _fd(pkg, mask, alpha, tau, fx, alphas=None):
    """J of the FP64 forward for (tau, fx) and either alpha or a batch of alpha fields."""
    batch = 1 if alphas is None else len(alphas)
    with pkg.Adjoint(NX, NY, tau, fx, 0.0, mask, precision="fp64", batch=batch,
                     checkpoint_every=STEPS) as a:
        a.set_alpha(alpha if alphas is None else np.stack(alphas))
        return a.forward(STEPS, WINDOW)


def test_gradient_matches_finite_differences(setup, adjoint64):
    pkg, mask, alpha, cells = setup
    J, g, _ = adjoint64
    h_fx, h_tau = FD_REL * FX, FD_REL * TAU
    d_fx = (_fd(pkg, mask, alpha, TAU, FX + h_fx)[0] - _fd(pkg, mask, alpha, TAU, FX - h_fx)[0]) / (2 * h_fx)
    d_tau = (_fd(pkg, mask, alpha, TAU + h_tau, FX)[0] - _fd(pkg, mask, alpha, TAU - h_tau, FX)[0]) / (2 * h_tau)
    assert g["fx"][0] == pytest.approx(d_fx, rel=1e-4)
    assert g["tau"][0] == pytest.approx(d_tau, rel=1e-4)
    fields = []
    for c in cells:
        for sgn in (1.0, -1.0):
            f = alpha.copy()
            f[c] += sgn * FD_REL * alpha[c]
            fields.append(f)
    Jb = _fd(pkg, mask, alpha, TAU, FX, alphas=fields)
    for k, c in enumerate(cells):
        d_a = (Jb[2 * k] - Jb[2 * k + 1]) / (2 * FD_REL * alpha[c])
        assert g["alpha"][0][c] == pytest.approx(d_a, rel=1e-4), f"alpha cell {c}"


def test_fp32_adjoint_matches_fp64(setup, adjoint64):
    pkg, mask, alpha, cells = setup
    J64, g64, _ = adjoint64
    with pkg.Adjoint(NX, NY, TAU, FX, 0.0, mask, precision="fp32", checkpoint_every=K) as a:
        a.set_alpha(alpha)
        J32 = a.forward(STEPS, WINDOW)[0]
        g32 = a.backward()
    assert J32 == pytest.approx(J64, rel=1e-4)
    # the parameter gradients to the finite-difference bar (measured on the 32-field batch:
    # 3e-6 for F_x, 3e-5 for tau); per-cell alpha gradients to 1e-3 on the seeded cells
    assert g32["fx"][0] == pytest.approx(g64["fx"][0], rel=1e-4)
    assert g32["tau"][0] == pytest.approx(g64["tau"][0], rel=1e-4)
    a32, a64 = g32["alpha"][0][cells], g64["alpha"][0][cells]
    assert np.max(np.abs(a32 - a64) / np.abs(a64)) < 1e-3


def test_batch_of_alpha_fields(setup):
    pkg, mask, alpha, cells = setup
    fields = [pkg.workloads.brinkman_field(NX, NY, seed=500 + k) for k in range(4)]
    for f in fields:
        f[mask != 0] = 0.0
    with pkg.Adjoint(NX, NY, TAU, FX, 0.0, mask, precision="fp64", batch=4, checkpoint_every=K) as a:
        a.set_alpha(np.stack(fields))
        Jb = a.forward(400, 50)
        gb = a.backward()
    for k in (0, 3):
        with pkg.Adjoint(NX, NY, TAU, FX, 0.0, mask, precision="fp64", checkpoint_every=K) as a:
            a.set_alpha(fields[k])
            J1 = a.forward(400, 50)[0]
            g1 = a.backward()
        assert Jb[k] == pytest.approx(J1, rel=1e-12)
        assert gb["fx"][k] == pytest.approx(g1["fx"][0], rel=1e-10)
        assert gb["tau"][k] == pytest.approx(g1["tau"][0], rel=1e-10)
        np.testing.assert_allclose(gb["alpha"][k], g1["alpha"][0], rtol=1e-9, atol=1e-18)


def test_batch_of_32_seeded_fields_full_run(setup):
    """The adjoint benchmark's batch: 32 distinct seeded alpha fields (seeds 1234..1265), the
    full 2000 steps with checkpoints every 100, FP32; instances 0 and 31 against single runs
    of their own fields."""
    pkg, mask, _, _ = setup
    fields = pkg.workloads.brinkman_batch(NX, NY, 32, mask, seed=1234)
    assert not np.array_equal(fields[0], fields[1])
    with pkg.Adjoint(NX, NY, TAU, FX, 0.0, mask, precision="fp32", batch=32, checkpoint_every=K) as a:
        a.set_alpha(fields)
        Jb = a.forward(STEPS, WINDOW)
        gb = a.backward()
    assert len(set(np.round(Jb, 12))) == 32
    for k in (0, 31):
        with pkg.Adjoint(NX, NY, TAU, FX, 0.0, mask, precision="fp32", checkpoint_every=K) as a:
            a.set_alpha(fields[k])
            J1 = a.forward(STEPS, WINDOW)[0]
            g1 = a.backward()
        assert Jb[k] == pytest.approx(J1, rel=1e-6)
        assert gb["fx"][k] == pytest.approx(g1["fx"][0], rel=1e-5)
        assert gb["tau"][k] == pytest.approx(g1["tau"][0], rel=1e-5)
        scale = np.max(np.abs(g1["alpha"][0]))
        np.testing.assert_allclose(gb["alpha"][k], g1["alpha"][0], rtol=1e-5, atol=1e-6 * scale)


def test_backward_cost_within_3x_forward(setup):
    pkg, mask, alpha, _ = setup
    with pkg.Adjoint(NX, NY, TAU, FX, 0.0, mask, precision="fp32", batch=32, checkpoint_every=K) as a:
        a.set_alpha(np.stack([alpha] * 32))
        a.forward(STEPS, WINDOW)
        a.backward()
        f, b = a.step_times()
    assert b / f <= 3.0, f"backward step {b * 1e6:.1f} us vs forward {f * 1e6:.1f} us"


def test_autograd_wrapper(setup, adjoint64):
    import torch

    from adjoint_autograd import LbmObjective
    pkg, mask, alpha, cells = setup
    J64, g64, _ = adjoint64
    fx = torch.tensor(FX, dtype=torch.float64, requires_grad=True)
    tau = torch.tensor(TAU, dtype=torch.float64, requires_grad=True)
    al = torch.from_numpy(alpha.copy()).requires_grad_(True)
    with pkg.Adjoint(NX, NY, TAU, FX, 0.0, mask, precision="fp64", checkpoint_every=K) as a:
        J = LbmObjective.apply(fx, tau, al, a, STEPS, WINDOW)
        (2.0 * J).backward()
    assert float(J.detach()) == pytest.approx(J64, rel=1e-12)
    assert float(fx.grad) == pytest.approx(2.0 * g64["fx"][0], rel=1e-10)
    assert float(tau.grad) == pytest.approx(2.0 * g64["tau"][0], rel=1e-10)
    np.testing.assert_allclose(al.grad.numpy()[cells], 2.0 * g64["alpha"][0][cells], rtol=1e-9)


# Ragged geometry: nx = 300 is not a multiple of the 256- or 512-cell tiles (partial last tile,
# row padding to the pitch), a disc across the x = 256 tile boundary and one across the periodic
# x wrap exercise bounce-back in both gathers at tile edges.
RNX, RNY = 300, 64


def _ragged(pkg):
    geo = pkg.geometry
    mask = pkg.workloads.adjoint_channel(RNX, RNY)
    mask = geo.add_disc(mask, RNX, RNY, 255.0, 30.0, 12.0)
    mask = geo.add_disc(mask, RNX, RNY, 3.0, 40.0, 8.0)
    alpha = pkg.workloads.brinkman_field(RNX, RNY, seed=99, wmin=4.0, wmax=12.0)
    alpha[mask != 0] = 0.0
    return mask.astype(np.uint8), alpha


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("cells", [1, 2])
def test_ragged_zero_alpha_is_plain_method(gpu_lib, orc, precision, cells):
    pkg = gpu_lib
    if precision == "fp64" and cells == 2:
        pytest.skip("two cells per lane is an FP32 tile shape")
    mask, _ = _ragged(pkg)
    real = "f32" if precision == "fp32" else "f64"
    s0 = orc.seeded_state(5, 1e-3, RNX, RNY, mask, real)
    with pkg.Adjoint(RNX, RNY, TAU, FX, 0.0, mask, precision=precision, checkpoint_every=40) as a:
        a.set_tiles(cells, cells)
        assert a.tiles() == (cells, cells)
        a.forward(120, 1, s0=s0)
        got = a.populations(0)
    with pkg.Solver(RNX, RNY, TAU, FX, 0.0, mask, precision=precision) as s:
        s.set_populations(s0)
        s.run(120)
        want = s.populations()
    assert np.array_equal(got, want)


def test_tile_shapes_agree(gpu_lib):
    """Both tile shapes of both sweeps: the same states and per-cell gradients bit for bit (the
    per-cell recursions do not depend on the tiling), the same objective and parameter
    gradients up to the order of their sums."""
    pkg = gpu_lib
    mask, alpha = _ragged(pkg)
    results = {}
    for shape in [(1, 1), (2, 2), (1, 2), (2, 1)]:
        with pkg.Adjoint(RNX, RNY, TAU, FX, 0.0, mask, precision="fp32", batch=2, checkpoint_every=70) as a:
            a.set_tiles(*shape)
            a.set_alpha(np.stack([alpha, 0.5 * alpha]))
            J = a.forward(500, 60)
            g = a.backward()
            results[shape] = (J, g, a.populations(1))
    J0, g0, s0 = results[(1, 1)]
    for shape, (J, g, s) in results.items():
        assert np.array_equal(s, s0), shape
        np.testing.assert_allclose(J, J0, rtol=1e-5)
        assert np.array_equal(g["alpha"], g0["alpha"]), shape
        np.testing.assert_allclose(g["fx"], g0["fx"], rtol=1e-5)
        np.testing.assert_allclose(g["tau"], g0["tau"], rtol=1e-5)


def test_ragged_gradient_matches_finite_differences(gpu_lib):
    """FP64 at the ragged size, checkpoints every 70 of 600 steps (a short last segment): the
    gradients with respect to fx and to the alpha cell of largest drag agree with central
    differences to 1e-4 relative."""
    pkg = gpu_lib
    mask, alpha = _ragged(pkg)
    steps, window = 600, 100

    def J(fx, al):
        with pkg.Adjoint(RNX, RNY, TAU, fx, 0.0, mask, precision="fp64", checkpoint_every=steps) as a:
            a.set_alpha(al)
            return a.forward(steps, window)[0]

    with pkg.Adjoint(RNX, RNY, TAU, FX, 0.0, mask, precision="fp64", checkpoint_every=70) as a:
        a.set_alpha(alpha)
        a.forward(steps, window)
        g = a.backward()
    h = FD_REL * FX
    assert g["fx"][0] == pytest.approx((J(FX + h, alpha) - J(FX - h, alpha)) / (2 * h), rel=1e-4)
    c = int(np.argmax(alpha))
    ap, am = alpha.copy(), alpha.copy()
    ap[c] += FD_REL * alpha[c]
    am[c] -= FD_REL * alpha[c]
    d_a = (J(FX, ap) - J(FX, am)) / (2 * FD_REL * alpha[c])
    assert g["alpha"][0][c] == pytest.approx(d_a, rel=1e-4)
