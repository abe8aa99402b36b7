"""Inversion driver pieces without a GPU: the regularisers and their
gradients, the cell-gradient operator (pinned to the reference's bed slope),
the optimisers (Adam, Descent, L-BFGS with backtracking), the optimiser
sequence, and the run-control settings."""
import numpy as np
import pytest

from hydrograd_gb import HostMesh
from hydrograd_gb.inversion import (LBFGS, Adam, CellGradient, Descent, Inversion, InversionSettings, backtracking,
                                    bound_loss, slope_loss)
from tests.golden_cases import load_fixture


def grad_op(d):
    return CellGradient(HostMesh(d).cell_faces(), d["cell_node_count"])


@pytest.mark.parametrize("name", ["fwd_bump", "fwd_savannah"])
def test_cell_gradient_is_minus_reference_bed_slope(name):
    """compute_scalar_gradients_from_cells and the bed slope S0 of
    update_bed_data are the same Green-Gauss map up to sign; S0_cells_truth is
    the reference's own output."""
    d = load_fixture(name)
    gx, gy = grad_op(d).apply(d["zb_cell_truth"])
    S0 = d["S0_cells_truth"].reshape(2, -1)
    scale = np.abs(S0).max()
    assert np.abs(gx + S0[0]).max() <= 1e-13 * scale
    assert np.abs(gy + S0[1]).max() <= 1e-13 * scale


def test_cell_gradient_transpose():
    d = load_fixture("fwd_savannah")
    G = grad_op(d)
    rng = np.random.default_rng(1)
    z, ax, ay = rng.normal(size=G.N), rng.normal(size=G.N), rng.normal(size=G.N)
    gx, gy = G.apply(z)
    assert abs(ax @ gx + ay @ gy - z @ G.transpose(ax, ay)) <= 1e-10 * np.abs(ax @ gx + ay @ gy)


def fd_check(f, x, g, n=6, seed=0, eps=1e-6):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        dirn = rng.normal(size=x.shape)
        fd = (f(x + eps * dirn) - f(x - eps * dirn)) / (2 * eps)
        assert abs(fd - g @ dirn) <= 1e-6 * max(abs(fd), 1e-12) + 1e-12


def test_bound_loss_gradient():
    p = np.array([0.005, 0.02, 0.05, 0.07, 0.1])
    val, g = bound_loss(p, 0.01, 0.06)
    r = 0.05
    assert np.isclose(val, (0.005 / r) ** 2 + (0.01 / r) ** 2 + (0.04 / r) ** 2)
    fd_check(lambda x: bound_loss(x, 0.01, 0.06)[0], p, g)


def test_slope_loss_gradient():
    d = load_fixture("fwd_savannah")
    G = grad_op(d)
    zb = d["zb_cell_truth"]
    val, g = slope_loss(zb, G, 0.05)
    assert val > 0   # the river bed has slopes above 0.05 somewhere
    fd_check(lambda x: slope_loss(x, G, 0.05)[0], zb, g, eps=1e-7)


def test_adam_matches_optimisers_jl():
    """Optimisers.Adam: the first step moves every coordinate by eta against
    the gradient's sign (bias-corrected moments); later steps follow
    m / (1 - b1^t) / (sqrt(v / (1 - b2^t)) + eps)."""
    opt = Adam(0.01)
    th = np.array([1.0, -2.0, 3.0])
    g1 = np.array([0.5, -3.0, 1e-3])
    th1 = opt.step(th, g1)
    np.testing.assert_allclose(th1, th - 0.01 * np.sign(g1) * np.abs(g1) / (np.abs(g1) + 1e-8), rtol=1e-12)
    g2 = np.array([0.1, 0.2, -0.3])
    th2 = opt.step(th1, g2)
    m = 0.9 * 0.1 * g1 + 0.1 * g2
    v = 0.999 * 0.001 * g1 ** 2 + 0.001 * g2 ** 2
    want = th1 - m / (1 - 0.81) / (np.sqrt(v / (1 - 0.999 ** 2)) + 1e-8) * 0.01
    np.testing.assert_allclose(th2, want, rtol=1e-12)
    np.testing.assert_allclose(Descent(0.1).step(th, g1), th - 0.1 * g1)


def test_settings_from_run_control():
    """The keys of the reference's inversion run-control block
    (examples/SWE_2D/inversion/*/run_control.json)."""
    opts = {"active_param_names": ["ManningN"], "inversion_bInversion_WSE_loss": True,
            "inversion_bInversion_uv_loss": True, "inversion_bInversion_bound_loss": True,
            "inversion_bInversion_slope_loss": False, "inversion_parameter_value_lower_bound": 0.01,
            "inversion_parameter_value_upper_bound": 0.06, "inversion_parameter_slope_upper_bound": 0.2,
            "inversion_optimizers": ["Adam", "LBFGS"], "inversion_learning_rates": [0.001, 0.01],
            "inversion_max_iterations": [300, 0], "inversion_save_frequency": 1, "inversion_save_checkpoint": True,
            "inversion_checkpoint_frequency": 10}
    s = InversionSettings.from_run_control(opts)
    assert (s.active_param, s.uv_loss, s.bound_loss, s.slope_loss) == ("ManningN", True, True, False)
    assert s.optimizers == ["Adam", "LBFGS"] and s.max_iterations == [300, 0]


def test_backtracking_takes_the_quadratic_minimiser_first():
    """phi(a) = (a - 0.3)^2 from a = 1: Armijo fails, the quadratic through
    phi(0), phi'(0) and phi(1) has its minimum at 0.3, inside [0.1, 0.5]."""
    phi = lambda a: (a - 0.3) ** 2
    a, pa, n = backtracking(phi, phi(0.0), -0.6)
    assert abs(a - 0.3) <= 1e-15 and pa <= 1e-30 and n == 2


def test_backtracking_keeps_steps_within_bounds():
    """A steep rise: the interpolated step is clamped to 0.1 of the last."""
    phi = lambda a: -a + 1e6 * a * a
    a, pa, n = backtracking(phi, 0.0, -1.0)
    assert pa <= 0.0 + 1e-4 * a * -1.0 and a < 1e-5 and n > 2


def test_lbfgs_minimizes_rosenbrock():
    def fg(x):
        return (100 * (x[1] - x[0] ** 2) ** 2 + (1 - x[0]) ** 2,
                np.array([-400 * x[0] * (x[1] - x[0] ** 2) - 2 * (1 - x[0]), 200 * (x[1] - x[0] ** 2)]))
    opt = LBFGS()
    x, f, conv = opt.minimize(fg, np.array([-1.2, 1.0]), 200)
    assert conv and np.abs(x - 1.0).max() <= 1e-8 and len(opt.S) <= 10


class QuadraticInversion(Inversion):
    """The driver's optimiser sequence on loss 0.5 |A theta - b|^2 (no device)."""

    def __init__(self, settings):
        self.s, self.case_path = settings, None
        r = np.random.default_rng(3)
        self.A, self.b = r.normal(size=(8, 4)), r.normal(size=8)

    def loss_and_grad(self, theta):
        e = self.A @ theta - self.b
        return (0.5 * e @ e, 0.0, 0.0, 0.0, 0.0, 0.0), self.A.T @ e, None


def test_optimiser_sequence_adam_then_lbfgs():
    """Adam for 5 iterations, then LBFGS to the least-squares solution; the
    histories hold one entry per iteration and the LBFGS stage converges."""
    s = InversionSettings(optimizers=["Adam", "LBFGS"], learning_rates=[0.01, 0.0], max_iterations=[5, 100],
                          rel_tols=[0.0, 1e-14])
    inv = QuadraticInversion(s)
    out = inv.run(np.zeros(4))
    x = np.linalg.lstsq(inv.A, inv.b, rcond=None)[0]
    assert np.abs(out["theta"] - x).max() <= 1e-6
    assert out["ITER"] == list(range(1, len(out["LOSS"]) + 1)) and 5 < len(out["LOSS"]) < 105
    assert out["LOSS"][-1] <= out["LOSS"][4]
