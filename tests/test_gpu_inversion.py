"""Final-state inversion loss (hg_final_loss_and_grad) and the inversion
driver on the device, against the oracle.

The loss value is checked against a numpy restatement of
compute_loss_inversion applied to the oracle's final state (FP64: 1e-12); the
gradients against central finite differences of the oracle's loss (1e-5 of the
largest component, as the probe-loss gradients are); FP32C gradients against
the FP64 ones (1e-5 normwise).
"""
import json
import os

import numpy as np
import pytest

from hydrograd_gb.inversion import Inversion, InversionSettings
from tests.golden_cases import initial_state, load_fixture
from tests.test_gpu_forward import setup_pair

pytestmark = pytest.mark.gpu

SQRT_EPS = np.sqrt(np.finfo(np.float64).eps)
NSTEPS, DT = 200, 0.05


def observed(d):
    """observed_data of the reference's inversion: the truth fields."""
    return dict(WSE_truth=d["xi_truth"] + d["wstill_truth"], u_truth=d["u_truth"], v_truth=d["v_truth"],
                zb_cell_truth=d["zb_cell_truth"])


def loss_np(Q, hstill, zbw, obs, use_wse=True, use_uv=True):
    """compute_loss_inversion's WSE and uv terms (swe_2D_inversion.jl:383-431)."""
    N = len(hstill)
    h = Q[:N] + hstill
    lw = luv = 0.0
    if use_wse:
        w = obs["WSE_truth"]
        r = ((h + zbw) - w) / ((w.max() - w.min()) + SQRT_EPS)
        lw = np.sum(r * r) / N
    if use_uv:
        u, v = obs["u_truth"], obs["v_truth"]
        vs = max(np.sqrt(u ** 2 + v ** 2).max(), np.finfo(np.float64).eps)
        lu = (Q[N:2 * N] / (h + SQRT_EPS) - u) / vs
        lv = (Q[2 * N:] / (h + SQRT_EPS) - v) / vs
        luv = (np.sum(lu * lu) + np.sum(lv * lv)) / N
    return lw, luv


def oracle_loss(o, Q0, obs, zbw):
    Q = o.rk2(Q0, NSTEPS, dt=DT, nthreads=4)
    return sum(loss_np(Q, o.hstill(), zbw, obs))


@pytest.fixture(scope="module")
def case():
    d = load_fixture("fwd_savannah")
    return d, observed(d)


def test_loss_value_matches_restatement(case):
    d, obs = case
    ctx, o, N = setup_pair(d, "fp64")
    Q0 = initial_state(d, N)
    r = ctx.final_loss_and_grad(Q0, NSTEPS, DT, wse=obs["WSE_truth"], u=obs["u_truth"], v=obs["v_truth"],
                                zb_wse=obs["zb_cell_truth"])
    Qo = o.rk2(Q0, NSTEPS, dt=DT, nthreads=4)
    lw, luv = loss_np(Qo, o.hstill(), obs["zb_cell_truth"], obs)
    assert abs(r["loss_wse"] - lw) <= 1e-12 * lw
    assert abs(r["loss_uv"] - luv) <= 1e-12 * luv
    assert abs(r["loss"] - (lw + luv)) <= 1e-12 * (lw + luv)
    np.testing.assert_allclose(r["Q"], Qo, rtol=0, atol=1e-10 * np.abs(Qo).max())


def test_zone_and_inlet_gradients_match_finite_differences(case):
    d, obs = case
    ctx, o, N = setup_pair(d, "fp64")
    Q0 = initial_state(d, N)
    r = ctx.final_loss_and_grad(Q0, NSTEPS, DT, wse=obs["WSE_truth"], u=obs["u_truth"], v=obs["v_truth"],
                                zb_wse=obs["zb_cell_truth"])
    mat, zones = d["mat_id"], np.array(d["manning_zones"], dtype=float)
    gz = np.bincount(mat, r["g_manning"], minlength=len(zones))
    fd = np.zeros_like(zones)
    for z in range(len(zones)):
        vals = []
        for s in (1, -1):
            zz = zones.copy()
            zz[z] += s * 1e-6
            o.set_manning_cells(zz[mat])
            vals.append(oracle_loss(o, Q0, obs, obs["zb_cell_truth"]))
        fd[z] = (vals[0] - vals[1]) / 2e-6
    o.set_manning_cells(zones[mat])
    assert np.abs(gz - fd).max() <= 1e-5 * np.abs(fd).max()
    q = np.array(d["inlet_q"], dtype=float)
    vals = []
    for s in (1, -1):
        o.set_inlet_q(q + s * 1e-6 * q)
        vals.append(oracle_loss(o, Q0, obs, obs["zb_cell_truth"]))
    o.set_inlet_q(q)
    fdq = (vals[0] - vals[1]) / (2e-6 * q[0])
    assert abs(r["g_inletq"][0] - fdq) <= 1e-5 * abs(fdq)


def test_active_zb_gradient_matches_finite_differences(case):
    """zb active: WSE_pred = h + zb (direct term) besides the bed slope and the
    exit-H ghost depth."""
    d, obs = case
    ctx, o, N = setup_pair(d, "fp64")
    Q0 = initial_state(d, N)
    zb = d["zb_cell_truth"].copy()
    r = ctx.final_loss_and_grad(Q0, NSTEPS, DT, wse=obs["WSE_truth"], u=obs["u_truth"], v=obs["v_truth"])
    rng = np.random.default_rng(3)
    for _ in range(2):
        dirn = rng.normal(0.0, 0.05, N)
        vals = []
        for s in (1, -1):
            z = zb + s * 1e-6 * dirn
            o.set_zb_cells(z)
            vals.append(oracle_loss(o, Q0, obs, z))
        fd = (vals[0] - vals[1]) / 2e-6
        assert abs(r["g_zb"] @ dirn - fd) <= 1e-5 * abs(fd)
    o.set_zb_cells(zb)


def test_fp32c_gradients_match_fp64(case):
    d, obs = case
    out = {}
    for prec in ("fp64", "fp32c"):
        ctx, _, N = setup_pair(d, prec)
        out[prec] = ctx.final_loss_and_grad(initial_state(d, N), NSTEPS, DT, wse=obs["WSE_truth"], u=obs["u_truth"],
                                            v=obs["v_truth"], zb_wse=obs["zb_cell_truth"])
    a, b = out["fp32c"], out["fp64"]
    assert abs(a["loss"] - b["loss"]) <= 1e-5 * b["loss"]
    for k in ("g_manning", "g_zb", "g_inletq"):
        assert np.abs(a[k] - b[k]).max() <= 1e-5 * np.abs(b[k]).max(), k


def test_driver_total_gradient_and_adam_iterations(case, tmp_path):
    """The driver's loss_total = pred + bound + slope with its gradient
    (finite differences of the device's own FP64 losses), then Adam
    iterations that lower the loss and write the reference's callback files."""
    d, obs = case
    ctx, _, N = setup_pair(d, "fp64")
    Q0 = initial_state(d, N)
    s = InversionSettings(active_param="zb", wse_loss=True, uv_loss=True, bound_loss=True, slope_loss=True,
                          lower_bound=float(d["zb_cell_truth"].min()) + 0.5, upper_bound=float(d["zb_cell_truth"].max()),
                          slope_upper_bound=0.01)
    inv = Inversion(ctx, d, Q0, NSTEPS, DT, obs, s, ckpt_every=40)
    zb = d["zb_cell_truth"].copy()
    parts, g, _ = inv.loss_and_grad(zb)
    assert parts[4] > 0 and parts[5] > 0     # both regularisers active at this zb
    assert np.isclose(parts[0], parts[1] + parts[4] + parts[5], rtol=1e-14)
    dirn = np.random.default_rng(5).normal(0.0, 0.05, N)
    fd = (inv.loss_and_grad(zb + 1e-6 * dirn)[0][0] - inv.loss_and_grad(zb - 1e-6 * dirn)[0][0]) / 2e-6
    assert abs(g @ dirn - fd) <= 1e-5 * abs(fd)

    mat = d["mat_id"]
    s2 = InversionSettings(active_param="ManningN", wse_loss=True, uv_loss=True, bound_loss=True,
                           lower_bound=0.01, upper_bound=0.06, optimizers=["Adam", "LBFGS"],
                           learning_rates=[0.002, 0.01], max_iterations=[8, 0], save_checkpoint=True,
                           checkpoint_frequency=4)
    inv2 = Inversion(ctx, d, Q0, NSTEPS, DT, obs, s2, mat_id=mat, case_path=str(tmp_path))
    res = inv2.run(np.full(len(d["manning_zones"]), 0.03))
    assert res["ITER"] == list(range(1, 9))
    assert res["LOSS"][-1] < res["LOSS"][0]
    cb = json.load(open(os.path.join(tmp_path, "inversion_callback_save_iter_8.json")))
    assert set(cb) == {"iter_number", "loss_total", "theta"} and cb["iter_number"] == 8
    assert np.isclose(cb["loss_total"], res["LOSS"][7])
    ck = json.load(open(os.path.join(tmp_path, "checkpoint_inversion_iter_8.json")))
    assert ck["ITER"] == list(range(1, 9)) and len(ck["PARS"]) == 8


def test_lbfgs_stage_after_adam_lowers_the_loss(case, tmp_path):
    """The reference's optimiser sequence with its LBFGS stage enabled: 4 Adam
    iterations, then up to 4 LBFGS iterations (backtracking line search on the
    device's loss and gradient) that lower the loss further, one history
    entry and callback file per iteration."""
    d, obs = case
    ctx, _, N = setup_pair(d, "fp64")
    Q0 = initial_state(d, N)
    s = InversionSettings(active_param="ManningN", wse_loss=True, uv_loss=True, optimizers=["Adam", "LBFGS"],
                          learning_rates=[0.002, 0.0], max_iterations=[4, 4])
    inv = Inversion(ctx, d, Q0, NSTEPS, DT, obs, s, mat_id=d["mat_id"], case_path=str(tmp_path))
    res = inv.run(np.full(len(d["manning_zones"]), 0.03))
    n = len(res["LOSS"])
    assert 5 <= n <= 8 and res["ITER"] == list(range(1, n + 1))
    assert res["LOSS"][-1] < res["LOSS"][3]
    assert os.path.exists(os.path.join(tmp_path, f"inversion_callback_save_iter_{n}.json"))
