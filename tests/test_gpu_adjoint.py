"""Adjoint gradients (hg_loss_and_grad) vs the oracle's forward-mode dual numbers
and central finite differences.

Loss = mean over steps and probes of (h_p^k - obs_kp)^2 over K fixed-dt SSP-RK2
steps; gradients w.r.t. the zone Manning n, per-cell zb (directional) and the
inlet Q.  Tolerances: FP64 adjoint vs dual numbers 1e-8 relative (both are the
exact derivative of the same discrete map); vs central differences (eps 1e-6)
1e-5 relative.
"""
import numpy as np
import pytest

from hydrograd_gb import SWE2D
from hydrograd_gb.workloads import Stream, river_triangles
from oracle.oracle import Oracle
from tests.golden_cases import initial_state, load_fixture, still_water

pytestmark = pytest.mark.gpu


def river():
    return river_triangles(n=24, L=400.0, inlet_q=100.0, pool_center=(60.0, 200.0), pool_radius=70.0)


def make_pair(case, zones=None):
    N = len(case["cell_node_count"])
    zones = case["manning_zones"] if zones is None else zones
    wst = case["wstill"] if "wstill" in case else still_water(case, N)
    ctx = SWE2D(case, precision="fp64")
    ctx.set_still_water(wst)
    ctx.set_manning_zones(case["mat_id"], zones)
    o = Oracle(case)
    o.set_wstill(wst)
    o.set_manning_cells(zones[case["mat_id"]])
    for obj in (ctx, o):
        if len(case["inlet_q"]):
            (obj.set_inlet_q)(case["inlet_q"])
        if len(case["exit_wse"]):
            (obj.set_exit_wse)(case["exit_wse"])
    return ctx, o, N


def observations(case, Q0, K, dt, probes, hidden_zones):
    """Probe depths of a run with hidden zone values (the 'truth' to invert)."""
    _, o, N = make_pair(case, hidden_zones)
    hs = o.hstill()
    obs = np.zeros((K, len(probes)))
    Q = Q0.copy()
    for k in range(K):
        Q = o.rk2(Q, 1, dt=dt)
        obs[k] = Q[probes] + hs[probes]
    return obs


def setup_problem(case, K, nprobe=16, seed=3, near_inlet=False, near_pool=False):
    N = len(case["cell_node_count"])
    Q0 = case["Q0"] if "Q0" in case else initial_state(case, N)
    ctx, o, _ = make_pair(case)
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    cxy = o.mesh_arrays()["centroids"].reshape(N, 2)
    if near_inlet and near_pool:   # half at the west (inlet) edge, half around the pool's rim
        west = np.argsort(cxy[:, 0])[:nprobe // 2]
        r = np.hypot(cxy[:, 0] - case["pool_center"][0], cxy[:, 1] - case["pool_center"][1])
        rim = np.argsort(np.abs(r - case["pool_radius"]))[:nprobe - nprobe // 2]
        probes = np.unique(np.concatenate([west, rim])).astype(np.int32)
    elif near_inlet:   # the cells closest to the west (inlet) edge
        probes = np.sort(np.argsort(cxy[:, 0])[:nprobe]).astype(np.int32)
    else:
        probes = np.unique((Stream(seed).uniform(4 * nprobe) * N).astype(np.int32))[:nprobe]
    hidden = case["manning_zones"] * (1.0 + 0.2 * np.sin(np.arange(len(case["manning_zones"])) + 1.0))
    obs = observations(case, Q0, K, dt, probes, hidden)
    return ctx, o, N, Q0, dt, probes, obs


def rel(a, b):
    return np.abs(a - b) / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("ckpt", [7, 40])
def test_adjoint_matches_dual_numbers_river(ckpt):
    case = river()
    K = 40
    ctx, o, N, Q0, dt, probes, obs = setup_problem(case, K)
    ctx.set_adjoint_tape(0)   # segments of exactly ckpt steps: the recomputation runs
    r = ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=ckpt)
    nz = len(case["manning_zones"])
    dman = np.stack([(case["mat_id"] == z).astype(float) for z in range(nz)])
    v = Stream(11).uniform(N, -1.0, 1.0)
    Qo, _, loss_o, dl_n = o.rk2_tangent(Q0, K, dt, d_manning=dman, probes=probes, obs=obs)
    _, _, _, dl_zb = o.rk2_tangent(Q0, K, dt, d_zb=v[None, :], probes=probes, obs=obs)
    _, _, _, dl_q = o.rk2_tangent(Q0, K, dt, d_inlet=np.ones((1, 1)), probes=probes, obs=obs)
    assert abs(r["loss"] - loss_o) <= 1e-10 * abs(loss_o)
    assert np.abs(r["Q"] - Qo).max() <= 1e-10 * np.abs(Qo).max()
    g_zone = np.array([r["g_manning"][case["mat_id"] == z].sum() for z in range(nz)])
    assert rel(g_zone, dl_n).max() <= 1e-8
    assert abs(r["g_zb"] @ v - dl_zb[0]) <= 1e-8 * abs(dl_zb[0])
    assert abs(r["g_inletq"][0] - dl_q[0]) <= 1e-8 * abs(dl_q[0])


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_checkpoint_interval_does_not_change_the_gradient(precision):
    """Segments of 4 and 30 steps (with recomputation), a byte budget of 5
    stage states (segments of 2, widened to the spacing of 4), and the
    automatic tape (all 30 steps kept): the same loss, gradients and final
    state, bit for bit."""
    case = river()
    K = 30
    _, o, N, Q0, dt, probes, obs = setup_problem(case, K)
    ctx = SWE2D(case, precision=precision)
    ctx.set_still_water(case["wstill"])
    ctx.set_manning_zones(case["mat_id"], case["manning_zones"])
    ctx.set_inlet_q(case["inlet_q"])
    ctx.set_exit_wse(case["exit_wse"])
    runs = []
    for tape, ckpt in ((0, 4), (0, 30), (5 * 24 * N, 4), (-1, 4)):
        ctx.set_adjoint_tape(tape)
        runs.append(ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=ckpt))
    a = runs[0]
    for b in runs[1:]:
        assert a["loss"] == b["loss"]
        for k in ("g_manning", "g_zb", "g_inletq", "Q"):
            assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_partial_gradient_requests_match(precision):
    """Asking for one gradient (the others NULL at the C-ABI) gives that
    gradient, the loss and the final state bit for bit as asking for all."""
    case = river()
    K = 20
    _, o, N, Q0, dt, probes, obs = setup_problem(case, K)
    ctx = SWE2D(case, precision=precision)
    ctx.set_still_water(case["wstill"])
    ctx.set_manning_zones(case["mat_id"], case["manning_zones"])
    ctx.set_inlet_q(case["inlet_q"])
    ctx.set_exit_wse(case["exit_wse"])
    full = ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=5)
    for want, key in ((("manning",), "g_manning"), (("zb",), "g_zb"), (("inletq",), "g_inletq")):
        r = ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=5, want=want)
        assert r["loss"] == full["loss"]
        assert np.array_equal(r["Q"], full["Q"])
        assert np.array_equal(r[key], full[key]), key
        for other in {"g_manning", "g_zb", "g_inletq"} - {key}:
            assert r[other] is None


def test_adjoint_vs_central_differences():
    """Central finite differences of the oracle loss, eps = 1e-6 (FP64)."""
    case = river()
    K = 30
    ctx, o, N, Q0, dt, probes, obs = setup_problem(case, K, near_inlet=True)
    r = ctx.loss_and_grad(Q0, K, dt, probes, obs)
    zones = case["manning_zones"].copy()
    eps = 1e-6
    for z in range(len(zones)):
        if not np.any(case["mat_id"] == z):
            continue
        lp = zones.copy(); lp[z] += eps
        lm = zones.copy(); lm[z] -= eps
        o.set_manning_cells(lp[case["mat_id"]]); fp, _ = o.rk2_loss(Q0, K, dt, probes, obs)
        o.set_manning_cells(lm[case["mat_id"]]); fm, _ = o.rk2_loss(Q0, K, dt, probes, obs)
        fd = (fp - fm) / (2 * eps)
        g = r["g_manning"][case["mat_id"] == z].sum()
        assert abs(g - fd) <= 1e-5 * max(abs(fd), 1e-12), (z, g, fd)
    o.set_manning_cells(zones[case["mat_id"]])
    q = case["inlet_q"].copy()
    eq = eps * q[0]                      # relative perturbation 1e-6 of Q
    o.set_inlet_q(q + eq); fp, _ = o.rk2_loss(Q0, K, dt, probes, obs)
    o.set_inlet_q(q - eq); fm, _ = o.rk2_loss(Q0, K, dt, probes, obs)
    fd = (fp - fm) / (2 * eq)
    assert abs(r["g_inletq"][0] - fd) <= 1e-5 * abs(fd), (r["g_inletq"][0], fd)


def test_adjoint_on_reference_bump_case():
    """The reference's sensitivity case geometry (inlet-Q, exit-H, symmetry), 3 zones."""
    d = load_fixture("sens_bump")
    K = 40
    ctx, o, N, Q0, dt, probes, obs = setup_problem(d, K, nprobe=12)
    r = ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=10)
    nz = len(d["manning_zones"])
    dman = np.stack([(d["mat_id"] == z).astype(float) for z in range(nz)])
    _, _, loss_o, dl_n = o.rk2_tangent(Q0, K, dt, d_manning=dman, probes=probes, obs=obs)
    g_zone = np.array([r["g_manning"][d["mat_id"] == z].sum() for z in range(nz)])
    assert abs(r["loss"] - loss_o) <= 1e-10 * abs(loss_o)
    assert rel(g_zone, dl_n).max() <= 1e-8


def test_fp32c_adjoint_error_vs_fp64():
    """FP32-compensated adjoint: zone-n and inlet-Q gradients within 1e-5 of the
    FP64 oracle's dual numbers; the per-cell zb gradient field within 1e-4
    (normwise) of the FP64 adjoint, itself checked against the oracle above."""
    case = river()
    K = 40
    ctx, o, N, Q0, dt, probes, obs = setup_problem(case, K, near_inlet=True, near_pool=True)
    c32 = SWE2D(case, precision="fp32c")
    c32.set_still_water(case["wstill"])
    c32.set_manning_zones(case["mat_id"], case["manning_zones"])
    c32.set_inlet_q(case["inlet_q"])
    c32.set_exit_wse(case["exit_wse"])
    r32 = c32.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=10)
    r64 = ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=10)
    nz = len(case["manning_zones"])
    dman = np.stack([(case["mat_id"] == z).astype(float) for z in range(nz)])
    _, _, _, dl_n = o.rk2_tangent(Q0, K, dt, d_manning=dman, probes=probes, obs=obs)
    _, _, _, dl_q = o.rk2_tangent(Q0, K, dt, d_inlet=np.ones((1, 1)), probes=probes, obs=obs)
    g_zone = np.array([r32["g_manning"][case["mat_id"] == z].sum() for z in range(nz)])
    assert rel(g_zone, dl_n).max() <= 1e-5
    assert abs(r32["g_inletq"][0] - dl_q[0]) <= 1e-5 * abs(dl_q[0])
    assert np.abs(r64["g_zb"]).max() > 1e-8 * np.abs(r64["g_manning"]).max()   # the probes see the bed
    assert np.abs(r32["g_zb"] - r64["g_zb"]).max() <= 1e-4 * np.abs(r64["g_zb"]).max()
    # state after the run
    for b in range(3):
        ref = r64["Q"][b * N:(b + 1) * N]
        assert np.abs(r32["Q"][b * N:(b + 1) * N] - ref).max() <= 1e-5 * max(np.abs(r64["Q"]).max(), 1e-300)
