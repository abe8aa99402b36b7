"""Gradients through fixed Tsit5 steps (hg_set_adjoint_integrator(HG_ADJ_TSIT5)).

The reference differentiates its Tsit5 solve (swe_2D_inversion.jl:304-339,
swe_2D_sensitivity.jl:80).  With the integrator set to Tsit5 the gradient
calls run nsteps fixed Tsit5 steps of dt (hg_integrate_tsit5 with adaptive =
0) and take the exact discrete adjoint of those steps.  Checked against the
oracle's forward-mode dual numbers of the same steps (hgo::tsit5_fixed_step,
1e-8 relative: both are the exact derivative of the same discrete map) and
central differences of the oracle's loss (eps 1e-6, 1e-5 relative), as the
SSP-RK2 adjoint is in tests/test_gpu_adjoint.py: the probe loss's zone-n,
inlet-Q and directional zb gradients, several checkpoint spacings, an inlet
hydrograph (central differences of a shift), and final-state
vector-Jacobian products (hg_final_vjp) against the duals' final-state
tangents.  FP32C contexts run the same adjoint on FP32 vectors (the unmasked
FP32 VJP kernels): against the same duals at FP32C tolerances, and through a
sigmoid n and a UDE closure against the FP64 device adjoint.
"""
import numpy as np
import pytest

from hydrograd_gb import HgError, SWE2D
from hydrograd_gb.workloads import Stream, river_triangles
from tests.test_gpu_adjoint import make_pair

pytestmark = pytest.mark.gpu

K = 24


def river():
    return river_triangles(n=24, L=400.0, inlet_q=100.0, pool_center=(60.0, 200.0), pool_radius=70.0)


@pytest.fixture(scope="module")
def problem():
    case = river()
    ctx, o, N = make_pair(case)
    Q0 = case["Q0"]
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    cxy = o.mesh_arrays()["centroids"].reshape(N, 2)
    r = np.hypot(cxy[:, 0] - case["pool_center"][0], cxy[:, 1] - case["pool_center"][1])
    probes = np.unique(np.concatenate([np.argsort(cxy[:, 0])[:8],
                                       np.argsort(np.abs(r - case["pool_radius"]))[:8]])).astype(np.int32)
    hs = o.hstill()
    # observations: the probe depths of a Tsit5 run with other zone values
    hidden = case["manning_zones"] * (1.0 + 0.2 * np.sin(np.arange(len(case["manning_zones"])) + 1.0))
    _, oh, _ = make_pair(case, hidden)
    obs = np.zeros((K, len(probes)))
    Q = Q0.copy()
    for k in range(K):
        _, Q = oh.tsit5_loss(Q, 1, dt, probes[:0], np.zeros((1, 0)))
        obs[k] = Q[probes] + hs[probes]
    zones = case["mat_id"]
    nz = len(case["manning_zones"])
    dman = np.zeros((nz, N))
    for z in range(nz):
        dman[z, zones == z] = 1.0
    v = Stream(5).uniform(N, -1.0, 1.0)
    dzb = v[None, :]
    Qo, dQ, L, dL = o.tsit5_tangent(Q0, K, dt, d_manning=dman, probes=probes, obs=obs, nthreads=4)
    _, dQz, _, dLz = o.tsit5_tangent(Q0, K, dt, d_zb=dzb, probes=probes, obs=obs, nthreads=4)
    _, dQq, _, dLq = o.tsit5_tangent(Q0, K, dt, d_inlet=np.ones((1, 1)), probes=probes, obs=obs, nthreads=4)
    ctx.set_adjoint_integrator("tsit5")
    return dict(case=case, ctx=ctx, o=o, N=N, Q0=Q0, dt=dt, probes=probes, obs=obs, Qo=Qo, L=L, dL=dL, dQ=dQ,
                v=v, dLz=dLz, dQz=dQz, dLq=dLq, dQq=dQq, zones=zones, nz=nz)


def zone_sums(g, zones, nz):
    return np.array([g[zones == z].sum() for z in range(nz)])


@pytest.mark.parametrize("ckpt", [5, 50])
def test_loss_and_gradients_match_dual_numbers(problem, ckpt):
    p = problem
    r = p["ctx"].loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=ckpt)
    assert abs(r["loss"] - p["L"]) <= 1e-12 * abs(p["L"])
    assert np.abs(r["Q"] - p["Qo"]).max() <= 1e-12 * np.abs(p["Qo"]).max()   # the same forward steps
    gz = zone_sums(r["g_manning"], p["zones"], p["nz"])
    assert np.abs(gz - p["dL"][:p["nz"]]).max() <= 1e-8 * np.abs(p["dL"][:p["nz"]]).max()
    assert abs(r["g_zb"] @ p["v"] - p["dLz"][0]) <= 1e-8 * abs(p["dLz"][0])
    assert abs(r["g_inletq"][0] - p["dLq"][0]) <= 1e-8 * abs(p["dLq"][0])


def test_checkpoint_spacing_does_not_change_the_gradient(problem):
    p = problem
    p["ctx"].set_adjoint_tape(0)   # segments of exactly ckpt_every steps
    try:
        a = p["ctx"].loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=5)
        b = p["ctx"].loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=K)
    finally:
        p["ctx"].set_adjoint_tape(-1)
    for k in ("g_manning", "g_zb", "g_inletq"):
        assert np.abs(a[k] - b[k]).max() <= 1e-12 * np.abs(b[k]).max()


def test_inlet_gradient_matches_central_differences(problem):
    p = problem
    o, case = p["o"], p["case"]
    r = p["ctx"].loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"])
    q0 = case["inlet_q"][0]
    eps = 1e-6 * q0
    o.set_inlet_q(np.array([q0 + eps]))
    lp, _ = o.tsit5_loss(p["Q0"], K, p["dt"], p["probes"], p["obs"])
    o.set_inlet_q(np.array([q0 - eps]))
    lm, _ = o.tsit5_loss(p["Q0"], K, p["dt"], p["probes"], p["obs"])
    o.set_inlet_q(case["inlet_q"])
    fd = (lp - lm) / (2 * eps)
    assert abs(r["g_inletq"][0] - fd) <= 1e-5 * abs(fd)


def test_final_vjp_matches_dual_numbers(problem):
    """lam^T dQ_K/dtheta for a random cotangent lam of the final state."""
    p = problem
    lam = Stream(11).uniform(3 * p["N"], -1.0, 1.0)
    r = p["ctx"].final_state_vjp(p["Q0"], K, p["dt"], lam)
    ref_n = p["dQ"][:p["nz"]] @ lam
    gz = zone_sums(r["g_manning"], p["zones"], p["nz"])
    assert np.abs(gz - ref_n).max() <= 1e-8 * np.abs(ref_n).max()
    assert abs(r["g_zb"] @ p["v"] - p["dQz"][0] @ lam) <= 1e-8 * abs(p["dQz"][0] @ lam)
    assert abs(r["g_inletq"][0] - p["dQq"][0] @ lam) <= 1e-8 * abs(p["dQq"][0] @ lam)


def test_hydrograph_run_matches_central_differences():
    """An inlet hydrograph, evaluated at every stage's own time t_s + c_i dt in
    the forward steps, the recomputation and the VJPs: the loss against the
    oracle's and the inlet-Q gradient -- the derivative w.r.t. a constant
    shift of the hydrograph -- against central differences of the oracle's
    loss with the hydrograph shifted (eps 1e-6 relative)."""
    case = river()
    ctx, o, N = make_pair(case)
    T = np.array([0.0, 3.0, 8.0])
    Qh = np.array([60.0, 140.0, 90.0])
    ctx.set_inlet_hydrograph(0, T, Qh)
    dt = 0.5 * o.cfl_dt(case["Q0"], 0.4)
    probes = np.arange(0, N, max(1, N // 12), dtype=np.int32)
    obs = np.full((K, len(probes)), 0.5)
    ctx.set_adjoint_integrator("tsit5")
    r = ctx.loss_and_grad(case["Q0"], K, dt, probes, obs, ckpt_every=7)
    loss = {}
    for sgn in (0.0, 1.0, -1.0):
        o.set_hydrograph(0, T, Qh + sgn * 1e-6 * Qh.mean())
        loss[sgn], _ = o.tsit5_loss(case["Q0"], K, dt, probes, obs)
    fd = (loss[1.0] - loss[-1.0]) / (2e-6 * Qh.mean())
    assert abs(r["loss"] - loss[0.0]) <= 1e-12 * abs(loss[0.0])
    assert abs(r["g_inletq"][0] - fd) <= 1e-5 * abs(fd)


def fp32c_ctx(case):
    c = SWE2D(case, precision="fp32c")
    c.set_still_water(case["wstill"])
    c.set_manning_zones(case["mat_id"], case["manning_zones"])
    c.set_inlet_q(case["inlet_q"])
    c.set_exit_wse(case["exit_wse"])
    c.set_adjoint_integrator("tsit5")
    return c


# FP32C against the FP64 duals: the forward states within 1e-5 of scale (the
# FP32C state error), the gradients within 1e-3 of their largest component
# (FP32 cotangents through 24 steps of six stages).
@pytest.mark.parametrize("ckpt", [5, 50])
def test_fp32c_loss_and_gradients_match_dual_numbers(problem, ckpt):
    p = problem
    c = fp32c_ctx(p["case"])
    r = c.loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=ckpt)
    assert np.abs(r["Q"] - p["Qo"]).max() <= 1e-5 * np.abs(p["Qo"]).max()
    assert abs(r["loss"] - p["L"]) <= 1e-4 * abs(p["L"])
    gz = zone_sums(r["g_manning"], p["zones"], p["nz"])
    assert np.abs(gz - p["dL"][:p["nz"]]).max() <= 1e-3 * np.abs(p["dL"][:p["nz"]]).max()
    assert abs(r["g_zb"] @ p["v"] - p["dLz"][0]) <= 1e-3 * abs(p["dLz"][0])
    assert abs(r["g_inletq"][0] - p["dLq"][0]) <= 1e-3 * abs(p["dLq"][0])


def test_fp32c_checkpoint_spacing_and_repeat_give_the_same_bits(problem):
    p = problem
    c = fp32c_ctx(p["case"])
    a = c.loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=5)
    b = c.loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=7)
    d = c.loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=5)
    for k in ("g_manning", "g_zb", "g_inletq"):
        np.testing.assert_array_equal(a[k], b[k])
        np.testing.assert_array_equal(a[k], d[k])
    assert a["loss"] == b["loss"] == d["loss"]


def test_fp32c_final_vjp_matches_dual_numbers(problem):
    p = problem
    c = fp32c_ctx(p["case"])
    lam = Stream(11).uniform(3 * p["N"], -1.0, 1.0)
    r = c.final_state_vjp(p["Q0"], K, p["dt"], lam)
    ref_n = p["dQ"][:p["nz"]] @ lam
    gz = zone_sums(r["g_manning"], p["zones"], p["nz"])
    assert np.abs(gz - ref_n).max() <= 1e-3 * np.abs(ref_n).max()
    assert abs(r["g_zb"] @ p["v"] - p["dQz"][0] @ lam) <= 1e-3 * abs(p["dQz"][0] @ lam)
    assert abs(r["g_inletq"][0] - p["dQq"][0] @ lam) <= 1e-3 * abs(p["dQq"][0] @ lam)


def test_adaptive_solve_steps_are_differentiated(problem):
    """hg_set_adjoint_steps: the accepted steps of an adaptive solve
    (hg_tsit5_steps), held fixed and differentiated.  Equal steps of dt give
    the fixed-step gradient bit for bit; the adaptive sequence's gradients
    agree with central differences of the device's own loss over the same
    steps (zone n, inlet Q; FP64), and FP32C with FP64 within 1e-3."""
    p = problem
    ctx, case = p["ctx"], p["case"]
    args = (p["probes"], p["obs"])
    ctx.set_adjoint_steps(np.full(K, p["dt"]))
    a = ctx.loss_and_grad(p["Q0"], K, p["dt"], *args, ckpt_every=5)
    ctx.set_adjoint_steps(None)
    b = ctx.loss_and_grad(p["Q0"], K, p["dt"], *args, ckpt_every=5)
    for k in ("g_manning", "g_zb", "g_inletq"):
        np.testing.assert_array_equal(a[k], b[k])
    assert a["loss"] == b["loss"]
    # the adaptive solve over the same span, and its steps
    ctx.integrate_tsit5(p["Q0"], 0.0, K * p["dt"])
    steps = ctx.tsit5_steps()
    M = len(steps)
    assert M >= 3 and abs(steps.sum() - K * p["dt"]) <= 1e-9 * K * p["dt"]
    assert np.ptp(steps) > 0.0   # not all one size
    obs = np.resize(p["obs"], (M, len(p["probes"])))
    ctx.set_adjoint_steps(steps)
    try:
        r = ctx.loss_and_grad(p["Q0"], M, 1.0, p["probes"], obs, ckpt_every=4)
        gz = zone_sums(r["g_manning"], p["zones"], p["nz"])
        zones = np.array(case["manning_zones"], dtype=float)
        loss = lambda: ctx.loss_and_grad(p["Q0"], M, 1.0, p["probes"], obs, ckpt_every=4)["loss"]
        for z in range(p["nz"]):
            e = 1e-6 * zones[z]
            lz = []
            for sgn in (1.0, -1.0):
                zz = zones.copy()
                zz[z] += sgn * e
                ctx.set_manning_zones(case["mat_id"], zz)
                lz.append(loss())
            ctx.set_manning_zones(case["mat_id"], zones)
            fd = (lz[0] - lz[1]) / (2 * e)
            assert abs(gz[z] - fd) <= 1e-5 * np.abs(gz).max(), z
        q0 = np.asarray(case["inlet_q"], dtype=float)
        lq = []
        for sgn in (1.0, -1.0):
            ctx.set_inlet_q(q0 + sgn * 1e-6 * q0)
            lq.append(loss())
        ctx.set_inlet_q(q0)
        fdq = (lq[0] - lq[1]) / (2e-6 * q0[0])
        assert abs(r["g_inletq"][0] - fdq) <= 1e-5 * abs(fdq)
        with pytest.raises(HgError):   # more steps than sizes given
            ctx.loss_and_grad(p["Q0"], M + 1, 1.0, p["probes"], np.resize(obs, (M + 1, len(p["probes"]))))
        for bad in ([p["dt"], -p["dt"]], [p["dt"], np.nan], [0.0]):   # sizes must be positive and finite
            with pytest.raises(HgError):
                ctx.set_adjoint_steps(bad)
        ctx.set_adjoint_steps(steps)   # a refused call leaves the sizes set before it
        c32 = fp32c_ctx(case)
        c32.set_adjoint_steps(steps)
        r32 = c32.loss_and_grad(p["Q0"], M, 1.0, p["probes"], obs, ckpt_every=4)
        g32 = zone_sums(r32["g_manning"], p["zones"], p["nz"])
        assert np.abs(g32 - gz).max() <= 1e-3 * np.abs(gz).max()
        assert abs(r32["g_inletq"][0] - r["g_inletq"][0]) <= 1e-3 * abs(r["g_inletq"][0])
    finally:
        ctx.set_adjoint_steps(None)


# Through a state-dependent resistance: every stage's VJP takes dL/dn back
# through the n function (or the UDE network) at that stage's own state.
# Against central differences of the oracle's fixed Tsit5 loss, which
# recomputes n in its RHS alike (tolerances and steps of
# tests/test_gpu_resistance_grad.py and tests/test_gpu_ude_grad.py).
RK = 16


def _flowing(c, o):
    N = len(c["cell_node_count"])
    hs = o.hstill()
    Q0 = c["Q0"].copy()
    Q0[N:2 * N] = 0.2 * (Q0[:N] + hs)   # a 0.2 m/s flow: the friction terms matter
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    probes = np.unique((Stream(5).uniform(40) * N).astype(np.int32))[:12]
    obs = np.tile(Q0[probes] + hs[probes] + 0.05, (RK, 1))
    return N, Q0, dt, probes, obs


def test_sigmoid_n_function_gradients_match_central_differences():
    from tests import test_gpu_resistance_grad as R
    c = R.case()
    params = R.PARAMS["sigmoid"]
    o = R.oracle(c, "sigmoid", params, None)
    N, Q0, dt, probes, obs = _flowing(c, o)
    ctx, _ = R.make(c, "fp64", "sigmoid", params)
    ctx.set_adjoint_integrator("tsit5")
    r = ctx.loss_and_grad(Q0, RK, dt, probes, obs, ckpt_every=5)
    gp = ctx.resistance_grad()

    def loss(pr=params, q=None):
        return R.oracle(c, "sigmoid", pr, None, q=q).tsit5_loss(Q0, RK, dt, probes, obs)[0]

    assert abs(r["loss"] - loss()) <= 1e-10 * abs(r["loss"])
    fd = np.zeros(4)
    for k in range(4):
        e = 1e-4 * max(abs(params[k]), 1e-2)
        up, dn = list(params), list(params)
        up[k] += e
        dn[k] -= e
        fd[k] = (loss(up) - loss(dn)) / (2 * e)
    assert np.abs(gp - fd).max() <= 1e-5 * np.abs(fd).max()
    q0 = np.asarray(c["inlet_q"], dtype=float)
    e = 1e-6 * q0[0]
    fdq = (loss(q=q0 + e) - loss(q=q0 - e)) / (2 * e)
    assert abs(r["g_inletq"][0] - fdq) <= 1e-5 * abs(fdq)
    # FP32C against the FP64 device adjoint
    c32, _ = R.make(c, "fp32c", "sigmoid", params)
    c32.set_adjoint_integrator("tsit5")
    r32 = c32.loss_and_grad(Q0, RK, dt, probes, obs, ckpt_every=5)
    assert abs(r32["loss"] - r["loss"]) <= 1e-4 * abs(r["loss"])
    assert np.abs(c32.resistance_grad() - gp).max() <= 1e-3 * np.abs(gp).max()
    assert abs(r32["g_inletq"][0] - r["g_inletq"][0]) <= 1e-3 * abs(r["g_inletq"][0])


@pytest.mark.parametrize("which", [0, 1, 2, 3, 4, 5])
def test_ude_gradients_match_central_differences(which):
    from tests import test_gpu_ude_grad as U
    spec = U.CASES[which]
    c = U.case()
    hidden, _ = U.NETS[spec[1]]
    theta = U.ude_params(spec[2], hidden, seed=20 + spec[1])
    o = U.oracle(c, spec, theta)
    N, Q0, dt, probes, obs = _flowing(c, o)
    ctx = U.make(c, "fp64", spec, theta)
    ctx.set_adjoint_integrator("tsit5")
    r = ctx.loss_and_grad(Q0, RK, dt, probes, obs, ckpt_every=5)
    g = ctx.ude_grad()

    def loss(th):
        return U.oracle(c, spec, th).tsit5_loss(Q0, RK, dt, probes, obs)[0]

    assert abs(r["loss"] - loss(theta)) <= 1e-10 * abs(r["loss"])
    v = Stream(17 + which).uniform(len(theta), -1.0, 1.0)
    fd = {}
    for e in (1e-4, 2e-4):   # Richardson's extrapolation of central differences along v
        fd[e] = (loss(theta + e * v) - loss(theta - e * v)) / (2 * e)
    fdr = (4 * fd[1e-4] - fd[2e-4]) / 3
    assert abs(g @ v - fdr) <= 1e-5 * np.linalg.norm(g) * np.linalg.norm(v)
    # FP32C against the FP64 device adjoint
    c32 = U.make(c, "fp32c", spec, theta)
    c32.set_adjoint_integrator("tsit5")
    r32 = c32.loss_and_grad(Q0, RK, dt, probes, obs, ckpt_every=5)
    assert abs(r32["loss"] - r["loss"]) <= 1e-4 * abs(r["loss"])
    assert np.linalg.norm(c32.ude_grad() - g) <= 1e-3 * np.linalg.norm(g)
