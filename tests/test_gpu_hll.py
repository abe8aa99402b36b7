"""The HLL Riemann solver (hg_set_riemann_solver) on the device vs the
oracle's hll_flux, through the C ABI, with the forward tests' error measures
and tolerances: FP64 RHS 1e-12, FP64 states after many steps 1e-10, FP32C
RHS 2e-5 and states 1e-5; the adjoint against the oracle's dual numbers
(FP64, 1e-8) and the FP32C adjoint against those (1e-5).  HLLC is refused as
the reference refuses it; switching solvers re-captures the step graphs."""
import numpy as np
import pytest

from hydrograd_gb import SWE2D, HgError
from hydrograd_gb.workloads import Stream, dam_break
from tests.test_gpu_forward import block_err, rhs_err, setup_pair, small_river

pytestmark = pytest.mark.gpu


def hll_pair(case, precision="fp64"):
    ctx, o, N = setup_pair(case, precision=precision)
    ctx.set_riemann_solver("HLL")
    o.set_riemann_solver("HLL")
    return ctx, o, N


@pytest.mark.parametrize("which", ["dam_break", "river_wet", "river_dry"])
def test_rhs_fp64_hll_matches_oracle(which):
    case = {"dam_break": lambda: dam_break(40, 8, 20.0, 4.0, x_gate=10.0), "river_wet": small_river,
            "river_dry": lambda: small_river(dry=True)}[which]()
    ctx, o, N = hll_pair(case)
    Q = case["Q0"]
    assert rhs_err(ctx.rhs(Q), o.rhs(Q), o, Q) <= 1e-12
    Qm = o.rk2(Q, 1 if which == "river_dry" else 40, cfl=0.4, nthreads=4)
    assert rhs_err(ctx.rhs(Qm), o.rhs(Qm), o, Qm) <= 1e-12


def test_rk2_fp64_hll_follows_oracle():
    case = small_river()
    ctx, o, N = hll_pair(case)
    Q, dts = ctx.integrate(case["Q0"], 300, cfl=0.4)
    Qr = case["Q0"].copy()
    for dt in dts:
        Qr = o.rk2(Qr, 1, dt=float(dt), nthreads=4)
    assert block_err(Q, Qr, N) <= 1e-10


def test_rhs_and_rk2_fp32c_hll_within_tolerance():
    case = small_river()
    ctx, o, N = hll_pair(case, precision="fp32c")
    Qm = o.rk2(case["Q0"], 40, cfl=0.4, nthreads=4)
    for Q in (case["Q0"], Qm):
        assert rhs_err(ctx.rhs(Q), o.rhs(Q), o, Q) <= 2e-5
    Q, dts = ctx.integrate(case["Q0"], 300, cfl=0.4)
    Qr = case["Q0"].copy()
    for dt in dts:
        Qr = o.rk2(Qr, 1, dt=float(dt), nthreads=4)
    assert block_err(Q, Qr, N) <= 1e-5


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_hll_lake_at_rest_stays_at_rest(precision):
    """A walled basin over an uneven bed, water at rest: 200 RK2 steps keep
    q at zero to rounding (FP32C: the own-pressure shift and the exact
    pressure jump keep the balance)."""
    case = dam_break(30, 10, 30.0, 10.0)
    x, y = case["node_xyz"][:, 0], case["node_xyz"][:, 1]
    case["node_xyz"][:, 2] = 0.3 * np.sin(0.4 * x) * np.cos(0.5 * y)
    N = len(case["cell_node_count"])
    ctx = SWE2D(case, precision=precision)
    ctx.set_still_water(np.full(N, 1.0))
    ctx.set_manning_zones(case["mat_id"], case["manning_zones"])
    ctx.set_riemann_solver("HLL")
    Q, _ = ctx.integrate(np.zeros(3 * N), 200, dt=0.02)
    assert np.abs(Q[N:]).max() <= (1e-12 if precision == "fp64" else 1e-7)
    assert np.abs(Q[:N]).max() <= (1e-12 if precision == "fp64" else 1e-7)


def test_solver_switch_recaptures_the_step_graph():
    """Steps replayed from a graph captured under Roe, then HLL: the HLL run
    equals the run without graphs, and differs from Roe's."""
    case = small_river()
    ctx, o, N = setup_pair(case, precision="fp32c")
    ctx.upload(case["Q0"])
    ctx.advance(60, cfl=0.4, graph=True)
    roe = ctx.download()
    ctx.set_riemann_solver("HLL")
    ctx.upload(case["Q0"])
    ctx.advance(60, cfl=0.4, graph=True)
    hll_graph = ctx.download()
    ctx.upload(case["Q0"])
    ctx.advance(60, cfl=0.4, graph=False)
    hll_plain = ctx.download()
    assert np.array_equal(hll_graph, hll_plain)
    assert not np.array_equal(hll_graph, roe)


def test_hllc_is_refused():
    case = small_river(n=8)
    ctx, _, _ = setup_pair(case)
    with pytest.raises(HgError) as e:
        ctx.set_riemann_solver("HLLC")
    assert e.value.code == 7


def test_hll_adjoint_matches_dual_numbers():
    """Gradients of the probe loss through 30 HLL steps w.r.t. the zone n and
    the inlet Q: the FP64 adjoint against the oracle's dual numbers (1e-8),
    the FP32C adjoint against the same (1e-5)."""
    case = small_river(n=24, L=400.0)
    ctx, o, N = hll_pair(case)
    c32, _, _ = hll_pair(case, precision="fp32c")
    K = 30
    Q0 = case["Q0"]
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    probes = np.unique((Stream(5).uniform(64) * N).astype(np.int32))[:16]
    obs = np.zeros((K, len(probes)))
    nz = len(case["manning_zones"])
    dman = np.stack([(case["mat_id"] == z).astype(float) for z in range(nz)])
    _, _, loss_o, dl_n = o.rk2_tangent(Q0, K, dt, d_manning=dman, probes=probes, obs=obs)
    _, _, _, dl_q = o.rk2_tangent(Q0, K, dt, d_inlet=np.ones((1, 1)), probes=probes, obs=obs)
    for c, tol in ((ctx, 1e-8), (c32, 1e-5)):
        r = c.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=10)
        g = np.array([r["g_manning"][case["mat_id"] == z].sum() for z in range(nz)])
        assert abs(r["loss"] - loss_o) <= max(tol, 1e-10) * abs(loss_o)
        assert np.abs(g - dl_n).max() <= tol * np.abs(dl_n).max()
        assert abs(r["g_inletq"][0] - dl_q[0]) <= tol * abs(dl_q[0])
