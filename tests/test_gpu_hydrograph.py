"""Inlet-Q hydrographs (hg_set_inlet_hydrograph) on a small copy of the
configuration-5 mesh (quad core, triangle band, meandering channel, per-cell n),
against the oracle evaluating the same hydrograph at the same stage times
(hgo::hydro_at).  Tolerances as in test_gpu_forward / test_gpu_adjoint: FP64
RHS 1e-12 of the flux scale, states 1e-10, adjoint vs dual numbers 1e-8,
vs central differences 1e-5; FP32C states 1e-5."""
import numpy as np
import pytest

from hydrograd_gb import SWE2D
from hydrograd_gb.workloads import cell_centroids, meander_mixed
from oracle.oracle import Oracle
from tests.test_gpu_forward import block_err, rhs_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    c = meander_mixed(n_core=40, n_band=8)
    # a hydrograph with a kink inside the runs below, scaled to this small reach
    c["hydrograph"] = (np.array([0.0, 20.0, 60.0]), np.array([50.0, 400.0, 150.0]))
    return c


def pair(case, precision="fp64", hydro=True):
    ctx = SWE2D(case, precision=precision)
    o = Oracle(case)
    ctx.set_still_water(case["wstill"])
    o.set_wstill(case["wstill"])
    ctx.set_manning_cells(case["manning_cells"])
    o.set_manning_cells(case["manning_cells"])
    for obj in (ctx, o):
        obj.set_inlet_q(case["inlet_q"])
        obj.set_exit_wse(case["exit_wse"])
    if hydro:
        t, q = case["hydrograph"]
        ctx.set_inlet_hydrograph(0, t, q)
        o.set_hydrograph(0, t, q)
    return ctx, o, len(case["cell_node_count"])


def q_at(case, t):
    T, Q = case["hydrograph"]
    return float(np.interp(t, T, Q))


def test_rhs_at_time(case):
    ctx, o, N = pair(case)
    Q0 = case["Q0"].copy()
    Q0[N:2 * N] = 0.05   # some flow everywhere
    for t in (0.0, 7.5, 33.0, 100.0):
        o.set_inlet_q([q_at(case, t)])
        assert rhs_err(ctx.rhs(Q0, t), o.rhs(Q0), o, Q0) <= 1e-12, t


@pytest.mark.parametrize("cfl", [False, True])
def test_rk2_with_hydrograph_matches_oracle(case, cfl):
    ctx, o, N = pair(case)
    Q0 = case["Q0"]
    if cfl:
        Qg, dts = ctx.integrate(Q0, 300, cfl=0.4)
        Qo, dto = o.rk2(Q0, 300, cfl=0.4, return_dts=True)
        assert np.abs(dts - dto).max() <= 1e-12 * dto.max()
    else:
        dt = 0.5 * o.cfl_dt(Q0, 0.4)
        Qg, _ = ctx.integrate(Q0, 300, dt=dt)
        Qo = o.rk2(Q0, 300, dt=dt)
    assert block_err(Qg, Qo, N) <= 1e-10
    ctx.set_inlet_hydrograph(0, [], [])   # back to the constant discharge
    Qc, _ = ctx.integrate(Q0, 50, dt=0.01)
    o2 = pair(case, hydro=False)[1]
    assert block_err(Qc, o2.rk2(Q0, 50, dt=0.01), N) <= 1e-10


def test_fp32c_fused_and_graph_steps(case):
    """FP32C with a hydrograph: the fused two-launch steps (one hydrograph
    launch before each), in a graph or not, against the FP64 path."""
    c64, _, N = pair(case, "fp64")
    c32, _, _ = pair(case, "fp32c")
    Q0 = case["Q0"]
    a, _ = c64.integrate(Q0, 400, cfl=0.4)
    b, _ = c32.integrate(Q0, 400, cfl=0.4)
    assert block_err(b, a, N) <= 1e-5
    c32.upload(Q0)
    c32.advance(400, cfl=0.4, graph=True)
    g = c32.download()
    assert block_err(g, b, N) <= 1e-6
    assert abs(c32.elapsed_time() - c64.elapsed_time()) <= 1e-6 * c64.elapsed_time()


def test_tsit5_with_hydrograph(case):
    ctx, o, N = pair(case)
    Q0 = case["Q0"]
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    T = 200 * dt
    Qg, sg = ctx.integrate_tsit5(Q0, 0.0, T, dt0=dt, adaptive=False)
    Qo, so = o.tsit5(Q0, 0.0, T, dt0=dt, adaptive=False, nthreads=4)
    assert sg == so
    assert block_err(Qg, Qo, N) <= 1e-10


def test_adjoint_with_hydrograph(case):
    """Gradient w.r.t. the per-cell n (directional) against the oracle's dual
    numbers; the inlet-Q gradient is the derivative w.r.t. a constant shift of
    the hydrograph, against central differences of the oracle's loss."""
    ctx, o, N = pair(case)
    Q0 = case["Q0"]
    K = 120
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    rng = np.random.default_rng(4)
    cx, _ = cell_centroids(case)
    probes = np.sort(np.argsort(cx)[:24]).astype(np.int32)   # next to the inlet, where the hydrograph acts
    hst = o.hstill()
    obs = np.tile(Q0[probes] + hst[probes], (K, 1)) + 0.01
    r = ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=30)
    v = rng.uniform(-1.0, 1.0, N)
    _, _, loss_o, dl = o.rk2_tangent(Q0, K, dt, d_manning=v[None, :], probes=probes, obs=obs, nthreads=4)
    assert abs(r["loss"] - loss_o) <= 1e-10 * loss_o
    assert abs(r["g_manning"] @ v - dl[0]) <= 1e-8 * abs(dl[0])
    t, q = case["hydrograph"]
    eps = 1e-6 * q.max()
    vals = []
    for s in (1, -1):
        o.set_hydrograph(0, t, q + s * eps)
        vals.append(o.rk2_loss(Q0, K, dt, probes, obs, nthreads=4)[0])
    o.set_hydrograph(0, t, q)
    fd = (vals[0] - vals[1]) / (2 * eps)
    assert abs(r["g_inletq"][0] - fd) <= 1e-5 * abs(fd)
