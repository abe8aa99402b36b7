"""Gradients through the UDE closures (hg_set_ude, hg_ude_grad).

The reference trains its networks by differentiating the solve
(swe_2D_UDE.jl:119 UDE_training, :522 compute_loss_UDE; the network in the
RHS at semi_discretize_swe_2D.jl:165-178,517-533).  The adjoint takes each
RHS evaluation's dL/dn (dL/dF of the flow-resistance closure) back through
the network by reverse mode: into the cells' states -- so the zb and inlet-Q
gradients include it -- and into the network's parameters, through Lux's
batch LayerNorm statistics too.  Checked against central differences of the
FP64 oracle, which evaluates the same network in its RHS: the parameter
gradient along random directions and on single parameters (Richardson's
extrapolation of central differences at eps 1e-4 and 2e-4; tolerance 1e-5 of
the gradient's norm), the inlet-Q gradient and a directional zb gradient (eps 1e-6, tolerance
1e-5 relative as tests/test_gpu_adjoint.py); the FP32C gradients against the
FP64 ones (tolerances of tests/test_gpu_resistance_grad.py)."""
import numpy as np
import pytest

from hydrograd_gb import SWE2D
from hydrograd_gb.workloads import Stream, river_triangles
from oracle.oracle import Oracle
from tests.resistance_cases import UDE_CASES, ude_params

pytestmark = pytest.mark.gpu

K, CKPT = 16, 5
NETS = {5: ([3, 3], ["tanh", "sigmoid"]), 6: ([4, 3], ["softplus", "tanh"]), 7: ([3, 2], ["tanh", "softplus"])}
ACT = {"relu": 0, "leakyrelu": 1, "sigmoid": 2, "tanh": 3, "softplus": 4}
CASES = [(c, kd, din, b, ob) for (c, kd, din, b) in UDE_CASES for ob in (True, False)]
IDS = ["%s-%s" % (c[0], "ln_batch" if c[4] else "ln_cell") for c in CASES]


def case():
    return river_triangles(n=16, L=400.0, inlet_q=100.0, pool_center=(60.0, 200.0), pool_radius=70.0)


def ks_of(N):
    return 0.05 + 0.02 * np.sin(np.arange(N))


def make(c, prec, spec, theta):
    choice, kind, din, bounds, ob = spec
    hidden, acts = NETS[kind]
    N = len(c["cell_node_count"])
    ctx = SWE2D(c, precision=prec)
    ctx.set_still_water(c["wstill"])
    ctx.set_manning_zones(c["mat_id"], c["manning_zones"])
    ctx.set_inlet_q(c["inlet_q"])
    ctx.set_exit_wse(c["exit_wse"])
    ctx.set_ude(choice, hidden, acts, theta, ks=ks_of(N) if kind == 6 else None, layernorm_over_batch=ob, **bounds)
    return ctx


def oracle(c, spec, theta, zb=None, q=None):
    choice, kind, din, bounds, ob = spec
    hidden, acts = NETS[kind]
    N = len(c["cell_node_count"])
    o = Oracle(c)
    o.set_wstill(c["wstill"])
    o.set_manning_cells(c["manning_zones"][c["mat_id"]])
    o.set_inlet_q(c["inlet_q"] if q is None else q)
    o.set_exit_wse(c["exit_wse"])
    if zb is not None:
        o.set_zb_cells(zb)
    o.set_ude(kind, din, hidden, [ACT[a] for a in acts], theta, bounds["output_bounds"], bounds["h_bounds"],
              bounds.get("u_bounds", (0.0, 1.0)), bounds.get("ks_bounds", (0.0, 1.0)),
              ks_of(N) if kind == 6 else None, ob)
    return o


@pytest.fixture(scope="module", params=CASES, ids=IDS)
def problem(request):
    spec = request.param
    c = case()
    N = len(c["cell_node_count"])
    hidden, _ = NETS[spec[1]]
    theta = ude_params(spec[2], hidden, seed=20 + spec[1])
    o = oracle(c, spec, theta)
    hs = o.hstill()
    Q0 = c["Q0"].copy()
    Q0[N:2 * N] = 0.2 * (Q0[:N] + hs)   # a 0.2 m/s flow: the friction and |q| terms matter
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    probes = np.unique((Stream(5).uniform(40) * N).astype(np.int32))[:12]
    obs = np.tile(Q0[probes] + hs[probes] + 0.05, (K, 1))
    ctx = make(c, "fp64", spec, theta)
    r = ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=CKPT)
    return dict(spec=spec, c=c, N=N, theta=theta, Q0=Q0, dt=dt, probes=probes, obs=obs, r=r, g=ctx.ude_grad())


def loss_of(p, theta=None, zb=None, q=None):
    o = oracle(p["c"], p["spec"], p["theta"] if theta is None else theta, zb=zb, q=q)
    return o.rk2_loss(p["Q0"], K, p["dt"], p["probes"], p["obs"])[0]


def test_loss_matches_oracle(problem):
    assert abs(problem["r"]["loss"] - loss_of(problem)) <= 1e-10 * abs(problem["r"]["loss"])


def test_parameter_gradient_vs_central_differences(problem):
    p = problem
    g, th = p["g"], p["theta"]
    assert g.shape == th.shape and np.isfinite(g).all() and np.abs(g).max() > 0.0
    scale = np.linalg.norm(g)
    e = 1e-4
    rng = np.random.default_rng(3)
    dirs = [rng.standard_normal(len(th)) for _ in range(2)]
    dirs = [v / np.linalg.norm(v) for v in dirs]
    for i in rng.choice(len(th), 4, replace=False):   # single parameters too
        v = np.zeros(len(th))
        v[i] = 1.0
        dirs.append(v)
    def central(v, h):
        return (loss_of(p, theta=th + h * v) - loss_of(p, theta=th - h * v)) / (2 * h)

    for v in dirs:
        # Richardson's extrapolation of two central differences: the per-cell
        # LayerNorm of 3 values is strongly curved, so eps^2 terms show at 1e-4
        fd = (4.0 * central(v, e) - central(v, 2 * e)) / 3.0
        assert abs(g @ v - fd) <= 1e-5 * scale, (g @ v, fd, scale)


def test_inlet_and_bed_gradients_vs_central_differences(problem):
    p = problem
    q0 = np.asarray(p["c"]["inlet_q"], dtype=float)
    e = 1e-6 * q0[0]
    fdq = (loss_of(p, q=q0 + e) - loss_of(p, q=q0 - e)) / (2 * e)
    assert abs(p["r"]["g_inletq"][0] - fdq) <= 1e-5 * abs(fdq)
    zb = p["c"]["zb_cells"]
    v = np.sin(np.arange(p["N"]) * 0.7)
    e = 1e-6
    fdz = (loss_of(p, zb=zb + e * v) - loss_of(p, zb=zb - e * v)) / (2 * e)
    g = float(p["r"]["g_zb"] @ v)
    assert abs(g - fdz) <= 1e-5 * max(abs(fdz), np.abs(p["r"]["g_zb"]).max())


def test_fp32c_gradients_match_fp64(problem):
    p = problem
    ctx = make(p["c"], "fp32c", p["spec"], p["theta"])
    r = ctx.loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=CKPT)
    g32 = ctx.ude_grad()
    assert abs(r["loss"] - p["r"]["loss"]) <= 1e-5 * abs(p["r"]["loss"])
    assert abs(r["g_inletq"][0] - p["r"]["g_inletq"][0]) <= 1e-4 * abs(p["r"]["g_inletq"][0])
    assert np.abs(r["g_zb"] - p["r"]["g_zb"]).max() <= 1e-4 * np.abs(p["r"]["g_zb"]).max()
    assert np.abs(g32 - p["g"]).max() <= 5e-4 * np.abs(p["g"]).max()


def test_gradients_reproduce_and_count_is_checked(problem):
    p = problem
    ctx = make(p["c"], "fp64", p["spec"], p["theta"])
    r = ctx.loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=CKPT)
    np.testing.assert_array_equal(ctx.ude_grad(), p["g"])   # fixed-order sums: the same bits
    np.testing.assert_array_equal(r["g_zb"], p["r"]["g_zb"])
    from hydrograd_gb import HgError
    from hydrograd_gb._lib import lib
    from hydrograd_gb.swe2d import _d
    buf = np.zeros(len(p["theta"]) + 1)
    with pytest.raises(HgError):
        ctx._chk(lib().hg_ude_grad(ctx.h, _d(buf), len(buf)))
