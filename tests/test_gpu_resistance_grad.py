"""Gradients through a state-dependent Manning n (hg_set_manning_function).

Every RHS evaluation recomputes n = f(h, Umag, ks) from its own state
(semi_discretize_swe_2D.jl:141-149, process_ManningN_2D.jl:149-213), so the
adjoint takes each evaluation's dL/dn back into that state through
dn/d(h, qx, qy) and into the function's parameters {n_lower, n_upper, k,
h_mid} (hg_resistance_grad).  Checked against central differences of the
FP64 oracle, which recomputes n in its RHS in the same way (eps 1e-6 relative
for the inlet and bed, 1e-4 for the parameters, whose loss derivatives are
small; tolerance 1e-5 relative as tests/test_gpu_adjoint.py): the parameter
gradient, the inlet-Q gradient and a directional zb gradient, for the power
law, the sigmoid, the inverse law and Cheng's n(h, Umag, ks); FP32C against
FP64 within 1e-4 of scale (tolerance of tests/test_gpu_adjoint.py's FP32C zb
field)."""
import numpy as np
import pytest

from hydrograd_gb import SWE2D
from hydrograd_gb.workloads import Stream, river_triangles
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

KINDS = {"power_law": 1, "sigmoid": 2, "inverse": 3, "h_Umag_ks": 4}
PARAMS = {"power_law": [0.02, 0.05, 0.3, 0.0], "sigmoid": [0.02, 0.06, 3.0, 0.8],
          "inverse": [0.02, 0.05, 1.5, 0.0], "h_Umag_ks": [0.0, 0.0, 0.0, 0.0]}
K, CKPT = 16, 5


def case():
    return river_triangles(n=16, L=400.0, inlet_q=100.0, pool_center=(60.0, 200.0), pool_radius=70.0)


def make(c, prec, fn, params):
    N = len(c["cell_node_count"])
    ks = 0.05 + 0.02 * np.sin(np.arange(N)) if fn == "h_Umag_ks" else None
    ctx = SWE2D(c, precision=prec)
    ctx.set_still_water(c["wstill"])
    ctx.set_manning_zones(c["mat_id"], c["manning_zones"])
    ctx.set_inlet_q(c["inlet_q"])
    ctx.set_exit_wse(c["exit_wse"])
    ctx.set_manning_function(fn, params, ks=ks)
    return ctx, ks


def oracle(c, fn, params, ks, zb=None, q=None):
    o = Oracle(c)
    o.set_wstill(c["wstill"])
    o.set_manning_cells(c["manning_zones"][c["mat_id"]])
    o.set_inlet_q(c["inlet_q"] if q is None else q)
    o.set_exit_wse(c["exit_wse"])
    if zb is not None:
        o.set_zb_cells(zb)
    o.set_resistance_fn(KINDS[fn], params, ks=ks)
    return o


@pytest.fixture(scope="module", params=list(KINDS))
def problem(request):
    fn = request.param
    c = case()
    N = len(c["cell_node_count"])
    params = PARAMS[fn]
    o = oracle(c, fn, params, None if fn != "h_Umag_ks" else 0.05 + 0.02 * np.sin(np.arange(N)))
    hs = o.hstill()
    Q0 = c["Q0"].copy()
    Q0[N:2 * N] = 0.2 * (Q0[:N] + hs)   # a 0.2 m/s flow: Cheng's n needs Re > 0
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    probes = np.unique((Stream(5).uniform(40) * N).astype(np.int32))[:12]
    obs = np.tile(Q0[probes] + hs[probes] + 0.05, (K, 1))
    ctx, ks = make(c, "fp64", fn, params)
    r = ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=CKPT)
    return dict(fn=fn, c=c, N=N, params=params, ks=ks, dt=dt, probes=probes, obs=obs, r=r, Q0=Q0,
                gp=ctx.resistance_grad())


def loss_of(p, params=None, zb=None, q=None):
    o = oracle(p["c"], p["fn"], p["params"] if params is None else params, p["ks"], zb=zb, q=q)
    return o.rk2_loss(p["Q0"], K, p["dt"], p["probes"], p["obs"])[0]


def test_loss_matches_oracle(problem):
    assert abs(problem["r"]["loss"] - loss_of(problem)) <= 1e-10 * abs(problem["r"]["loss"])


def test_parameter_gradient_vs_central_differences(problem):
    p = problem
    if p["fn"] == "h_Umag_ks":
        np.testing.assert_array_equal(p["gp"], 0.0)   # Cheng's n has no parameters
        return
    used = 4 if p["fn"] == "sigmoid" else 3
    fd = np.zeros(4)
    for k in range(used):
        e = 1e-4 * max(abs(p["params"][k]), 1e-2)   # 1e-6 is in the loss's rounding for the small dL/dp
        up, dn = list(p["params"]), list(p["params"])
        up[k] += e
        dn[k] -= e
        fd[k] = (loss_of(p, params=up) - loss_of(p, params=dn)) / (2 * e)
    assert np.abs(p["gp"][:used] - fd[:used]).max() <= 1e-5 * np.abs(fd[:used]).max()
    assert np.abs(p["gp"]).max() > 0.0


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
    ctx, _ = make(p["c"], "fp32c", p["fn"], p["params"])
    r = ctx.loss_and_grad(p["Q0"], K, p["dt"], p["probes"], p["obs"], ckpt_every=CKPT)
    g32 = ctx.resistance_grad()
    assert abs(r["loss"] - p["r"]["loss"]) <= 1e-5 * abs(p["r"]["loss"])
    assert abs(r["g_inletq"][0] - p["r"]["g_inletq"][0]) <= 1e-4 * abs(p["r"]["g_inletq"][0])
    assert np.abs(r["g_zb"] - p["r"]["g_zb"]).max() <= 1e-4 * np.abs(p["r"]["g_zb"]).max()
    if p["fn"] != "h_Umag_ks":
        # dL/dp sums terms of both signs over every cell and stage; the sum is
        # smaller than its terms, so the FP32C adjoint's error shows larger in it
        assert np.abs(g32 - p["gp"]).max() <= 5e-4 * np.abs(p["gp"]).max()
