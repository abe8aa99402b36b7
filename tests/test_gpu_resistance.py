"""State-dependent flow resistance on the device vs the oracle, through the C ABI.

Tolerances as in test_gpu_forward: FP64 RHS 1e-12 of the flux scale, states
1e-10; FP32C RHS 2e-5 of the flux scale, states 1e-5.  The reference's own
final states of its variable-n example cases: 2e-3 of scale, as the oracle is
pinned (test_resistance.py).
"""
import numpy as np
import pytest

from hydrograd_gb import HgError
from hydrograd_gb._lib import ACTIVATIONS
from tests.golden_cases import initial_state, load_fixture
from tests.resistance_cases import UDE_CASES, truth_state, ude_params
from tests.test_gpu_forward import block_err, rhs_err, setup_pair

pytestmark = pytest.mark.gpu

RHS_TOL = {"fp64": 1e-12, "fp32c": 2e-5}
STATE_TOL = {"fp64": 1e-10, "fp32c": 1e-5}
# the four n functions: the shipped cases' sigmoid and h_Umag_ks, plus power
# law and inverse with parameters of the same range
FN_CASES = [("fwd_bump_nh", "sigmoid", None), ("fwd_savannah_nks", "h_Umag_ks", None),
            ("fwd_bump_nh", "power_law", (0.03, 0.06, 0.5)), ("fwd_savannah_nks", "inverse", (0.02, 0.07, 2.0))]
KIND = {"power_law": 1, "sigmoid": 2, "inverse": 3, "h_Umag_ks": 4}


def states(d, N):
    return [initial_state(d, N), truth_state(d)]


def set_fn(ctx, o, d, fn, params):
    p = d["res_params"] if params is None else np.array(params + (0.0,) * (4 - len(params)))
    ks = d.get("ks_cells") if fn == "h_Umag_ks" else None
    ctx.set_manning_function(fn, p, ks)
    o.set_resistance_fn(KIND[fn], p, ks)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("name,fn,params", FN_CASES, ids=[f"{c[0]}-{c[1]}" for c in FN_CASES])
def test_manning_function_rhs_matches_oracle(name, fn, params, precision):
    d = load_fixture(name)
    ctx, o, N = setup_pair(d, precision)
    set_fn(ctx, o, d, fn, params)
    for Q in states(d, N):
        assert rhs_err(ctx.rhs(Q), o.rhs(Q), o, Q) <= RHS_TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("name", ["fwd_bump_nh", "fwd_savannah_nks"])
def test_variable_n_cases_reach_reference_final_state(name, precision):
    """Device Tsit5 with n recomputed in every RHS: fixed steps against the
    oracle's fixed steps, adaptive steps (the case's dt as the first step, as
    the reference's solve call takes it) against the reference's final state."""
    d = load_fixture(name)
    ctx, o, N = setup_pair(d, precision)
    fn = {2: "sigmoid", 4: "h_Umag_ks"}[int(d["res_kind"])]
    set_fn(ctx, o, d, fn, None)
    Q0 = initial_state(d, N)
    T = float(d["tspan"][1])
    Qg, _ = ctx.integrate_tsit5(Q0, 0.0, T, dt0=float(d["dt"]))
    ref = truth_state(d)
    scale = max(np.abs(ref[:N]).max(), np.abs(ref[N:]).max())
    assert np.abs(Qg - ref).max() <= 2e-3 * scale
    T1 = T / 20
    n = int(np.ceil(T1 / (0.9 * o.cfl_dt(Q0, 0.4))))
    Qf, _ = ctx.integrate_tsit5(Q0, 0.0, T1, dt0=T1 / n, adaptive=False)
    Qo, _ = o.tsit5(Q0, 0.0, T1, dt0=T1 / n, adaptive=False, nthreads=4)
    assert block_err(Qf, Qo, N) <= STATE_TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("over_batch", [True, False], ids=["ln_batch", "ln_cell"])
@pytest.mark.parametrize("choice,kind,in_dim,bounds", UDE_CASES, ids=[c[0] for c in UDE_CASES])
def test_ude_rhs_and_steps_match_oracle(choice, kind, in_dim, bounds, over_batch, precision):
    d = load_fixture("fwd_savannah_nks")
    ctx, o, N = setup_pair(d, precision)
    hidden, acts = [3, 3], ["tanh", "tanh"]
    p = ude_params(in_dim, hidden, seed=10 + kind)
    ks = d["ks_cells"] if kind == 6 else None
    ctx.set_ude(choice, hidden, acts, p, ks=ks, layernorm_over_batch=over_batch, **bounds)
    o.set_ude(kind, in_dim, hidden, [3, 3], p, bounds["output_bounds"], bounds["h_bounds"],
              bounds.get("u_bounds", (0.0, 1.0)), bounds.get("ks_bounds", (0.0, 1.0)), ks, over_batch)
    for Q in states(d, N):
        assert rhs_err(ctx.rhs(Q), o.rhs(Q), o, Q) <= RHS_TOL[precision]
    Q0 = initial_state(d, N)
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    Qg, _ = ctx.integrate(Q0, 50, dt=dt)
    Qo = o.rk2(Q0, 50, dt=dt, nthreads=4)
    assert block_err(Qg, Qo, N) <= STATE_TOL[precision]


WIDTHS = [([8, 8], ["tanh", "tanh"]), ([16, 5], ["sigmoid", "softplus"]), ([2], ["relu"]),
          ([4, 9, 3], ["leakyrelu", "tanh", "sigmoid"])]


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("over_batch", [True, False], ids=["ln_batch", "ln_cell"])
@pytest.mark.parametrize("hidden,acts", WIDTHS, ids=["8-8", "16-5", "2", "4-9-3"])
def test_ude_widths_match_oracle(hidden, acts, over_batch, precision):
    """Networks of every register width the forward kernels take (4, 8, 16
    values a layer) and depths 1 to 3."""
    d = load_fixture("fwd_savannah_nks")
    ctx, o, N = setup_pair(d, precision)
    bounds = dict(output_bounds=(0.03, 0.06), h_bounds=(0.1, 0.5))
    p = ude_params(1, hidden, seed=40 + sum(hidden))
    ctx.set_ude("ManningN_h", hidden, acts, p, layernorm_over_batch=over_batch, **bounds)
    o.set_ude(5, 1, hidden, [ACTIVATIONS[a] for a in acts], p, bounds["output_bounds"], bounds["h_bounds"],
              (0.0, 1.0), (0.0, 1.0), None, over_batch)
    for Q in states(d, N):
        assert rhs_err(ctx.rhs(Q), o.rhs(Q), o, Q) <= RHS_TOL[precision]
    Q0 = initial_state(d, N)
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    Qg, _ = ctx.integrate(Q0, 20, dt=dt)
    Qo = o.rk2(Q0, 20, dt=dt, nthreads=4)
    assert block_err(Qg, Qo, N) <= STATE_TOL[precision]


@pytest.mark.parametrize("solver", ["Roe", "HLL"])
@pytest.mark.parametrize("name,fn,params", FN_CASES, ids=[f"{c[0]}-{c[1]}" for c in FN_CASES])
def test_fused_fp32c_steps_with_n_functions(name, fn, params, solver):
    """The fused FP32C steps evaluate the n function in the stage kernel
    (both Riemann solvers): CFL steps against the oracle's steps of the same
    sizes, and the resident steps (hg_advance) the same as hg_integrate's."""
    d = load_fixture(name)
    ctx, o, N = setup_pair(d, "fp32c")
    set_fn(ctx, o, d, fn, params)
    ctx.set_riemann_solver(solver)
    o.set_riemann_solver(solver)
    Q0 = initial_state(d, N)
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    Qg, _ = ctx.integrate(Q0, 60, dt=dt)
    Qo = o.rk2(Q0, 60, dt=dt, nthreads=4)
    assert block_err(Qg, Qo, N) <= STATE_TOL["fp32c"]
    ctx.upload(Q0)
    ctx.advance(60, dt=dt, graph=True)
    assert block_err(ctx.download(), Qg, N) <= 1e-6


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_graph_steps_and_constant_restore(precision):
    """Resident steps (hg_advance, captured in a graph) see the state-dependent
    n like hg_integrate does; switching back to "constant" restores the zones'
    n; gradients run through the function (their values are checked in
    tests/test_gpu_resistance_grad.py)."""
    d = load_fixture("fwd_bump_nh")
    ctx, o, N = setup_pair(d, precision)
    Q0 = initial_state(d, N)
    rhs_const = ctx.rhs(Q0)
    set_fn(ctx, o, d, "sigmoid", None)
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    Qi, _ = ctx.integrate(Q0, 120, dt=dt)
    ctx.upload(Q0)
    ctx.advance(120, dt=dt, graph=True)
    Qa = ctx.download()
    assert block_err(Qa, Qi, N) <= (0.0 if precision == "fp64" else 1e-6)
    r = ctx.loss_and_grad(Q0, 5, dt, [0, 1], np.full((5, 2), 0.1))   # one observation per step and probe
    assert np.isfinite(r["loss"]) and np.isfinite(ctx.resistance_grad()).all()
    ctx.set_manning_function("constant")
    np.testing.assert_array_equal(ctx.rhs(Q0), rhs_const)


def test_resistance_argument_errors():
    d = load_fixture("fwd_bump_nh")
    ctx, _, N = setup_pair(d, "fp64")
    with pytest.raises(HgError, match="k must be"):
        ctx.set_manning_function("sigmoid", (0.03, 0.06, -1.0, 0.3))
    with pytest.raises(HgError, match="h_mid"):
        ctx.set_manning_function("sigmoid", (0.03, 0.06, 100.0, 0.0))
    with pytest.raises(HgError, match="ks"):
        ctx.set_manning_function("h_Umag_ks")
    with pytest.raises(HgError, match="network parameters"):
        ctx.set_ude("ManningN_h", [3, 3], ["tanh", "tanh"], np.zeros(5), (0.03, 0.06), (0.1, 0.5))
    with pytest.raises(HgError, match="widths"):
        ctx.set_ude("ManningN_h", [17], ["tanh"], np.zeros(17 * 4 + 18), (0.03, 0.06), (0.1, 0.5))
