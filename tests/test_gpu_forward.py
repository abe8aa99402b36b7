"""CUDA forward path vs the oracle, through the C ABI.

Error measures (normwise relative):
  RHS:    max|gpu - oracle| / max(max|oracle|, S), S = the flux scale of the
          state, max_c (g h^2/2 + |q|^2/h) * perimeter_c / area_c: the size of
          the terms the RHS sums, so that a residual that cancels to ~0 (a
          near-steady state) is judged against what was summed.
  State:  per block b, max|gpu_b - oracle_b| / max(max|oracle_b|, 1e-3 max|oracle|).
Tolerances: FP64 path 1e-12 for one RHS, 1e-10 after many steps;
            FP32C path 2e-5 for one RHS, 1e-5 for states.
"""
import numpy as np
import pytest

from hydrograd_gb import SWE2D, SWE2DExtraParameters, HgError, custom_ODE_solve, swe_2d_rhs
from hydrograd_gb.workloads import dam_break, river_triangles
from oracle.oracle import Oracle
from tests.golden_cases import initial_state, load_fixture, still_water

pytestmark = pytest.mark.gpu


def block_err(a, b, N):
    """State error (see module docstring)."""
    out = []
    for k in range(3):
        ref = b[k * N:(k + 1) * N]
        scale = max(np.abs(ref).max(), np.abs(b).max() * 1e-3, 1e-300)
        out.append(np.abs(a[k * N:(k + 1) * N] - ref).max() / scale)
    return max(out)


def flux_scale(o, Q, g=9.81, h_small=1e-3):
    N = o.n_cells
    m = o.mesh_arrays()
    lengths = m["face_lengths"][m["cell_faces"].reshape(N, 8)]
    per = np.where(np.arange(8)[None, :] < o._keep["cell_node_count"][:, None], lengths, 0.0).sum(axis=1)
    h = np.maximum(Q[:N] + o.hstill(), h_small)
    q2 = Q[N:2 * N] ** 2 + Q[2 * N:] ** 2
    return np.max((0.5 * g * h * h + q2 / h) * per / m["areas"])


def rhs_err(a, b, o, Q):
    """RHS error (see module docstring)."""
    scale = max(np.abs(b).max(), flux_scale(o, Q))
    return np.abs(a - b).max() / scale


def small_river(n=32, L=500.0, dry=False):
    """A small copy of the benchmark reach (dry=True: dry bed outside the pool)."""
    return river_triangles(n=n, L=L, inlet_q=500.0 * L / 2000.0, pool_center=(0.15 * L, 0.5 * L),
                           pool_radius=0.175 * L, dry_land=dry)


def setup_pair(case, precision="fp64", order="hilbert", manning=None):
    N = len(case["cell_node_count"])
    ctx = SWE2D(case, precision=precision, order=order)
    o = Oracle(case)
    wst = case["wstill"] if "wstill" in case else still_water(case, N)
    ctx.set_still_water(wst)
    o.set_wstill(wst)
    n_cells = case["manning_zones"][case["mat_id"]] if manning is None else manning
    ctx.set_manning_zones(case["mat_id"], case["manning_zones"])
    o.set_manning_cells(n_cells)
    if len(case["inlet_q"]):
        ctx.set_inlet_q(case["inlet_q"])
        o.set_inlet_q(case["inlet_q"])
    if len(case["exit_wse"]):
        ctx.set_exit_wse(case["exit_wse"])
        o.set_exit_wse(case["exit_wse"])
    return ctx, o, N


def golden_states(name):
    d = load_fixture(name)
    N = len(d["cell_node_count"])
    Q0 = initial_state(d, N)
    h = d["h_truth"]
    Qt = np.concatenate([d["xi_truth"], d["u_truth"] * (h + 1e-3), d["v_truth"] * (h + 1e-3)])
    return d, [Q0, Qt]


@pytest.mark.parametrize("name", ["fwd_bump", "fwd_uniform", "fwd_savannah"])
@pytest.mark.parametrize("order", ["none", "rcm", "hilbert"])
def test_rhs_fp64_matches_oracle_on_reference_cases(name, order):
    d, states = golden_states(name)
    ctx, o, N = setup_pair(d, order=order)
    for Q in states:
        assert rhs_err(ctx.rhs(Q), o.rhs(Q), o, Q) <= 1e-12


def test_bed_slope_on_device_context_matches_reference_truth():
    d = load_fixture("fwd_savannah")
    ctx, _, N = setup_pair(d)
    S0t = d["S0_cells_truth"].reshape(2, -1).T
    assert np.array_equal(ctx.bed()["S0"], S0t)


@pytest.mark.parametrize("which", ["dam_break", "river_wet", "river_dry"])
def test_rhs_fp64_dam_break_and_wet_dry_fronts(which):
    case = {"dam_break": dam_break, "river_wet": small_river, "river_dry": lambda: small_river(dry=True)}[which]()
    ctx, o, N = setup_pair(case)
    Q = case["Q0"]
    assert rhs_err(ctx.rhs(Q), o.rhs(Q), o, Q) <= 1e-12
    # advance the oracle so that fronts, dry cells and inlet/exit ghosts are exercised
    # (a dry bed only briefly: the reference scheme floods dry cells unstably)
    Qm = o.rk2(Q, 1 if which == "river_dry" else 40, cfl=0.4, nthreads=4)
    assert rhs_err(ctx.rhs(Qm), o.rhs(Qm), o, Qm) <= 1e-12


def test_rk2_dam_break_1000_steps_fp64():
    """Configuration 1: 200x40 quads, dt = 0.01 s, 1,000 SSP-RK2 steps."""
    case = dam_break()
    ctx, o, N = setup_pair(case)
    Q, dts = ctx.integrate(case["Q0"], 1000, method="rk2", dt=0.01)
    Qr = o.rk2(case["Q0"], 1000, dt=0.01, nthreads=8)
    assert np.all(dts == 0.01)
    assert block_err(Q, Qr, N) <= 1e-10


def test_rk2_cfl_river_fp64_follows_oracle():
    case = small_river()
    ctx, o, N = setup_pair(case)
    Q, dts = ctx.integrate(case["Q0"], 300, method="rk2", cfl=0.4)
    assert abs(dts[0] - o.cfl_dt(case["Q0"], 0.4)) <= 1e-14 * dts[0]
    Qr = case["Q0"].copy()
    for dt in dts:
        Qr = o.rk2(Qr, 1, dt=float(dt), nthreads=4)
    assert block_err(Q, Qr, N) <= 1e-10
    # the CFL steps the device chose are the oracle's CFL steps of its own states
    Qc, dtc = o.rk2(case["Q0"], 300, cfl=0.4, nthreads=4, return_dts=True)
    assert np.abs(dtc - dts).max() <= 1e-10 * dts.max()


def test_euler_reference_loop_matches_oracle():
    """custom_ODE_solve (custom_ODE_solvers.jl:36-95) with its xi-as-h clamp."""
    case = dam_break(40, 8, 20.0, 4.0)
    ctx, o, N = setup_pair(case)
    p = SWE2DExtraParameters(ctx)
    sol = custom_ODE_solve(case["Q0"], None, p, (0.0, 0.5), 0.01)
    assert sol.shape == (3 * N, 51)
    Qr = o.euler_reference(case["Q0"], 51, 0.01)
    assert block_err(sol[:, -1], Qr, N) <= 1e-12


def test_active_parameter_injection_matches_oracle():
    """swe_2d_rhs with params_vector = zone n, zb cells, inlet Q (semi_discretize_swe_2D.jl:112-199)."""
    d = load_fixture("sens_bump")
    ctx, o, N = setup_pair(d)
    Q = initial_state(d, N)
    o2 = Oracle(d)
    o2.set_wstill(still_water(d, N)); o2.set_inlet_q(d["inlet_q"]); o2.set_exit_wse(d["exit_wse"])
    # ManningN
    pz = np.array([0.021, 0.034, 0.027])
    pe = SWE2DExtraParameters(ctx, "ManningN", mat_id=d["mat_id"])
    o2.set_manning_cells(pz[d["mat_id"]])
    assert rhs_err(swe_2d_rhs(None, Q, pz, 0.0, pe), o2.rhs(Q), o2, Q) <= 1e-12
    # zb (hstill kept)
    zb = o2.bed()[0] + 0.01 * np.sin(np.arange(N))
    pe = SWE2DExtraParameters(ctx, "zb")
    o2.set_zb_cells(zb)
    assert rhs_err(swe_2d_rhs(None, Q, zb, 0.0, pe), o2.rhs(Q), o2, Q) <= 1e-12
    # inlet Q, in-place form
    pe = SWE2DExtraParameters(ctx, "Q", bInPlaceODE=True)
    o2.set_inlet_q([0.25])
    out = np.zeros(3 * N)
    r = swe_2d_rhs(out, Q, np.array([0.25]), 0.0, pe)
    assert r is out
    assert rhs_err(out, o2.rhs(Q), o2, Q) <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_runs_are_bitwise_deterministic(precision):
    case = small_river(24, 400.0)
    ctx, _, _ = setup_pair(case, precision=precision)
    a, _ = ctx.integrate(case["Q0"], 100, cfl=0.4)
    b, _ = ctx.integrate(case["Q0"], 100, cfl=0.4)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_device_resident_graph_path_equals_integrate(precision):
    case = small_river(24, 400.0)
    ctx, _, _ = setup_pair(case, precision=precision)
    a, dts = ctx.integrate(case["Q0"], 120, cfl=0.4)
    ctx.upload(case["Q0"])
    ctx.advance(120, cfl=0.4, graph=True)
    b = ctx.download()
    assert np.array_equal(a, b)
    assert abs(ctx.elapsed_time() - dts.sum()) <= 1e-12 * dts.sum()


@pytest.mark.parametrize("order", ["none", "hilbert"])
def test_rhs_fp32c_within_tolerance(order):
    case = small_river()
    ctx, o, N = setup_pair(case, precision="fp32c", order=order)
    Qm = o.rk2(case["Q0"], 40, cfl=0.4, nthreads=4)
    dry = small_river(dry=True)
    for Q in (case["Q0"], Qm):
        assert rhs_err(ctx.rhs(Q), o.rhs(Q), o, Q) <= 2e-5
    ctx, o, N = setup_pair(dry, precision="fp32c", order=order)
    Qd = o.rk2(dry["Q0"], 1, cfl=0.4, nthreads=4)
    for Q in (dry["Q0"], Qd):
        assert rhs_err(ctx.rhs(Q), o.rhs(Q), o, Q) <= 2e-5


def test_rk2_fp32c_state_error_vs_fp64_oracle():
    case = small_river()
    ctx, o, N = setup_pair(case, precision="fp32c")
    Q, dts = ctx.integrate(case["Q0"], 300, cfl=0.4)
    Qr = case["Q0"].copy()
    for dt in dts:
        Qr = o.rk2(Qr, 1, dt=float(dt), nthreads=4)
    assert block_err(Q, Qr, N) <= 1e-5


def test_dry_inlet_is_reported():
    case = river_triangles(n=16, L=400.0, pool_center=(300.0, 300.0), pool_radius=40.0, dry_land=True)
    ctx, _, _ = setup_pair(case)
    with pytest.raises(HgError) as e:
        ctx.rhs(case["Q0"])
    assert e.value.code == 6


def test_nonfinite_state_is_reported():
    case = dam_break(20, 4, 10.0, 2.0)
    ctx, _, N = setup_pair(case)
    Q = case["Q0"].copy()
    Q[N + 3] = np.nan
    with pytest.raises(HgError) as e:
        ctx.integrate(Q, 2, dt=0.01)
    assert e.value.code == 5


def test_initial_depth_check():
    case = dam_break(20, 4, 10.0, 2.0)
    ctx, _, N = setup_pair(case)
    Q = case["Q0"].copy()
    ctx.check_initial_state(Q)
    Q[5] = 1e-4
    with pytest.raises(HgError):
        ctx.check_initial_state(Q)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("name", ["fwd_bump", "fwd_uniform", "fwd_savannah"])
def test_shipped_cases_reach_reference_final_state(name, precision):
    """The reference's example cases (read from their SRH-2D files by
    hydrograd_gb.srh2d into the fixtures) run on the device with SSP-RK2 to the
    case's end time, against the final state of the reference's own Tsit5 run
    (abstol 1e-6, reltol 1e-3), as the oracle is checked: within 2e-3 of scale."""
    d = load_fixture(name)
    N = len(d["cell_node_count"])
    ctx, o, _ = setup_pair(d, precision)
    Q0 = initial_state(d, N)
    T = float(d["tspan"][1])
    nsteps = int(np.ceil(T / (0.8 * o.cfl_dt(Q0, 0.4))))
    Q, _ = ctx.integrate(Q0, nsteps, dt=T / nsteps)
    h = d["h_truth"]
    ref = np.concatenate([d["xi_truth"], d["u_truth"] * (h + 1e-3), d["v_truth"] * (h + 1e-3)])
    scale = max(np.abs(ref[:N]).max(), np.abs(ref[N:]).max())
    assert np.abs(Q - ref).max() <= 2e-3 * scale


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_collapsing_cfl_step_is_reported(precision):
    """The dry-bed pool of the reach diverges under SSP-RK2 at CFL 0.4 (a
    property of the reference scheme, see tests/test_dry_bed.py): its third
    CFL step is about 6e-6 s, far below the reference's dt_min of 0.001 s
    (swe_2D_constants.jl:9, solve_swe_2D.jl:83).  The stepping call reports
    it as HG_ERR_STATE; with the check off (dt_min = 0) the same steps pass."""
    case = river_triangles(n=32, dry_land=True)
    ctx, _, _ = setup_pair(case, precision)
    with pytest.raises(HgError) as e:
        ctx.integrate(case["Q0"], 3, cfl=0.4)
    assert e.value.code == 5
    assert "dt_min" in str(e.value) or "non-finite" in str(e.value)
    ctx.set_dt_min(0.0)
    _, dts = ctx.integrate(case["Q0"], 2, cfl=0.4)
    assert dts.min() > 0.0
    ctx.set_dt_min(0.001)
    ctx.integrate(case["Q0"], 1, cfl=0.4)     # the first step is 0.63 s: accepted
