"""Pin the oracle against the reference's own shipped outputs.

The fixtures in tests/golden/*.npz were produced by tests/golden/make_golden.py
from Hydrograd.jl's example cases.  These tests need no GPU.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from tests.golden_cases import load_case, initial_state

FWD = ["fwd_bump", "fwd_uniform", "fwd_savannah"]


@pytest.mark.parametrize("name", FWD)
def test_bed_slope_matches_reference_truth(name):
    # S0_cells_truth = update_bed_data(...) (process_bed_2D.jl:46-66): geometry + Green-Gauss.
    d, o = load_case(name)
    zb, S0, _ = o.bed()
    S0t = d["S0_cells_truth"].reshape(2, -1).T
    assert np.array_equal(zb, d["zb_cell_truth"])
    assert np.max(np.abs(S0 - S0t)) <= 1e-15 * max(1.0, np.abs(S0t).max())


@pytest.mark.parametrize("name", FWD)
def test_manning_zones_and_friction_match_reference_truth(name):
    # friction_x/y_truth from compute_friction_terms at the truth state
    # (process_forward_simulation_results_2D.jl:45-47; semi_discretize_swe_2D.jl:544-547).
    d, o = load_case(name)
    n = d["manning_zones"][d["mat_id"]]
    assert np.array_equal(n, d["ManningN_cells_truth"])
    h = d["h_truth"]
    qx = d["u_truth"] * (h + 1e-3)
    qy = d["v_truth"] * (h + 1e-3)
    fx, fy = o.friction(h, qx, qy)
    scale = max(np.abs(d["friction_x_truth"]).max(), np.abs(d["friction_y_truth"]).max())
    assert np.abs(fx - d["friction_x_truth"]).max() <= 1e-12 * scale
    assert np.abs(fy - d["friction_y_truth"]).max() <= 1e-12 * scale


@pytest.mark.parametrize("name", FWD)
def test_still_water_depth_matches_reference_truth(name):
    d, o = load_case(name)
    assert np.array_equal(o.hstill(), d["hstill_truth"])


@pytest.mark.parametrize("name,tol", [("fwd_bump", 2e-3), ("fwd_uniform", 2e-3), ("fwd_savannah", 2e-3)])
def test_forward_run_reaches_reference_final_state(name, tol):
    """SSP-RK2 + CFL run of the oracle RHS to the case's end time vs the
    reference's Tsit5 (abstol 1e-6, reltol 1e-3) final state.  A wrong flux,
    source or ghost state gives O(1) differences here."""
    d, o = load_case(name)
    N = o.n_cells
    Q = initial_state(d, N)
    T = float(d["tspan"][1])
    t = 0.0
    while t < T - 1e-12:
        dt = min(o.cfl_dt(Q, 0.4), T - t)
        Q = o.rk2(Q, 1, dt=dt, nthreads=4)
        t += dt
    h = d["h_truth"]
    ref = np.concatenate([d["xi_truth"], d["u_truth"] * (h + 1e-3), d["v_truth"] * (h + 1e-3)])
    for b in range(3):
        scale = max(np.abs(ref[: N]).max(), np.abs(ref[N:]).max())
        assert np.abs(Q[b * N:(b + 1) * N] - ref[b * N:(b + 1) * N]).max() <= tol * scale


@pytest.mark.slow
def test_dual_number_jacobian_matches_reference_forwarddiff_sensitivity():
    """ForwardDiff.jacobian of the final state w.r.t. the zone Manning n
    (swe_2D_sensitivity.jl:80), shipped as sensitivity_results.json, vs the
    oracle's own dual-number tangent through 200 s of SSP-RK2."""
    d, o = load_case("sens_bump")
    N = o.n_cells
    Q0 = initial_state(d, N)
    T = float(d["tspan"][1])
    dt = o.cfl_dt(Q0, 0.4)
    nst = int(np.ceil(T / dt))
    dt = T / nst
    nz = d["manning_zones"]
    dman = np.stack([(d["mat_id"] == k).astype(float) for k in range(len(nz))])
    _, dQ, _, _ = o.rk2_tangent(Q0, nst, dt, d_manning=dman, nthreads=4)
    S = d["sensitivity"].reshape(len(nz), 3 * N)
    scale = np.abs(S).max()
    assert np.abs(dQ - S).max() <= 1e-4 * scale
