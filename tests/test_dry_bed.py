"""The reference scheme on a dry bed, measured with the oracle (no GPU).

Configuration 2 is written as "initially dry except a 1.5 m pool, which gives
moving wet/dry fronts".  These tests pin what the reference's scheme does
with that start on a small copy of the reach (river_triangles(32,
dry_land=True): 2,048 triangles, 62.5 m cells, a 350 m pool touching the
inlet-Q edge, every other cell at h = h_small):

* SSP-RK2 with the CFL step diverges within three steps, at CFL 0.4 and at
  CFL 0.1: at a dry bank the Roe solver's wall branch keeps the dry side's
  xi (swe_2D_solvers.jl:23-53), a flooded cell receives the full one-sided
  pressure as momentum while nearly empty, and its Manning friction
  (h + h_small)^(-7/3) (semi_discretize_swe_2D.jl:544-547) makes the next
  step unstable; the CFL step collapses far below dt_min (0.001 s).
* The reference's own integrator, Tsit5 with abstol 1e-6 / reltol 1e-3
  (swe_2D_forward_simulation.jl:37-39), has no state clamp (the RHS clamps
  only its own copy of h, semi_discretize_swe_2D.jl:101-106): cells drain
  below their bed within 0.5 s and the run diverges by 30 s.
* The reference's Euler loop clamps xi as if it were h
  (custom_ODE_solvers.jl:19-26): with a still-water level above the dry
  bed its first step floods every dry cell below that level.
* A fixed step equal to the initial state's CFL step at CFL 0.003 (0.0047 s)
  stays bounded for 400 steps while the fronts move (at CFL 0.01, 0.016 s,
  it diverges after 18); that regime is the one the GPU front tests
  (tests/test_gpu_fronts.py) and the bench's dry-start leg use.
"""
import os

import numpy as np
import pytest

from hydrograd_gb.workloads import river_triangles
from oracle.oracle import Oracle

THREADS = min(8, os.cpu_count() or 1)
DT_MIN = 0.001   # swe_2D_consts.dt_min (solve_swe_2D.jl:83,98)


@pytest.fixture(scope="module")
def dry():
    case = river_triangles(n=32, dry_land=True)
    o = Oracle(case)
    o.set_wstill(case["wstill"])
    o.set_manning_cells(case["manning_zones"][case["mat_id"]])
    o.set_inlet_q(case["inlet_q"])
    o.set_exit_wse(case["exit_wse"])
    N = len(case["cell_node_count"])
    hst = case["wstill"] - case["zb_cells"]
    return case, o, N, hst


@pytest.mark.parametrize("cfl", [0.4, 0.1])
def test_ssp_rk2_cfl_diverges_within_three_steps(dry, cfl):
    case, o, N, _ = dry
    Q = case["Q0"].copy()
    dts = []
    for _ in range(3):
        Q, d = o.rk2(Q, 1, cfl=cfl, return_dts=True)
        dts.append(d[0])
    assert np.abs(Q[N:]).max() > 1e4
    assert dts[0] > 0.1 and min(dts) < DT_MIN   # a 0.16-0.63 s step, then a collapse


def test_small_fixed_step_stays_bounded_and_the_fronts_move(dry):
    case, o, N, hst = dry
    dt = o.cfl_dt(case["Q0"], 0.003)
    wet0 = case["Q0"][:N] + hst > 2e-3
    Q = o.rk2(case["Q0"], 400, dt=dt, nthreads=THREADS)
    wet = Q[:N] + hst > 2e-3
    assert np.isfinite(Q).all() and np.abs(Q[N:]).max() < 10.0
    assert (wet & ~wet0).sum() >= 10          # cells flooded by the moving front


def test_reference_tsit5_drains_cells_below_the_bed_and_diverges(dry):
    case, o, N, hst = dry
    Q, _ = o.tsit5(case["Q0"], 0.0, 0.5, max_steps=100000, nthreads=THREADS)
    assert (Q[:N] + hst).min() < 0.0          # negative depth: no state clamp in the ODE solve
    Q, _ = o.tsit5(case["Q0"], 0.0, 30.0, max_steps=100000, nthreads=THREADS)
    assert np.abs(Q[N:]).max() > 1e4


def test_reference_euler_loop_floods_the_dry_bed(dry):
    case, o, N, hst = dry
    dry0 = case["Q0"][:N] + hst <= 1.0001e-3
    Q = o.euler_reference(case["Q0"], 1, 0.01)
    h = Q[:N] + hst
    below = dry0 & (hst > 0.0)                # dry cells whose bed lies below the still-water level
    assert below.sum() > 1000
    # xi clamped to h_small: depth = hstill + h_small, water up to the still-water level
    assert np.allclose(h[below], hst[below] + 1e-3, rtol=0, atol=1e-9)


def test_a_film_far_thinner_than_fp32_resolution_switches_on_the_bed_slope_source(dry):
    """Why FP32 flux arithmetic cannot follow the reference on a dry bed: the
    RHS jumps at h = h_small.  A cell whose depth exceeds h_small by 1e-12 m
    is wet, so its momentum source (h > h_small) g xi S0
    (semi_discretize_swe_2D.jl:463,474-475) is on -- with xi = h - hstill
    about -hstill, an O(0.1) m^2/s^2 acceleration -- while its dry
    neighbours' one-sided fluxes carry the h-based pressure
    (swe_2D_solvers.jl:54-75), which does not balance it.  1e-12 m is 1e-12
    of the state's scale, far below what FP32 (24-bit) flux arithmetic
    resolves."""
    case, o, N, hst = dry
    Q = case["Q0"].copy()
    dry0 = Q[:N] + hst <= 1.0001e-3
    r0 = o.rhs(Q)
    # dry cells below still water away from the pool: no momentum change
    cand = np.nonzero(dry0 & (hst > 0.5) & (r0[N:2 * N] == 0.0) & (r0[2 * N:] == 0.0))[0]
    assert len(cand) > 500
    acc = []
    for c in cand[:: max(1, len(cand) // 20)]:
        Qf = Q.copy()
        Qf[c] = 1e-3 + 1e-12 - hst[c]                   # a film 1e-12 m above h_small
        r1 = o.rhs(Qf)
        acc.append(np.hypot(r1[N + c], r1[2 * N + c]))
    assert np.median(acc) > 1e-2


def test_films_spread_ahead_of_the_front_in_fp64():
    """The reference's own FP64 run (river_triangles(128, dry_land=True),
    32,768 cells, fixed dt = the CFL-0.01 step) wets cells far ahead of the
    pool with films of 1e-13-1e-9 m: after 50 steps (0.14 s, in which the
    pool's edge moves about half a metre) they reach more than 1 km from the
    pool's centre, a numerical precursor moving about a cell per step.  The
    same run with FMA contraction, or with the wet state perturbed by 1e-6,
    reproduces them to 1e-12, so they are systematic FP64 arithmetic -- of a
    size that FP32 flux arithmetic does not produce, which is why the FP32C
    path departs from FP64 at dry fronts (tests/test_gpu_fronts.py)."""
    from hydrograd_gb.workloads import cell_centroids
    case = river_triangles(n=128, dry_land=True)
    N = len(case["cell_node_count"])
    hst = case["wstill"] - case["zb_cells"]
    o = Oracle(case)
    o.set_wstill(case["wstill"])
    o.set_manning_cells(case["manning_zones"][case["mat_id"]])
    o.set_inlet_q(case["inlet_q"])
    o.set_exit_wse(case["exit_wse"])
    Q = o.rk2(case["Q0"], 50, dt=o.cfl_dt(case["Q0"], 0.01), nthreads=THREADS)
    h = Q[:N] + hst
    films = (h > 1e-3) & (h < 1e-3 + 1e-9)
    thin = (h > 1e-3) & (h < 1e-3 + 1e-5)
    cx, cy = cell_centroids(case)
    assert films.sum() >= 10
    assert np.hypot(cx - 300.0, cy - 1000.0)[thin].max() > 1000.0


def test_the_fronts_amplify_rounding_sized_perturbations():
    """How far apart two runs at the fronts may be when their arithmetic differs.
    FP64 runs of the dry-pool start (river_triangles(128, dry_land=True),
    32,768 cells, fixed dt = the CFL-0.01 step), one of them with a seeded
    relative perturbation added to the wet cells' depth and momenta after every
    step: at 1e-7 -- FP32's rounding -- the two part by about 1e-2 of the
    state within 20 steps, because a perturbation of that size decides whether
    a dry cell takes a film this step or a later one (the films of the test
    above; a film then grows to centimetres under its neighbour's one-sided
    pressure); at 1e-14 they stay 1e-13 apart.  The FP32C path's flux
    arithmetic rounds at 1e-7, so at dry fronts it departs from FP64 by this
    much at the first film it seeds differently; on wet states it keeps to
    FP64 within 2e-7 over 2,000 steps."""
    case = river_triangles(n=128, dry_land=True)
    N = len(case["cell_node_count"])
    hst = case["wstill"] - case["zb_cells"]
    o = Oracle(case)
    o.set_wstill(case["wstill"])
    o.set_manning_cells(case["manning_zones"][case["mat_id"]])
    o.set_inlet_q(case["inlet_q"])
    o.set_exit_wse(case["exit_wse"])
    dt = o.cfl_dt(case["Q0"], 0.01)
    steps = 20

    def run(amp):
        rng = np.random.default_rng(7)
        Q = case["Q0"].copy()
        for _ in range(steps):
            Q = o.rk2(Q, 1, dt=dt, nthreads=THREADS)
            if amp > 0.0:
                wet = Q[:N] + hst > 1.0e-3
                nw = int(wet.sum())
                h = Q[:N][wet] + hst[wet]
                Q[:N][wet] = h * (1.0 + amp * rng.standard_normal(nw)) - hst[wet]
                Q[N:2 * N][wet] *= 1.0 + amp * rng.standard_normal(nw)
                Q[2 * N:][wet] *= 1.0 + amp * rng.standard_normal(nw)
        return Q

    clean = run(0.0)
    scale = np.abs(clean).max()
    part = {amp: np.abs(run(amp) - clean).max() / scale for amp in (1e-7, 1e-14)}
    assert part[1e-7] > 1e-3
    assert part[1e-14] < 1e-11
