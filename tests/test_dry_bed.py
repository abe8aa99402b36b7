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
