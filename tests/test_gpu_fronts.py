"""FP64 and FP32C at moving wet/dry fronts: configuration 2's dry-pool start.

The reach starts dry (h = h_small) except a 1.5 m pool touching the inlet-Q
edge; the pool spreads over the dry bed, so cells change from dry to wet
during the run and every dry/wet branch of the Roe solver
(swe_2D_solvers.jl:16-76) and the depth clamp (semi_discretize_swe_2D.jl:101-106)
is taken at the fronts.  The reference scheme diverges on this start at any
CFL-sized step (tests/test_dry_bed.py), so the runs take a fixed step: the
initial state's CFL step at CFL 0.01, 1/40 of the CFL-0.4 step.

Tolerances (as in test_gpu_forward.py): the FP64 path within 1e-10 of the
oracle after many steps; the FP32C path within 1e-5 of the FP64 oracle, per
state block (max |error| / max(max |block|, 1e-3 max |state|)), over the
whole mesh and over the front cells alone.
"""
import numpy as np
import pytest

from hydrograd_gb.workloads import river_triangles
from tests.test_gpu_forward import block_err, setup_pair

pytestmark = pytest.mark.gpu

STEPS = 300


@pytest.fixture(scope="module")
def front_run():
    case = river_triangles(n=64, dry_land=True)
    N = len(case["cell_node_count"])
    _, o, _ = setup_pair(case, "fp64")
    dt = o.cfl_dt(case["Q0"], 0.01)
    ref = o.rk2(case["Q0"], STEPS, dt=dt, nthreads=8)
    hst = case["wstill"] - case["zb_cells"]
    wet0 = case["Q0"][:N] + hst > 1.5e-3
    wet1 = ref[:N] + hst > 1.5e-3
    return case, N, dt, ref, wet0, wet1


def front_err(a, b, N, cells):
    """Per-block error over the front cells, scaled as block_err."""
    out = []
    for k in range(3):
        blk = b[k * N:(k + 1) * N]
        scale = max(np.abs(blk).max(), np.abs(b).max() * 1e-3, 1e-300)
        out.append(np.abs(a[k * N:(k + 1) * N][cells] - blk[cells]).max() / scale)
    return max(out)


def test_fronts_move(front_run):
    _, _, _, ref, wet0, wet1 = front_run
    assert (wet1 & ~wet0).sum() >= 25
    assert np.isfinite(ref).all()


def test_fp64_matches_oracle_at_fronts(front_run):
    case, N, dt, ref, _, _ = front_run
    ctx, _, _ = setup_pair(case, "fp64")
    Q, _ = ctx.integrate(case["Q0"], STEPS, dt=dt)
    assert block_err(Q, ref, N) <= 1e-10


def test_fp32c_within_1e5_of_fp64_at_fronts(front_run):
    case, N, dt, ref, wet0, wet1 = front_run
    ctx, _, _ = setup_pair(case, "fp32c")
    Q, _ = ctx.integrate(case["Q0"], STEPS, dt=dt)
    front = np.nonzero(wet0 != wet1)[0]
    assert block_err(Q, ref, N) <= 1e-5
    assert front_err(Q, ref, N, front) <= 1e-5
    # the same cells are wet at the end (no wet/dry decision flipped)
    hst = case["wstill"] - case["zb_cells"]
    assert ((Q[:N] + hst > 1.5e-3) == wet1).all()
