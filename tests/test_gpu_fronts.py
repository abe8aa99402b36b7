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


# The same start on a finer mesh (131,072 cells, 15.6 m).  Here the scheme
# seeds its first films within 20 steps: a dry cell whose inflows cancel to
# ~1e-11 of their size takes a film of ~1e-13 m, which the neighbour's
# one-sided pressure then grows to ~1e-4 m within a few steps
# (tests/test_dry_bed.py pins both the seed and how the fronts amplify
# rounding-sized differences).  Whether a seed forms hangs on differences far
# below FP32's resolution, so FP32C and FP64 part at the first one; before it
# FP32C holds the 1e-5 contract at the fronts.
SEED_FREE_STEPS = 15


@pytest.fixture(scope="module")
def fine_run():
    case = river_triangles(n=256, dry_land=True)
    N = len(case["cell_node_count"])
    _, o, _ = setup_pair(case, "fp64")
    dt = o.cfl_dt(case["Q0"], 0.01)
    ref = o.rk2(case["Q0"], SEED_FREE_STEPS, dt=dt, nthreads=8)
    hst = case["wstill"] - case["zb_cells"]
    return case, N, dt, ref, hst


def test_fp32c_within_1e5_of_fp64_at_fronts_on_a_fine_mesh(fine_run):
    case, N, dt, ref, hst = fine_run
    wet0 = case["Q0"][:N] + hst > 1.5e-3
    wet1 = ref[:N] + hst > 1.5e-3
    assert (wet1 & ~wet0).sum() >= 20   # the fronts moved
    ctx, _, _ = setup_pair(case, "fp32c")
    Q, _ = ctx.integrate(case["Q0"], SEED_FREE_STEPS, dt=dt)
    front = np.nonzero(wet0 != wet1)[0]
    assert block_err(Q, ref, N) <= 1e-5
    assert front_err(Q, ref, N, front) <= 1e-5
    # every cell is dry (clamped, h = h_small) in both precisions or in neither
    dry64 = ref[:N] + hst <= 1.0e-3
    dry32 = Q[:N] + hst <= 1.0e-3 * (1 + 1e-9)
    assert (dry64 == dry32).all()


def test_fp32c_gradients_match_fp64_at_fronts(front_run):
    """The FP32C reverse sweep differentiates the branches its forward pass took
    (the same FP64 wall test): gradients of a probe-depth loss over 100 steps of
    the moving fronts, FP32C against FP64, within 1e-5 of each field's scale."""
    case, N, dt, _, wet0, wet1 = front_run
    probes = np.nonzero(wet1 & ~wet0)[0][::4][:32].astype(np.int32)   # cells the fronts reach
    K = 100
    obs = np.full((K, len(probes)), 2.0e-3)
    out = {}
    for prec in ("fp32c", "fp64"):
        ctx, _, _ = setup_pair(case, prec)
        out[prec] = ctx.loss_and_grad(case["Q0"], K, dt, probes, obs, ckpt_every=25)
    a, b = out["fp32c"], out["fp64"]
    assert abs(a["loss"] - b["loss"]) <= 1e-5 * abs(b["loss"])
    for k in ("g_manning", "g_zb", "g_inletq"):
        assert np.abs(a[k] - b[k]).max() <= 1e-5 * np.abs(b[k]).max(), k
    assert np.abs(b["g_manning"]).max() > 0.0 and np.abs(b["g_zb"]).max() > 0.0
