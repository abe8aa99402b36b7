"""Vector-Jacobian products of the final state (hg_final_vjp) and the zone-n
Jacobian built from them (hydrograd_gb.sensitivity, what the reference's
sensitivity analysis computes with ForwardDiff.jacobian).

* Jacobian rows: the FP64 adjoint against the oracle's forward-mode dual
  numbers of the same fixed-dt SSP-RK2 run (1e-8 of the Jacobian's scale); the
  FP32C adjoint against the same (1e-4 of scale: a single state entry's
  derivative, not an aggregate).
* A cotangent formed on the host from the WSE loss gives the gradients of
  hg_final_loss_and_grad (1e-12).
"""
import numpy as np
import pytest

from hydrograd_gb.sensitivity import flatten_like_reference, zone_manning_jacobian
from hydrograd_gb.workloads import Stream
from tests.test_gpu_forward import setup_pair, small_river

pytestmark = pytest.mark.gpu


def problem():
    case = small_river(n=12, L=300.0)
    return case, len(case["cell_node_count"])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("fp32c", 1e-4)])
def test_zone_jacobian_rows_match_dual_numbers(precision, tol):
    case, N = problem()
    ctx, o, _ = setup_pair(case, precision=precision)
    K = 40
    Q0 = case["Q0"]
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    nz = len(case["manning_zones"])
    dman = np.stack([(case["mat_id"] == z).astype(float) for z in range(nz)])
    _, dQ, _, _ = o.rk2_tangent(Q0, K, dt, d_manning=dman, nthreads=4)   # [nz, 3N]
    wet = np.flatnonzero(np.abs(dQ).max(axis=0) > 1e-6 * np.abs(dQ).max())
    rows = np.sort(Stream(9).uniform(24) * len(wet)).astype(int)
    rows = np.unique(wet[rows])
    J = zone_manning_jacobian(ctx, Q0, K, dt, case["mat_id"], nz, rows=rows, ckpt_every=10)
    ref = dQ[:, rows].T
    assert np.abs(J - ref).max() <= tol * np.abs(dQ).max()
    assert flatten_like_reference(J).shape == (len(rows) * nz,)


def test_wse_cotangent_reproduces_the_final_loss_gradient():
    case, N = problem()
    ctx, o, _ = setup_pair(case, precision="fp64")
    K = 30
    Q0 = case["Q0"]
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    hst = o.hstill()
    wse = case["wstill"] + 0.05 * Stream(4).uniform(N, -1.0, 1.0)
    zb = case["zb_cells"]
    r = ctx.final_loss_and_grad(Q0, K, dt, wse=wse, zb_wse=zb, ckpt_every=10)
    Q = r["Q"]
    h = Q[:N] + hst
    den = (wse.max() - wse.min()) + np.sqrt(np.finfo(float).eps)
    lam = np.zeros(3 * N)
    lam[:N] = 2.0 * ((h + zb) - wse) / den / den / N   # dL/dxi of the WSE term
    lam[:N] *= h > 1e-3                                 # clamped cells do not depend on their inputs
    v = ctx.final_state_vjp(Q0, K, dt, lam, ckpt_every=10)
    for k in ("g_manning", "g_zb", "g_inletq"):
        assert np.abs(v[k] - r[k]).max() <= 1e-12 * max(np.abs(r[k]).max(), 1e-300), k
    assert np.array_equal(v["Q"], r["Q"])
