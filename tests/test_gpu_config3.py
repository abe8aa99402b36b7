"""Configuration 3: the adjoint of 500 fixed-dt SSP-RK2 steps, 64 probes whose
observations come from a run with hidden zone values of n, gradients w.r.t. the
5 zone values of n, the per-cell bed elevation (at a bed perturbed by a seeded
FP32 field of standard deviation 0.05 m, and along that field) and the inlet Q,
checkpoints every 50.

* The 2,048-cell copy (32 x 32 x 2): the FP64 adjoint against the oracle's
  dual numbers (1e-8, the exact derivative of the same discrete map) and
  central differences of the oracle (eps 1e-6, FP64; 1e-5).
* 250,632 cells (354 x 354 x 2): the FP32C adjoint against the FP64 adjoint
  (1e-5 relative for the zone, inlet and directional bed gradients).
"""
import numpy as np
import pytest

from hydrograd_gb import SWE2D
from hydrograd_gb.workloads import Stream, probes_and_perturbation, river_triangles
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

K, CKPT = 500, 50


def configure(obj, case, zones, zb):
    """The same parameters on a fresh device context or oracle (hstill = wstill
    - the mesh's zb, fixed before the bed is perturbed, as in the reference)."""
    if isinstance(obj, SWE2D):
        obj.set_still_water(case["wstill"])
        obj.set_manning_zones(case["mat_id"], zones)
    else:
        obj.set_wstill(case["wstill"])
        obj.set_manning_cells(zones[case["mat_id"]])
    obj.set_zb_cells(zb)
    obj.set_inlet_q(case["inlet_q"])
    obj.set_exit_wse(case["exit_wse"])


def problem(n):
    case = river_triangles(n=n)
    N = len(case["cell_node_count"])
    probes, dz = probes_and_perturbation(case, n_probe=64, seed=5, zb_sigma=0.05, inlet_share=0.25)
    zb = case["zb_cells"] + dz
    hidden = Stream(17).uniform(len(case["manning_zones"]), 0.02, 0.06)
    return case, N, probes, dz, zb, hidden


def device_obs(case, zb, hidden, Q0, dt, probes):
    """Probe depths of K steps with the hidden zone values, on the FP64 device path."""
    c = SWE2D(case, precision="fp64")
    configure(c, case, hidden, zb)
    hst = case["wstill"] - zb
    c.upload(Q0)
    obs = np.zeros((K, len(probes)))
    for k in range(K):
        c.advance(1, dt=dt, graph=False)
        q = c.download()
        obs[k] = q[probes] + hst[probes]
    return obs


def test_config3_small_copy_vs_oracle():
    case, N, probes, dz, zb, hidden = problem(32)
    assert N == 2048
    oh = Oracle(case)                 # the run with the hidden zone values
    configure(oh, case, hidden, zb)
    Q0 = case["Q0"]
    dt = 0.5 * oh.cfl_dt(Q0, 0.4)
    obs = np.zeros((K, len(probes)))
    hst = oh.hstill()
    Q = Q0.copy()
    for k in range(K):
        Q = oh.rk2(Q, 1, dt=dt)
        obs[k] = Q[probes] + hst[probes]
    zones = case["manning_zones"]
    o = Oracle(case)
    configure(o, case, zones, zb)
    ctx = SWE2D(case, precision="fp64")
    configure(ctx, case, zones, zb)
    r = ctx.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=CKPT)
    nz = len(zones)
    g_zone = np.bincount(case["mat_id"], r["g_manning"], minlength=nz)
    dman = np.stack([(case["mat_id"] == z).astype(float) for z in range(nz)])
    _, _, loss_o, dl_n = o.rk2_tangent(Q0, K, dt, d_manning=dman, probes=probes, obs=obs, nthreads=4)
    _, _, _, dl_zb = o.rk2_tangent(Q0, K, dt, d_zb=dz[None, :], probes=probes, obs=obs, nthreads=4)
    _, _, _, dl_q = o.rk2_tangent(Q0, K, dt, d_inlet=np.ones((1, 1)), probes=probes, obs=obs, nthreads=4)
    assert abs(r["loss"] - loss_o) <= 1e-10 * loss_o
    assert np.abs(g_zone - dl_n).max() <= 1e-8 * np.abs(dl_n).max()
    assert abs(r["g_zb"] @ dz - dl_zb[0]) <= 1e-8 * abs(dl_zb[0])
    assert abs(r["g_inletq"][0] - dl_q[0]) <= 1e-8 * abs(dl_q[0])
    # central differences of the oracle's loss, eps 1e-6
    eps = 1e-6
    for z in range(nz):
        vals = []
        for s in (1, -1):
            zz = zones.copy()
            zz[z] += s * eps
            o.set_manning_cells(zz[case["mat_id"]])
            vals.append(o.rk2_loss(Q0, K, dt, probes, obs, nthreads=4)[0])
        fd = (vals[0] - vals[1]) / (2 * eps)
        assert abs(g_zone[z] - fd) <= 1e-5 * np.abs(dl_n).max(), z
    o.set_manning_cells(zones[case["mat_id"]])
    vals = []
    for s in (1, -1):
        o.set_zb_cells(zb + s * eps * dz)
        vals.append(o.rk2_loss(Q0, K, dt, probes, obs, nthreads=4)[0])
    o.set_zb_cells(zb)
    fd = (vals[0] - vals[1]) / (2 * eps)
    assert abs(r["g_zb"] @ dz - fd) <= 1e-5 * abs(fd)


def test_config3_fp32c_vs_fp64_at_250k():
    case, N, probes, dz, zb, hidden = problem(354)
    assert N == 250632
    Q0 = case["Q0"]
    ctx64 = SWE2D(case, precision="fp64")
    configure(ctx64, case, case["manning_zones"], zb)
    o = Oracle(case)
    configure(o, case, case["manning_zones"], zb)
    dt = 0.5 * o.cfl_dt(Q0, 0.4)
    obs = device_obs(case, zb, hidden, Q0, dt, probes)
    ctx32 = SWE2D(case, precision="fp32c")
    configure(ctx32, case, case["manning_zones"], zb)
    a = ctx64.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=CKPT)
    b = ctx32.loss_and_grad(Q0, K, dt, probes, obs, ckpt_every=CKPT)
    nz = len(case["manning_zones"])
    ga = np.bincount(case["mat_id"], a["g_manning"], minlength=nz)
    gb = np.bincount(case["mat_id"], b["g_manning"], minlength=nz)
    assert a["loss"] > 0 and abs(b["loss"] - a["loss"]) <= 1e-5 * a["loss"]
    assert np.abs(gb - ga).max() <= 1e-5 * np.abs(ga).max()
    assert abs(b["g_inletq"][0] - a["g_inletq"][0]) <= 1e-5 * abs(a["g_inletq"][0])
    assert abs(b["g_zb"] @ dz - a["g_zb"] @ dz) <= 1e-5 * abs(a["g_zb"] @ dz)
