"""Ensembles (hg_ensemble_create): members stepped together give each member's
own single-context result, and in CFL stepping every member takes its own
step.

In FP64 every member's state after K fixed-dt steps is bit-identical to a
context of its own (gather-form sums in the mesh's slot order, inlet totals in
NodeString order: nothing depends on the other members or on the cell order).
The FP32C path sums inlet totals from per-block partials, and a member's
cells fall into other blocks in the ensemble than in its own context, so
there the match is to rounding.  The ensemble's loss is the mean over all members' probes, so member
m's gradients are its own, scaled by P_m / P.
"""
import numpy as np
import pytest

from hydrograd_gb import SWE2D, SWE2DEnsemble
from hydrograd_gb.workloads import Stream, dam_break, river_triangles

pytestmark = pytest.mark.gpu


def _meshes():
    return [river_triangles(n=12, L=400.0, inlet_q=100.0, pool_center=(60.0, 200.0), pool_radius=70.0),
            dam_break(20, 4, 10.0, 2.0),
            river_triangles(n=10, L=300.0, seed=3, inlet_q=60.0, pool_center=(150.0, 150.0), pool_radius=60.0)]


# member -> (mesh, zone-n scale, inlet Q scale)
MEMBERS = [(0, 1.0, 1.0), (1, 1.0, 1.0), (0, 1.3, 0.7), (2, 0.8, 1.2)]


def _member_params(case, zscale, qscale):
    return dict(wstill=case["wstill"], mat_id=case["mat_id"], zones=case["manning_zones"] * zscale,
                inlet_q=np.asarray(case["inlet_q"], dtype=float) * qscale, exit_wse=np.asarray(case["exit_wse"]),
                Q0=case["Q0"])


def _single(case, p, precision):
    c = SWE2D(case, precision=precision)
    c.set_still_water(p["wstill"])
    c.set_manning_zones(p["mat_id"], p["zones"])
    if len(p["inlet_q"]):
        c.set_inlet_q(p["inlet_q"])
    if len(p["exit_wse"]):
        c.set_exit_wse(p["exit_wse"])
    return c


def _ensemble(meshes, params, precision):
    e = SWE2DEnsemble(meshes, [m for m, _, _ in MEMBERS], precision=precision)
    e.set_still_water(e.concat([p["wstill"] for p in params]))
    # zone ids made distinct per member: member m's zones follow members 0..m-1's
    mat, zones, base = [], [], 0
    for p in params:
        mat.append(np.asarray(p["mat_id"]) + base)
        zones.append(p["zones"])
        base += len(p["zones"])
    e.set_manning_zones(np.concatenate(mat).astype(np.int32), np.concatenate(zones))
    e.set_inlet_q(e.concat([p["inlet_q"] for p in params], "inlet"))
    e.set_exit_wse(e.concat([p["exit_wse"] for p in params], "exit"))
    return e


def _setup(precision):
    meshes = _meshes()
    params = [_member_params(meshes[m], zs, qs) for m, zs, qs in MEMBERS]
    return meshes, params, _ensemble(meshes, params, precision)


def test_layout_counts_members_cells_and_boundaries():
    meshes, params, e = _setup("fp64")
    sizes = [len(meshes[m]["cell_node_count"]) for m, _, _ in MEMBERS]
    assert e.n_members == len(MEMBERS)
    assert list(np.diff(e.cell_offset)) == sizes
    assert list(np.diff(e.inlet_offset)) == [len(meshes[m]["inlet_q"]) for m, _, _ in MEMBERS]
    assert list(np.diff(e.exit_offset)) == [len(meshes[m]["exit_wse"]) for m, _, _ in MEMBERS]
    assert e.n_cells == sum(sizes)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_members_match_their_own_contexts(precision):
    meshes, params, e = _setup(precision)
    K = 40
    dts = []
    for (m, _, _), p in zip(MEMBERS, params):
        c = _single(meshes[m], p, "fp64")
        dts.append(c.integrate(p["Q0"], 1, cfl=0.4)[1][0])
    dt = 0.5 * min(dts)
    qe, _ = e.integrate(e.concat([p["Q0"] for p in params], "state"), K, dt=dt)
    for (m, _, _), p, q in zip(MEMBERS, params, e.split(qe, "state")):
        qs, _ = _single(meshes[m], p, precision).integrate(p["Q0"], K, dt=dt)
        if precision == "fp64":
            np.testing.assert_array_equal(q, qs)
        else:
            assert np.abs(q - qs).max() <= 1e-6 * np.abs(qs).max()


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_each_member_takes_its_own_cfl_steps(precision):
    """CFL stepping: every member forms its step from its own cells and keeps
    its own time (hg_ensemble_steps), so its trajectory is the one it has
    alone (swe_2D_forward_simulation.jl:24-39 solves one problem per run).
    FP64: bit for bit, steps and states, with a hydrograph on one member
    (evaluated at that member's own stage times).  FP32C: the ensemble's
    unfused stages against the single context's fused ones, within 1e-5."""
    meshes, params, e = _setup(precision)
    hydro = (np.array([0.0, 2.0, 5.0]), np.array([100.0, 180.0, 60.0]))
    e.set_inlet_hydrograph(int(e.inlet_offset[2]), *hydro)      # member 2's inlet (mesh 0)
    K = 30
    qe, dts_e = e.integrate(e.concat([p["Q0"] for p in params], "state"), K, cfl=0.4)
    dts, t = e.steps(K)
    np.testing.assert_array_equal(dts[:, 0], dts_e)              # the context's own record is member 0's
    assert not np.array_equal(dts[:, 1], dts[:, 0])              # the members' steps differ
    assert not np.array_equal(dts[:, 3], dts[:, 0])
    for i, (((m, _, _), p), q) in enumerate(zip(zip(MEMBERS, params), e.split(qe, "state"))):
        c = _single(meshes[m], p, precision)
        if i == 2:
            c.set_inlet_hydrograph(0, *hydro)
        qs, dts_s = c.integrate(p["Q0"], K, cfl=0.4)
        if precision == "fp64":
            np.testing.assert_array_equal(dts[:, i], dts_s)
            np.testing.assert_array_equal(q, qs)
            assert t[i] == c.elapsed_time()
        else:
            assert np.abs(dts[:, i] - dts_s).max() <= 1e-5 * dts_s.max()
            assert np.abs(q - qs).max() <= 1e-5 * np.abs(qs).max()


def test_member_gradients_are_their_own_scaled_by_probe_share():
    meshes, params, e = _setup("fp64")
    K = 12
    dt = 0.5 * e.integrate(e.concat([p["Q0"] for p in params], "state"), 1, cfl=0.4)[1][0]
    probes, obs, singles = [], [], []
    for i, ((m, _, _), p) in enumerate(zip(MEMBERS, params)):
        N = len(meshes[m]["cell_node_count"])
        c = _single(meshes[m], p, "fp64")
        h0 = p["Q0"][:N] + c.bed()["hstill"]
        pr = np.unique((Stream(20 + i).uniform(12) * N).astype(np.int32))[:4 + i]
        ob = np.tile(h0[pr] + 0.05, (K, 1))
        singles.append(c.loss_and_grad(p["Q0"], K, dt, pr, ob, ckpt_every=5))
        probes.append(pr + e.cell_offset[i])
        obs.append(ob)
    P = np.array([len(pr) for pr in probes])
    r = e.loss_and_grad(e.concat([p["Q0"] for p in params], "state"), K, dt, np.concatenate(probes),
                        np.concatenate(obs, axis=1), ckpt_every=5)
    w = P / P.sum()
    assert abs(r["loss"] - sum(wi * s["loss"] for wi, s in zip(w, singles))) <= 1e-12 * abs(r["loss"])
    for i, (gn, gz, gq) in enumerate(zip(e.split(r["g_manning"]), e.split(r["g_zb"]), e.split(r["g_inletq"], "inlet"))):
        s = singles[i]
        for got, ref in ((gn, s["g_manning"]), (gz, s["g_zb"]), (gq, s["g_inletq"])):
            if len(ref):
                assert np.abs(got - w[i] * ref).max() <= 1e-10 * max(np.abs(w[i] * ref).max(), 1e-300)
