"""hg_rhs_device_noalloc: the RHS entry point that allocates nothing.

It is meant for callers that cannot allocate device memory while their time
loop runs (an integrator using CUDA.jl's memory pool, or a step recorded into
a CUDA graph).  These tests call it through the C ABI with device buffers the
test owns, twice in a row, and compare with the ordinary hg_rhs entry point
at the FP64 RHS tolerance (1e-12 of the flux scale, see test_gpu_forward.py).
"""
import ctypes

import numpy as np
import pytest

from hydrograd_gb import HgError, HostMesh, SWE2D
from hydrograd_gb._lib import lib
from hydrograd_gb.workloads import dam_break, river_triangles

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _river():
    return river_triangles(n=24, L=400.0, inlet_q=100.0, pool_center=(60.0, 200.0), pool_radius=70.0)


def _ctx(case):
    ctx = SWE2D(case, precision="fp64", order="hilbert")
    ctx.set_still_water(case["wstill"])
    ctx.set_manning_zones(case["mat_id"], case["manning_zones"])
    if len(case["inlet_q"]):
        ctx.set_inlet_q(case["inlet_q"])
    if len(case["exit_wse"]):
        ctx.set_exit_wse(case["exit_wse"])
    return ctx


def _noalloc(ctx, dq_in, dq_out, flags):
    return lib().hg_rhs_device_noalloc(ctx.h, ctypes.c_void_p(dq_in.data_ptr()), ctypes.c_void_p(dq_out.data_ptr()),
                                       ctypes.c_void_p(flags.data_ptr()), None)


def test_noalloc_rhs_matches_hg_rhs_on_two_calls():
    case = _river()
    N = len(case["cell_node_count"])
    ctx = _ctx(case)
    perm = HostMesh(case).order("hilbert")        # perm[device id] = caller id
    dev = torch.device("cuda:0")
    flags = torch.full((1,), -1, dtype=torch.int32, device=dev)
    Q1 = case["Q0"]
    Q2 = Q1.copy()
    Q2[N:2 * N] += 0.05 * np.sin(np.arange(N))     # a second, different state
    for Q in (Q1, Q2):
        ref = ctx.rhs(Q)
        q_dev = torch.from_numpy(np.concatenate([Q[b * N:(b + 1) * N][perm] for b in range(3)])).to(dev)
        out = torch.full((3 * N,), np.nan, dtype=torch.float64, device=dev)
        assert _noalloc(ctx, q_dev, out, flags) == 0
        torch.cuda.synchronize()
        got_dev = out.cpu().numpy()
        got = np.empty(3 * N)
        for b in range(3):
            got[b * N + perm] = got_dev[b * N:(b + 1) * N]
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(got - ref).max() <= 1e-12 * scale
        assert int(flags.item()) == 0


def test_noalloc_reports_dry_inlet_in_flags():
    case = river_triangles(n=16, L=400.0, pool_center=(300.0, 300.0), pool_radius=40.0, dry_land=True)
    N = len(case["cell_node_count"])
    ctx = _ctx(case)
    perm = HostMesh(case).order("hilbert")
    dev = torch.device("cuda:0")
    q_dev = torch.from_numpy(np.concatenate([case["Q0"][b * N:(b + 1) * N][perm] for b in range(3)])).to(dev)
    out = torch.zeros(3 * N, dtype=torch.float64, device=dev)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    assert _noalloc(ctx, q_dev, out, flags) == 0
    torch.cuda.synchronize()
    assert int(flags.item()) & 2


def test_noalloc_rejects_too_many_inlet_boundaries():
    case = dam_break(80, 4, 40.0, 2.0)
    # 65 one-edge inlet-Q NodeStrings along the south edge (nodes 0..80)
    strings = [np.array([k, k + 1], dtype=np.int32) for k in range(65)]
    case.update(string_ids=np.arange(1, 66, dtype=np.int32),
                string_offsets=np.cumsum([0] + [2] * 65).astype(np.int32),
                string_nodes=np.concatenate(strings), string_bc=np.full(65, 2, dtype=np.int32),
                inlet_q=np.full(65, 0.01))
    ctx = _ctx(case)
    N = len(case["cell_node_count"])
    dev = torch.device("cuda:0")
    q = torch.zeros(3 * N, dtype=torch.float64, device=dev)
    rc = lib().hg_rhs_device_noalloc(ctx.h, ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(q.data_ptr()), None, None)
    assert rc == 1
    with pytest.raises(HgError, match="at most 64"):
        ctx._chk(rc)


def test_noalloc_refuses_hydrograph_and_state_dependent_resistance():
    """A hydrograph makes the inlet Q depend on the time, which this entry
    point does not take; a state-dependent resistance writes the context's
    own per-cell n before every RHS.  Both are refused (HG_ERR_UNSUPPORTED),
    and the context works again once the option is removed."""
    case = _river()
    N = len(case["cell_node_count"])
    dev = torch.device("cuda:0")
    q = torch.from_numpy(case["Q0"].copy()).to(dev)
    out = torch.zeros(3 * N, dtype=torch.float64, device=dev)
    ctx = _ctx(case)
    ctx.set_inlet_hydrograph(0, [0.0, 100.0], [50.0, 150.0])
    rc = _noalloc(ctx, q, out, torch.zeros(1, dtype=torch.int32, device=dev))
    assert rc == 7
    with pytest.raises(HgError, match="hydrograph"):
        ctx._chk(rc)
    ctx.set_inlet_hydrograph(0, [], [])
    assert _noalloc(ctx, q, out, torch.zeros(1, dtype=torch.int32, device=dev)) == 0
    ctx.set_manning_function("sigmoid", {"n_lower": 0.02, "n_upper": 0.05, "k": 4.0, "h_mid": 0.5})
    rc = _noalloc(ctx, q, out, torch.zeros(1, dtype=torch.int32, device=dev))
    assert rc == 7
    with pytest.raises(HgError, match="resistance"):
        ctx._chk(rc)
    ctx.set_manning_function("constant")
    assert _noalloc(ctx, q, out, torch.zeros(1, dtype=torch.int32, device=dev)) == 0
    torch.cuda.synchronize()
