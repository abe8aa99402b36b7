"""State-dependent flow resistance without a GPU: the oracle's Manning n
functions against the reference's own truth fields, its variable-n runs
against the reference's final states, and its UDE network against an
independent numpy restatement of the Lux chain."""
import numpy as np
import pytest

from oracle.oracle import manning_fn
from tests.golden_cases import initial_state, load_case
from tests.resistance_cases import UDE_CASES, truth_state, ude_param_count, ude_params

VAR_CASES = ["fwd_bump_nh", "fwd_savannah_nks"]   # sigmoid n(h); Cheng's n(h, Umag, ks)


@pytest.mark.parametrize("name", VAR_CASES)
def test_manning_functions_match_reference_truth(name):
    """ManningN_cells_truth (and h/ks, f, Re of h_Umag_ks) were computed by the
    reference's update_ManningN_forward_simulation at the truth state with
    Umag from u = q / (h + h_small) (process_forward_simulation_results_2D.jl:26-38)."""
    d, _ = load_case(name)
    umag = np.sqrt(d["u_truth"] ** 2 + d["v_truth"] ** 2)
    n, hks, f, re = manning_fn(int(d["res_kind"]), d["res_params"], d["h_truth"], umag, d.get("ks_cells"))
    assert np.abs(n / d["ManningN_cells_truth"] - 1).max() <= 1e-14
    if "Re_cells_truth" in d:
        assert np.abs(hks / d["h_ks_cells_truth"] - 1).max() <= 1e-15
        assert np.abs(re / d["Re_cells_truth"] - 1).max() <= 1e-15
        assert np.abs(f / d["friction_factor_cells_truth"] - 1).max() <= 1e-14


@pytest.mark.parametrize("name", VAR_CASES)
def test_variable_n_run_reaches_reference_final_state(name):
    """Tsit5 (abstol 1e-6, reltol 1e-3, the case's dt as the first step, as
    the reference's solve call takes it) with n recomputed from the state in
    every RHS lands within 2e-3 of scale of the reference's final state; the
    same run with the zones' constant n does not (>= 0.05 of scale)."""
    d, o = load_case(name)
    N = o.n_cells
    Q0 = initial_state(d, N)
    T = float(d["tspan"][1])
    ref = truth_state(d)
    scale = max(np.abs(ref[:N]).max(), np.abs(ref[N:]).max())
    o.set_resistance_fn(int(d["res_kind"]), d["res_params"], d.get("ks_cells"))
    Q, _ = o.tsit5(Q0, 0.0, T, dt0=float(d["dt"]), nthreads=4)
    assert np.abs(Q - ref).max() <= 2e-3 * scale
    o.set_resistance_fn(0)
    Qc, _ = o.tsit5(Q0, 0.0, T, dt0=float(d["dt"]), nthreads=4)
    assert np.abs(Qc - ref).max() >= 0.05 * scale


def lux_chain(x, hidden, acts, p, out_bounds, over_batch):
    """Independent restatement: x [in, cells] -> [cells] (column = cell, as Lux batches)."""
    f = {"tanh": np.tanh, "relu": lambda v: np.maximum(v, 0.0), "sigmoid": lambda v: 1.0 / (1.0 + np.exp(-v)),
         "leakyrelu": lambda v: np.where(v > 0, v, 0.01 * v), "softplus": lambda v: np.log1p(np.exp(v))}
    off, a = 0, x
    for w, act in zip(hidden, acts):
        din = a.shape[0]
        W = p[off:off + w * din].reshape(din, w).T     # column-major (w x din)
        off += w * din
        b = p[off:off + w]; off += w
        z = f[act](W @ a + b[:, None])
        sc, bi = p[off:off + w], p[off + w:off + 2 * w]; off += 2 * w
        if over_batch:
            mu, var = z.mean(), z.var()
        else:
            mu, var = z.mean(axis=0, keepdims=True), z.var(axis=0, keepdims=True)
        a = (z - mu) / np.sqrt(var + np.float64(np.float32(1e-5))) * sc[:, None] + bi[:, None]
    din = a.shape[0]
    W, b = p[off:off + din], p[off + din]
    y = W @ a + b
    return out_bounds[0] + (out_bounds[1] - out_bounds[0]) / (1.0 + np.exp(-y))


@pytest.mark.parametrize("over_batch", [True, False])
@pytest.mark.parametrize("choice,kind,in_dim,bounds", UDE_CASES, ids=[c[0] for c in UDE_CASES])
def test_oracle_ude_network_matches_numpy_restatement(choice, kind, in_dim, bounds, over_batch):
    d, o = load_case("fwd_savannah_nks")
    N = o.n_cells
    hidden, acts = [3, 4], ["tanh", "softplus"]
    p = ude_params(in_dim, hidden, seed=kind)
    assert len(p) == ude_param_count(in_dim, hidden)
    ks = d["ks_cells"]
    o.set_ude(kind, in_dim, hidden, [3, 4], p, bounds["output_bounds"], bounds["h_bounds"],
              bounds.get("u_bounds", (0.0, 1.0)), bounds.get("ks_bounds", (0.0, 1.0)), ks, over_batch)
    Q = truth_state(d)
    got = o.resistance_cells(Q)
    h = np.maximum(Q[:N] + o.hstill(), 1e-3)
    dry = Q[:N] + o.hstill() <= 1e-3
    qx, qy = np.where(dry, 0.0, Q[N:2 * N]), np.where(dry, 0.0, Q[2 * N:])
    nrm = lambda v, b: 2.0 * (v - b[0]) / (b[1] - b[0]) - 1.0
    x = [nrm(h, bounds["h_bounds"])]
    if kind == 6:
        x += [nrm(np.hypot(qx / h, qy / h), bounds["u_bounds"]), nrm(ks, bounds["ks_bounds"])]
    elif kind == 7:
        hb, ub = bounds["h_bounds"], bounds["u_bounds"]
        x += [nrm(np.sqrt(qx ** 2 + qy ** 2 + 2.220446049250313e-16), (hb[0] * ub[0], hb[1] * ub[1]))]
    want = lux_chain(np.array(x), hidden, acts, p, bounds["output_bounds"], over_batch)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
