"""Tsit5 without a GPU: the library's tableau (through the C ABI) satisfies
the order conditions of the Tsitouras 5(4) pair, and the oracle's Tsit5
(hgo::tsit5) reaches the final states of the reference's own Tsit5 runs
(abstol 1e-6, reltol 1e-3) of its shipped example cases."""
import ctypes

import numpy as np
import pytest

from tests.golden_cases import initial_state, load_case


def tableau():
    from hydrograd_gb._lib import lib
    c, a, b, bt = np.zeros(7), np.zeros(49), np.zeros(7), np.zeros(7)
    p = ctypes.POINTER(ctypes.c_double)
    assert lib().hg_tsit5_tableau(*(v.ctypes.data_as(p) for v in (c, a, b, bt))) == 0
    return c, a.reshape(7, 7), b, bt


def test_tableau_order_conditions():
    c, A, b, bt = tableau()
    assert np.abs(A.sum(axis=1) - c).max() < 1e-14            # row sums = nodes
    assert np.allclose(A[6], b, rtol=0, atol=0)               # first same as last
    assert abs(bt.sum()) < 1e-15                              # error weights sum to zero
    bh = b - bt                                               # the embedded 4th-order weights
    for w, order in ((b, 5), (bh, 4)):
        # quadrature conditions sum_i w_i c_i^(k-1) = 1/k
        for k in range(1, order + 1):
            assert abs(w @ c ** (k - 1) - 1.0 / k) < 1e-13, (order, k)
        # tree conditions up to order 4 on the same weights
        assert abs(w @ (A @ c) - 1 / 6) < 1e-13
        assert abs(w @ (c * (A @ c)) - 1 / 8) < 1e-13
        assert abs(w @ (A @ c ** 2) - 1 / 12) < 1e-13
        assert abs(w @ (A @ (A @ c)) - 1 / 24) < 1e-13
    # fifth-order trees of b
    assert abs(b @ (c ** 2 * (A @ c)) - 1 / 10) < 1e-13
    assert abs(b @ (A @ c ** 3) - 1 / 20) < 1e-13
    assert abs(b @ ((A @ c) ** 2) - 1 / 20) < 1e-13
    assert abs(b @ (A @ (A @ (A @ c))) - 1 / 120) < 1e-13


@pytest.mark.parametrize("name", ["fwd_bump", "fwd_uniform", "fwd_savannah"])
def test_oracle_tsit5_reaches_reference_final_state(name):
    """The reference ran these cases with Tsit5 at abstol 1e-6, reltol 1e-3;
    the restated Tsit5 at the same tolerances lands within 1e-3 of scale of
    its final state (the SSP-RK2 pin of the oracle allows 2e-3)."""
    d, o = load_case(name)
    N = o.n_cells
    Q, (acc, rej, ev) = o.tsit5(initial_state(d, N), float(d["tspan"][0]), float(d["tspan"][1]),
                                abstol=1e-6, reltol=1e-3, nthreads=4)
    assert ev == 6 * (acc + rej) + 2                          # K1 + starting-step probe, 6 per step attempt
    h = d["h_truth"]
    ref = np.concatenate([d["xi_truth"], d["u_truth"] * (h + 1e-3), d["v_truth"] * (h + 1e-3)])
    scale = max(np.abs(ref[:N]).max(), np.abs(ref[N:]).max())
    assert np.abs(Q - ref).max() <= 1e-3 * scale


def test_oracle_tsit5_fixed_steps_fifth_order():
    """Fixed steps (adaptive=False): halving dt divides the error by about
    2^5 on a smooth flow (the bump case over 20 CFL steps), measured against a
    run with 8x smaller steps."""
    d, o = load_case("fwd_bump")
    N = o.n_cells
    Q0 = initial_state(d, N)
    T = 20 * o.cfl_dt(Q0, 0.4)
    ref, _ = o.tsit5(Q0, 0.0, T, dt0=T / 640, adaptive=False, nthreads=4)
    errs = []
    for n in (20, 40, 80):
        Q, (acc, rej, ev) = o.tsit5(Q0, 0.0, T, dt0=T / n, adaptive=False, nthreads=4)
        assert (acc, rej, ev) == (n, 0, 6 * n + 1)
        errs.append(np.abs(Q - ref).max())
    assert errs[0] / errs[1] > 24 and errs[1] / errs[2] > 24


def test_oracle_tsit5_converges_with_tolerance():
    """Tightening the tolerance by 1e3 moves the final state toward the
    tight-tolerance solution: the error follows the tolerance."""
    d, o = load_case("fwd_bump")
    N = o.n_cells
    Q0 = initial_state(d, N)
    fine, _ = o.tsit5(Q0, 0.0, 20.0, abstol=1e-12, reltol=1e-10, nthreads=4)
    coarse, _ = o.tsit5(Q0, 0.0, 20.0, abstol=1e-6, reltol=1e-3, nthreads=4)
    mid, _ = o.tsit5(Q0, 0.0, 20.0, abstol=1e-9, reltol=1e-6, nthreads=4)
    e_coarse, e_mid = np.abs(coarse - fine).max(), np.abs(mid - fine).max()
    assert e_mid < 0.05 * e_coarse


def test_oracle_tsit5_lake_at_rest():
    """Still water stays still under adaptive steps (well-balanced RHS): the
    controller grows the step to its cap and the state does not move."""
    d, o = load_case("fwd_bump")
    N = o.n_cells
    Q0 = np.zeros(3 * N)
    wstill = float(d["ic_const"][1])                          # xi = 0: the water surface at wstill
    o.set_inlet_q(np.zeros_like(d["inlet_q"]))
    o.set_exit_wse(np.full_like(d["exit_wse"], wstill))
    Q, (_, rej, _) = o.tsit5(Q0, 0.0, 50.0, nthreads=4)
    assert rej == 0
    assert np.abs(Q).max() < 1e-10
