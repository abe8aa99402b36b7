"""Device Tsit5 (hg_integrate_tsit5) vs the oracle's Tsit5 (hgo::tsit5), the
same algorithm: Tsitouras 5(4) pair, weighted RMS error norm, PI controller,
Hairer's starting step, steps clamped onto save times and the end time.

Fixed steps: FP64 states within 1e-10 of the oracle (normwise per block, as in
test_gpu_forward) over the cases' whole time spans; the FP32-compensated RHS
within 1e-5.

Adaptive steps: once the step size sits at the explicit stability limit, the
controller feeds round-off back into the step sizes and two runs that differ
in the last bit of one sum drift apart (two CPU restatements that differ only
in summation order: 1e-14 apart after 18 steps, 3e-13 after 28, 2e-8 after
110).  So the adaptive runs are compared step for step over their first 10-16
steps (same step counts, 1e-10), and over the whole span against the
reference's own Tsit5 final state (2e-3 of scale, twice the runs' reltol).
"""
import numpy as np
import pytest

from hydrograd_gb import HgError
from tests.golden_cases import initial_state, load_fixture
from tests.test_gpu_forward import block_err, setup_pair

pytestmark = pytest.mark.gpu

CASES = ["fwd_bump", "fwd_uniform", "fwd_savannah"]
STATE_TOL = {"fp64": 1e-10, "fp32c": 1e-5}


def truth(d, N):
    h = d["h_truth"]
    return np.concatenate([d["xi_truth"], d["u_truth"] * (h + 1e-3), d["v_truth"] * (h + 1e-3)])


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("name", CASES)
def test_fixed_step_tsit5_matches_oracle(name, precision):
    d = load_fixture(name)
    ctx, o, N = setup_pair(d, precision)
    Q0 = initial_state(d, N)
    T = float(d["tspan"][1])
    n = int(np.ceil(T / (0.9 * o.cfl_dt(Q0, 0.4))))
    Qg, sg = ctx.integrate_tsit5(Q0, 0.0, T, dt0=T / n, adaptive=False)
    Qo, so = o.tsit5(Q0, 0.0, T, dt0=T / n, adaptive=False, nthreads=4)
    assert sg == so == (n, 0, 6 * n + 1)
    assert block_err(Qg, Qo, N) <= STATE_TOL[precision]


@pytest.mark.parametrize("name", CASES)
def test_adaptive_tsit5_matches_oracle_step_for_step(name):
    d = load_fixture(name)
    ctx, o, N = setup_pair(d, "fp64")
    Q0 = initial_state(d, N)
    T = 50 * o.cfl_dt(Q0, 0.4)                                # 10 to 16 adaptive steps
    Qg, sg = ctx.integrate_tsit5(Q0, 0.0, T)
    Qo, so = o.tsit5(Q0, 0.0, T, nthreads=4)
    assert sg == so
    assert block_err(Qg, Qo, N) <= 1e-10


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("name", CASES)
def test_adaptive_tsit5_reaches_reference_final_state(name, precision):
    """The reference ran these cases with Tsit5 (abstol 1e-6, reltol 1e-3);
    the device run at the same tolerances lands within 2e-3 of scale of its
    final state -- twice the runs' relative tolerance: the two adaptive runs
    take different steps, and an FP32C run's steps follow its rounding --
    with step counts within 5% of the oracle's."""
    d = load_fixture(name)
    ctx, o, N = setup_pair(d, precision)
    Q0 = initial_state(d, N)
    T = float(d["tspan"][1])
    Qg, (acc, _, _) = ctx.integrate_tsit5(Q0, 0.0, T, abstol=1e-6, reltol=1e-3)
    _, (acc_o, _, _) = o.tsit5(Q0, 0.0, T, abstol=1e-6, reltol=1e-3, nthreads=4)
    assert abs(acc - acc_o) <= max(2, acc_o // 20)
    ref = truth(d, N)
    scale = max(np.abs(ref[:N]).max(), np.abs(ref[N:]).max())
    assert np.abs(Qg - ref).max() <= 2e-3 * scale


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_tsit5_saveat(precision):
    """Save times are stepped onto: with fixed steps the state saved at T/2
    is the oracle's run from 0 to T/2; the last save is the final state."""
    d = load_fixture("fwd_bump")
    ctx, o, N = setup_pair(d, precision)
    Q0 = initial_state(d, N)
    T = float(d["tspan"][1])
    dt = T / 4000
    Qg, _, saves = ctx.integrate_tsit5(Q0, 0.0, T, dt0=dt, adaptive=False, saveat=[0.5 * T, T])
    np.testing.assert_array_equal(saves[1], Qg)
    Qh, _ = o.tsit5(Q0, 0.0, 0.5 * T, dt0=dt, adaptive=False, nthreads=4)
    assert block_err(saves[0], Qh, N) <= STATE_TOL[precision]
    # adaptive: the saved states sit at the requested times
    Qa, _, sa = ctx.integrate_tsit5(Q0, 0.0, T, saveat=[0.25 * T, T])
    np.testing.assert_array_equal(sa[1], Qa)
    ref = truth(d, N)
    assert np.abs(sa[0] - ref).max() > 10 * np.abs(Qa - ref).max()   # mid-run, not yet near the final state


def test_tsit5_argument_errors():
    d = load_fixture("fwd_bump")
    ctx, _, N = setup_pair(d, "fp64")
    Q0 = initial_state(d, N)
    with pytest.raises(HgError):
        ctx.integrate_tsit5(Q0, 1.0, 1.0)                       # empty time span
    with pytest.raises(HgError):
        ctx.integrate_tsit5(Q0, 0.0, 10.0, saveat=[5.0, 2.0])   # save times must ascend
    with pytest.raises(HgError):
        ctx.integrate_tsit5(Q0, 0.0, 10.0, saveat=[11.0])       # outside (t0, t1]
    with pytest.raises(HgError, match="dt0"):
        ctx.integrate_tsit5(Q0, 0.0, 10.0, adaptive=False)      # fixed steps need dt0
    with pytest.raises(HgError, match="max_steps"):
        ctx.integrate_tsit5(Q0, 0.0, 100.0, max_steps=3)
    # the context stays usable after the errors
    Q, (acc, _, _) = ctx.integrate_tsit5(Q0, 0.0, 1.0)
    assert acc > 0 and np.isfinite(Q).all()
