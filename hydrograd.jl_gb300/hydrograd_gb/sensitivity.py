"""Sensitivity of the final state to the zone Manning n -- what the
reference's sensitivity analysis computes with ForwardDiff.jacobian
(src/applications/sensitivity_analysis/swe_2D_sensitivity.jl): the Jacobian
dQ_K / dn_zone of the state after nsteps SSP-RK2 steps of dt, 3n x n_zones,
flattened column-major as sensitivity_results.json holds it.

Each row is one vector-Jacobian product on the device (hg_final_vjp with a unit
cotangent; the per-cell n gradient summed over each zone's cells), so a full
Jacobian costs 3n adjoint runs: sized for the reference's example meshes
(hundreds to a few thousand cells).  rows restricts it to some state entries.
"""
import numpy as np


def zone_manning_jacobian(ctx, Q0, nsteps, dt, mat_id, n_zones, rows=None, ckpt_every=50):
    """J[r, z] = d Q_K[r] / d n_z for the state entries r (default: all 3 n)."""
    N = ctx.n_cells
    mat_id = np.asarray(mat_id)
    rows = np.arange(3 * N) if rows is None else np.asarray(rows)
    J = np.zeros((len(rows), n_zones))
    lam = np.zeros(3 * N)
    for i, r in enumerate(rows):
        lam[r] = 1.0
        g = ctx.final_state_vjp(Q0, nsteps, dt, lam, ckpt_every=ckpt_every, want=("manning",))["g_manning"]
        J[i] = np.bincount(mat_id, g, minlength=n_zones)
        lam[r] = 0.0
    return J


def flatten_like_reference(J):
    """ForwardDiff.jacobian's matrix flattened column-major (vec(J) in Julia)."""
    return np.asarray(J).flatten(order="F")
