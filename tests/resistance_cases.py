"""Helpers for the state-dependent resistance tests (tests only): seeded UDE
networks in Lux's flattened parameter order and the truth state of a fixture."""
import numpy as np


def ude_param_count(in_dim, hidden):
    n, din = 0, in_dim
    for w in hidden:
        n += w * din + 3 * w
        din = w
    return n + din + 1


def ude_params(in_dim, hidden, seed):
    """Glorot-uniform weights, small random biases and LayerNorm affine terms
    (a trained network's, not an initial one's, so that every term matters)."""
    rng = np.random.default_rng(seed)
    out, din = [], in_dim
    for w in hidden:
        lim = np.sqrt(6.0 / (din + w))
        out += [rng.uniform(-lim, lim, w * din), rng.uniform(-0.2, 0.2, w),
                rng.uniform(0.5, 1.5, w), rng.uniform(-0.3, 0.3, w)]
        din = w
    lim = np.sqrt(6.0 / (din + 1))
    out += [rng.uniform(-lim, lim, din), rng.uniform(-0.2, 0.2, 1)]
    return np.concatenate(out)


def truth_state(d):
    h = d["h_truth"]
    return np.concatenate([d["xi_truth"], d["u_truth"] * (h + 1e-3), d["v_truth"] * (h + 1e-3)])


# (choice, kind, in_dim, bounds) of the three UDE closures, with the bounds of
# the reference's example run-control files
UDE_CASES = [
    ("ManningN_h", 5, 1, dict(output_bounds=(0.03, 0.06), h_bounds=(0.1, 0.5))),
    ("ManningN_h_Umag_ks", 6, 3, dict(output_bounds=(0.02, 0.08), h_bounds=(0.0, 3.0), u_bounds=(0.0, 2.0),
                                      ks_bounds=(0.0, 0.5))),
    ("FlowResistance", 7, 2, dict(output_bounds=(0.0, 0.03), h_bounds=(0.1, 0.5), u_bounds=(0.0, 1.0))),
]
