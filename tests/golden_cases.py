"""Helpers to open the golden fixtures (tests only)."""
import os

import numpy as np

from oracle.oracle import Oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_fixture(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def load_case(name):
    """Oracle set up as solve_swe_2D.jl:148-221 does for the case."""
    d = load_fixture(name)
    o = Oracle(d)
    o.set_manning_cells(d["manning_zones"][d["mat_id"]])
    o.set_wstill(still_water(d, o.n_cells))
    o.set_inlet_q(d["inlet_q"])
    o.set_exit_wse(d["exit_wse"])
    return d, o


def still_water(d, N):
    if "ic_const" in d:
        return np.full(N, float(d["ic_const"][1]))
    return np.asarray(d["ic_wstill"], float)


def initial_state(d, N):
    """Q0 = [xi; q_x; q_y] with xi = wse - wstill (process_ICs_2D.jl:48-87)."""
    if "ic_const" in d:
        wse, wstill, qx, qy = (float(v) for v in d["ic_const"])
        return np.concatenate([np.full(N, wse - wstill), np.full(N, qx), np.full(N, qy)])
    return np.concatenate([d["ic_wse"] - d["ic_wstill"], d["ic_qx"], d["ic_qy"]])
