"""The face-once FP32C stage kernel (k_stage_face_f32).

It evaluates each wet-wet face once (its two cells' terms from one flux) where
the gather kernels evaluate it from each side, so its results differ from
theirs in the last bits; it is checked like the FP32C path itself: against the
FP64 oracle within 1e-5 per state block (test_gpu_forward.py's measure), at
moving wet/dry fronts, with the HLL solver, and bit for bit between runs.
Each check runs in a child process with HG_STAGE_KERNEL=face (read once per
process)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import hashlib, json, sys
sys.path.insert(0, %(root)r); sys.path.insert(0, %(pkg)r)
import numpy as np
from hydrograd_gb import SWE2D
from hydrograd_gb.workloads import river_triangles
from oracle.oracle import Oracle
def pair(case, solver="Roe"):
    c = SWE2D(case, precision="fp32c")
    o = Oracle(case)
    c.set_still_water(case["wstill"]); o.set_wstill(case["wstill"])
    c.set_manning_zones(case["mat_id"], case["manning_zones"]); o.set_manning_cells(case["manning_zones"][case["mat_id"]])
    c.set_inlet_q(case["inlet_q"]); o.set_inlet_q(case["inlet_q"])
    c.set_exit_wse(case["exit_wse"]); o.set_exit_wse(case["exit_wse"])
    c.set_riemann_solver(solver); o.set_riemann_solver(solver)
    return c, o
def block_err(a, b, N):
    return max(float(np.abs(a[k*N:(k+1)*N] - b[k*N:(k+1)*N]).max()
                     / max(np.abs(b[k*N:(k+1)*N]).max(), 1e-3 * np.abs(b).max())) for k in range(3))
out = {}
case = river_triangles(n=64)
N = len(case["cell_node_count"])
for solver in ("Roe", "HLL"):
    c, o = pair(case, solver)
    Q, dts = c.integrate(case["Q0"], 300, cfl=0.4)
    ref = case["Q0"].copy()
    for d in dts:
        ref = o.rk2(ref, 1, dt=float(d), nthreads=8)
    out["wet_" + solver] = block_err(Q, ref, N)
    out["kernel_" + solver] = c.autotune(0)
    c.upload(case["Q0"]); c.advance(120, cfl=0.4, graph=True); a = c.download()
    c.upload(case["Q0"]); c.advance(120, cfl=0.4, graph=True); b = c.download()
    out["repeat_" + solver] = bool(np.array_equal(a, b))
    out["hash_" + solver] = hashlib.sha256(a.tobytes()).hexdigest()
dry = river_triangles(n=64, dry_land=True)
N = len(dry["cell_node_count"])
c, o = pair(dry)
dt = o.cfl_dt(dry["Q0"], 0.01)
Q, _ = c.integrate(dry["Q0"], 300, dt=dt)
out["dry"] = block_err(Q, o.rk2(dry["Q0"], 300, dt=dt, nthreads=8), N)
print(json.dumps(out))
"""


_RUNS = {}


def _run(kernel):
    if kernel in _RUNS:
        return _RUNS[kernel]
    env = dict(os.environ)
    env["HG_STAGE_KERNEL"] = kernel
    code = CHILD % {"root": ROOT, "pkg": os.path.join(ROOT, "hydrograd.jl_gb300")}
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    _RUNS[kernel] = json.loads(r.stdout.strip().splitlines()[-1])
    return _RUNS[kernel]


@pytest.fixture(scope="module")
def face_run():
    return _run("face")


def test_face_kernel_is_the_one_running(face_run):
    assert face_run["kernel_Roe"] == 3 and face_run["kernel_HLL"] == 3


@pytest.mark.parametrize("solver", ["Roe", "HLL"])
def test_face_kernel_within_1e5_of_fp64_oracle(face_run, solver):
    assert face_run["wet_" + solver] <= 1e-5


def test_face_kernel_at_wet_dry_fronts(face_run):
    assert face_run["dry"] <= 1e-5


@pytest.mark.parametrize("solver", ["Roe", "HLL"])
def test_face_kernel_is_bit_reproducible(face_run, solver):
    assert face_run["repeat_" + solver]
