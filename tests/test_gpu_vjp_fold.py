"""The FP32C reverse sweep with the boundary faces folded into the pipelined
interior VJP (their flux Jacobians formed once per checkpoint segment,
k_bnd_jac_f32) against the separate boundary + combine kernels
(HG_VJP_FOLD=0, read once per process): the same loss, gradients within FP32
rounding of each other (1e-5 of each field's scale), and the folded sweep
reproducing its own bits run to run."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, %(pkg)r)
import numpy as np
from hydrograd_gb import SWE2D
from hydrograd_gb.workloads import river_triangles, probes_and_perturbation
case = river_triangles(n=%(n)d)
c = SWE2D(case, precision="fp32c")
c.set_still_water(case["wstill"]); c.set_manning_zones(case["mat_id"], case["manning_zones"])
c.set_inlet_q(case["inlet_q"]); c.set_exit_wse(case["exit_wse"])
c.set_adjoint_tape(0)   # segments of exactly ckpt_every steps
dt = 0.5 * c.integrate(case["Q0"], 1, cfl=0.4)[1][0]
probes, _ = probes_and_perturbation(case, 48)
K = 30
obs = np.tile(case["Q0"][probes] + 0.01, (K, 1))
out = {}
for ck in (7, 50):   # several segments (recomputed states), and one
    r = c.loss_and_grad(case["Q0"], K, dt, probes, obs, ckpt_every=ck)
    r2 = c.loss_and_grad(case["Q0"], K, dt, probes, obs, ckpt_every=ck)
    same = all(np.array_equal(r[k], r2[k]) for k in ("g_manning", "g_zb", "g_inletq")) and r["loss"] == r2["loss"]
    out[ck] = (r, same)
np.savez(sys.argv[1], **{"%%s_%%d" %% (k, ck): np.atleast_1d(v[0][k]) for ck, v in out.items()
                         for k in ("loss", "g_manning", "g_zb", "g_inletq")},
         same=np.array([out[7][1], out[50][1]]))
"""


def run(tmp_path, tag, env_extra, n=120):
    env = dict(os.environ)
    env.pop("HG_VJP_FOLD", None)
    env.update(env_extra)
    f = str(tmp_path / ("%s.npz" % tag))
    code = CHILD % {"pkg": os.path.join(ROOT, "hydrograd.jl_gb300"), "n": n}
    r = subprocess.run([sys.executable, "-c", code, f], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return dict(np.load(f))


def test_folded_boundary_vjp_matches_separate_kernels(tmp_path):
    fold = run(tmp_path, "fold", {})
    sep = run(tmp_path, "sep", {"HG_VJP_FOLD": "0"})
    assert fold["same"].all() and sep["same"].all()
    for ck in (7, 50):
        assert fold["loss_%d" % ck][0] == sep["loss_%d" % ck][0]
        for k in ("g_manning", "g_zb", "g_inletq"):
            a, b = fold["%s_%d" % (k, ck)], sep["%s_%d" % (k, ck)]
            assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max(), (k, ck)
    # the segment length does not change the gradients (recomputation repeats the forward pass)
    for k in ("g_manning", "g_zb", "g_inletq"):
        np.testing.assert_array_equal(fold["%s_7" % k], fold["%s_50" % k])
