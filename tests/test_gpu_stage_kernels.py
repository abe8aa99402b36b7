"""The autotuner's candidates (hg_autotune): within a family every kernel and
shape computes the same results, and the choice is cached per mesh and GPU.

Each candidate is forced in a child process (HG_STAGE_KERNEL, HG_STAGE_VARIANT,
HG_STAGE_FAMILY, read once per process) and the states after graph-captured CFL
steps and hg_integrate steps are compared bit for bit:
  family 0 (gather): gather in its four shapes (256-cell blocks with the
                     register budget of 4 and 3 blocks per SM, 512-cell blocks,
                     128-cell blocks), pipe, tma, and the autotuned default
                     (the family of a new context);
  family 1 (face):   face with both budgets, and the family's autotuned choice.
Unfused steps take a fixed kernel (pipe where it can run, so runs
reproduce); their gather instance agrees within 1e-6.  hg_autotune leaves the
resident state as it was; a second context on the same mesh takes the cached
choice without timing the candidates (hg_autotune_info's source)."""
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
sys.path.insert(0, %(pkg)r)
import numpy as np
from hydrograd_gb import SWE2D
from hydrograd_gb.workloads import river_triangles
def ctx_for(case):
    c = SWE2D(case, precision="fp32c")
    c.set_still_water(case["wstill"]); c.set_manning_zones(case["mat_id"], case["manning_zones"])
    c.set_inlet_q(case["inlet_q"]); c.set_exit_wse(case["exit_wse"])
    return c
case = river_triangles(n=120)
c = ctx_for(case)
c.upload(case["Q0"]); c.advance(150, cfl=0.4, graph=True); a = c.download()
b, _ = c.integrate(case["Q0"], 80, cfl=0.4)
info = c.autotune_info()
# unfused steps (a state-dependent n makes every stage a plain launch)
c.set_manning_function("inverse", (0.03, 0.05, 2.0))
u, _ = c.integrate(case["Q0"], 60, cfl=0.4)
h = lambda v: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()
np.save(sys.argv[1], u)
print(json.dumps({"advance": h(a), "integrate": h(b), "unfused": h(u), "kernel": info[0], "variant": info[1],
                  "source": info[2]}))
"""


def run_child(tag, env_extra, tmp_path):
    env = dict(os.environ)
    for k in ("HG_STAGE_KERNEL", "HG_STAGE_VARIANT", "HG_STAGE_FAMILY"):
        env.pop(k, None)
    env["HG_AUTOTUNE_CACHE"] = str(tmp_path / ("cache_%s.json" % tag))
    env.update(env_extra)
    code = CHILD % {"pkg": os.path.join(ROOT, "hydrograd.jl_gb300")}
    f = str(tmp_path / ("u_%s.npy" % tag))
    r = subprocess.run([sys.executable, "-c", code, f], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    out["u"] = np.load(f)
    return out


def test_gather_family_candidates_give_identical_states(tmp_path):
    runs = {
        "gather0": run_child("g0", {"HG_STAGE_KERNEL": "gather", "HG_STAGE_VARIANT": "0"}, tmp_path),
        "gather1": run_child("g1", {"HG_STAGE_KERNEL": "gather", "HG_STAGE_VARIANT": "1"}, tmp_path),
        "gather512": run_child("g2", {"HG_STAGE_KERNEL": "gather", "HG_STAGE_VARIANT": "2"}, tmp_path),
        "gather128": run_child("g3", {"HG_STAGE_KERNEL": "gather", "HG_STAGE_VARIANT": "3"}, tmp_path),
        "pipe": run_child("p", {"HG_STAGE_KERNEL": "pipe"}, tmp_path),
        "tma": run_child("t", {"HG_STAGE_KERNEL": "tma"}, tmp_path),
        "tuned": run_child("d", {}, tmp_path),
    }
    assert runs["pipe"]["kernel"] == 1 and runs["tma"]["kernel"] == 2 and runs["gather1"]["variant"] == 1
    assert runs["gather512"]["variant"] == 2 and runs["gather128"]["variant"] == 3
    assert runs["tuned"]["kernel"] in (0, 1, 2) and runs["tuned"]["source"] == 1
    for k, r in runs.items():
        assert r["advance"] == runs["gather0"]["advance"], k
        assert r["integrate"] == runs["gather0"]["integrate"], k
    # unfused: the tuned run takes the pipelined kernel, as a forced one
    assert runs["tuned"]["unfused"] == runs["pipe"]["unfused"]
    u, g = runs["pipe"]["u"], runs["gather0"]["u"]
    assert np.abs(u - g).max() <= 1e-6 * np.abs(g).max()


def test_face_family_candidates_give_identical_states(tmp_path):
    runs = {
        "face0": run_child("f0", {"HG_STAGE_KERNEL": "face", "HG_STAGE_VARIANT": "0"}, tmp_path),
        "face1": run_child("f1", {"HG_STAGE_KERNEL": "face", "HG_STAGE_VARIANT": "1"}, tmp_path),
        "tuned": run_child("fd", {"HG_STAGE_FAMILY": "face"}, tmp_path),
    }
    assert runs["tuned"]["kernel"] == 3 and runs["tuned"]["source"] == 1
    for k, r in runs.items():
        assert r["advance"] == runs["face0"]["advance"], k
        assert r["integrate"] == runs["face0"]["integrate"], k


def test_cached_choice_is_reused_without_timing(tmp_path, monkeypatch):
    cache = tmp_path / "autotune.json"
    monkeypatch.setenv("HG_AUTOTUNE_CACHE", str(cache))
    sys.path.insert(0, os.path.join(ROOT, "hydrograd.jl_gb300"))
    from hydrograd_gb import SWE2D
    from hydrograd_gb.workloads import river_triangles

    def ctx_for(case):
        c = SWE2D(case, precision="fp32c")
        c.set_still_water(case["wstill"])
        c.set_manning_zones(case["mat_id"], case["manning_zones"])
        c.set_inlet_q(case["inlet_q"])
        c.set_exit_wse(case["exit_wse"])
        return c

    case = river_triangles(n=100)
    a = ctx_for(case)
    a.upload(case["Q0"])
    a.advance(4, cfl=0.4)
    ka, va, sa = a.autotune_info()
    assert sa == 1 and cache.exists()
    entries = json.load(open(cache))["entries"]
    assert len(entries) == 1 and list(entries.values())[0]["kernel"] == ka
    b = ctx_for(case)
    b.upload(case["Q0"])
    l0 = b.launch_count()
    b.advance(4, cfl=0.4, graph=False)
    kb, vb, sb = b.autotune_info()
    assert (kb, vb, sb) == (ka, va, 2)
    # no candidate timing: the steps' own launches only (prime 3 + 2 per step)
    assert b.launch_count() - l0 <= 3 + 2 * 4
    # another mesh is another key
    other = river_triangles(n=90)
    c = ctx_for(other)
    c.upload(other["Q0"])
    c.advance(2, cfl=0.4)
    assert c.autotune_info()[2] == 1
    assert len(json.load(open(cache))["entries"]) == 2


def test_autotune_keeps_the_state():
    sys.path.insert(0, os.path.join(ROOT, "hydrograd.jl_gb300"))
    from hydrograd_gb import SWE2D
    from hydrograd_gb.workloads import river_triangles
    case = river_triangles(n=120)
    c = SWE2D(case, precision="fp32c")
    c.set_still_water(case["wstill"])
    c.set_manning_zones(case["mat_id"], case["manning_zones"])
    c.set_inlet_q(case["inlet_q"])
    c.set_exit_wse(case["exit_wse"])
    c.upload(case["Q0"])
    c.advance(20, cfl=0.4)
    before = c.download()
    k = c.autotune(2)
    assert k in (0, 1, 2, 3)
    np.testing.assert_array_equal(c.download(), before)
    c.advance(20, cfl=0.4)   # and the context steps on
    assert np.isfinite(c.download()).all()
