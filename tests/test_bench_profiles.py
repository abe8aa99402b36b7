"""The committed ncu summaries bench.py reads for its roofline `traffic`
(per-cell DRAM bytes of one launch): each exists under profiles/, names the
command that made it, and gives a per-cell figure near the kernel's
algorithmic bytes (within 2x either way: well above means re-reads, well below
a capture of another kernel)."""
import os

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (summary, algorithmic bytes per cell at the 1M-cell reach's 1.5014 faces per cell)
FP32C_STAGE = 72 + 1.5014 * 20
CASES = [(bench.STAGE_KERNELS[k][1], FP32C_STAGE) for k in bench.STAGE_KERNELS if bench.STAGE_KERNELS[k][1]]
CASES += [("k_stage_f32_t128_river_tri_1M.md", FP32C_STAGE),
          (bench.VJP_PROFILE, 120 + 1.5014 * 32)]


@pytest.mark.parametrize("name,algorithmic", CASES, ids=[c[0] for c in CASES])
def test_profile_summary_gives_the_traffic(name, algorithmic):
    path = os.path.join(ROOT, "profiles", name)
    assert os.path.exists(path), name
    text = open(path).read()
    assert "ncu" in text and "--clock-control none" in text   # the command that made it
    b = bench.profile_traffic("fp32c", name=name)
    assert b is not None
    assert 0.5 * algorithmic <= b <= 2.0 * algorithmic


def test_fp64_stage_summary_gives_the_traffic():
    b = bench.profile_traffic("fp64")
    assert b is not None and 72 <= b <= 2 * (96 + 1.5014 * 32)
