"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute calls; runs without a GPU)."""
import ctypes
import glob
import os
import re

import pytest

from hydrograd_gb import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*int\s+(hg_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "hg_create" in names and "hg_rhs" in names and "hg_loss_and_grad" in names


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header():
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_abi_version():
    assert _lib.lib().hg_abi_version() == 1


def test_create_without_device_fails_loudly():
    """No CPU fallback: on a machine without a GPU hg_create must fail."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from hydrograd_gb import SWE2D, HgError
    from hydrograd_gb.workloads import dam_break
    with pytest.raises(HgError) as e:
        SWE2D(dam_break(8, 4, 4.0, 2.0))
    assert e.value.code == 4


def test_setters_reject_a_null_context():
    """Argument checks on the host, before any device work: a null context is
    HG_ERR_ARG (1), also for hg_set_dt_min."""
    L = _lib.lib()
    assert L.hg_set_dt_min(None, 0.001) == 1
    assert L.hg_set_riemann_solver(None, 0) == 1
