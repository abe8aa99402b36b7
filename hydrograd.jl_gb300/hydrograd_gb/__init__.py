"""GB300-native shallow-water RHS, time stepping and adjoint for Hydrograd.jl's hot path.

The compute path is libhydrograd_gb.so (hand-written sm_103a CUDA kernels
behind the C ABI in include/hydrograd_gb.h).  This package is the Python host
mirror of the reference's ODE-RHS / parameter interface plus the synthetic
workload generators used by the tests and the benchmark.
"""
from ._lib import HgError, lib  # noqa: F401
from .swe2d import (HostMesh, MeshDesc, PinnedBuffer, SWE2D, SWE2DEnsemble, SWE2DExtraParameters,  # noqa: F401
                    custom_ODE_solve,
                    swe_2d_rhs)
