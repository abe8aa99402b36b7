"""Loads libhydrograd_gb.so (the C ABI declared in include/hydrograd_gb.h).

There is no fallback: if the shared library is missing or fails to load, every
entry point raises.  Build it with ``python hydrograd.jl_gb300/build.py`` (or
``__graft_entry__.build()``).
"""
import ctypes
import os

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "build", "libhydrograd_gb.so")

HG_OK = 0
HG_FP64 = 0
HG_FP32C = 1
HG_ORDER_NONE, HG_ORDER_RCM, HG_ORDER_HILBERT = 0, 1, 2
BC_NONE, BC_WALL, BC_SYMM, BC_INLETQ, BC_EXITH = -1, 0, 1, 2, 3
# hg_resistance
RES_CONSTANT, RES_POWER_LAW, RES_SIGMOID, RES_INVERSE, RES_H_UMAG_KS = 0, 1, 2, 3, 4
RES_UDE_MANNING_H, RES_UDE_MANNING_H_UMAG_KS, RES_UDE_FLOW_RESISTANCE = 5, 6, 7
# hg_activation
ACTIVATIONS = {"relu": 0, "leakyrelu": 1, "sigmoid": 2, "tanh": 3, "softplus": 4}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p


class HgMeshDesc(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int32), ("node_x", _dp), ("node_y", _dp), ("node_z", _dp),
                ("n_cells", ctypes.c_int32), ("cell_node_count", _ip), ("cell_nodes", _ip),
                ("n_strings", ctypes.c_int32), ("string_ids", _ip), ("string_offsets", _ip),
                ("string_nodes", _ip), ("string_bc", _ip)]


class HgEnsembleDesc(ctypes.Structure):
    _fields_ = [("n_meshes", ctypes.c_int32), ("meshes", ctypes.POINTER(HgMeshDesc)),
                ("n_members", ctypes.c_int32), ("member_mesh", _ip)]


class HgUdeDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("n_hidden", ctypes.c_int32), ("hidden", _ip), ("activation", _ip),
                ("params", _dp), ("n_params", ctypes.c_int32), ("output_bounds", ctypes.c_double * 2),
                ("h_bounds", ctypes.c_double * 2), ("u_bounds", ctypes.c_double * 2),
                ("ks_bounds", ctypes.c_double * 2), ("ks_cells", _dp), ("layernorm_over_batch", ctypes.c_int32)]


class HgFinalObs(ctypes.Structure):
    _fields_ = [("wse", _dp), ("u", _dp), ("v", _dp), ("zb_wse", _dp)]


class HgConsts(ctypes.Structure):
    _fields_ = [("g", ctypes.c_double), ("k_n", ctypes.c_double), ("h_small", ctypes.c_double),
                ("riemann", ctypes.c_int32), ("order", ctypes.c_int32)]


# name -> argtypes (all return int status)
SIGNATURES = {
    "hg_abi_version": [],
    "hg_last_error": [_vp, ctypes.c_char_p, ctypes.c_int32],
    "hg_mesh_build": [ctypes.POINTER(HgMeshDesc), ctypes.POINTER(_vp)],
    "hg_mesh_free": [_vp],
    "hg_mesh_sizes": [_vp, _ip],
    "hg_mesh_cell_faces": [_vp, _ip, _dp, _dp, _dp, _dp],
    "hg_mesh_order": [_vp, ctypes.c_int32, _ip],
    "hg_create": [ctypes.POINTER(HgMeshDesc), ctypes.POINTER(HgConsts), ctypes.c_int32, ctypes.c_int32,
                  ctypes.POINTER(_vp)],
    "hg_ensemble_create": [ctypes.POINTER(HgEnsembleDesc), ctypes.POINTER(HgConsts), ctypes.c_int32, ctypes.c_int32,
                           ctypes.POINTER(_vp)],
    "hg_ensemble_layout": [_vp, _ip, _ip, _ip, _ip],
    "hg_ensemble_steps": [_vp, ctypes.c_int32, _dp, _dp],
    "hg_destroy": [_vp],
    "hg_sizes": [_vp, _ip],
    "hg_set_still_water": [_vp, _dp],
    "hg_set_manning_zones": [_vp, _ip, ctypes.c_int32, _dp],
    "hg_set_manning_cells": [_vp, _dp],
    "hg_set_zb_cells": [_vp, _dp],
    "hg_set_inlet_hydrograph": [_vp, ctypes.c_int32, ctypes.c_int32, _dp, _dp],
    "hg_set_manning_function": [_vp, ctypes.c_int32, _dp, ctypes.c_int32, _dp],
    "hg_set_ude": [_vp, ctypes.POINTER(HgUdeDesc)],
    "hg_resistance_grad": [_vp, _dp],
    "hg_ude_grad": [_vp, _dp, ctypes.c_int64],
    "hg_set_inlet_q": [_vp, _dp, ctypes.c_int32],
    "hg_set_exit_wse": [_vp, _dp, ctypes.c_int32],
    "hg_get_bed": [_vp, _dp, _dp, _dp, _dp],
    "hg_rhs": [_vp, _dp, ctypes.c_double, _dp],
    "hg_check_initial_state": [_vp, _dp],
    "hg_integrate": [_vp, _dp, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                     ctypes.c_int32, _dp, _dp],
    "hg_integrate_tsit5": [_vp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                           ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _dp, _dp, _ip],
    "hg_tsit5_tableau": [_dp, _dp, _dp, _dp],
    "hg_state_upload": [_vp, _dp],
    "hg_state_download": [_vp, _dp],
    "hg_advance": [_vp, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_int32],
    "hg_synchronize": [_vp],
    "hg_elapsed_time": [_vp, _dp],
    "hg_final_loss_and_grad": [_vp, _dp, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.POINTER(HgFinalObs),
                               _dp, _dp, _dp, _dp, _dp],
    "hg_loss_and_grad": [_vp, _dp, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, _ip, _dp, ctypes.c_int32, _dp,
                         _dp, _dp, _dp, _dp],
    "hg_launch_count": [_vp, ctypes.POINTER(ctypes.c_int64)],
    "hg_autotune": [_vp, ctypes.c_int32, _ip],
    "hg_autotune_info": [_vp, _ip, _ip, _ip],
    "hg_set_stage_family": [_vp, ctypes.c_int32],
    "hg_set_adjoint_tape": [_vp, ctypes.c_int64],
    "hg_set_riemann_solver": [_vp, ctypes.c_int32],
    "hg_set_dt_min": [_vp, ctypes.c_double],
    "hg_set_adjoint_integrator": [_vp, ctypes.c_int32],
    "hg_set_adjoint_steps": [_vp, _dp, ctypes.c_int32],
    "hg_tsit5_steps": [_vp, _dp, ctypes.c_int32, _ip],
    "hg_final_vjp": [_vp, _dp, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, _dp, _dp, _dp, _dp, _dp],
    "hg_time_stage_kernel": [_vp, ctypes.c_int32, ctypes.c_int32, _dp],
    "hg_time_vjp_kernel": [_vp, ctypes.c_int32, ctypes.c_int32, _dp],
    "hg_flush_l2": [_vp],
    "hg_advance_timed": [_vp, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_int32, _dp],
    "hg_rhs_device_noalloc": [_vp, _vp, _vp, _vp, _vp],
    "hg_pinned_alloc": [ctypes.c_int64, ctypes.POINTER(_vp)],
    "hg_pinned_free": [_vp],
}

_lib = None


class HgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"hydrograd_gb error {code}: {msg}")
        self.code = code


def lib():
    """The loaded library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise HgError(-1, f"{LIB_PATH} not found: build it with hydrograd.jl_gb300/build.py "
                              "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = L
    return _lib


def last_error(ctx=None):
    buf = ctypes.create_string_buffer(1024)
    lib().hg_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, ctx=None):
    if rc != HG_OK:
        raise HgError(rc, last_error(ctx))
    return rc
