"""Host-side mirror of Hydrograd.jl's ODE-RHS / parameter interface over the C ABI.

Hydrograd builds ``ODEFunction((u, p, t) -> swe_2d_rhs(du, u, p, t, swe_extra_params))``
(src/applications/solve_swe_2D.jl:281-307) and hands it to SciML or to its own
Euler loop.  This module gives the same shapes over libhydrograd_gb.so:

* :class:`SWE2D` -- one device context: mesh, boundary conditions, parameters
  and state buffers (what ``SWE2D_Extra_Parameters`` holds,
  src/applications/application_commons.jl:7-44).
* :func:`swe_2d_rhs` -- ``swe_2d_rhs(dQdt, Q, params_vector, t, p_extra)`` with
  the reference's active-parameter injection (semi_discretize_swe_2D.jl:112-199).
* :func:`custom_ODE_solve` -- the reference's forward-Euler loop
  (src/ode_solvers/custom_ODE_solvers.jl:36-95).

Every call goes to the CUDA library; a missing library raises (no fallback).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import HgConsts, HgEnsembleDesc, HgFinalObs, HgMeshDesc, HgUdeDesc, check, lib

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)

PRECISIONS = {"fp64": _lib.HG_FP64, "fp32c": _lib.HG_FP32C}
ORDERS = {"none": _lib.HG_ORDER_NONE, "rcm": _lib.HG_ORDER_RCM, "hilbert": _lib.HG_ORDER_HILBERT}


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


class MeshDesc:
    """hg_mesh_desc over numpy arrays kept alive by this object.

    ``case`` holds node_xyz [n,3], cell_nodes [n,8] (0-based, -1 padded),
    cell_node_count [n], string_ids, string_offsets, string_nodes, string_bc.
    """

    def __init__(self, case):
        xyz = np.asarray(case["node_xyz"], dtype=np.float64)
        self.x = np.ascontiguousarray(xyz[:, 0])
        self.y = np.ascontiguousarray(xyz[:, 1])
        self.z = np.ascontiguousarray(xyz[:, 2])
        self.cnt = np.ascontiguousarray(case["cell_node_count"], dtype=np.int32)
        self.cn = np.ascontiguousarray(case["cell_nodes"], dtype=np.int32)
        self.sid = np.ascontiguousarray(case.get("string_ids", np.zeros(0)), dtype=np.int32)
        self.soff = np.ascontiguousarray(case.get("string_offsets", np.zeros(1)), dtype=np.int32)
        self.snod = np.ascontiguousarray(case.get("string_nodes", np.zeros(0)), dtype=np.int32)
        self.sbc = np.ascontiguousarray(case.get("string_bc", np.zeros(0)), dtype=np.int32)
        if self.cn.shape != (len(self.cnt), 8):
            raise ValueError("cell_nodes must be [n_cells, 8]")
        self.desc = HgMeshDesc(len(self.x), _d(self.x), _d(self.y), _d(self.z), len(self.cnt), _i(self.cnt),
                               _i(self.cn), len(self.sid), _i(self.sid), _i(self.soff), _i(self.snod), _i(self.sbc))


class HostMesh:
    """Host-only mesh topology (hg_mesh_build): no device needed."""

    def __init__(self, case):
        self._desc = MeshDesc(case)
        h = ctypes.c_void_p()
        check(lib().hg_mesh_build(ctypes.byref(self._desc.desc), ctypes.byref(h)))
        self.h = h
        s = np.zeros(8, np.int32)
        check(lib().hg_mesh_sizes(self.h, _i(s)))
        (self.n_cells, self.n_faces, self.n_ghosts, self.n_inletq, self.n_exith, self.n_wall, self.n_symm,
         self.max_cell_faces) = map(int, s)

    def __del__(self):
        if getattr(self, "h", None):
            lib().hg_mesh_free(self.h)
            self.h = None

    def cell_faces(self):
        N = self.n_cells
        nbr = np.zeros(N * 8, np.int32)
        nrm = np.zeros(N * 16)
        ln = np.zeros(N * 8)
        ar = np.zeros(N)
        ce = np.zeros(N * 2)
        check(lib().hg_mesh_cell_faces(self.h, _i(nbr), _d(nrm), _d(ln), _d(ar), _d(ce)))
        return dict(nbr=nbr.reshape(N, 8), normals=nrm.reshape(N, 8, 2), lengths=ln.reshape(N, 8), areas=ar,
                    centroids=ce.reshape(N, 2))

    def order(self, order="hilbert"):
        p = np.zeros(self.n_cells, np.int32)
        check(lib().hg_mesh_order(self.h, ORDERS[order], _i(p)))
        return p


class SWE2D:
    """A device context: the compiled RHS with its mesh, BCs, parameters and state."""

    def __init__(self, case, precision="fp64", order="hilbert", g=9.81, k_n=1.0, h_small=1.0e-3, device=0):
        self._desc = MeshDesc(case)
        k = HgConsts(g, k_n, h_small, 0, ORDERS[order])
        h = ctypes.c_void_p()
        check(lib().hg_create(ctypes.byref(self._desc.desc), ctypes.byref(k), PRECISIONS[precision], device,
                              ctypes.byref(h)))
        self._init_handle(h, precision, h_small)

    def _init_handle(self, h, precision, h_small):
        self.h = h
        self.precision = precision
        s = np.zeros(8, np.int32)
        check(lib().hg_sizes(self.h, _i(s)), self.h)
        (self.n_cells, self.n_faces, self.n_ghosts, self.n_inletq, self.n_exith, self.n_wall, self.n_symm,
         self.max_cell_faces) = map(int, s)
        self.h_small = h_small

    def close(self):
        if getattr(self, "h", None):
            lib().hg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _chk(self, rc):
        return check(rc, self.h)

    # -- parameters ------------------------------------------------------------
    def set_still_water(self, wstill):
        w = np.ascontiguousarray(np.broadcast_to(np.asarray(wstill, np.float64), (self.n_cells,)))
        self._chk(lib().hg_set_still_water(self.h, _d(w)))

    def set_manning_zones(self, mat_id, n_zone):
        m = np.ascontiguousarray(mat_id, dtype=np.int32)
        z = np.ascontiguousarray(n_zone, dtype=np.float64)
        self._chk(lib().hg_set_manning_zones(self.h, _i(m), len(z), _d(z)))

    def set_manning_cells(self, n):
        self._chk(lib().hg_set_manning_cells(self.h, _d(np.ascontiguousarray(n, dtype=np.float64))))

    def set_zb_cells(self, zb):
        self._chk(lib().hg_set_zb_cells(self.h, _d(np.ascontiguousarray(zb, dtype=np.float64))))

    def set_inlet_hydrograph(self, group, t, q):
        """Time-varying discharge of inlet-Q boundary `group` (hg_set_inlet_hydrograph);
        empty t returns it to its set_inlet_q value."""
        t = np.ascontiguousarray(t, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        self._hydro = getattr(self, "_hydro", {})
        self._hydro[group] = (t, q)
        self._chk(lib().hg_set_inlet_hydrograph(self.h, int(group), len(t), _d(t) if len(t) else None,
                                                _d(q) if len(q) else None))

    def set_manning_function(self, kind, params=(), ks=None):
        """Manning's n as a function of the state (ManningN_option "variable",
        process_ManningN_2D.jl:102-213): kind "power_law" / "sigmoid" / "inverse"
        with params {n_lower, n_upper, k[, h_mid]}, or "h_Umag_ks" with ks per
        cell; "constant" returns to the cells' n."""
        kinds = {"constant": _lib.RES_CONSTANT, "power_law": _lib.RES_POWER_LAW, "sigmoid": _lib.RES_SIGMOID,
                 "inverse": _lib.RES_INVERSE, "h_Umag_ks": _lib.RES_H_UMAG_KS}
        k = kinds[kind] if isinstance(kind, str) else int(kind)
        if isinstance(params, dict):
            params = [params.get(n, 0.0) for n in ("n_lower", "n_upper", "k", "h_mid")]
        p = np.ascontiguousarray(params, dtype=np.float64)
        self._res_ks = None if ks is None else np.ascontiguousarray(ks, dtype=np.float64)
        self._ude_nparams = 0
        self._chk(lib().hg_set_manning_function(self.h, k, _d(p) if len(p) else None, len(p), _d(self._res_ks)))

    def resistance_grad(self):
        """dL/d{n_lower, n_upper, k, h_mid} of the state-dependent n function
        from the last gradient call (hg_resistance_grad)."""
        g = np.zeros(4)
        self._chk(lib().hg_resistance_grad(self.h, _d(g)))
        return g

    def ude_grad(self):
        """dL/dparams of the UDE network from the last gradient call, in the
        parameters' order (hg_ude_grad)."""
        g = np.zeros(getattr(self, "_ude_nparams", 0))
        self._chk(lib().hg_ude_grad(self.h, _d(g), len(g)))
        return g

    def set_ude(self, choice, hidden, activations, params, output_bounds, h_bounds, u_bounds=(0.0, 1.0),
                ks_bounds=(0.0, 1.0), ks=None, layernorm_over_batch=True):
        """A UDE closure in the RHS (process_ManningN_2D.jl:216-273,
        process_FlowResistance_UDE.jl:3-45): choice "ManningN_h",
        "ManningN_h_Umag_ks" or "FlowResistance"; the network of
        process_UDE.jl:3-56 with hidden widths, activation names and its
        parameters in Lux's flattened order (hg_ude_desc)."""
        kinds = {"ManningN_h": _lib.RES_UDE_MANNING_H, "ManningN_h_Umag_ks": _lib.RES_UDE_MANNING_H_UMAG_KS,
                 "FlowResistance": _lib.RES_UDE_FLOW_RESISTANCE}
        hid = np.ascontiguousarray(hidden, dtype=np.int32)
        act = np.ascontiguousarray([_lib.ACTIVATIONS[a] if isinstance(a, str) else a for a in activations],
                                   dtype=np.int32)
        prm = np.ascontiguousarray(params, dtype=np.float64)
        ks = None if ks is None else np.ascontiguousarray(ks, dtype=np.float64)
        self._ude_keep = (hid, act, prm, ks)
        self._ude_nparams = len(prm)
        pair = ctypes.c_double * 2
        d = HgUdeDesc(kinds[choice] if isinstance(choice, str) else int(choice), len(hid), _i(hid), _i(act), _d(prm),
                      len(prm), pair(*output_bounds), pair(*h_bounds), pair(*u_bounds), pair(*ks_bounds), _d(ks),
                      1 if layernorm_over_batch else 0)
        self._chk(lib().hg_set_ude(self.h, ctypes.byref(d)))

    def set_inlet_q(self, q):
        q = np.ascontiguousarray(np.atleast_1d(q), dtype=np.float64)
        self._chk(lib().hg_set_inlet_q(self.h, _d(q), len(q)))

    def set_exit_wse(self, w):
        w = np.ascontiguousarray(np.atleast_1d(w), dtype=np.float64)
        self._chk(lib().hg_set_exit_wse(self.h, _d(w), len(w)))

    def bed(self):
        N = self.n_cells
        zb, S0, man, hst = np.zeros(N), np.zeros(2 * N), np.zeros(N), np.zeros(N)
        self._chk(lib().hg_get_bed(self.h, _d(zb), _d(S0), _d(man), _d(hst)))
        return dict(zb=zb, S0=S0.reshape(N, 2), manning=man, hstill=hst)

    # -- forward -----------------------------------------------------------------
    def check_initial_state(self, Q):
        self._chk(lib().hg_check_initial_state(self.h, _d(np.ascontiguousarray(Q, dtype=np.float64))))

    def rhs(self, Q, t=0.0, out=None):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        if out is None:
            out = np.empty_like(Q)
        self._chk(lib().hg_rhs(self.h, _d(Q), float(t), _d(out)))
        return out

    def integrate(self, Q, nsteps, method="rk2", dt=None, cfl=0.4, save_every=0, inplace=False):
        """nsteps explicit steps from Q; returns (Q, dts[, saves]).  With
        inplace=True a C-contiguous float64 Q (e.g. a PinnedBuffer's array) is
        advanced where it lies, as hg_integrate does with its host buffer."""
        if inplace:
            if not (isinstance(Q, np.ndarray) and Q.dtype == np.float64 and Q.flags.c_contiguous and Q.flags.writeable):
                raise ValueError("inplace needs a writable C-contiguous float64 array")
        else:
            Q = np.array(Q, dtype=np.float64)
        dts = np.zeros(max(nsteps, 1))
        saves = np.zeros((nsteps // save_every, Q.size)) if save_every > 0 else None
        m = {"rk2": 0, "euler": 1}[method]
        self._chk(lib().hg_integrate(self.h, _d(Q), 0.0, int(nsteps), m, float(dt) if dt else -1.0, float(cfl),
                                     int(save_every), _d(saves), _d(dts)))
        if saves is not None:
            return Q, dts[:nsteps], saves
        return Q, dts[:nsteps]

    def integrate_tsit5(self, Q, t0, t1, abstol=1e-6, reltol=1e-3, dt0=None, adaptive=True, max_steps=0,
                        saveat=None):
        """Tsit5 (Tsitouras 5(4)) from t0 to t1 on the device, as
        solve(prob, Tsit5(); abstol, reltol, saveat) integrates the reference's
        ODE problem (adaptive=False: fixed steps of dt0).  Returns (Q, stats[,
        saves]) with stats = (accepted, rejected, RHS evaluations) and saves[i]
        the state at saveat[i]."""
        Q = np.array(Q, dtype=np.float64)
        ts = np.ascontiguousarray(saveat if saveat is not None else [], dtype=np.float64)
        saves = np.zeros((len(ts), Q.size)) if len(ts) else None
        st = np.zeros(3, dtype=np.int32)
        self._chk(lib().hg_integrate_tsit5(self.h, _d(Q), float(t0), float(t1), float(abstol), float(reltol),
                                           float(dt0) if dt0 else -1.0, 1 if adaptive else 0, int(max_steps), len(ts),
                                           _d(ts) if len(ts) else None, _d(saves), _i(st)))
        stats = tuple(int(v) for v in st)
        return (Q, stats, saves) if saves is not None else (Q, stats)

    def tsit5_steps(self):
        """hg_tsit5_steps: the step sizes the last integrate_tsit5 accepted."""
        cnt = np.zeros(1, dtype=np.int32)
        self._chk(lib().hg_tsit5_steps(self.h, None, 0, _i(cnt)))
        out = np.zeros(int(cnt[0]))
        if len(out):
            self._chk(lib().hg_tsit5_steps(self.h, _d(out), len(out), _i(cnt)))
        return out

    def set_adjoint_steps(self, dts=None):
        """hg_set_adjoint_steps: the step sizes the Tsit5 adjoint
        differentiates (e.g. tsit5_steps() of an adaptive run); None: steps of
        the gradient call's dt."""
        d = np.ascontiguousarray(dts if dts is not None else [], dtype=np.float64)
        self._chk(lib().hg_set_adjoint_steps(self.h, _d(d) if len(d) else None, len(d)))

    def upload(self, Q):
        self._chk(lib().hg_state_upload(self.h, _d(np.ascontiguousarray(Q, dtype=np.float64))))

    def download(self, out=None):
        if out is None:
            out = np.empty(3 * self.n_cells)
        self._chk(lib().hg_state_download(self.h, _d(out)))
        return out

    def advance(self, nsteps, dt=None, cfl=0.4, graph=True):
        self._chk(lib().hg_advance(self.h, int(nsteps), float(dt) if dt else -1.0, float(cfl), 1 if graph else 0))

    def advance_timed(self, nsteps, dt=None, cfl=0.4, flush_l2=True):
        """Device time (ms) of nsteps RK2 steps, each timed by CUDA events."""
        ms = np.zeros(1)
        self._chk(lib().hg_advance_timed(self.h, int(nsteps), float(dt) if dt else -1.0, float(cfl),
                                         1 if flush_l2 else 0, _d(ms)))
        return float(ms[0])

    def synchronize(self):
        self._chk(lib().hg_synchronize(self.h))

    def elapsed_time(self):
        t = np.zeros(1)
        self._chk(lib().hg_elapsed_time(self.h, _d(t)))
        return float(t[0])

    def launch_count(self):
        c = ctypes.c_int64()
        self._chk(lib().hg_launch_count(self.h, ctypes.byref(c)))
        return int(c.value)

    def autotune(self, reps=3):
        """hg_autotune: time the FP32C stage kernels of the context's family on
        the resident state and keep (and cache) the fastest; returns the kernel
        (0 gather, 1 pipe, 2 tma, 3 face).  reps=0 only reports the current one."""
        k = np.zeros(1, np.int32)
        self._chk(lib().hg_autotune(self.h, int(reps), _i(k)))
        return int(k[0])

    def autotune_info(self):
        """(kernel, variant, source) of the stage-kernel choice (hg_autotune_info;
        source 0 default, 1 timed, 2 cache file, 3 forced)."""
        v = np.zeros(3, np.int32)
        self._chk(lib().hg_autotune_info(self.h, _i(v[0:1]), _i(v[1:2]), _i(v[2:3])))
        return tuple(int(x) for x in v)

    def set_stage_family(self, family):
        """hg_set_stage_family: "gather" (gather / pipe / tma) or "face"."""
        self._chk(lib().hg_set_stage_family(self.h, {"gather": 0, "face": 1}[family]))

    def final_state_vjp(self, Q0, nsteps, dt, lam, ckpt_every=50, want=("manning", "zb", "inletq")):
        """hg_final_vjp: gradients of lam . Q_K (Q_K the state after nsteps
        SSP-RK2 steps of dt) w.r.t. the per-cell n, zb and the inlet Q."""
        N = self.n_cells
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        if lam.size != 3 * N:
            raise ValueError("lam: one value per state entry (3 n)")
        gn = np.zeros(N) if "manning" in want else None
        gz = np.zeros(N) if "zb" in want else None
        gq = np.zeros(max(self.n_inletq, 1)) if "inletq" in want else None
        Qf = np.zeros(3 * N)
        self._chk(lib().hg_final_vjp(self.h, _d(np.ascontiguousarray(Q0, dtype=np.float64)), int(nsteps), float(dt),
                                     int(ckpt_every), _d(lam), _d(gn), _d(gz), _d(gq), _d(Qf)))
        return dict(g_manning=gn, g_zb=gz, g_inletq=None if gq is None else gq[:self.n_inletq], Q=Qf)

    def set_riemann_solver(self, name):
        """hg_set_riemann_solver: "Roe" (the reference's, the default) or
        "HLL" (Harten-Lax-van Leer with Einfeldt's wave speeds); "HLLC" is
        refused (HgError), as the reference raises an error for it."""
        kinds = {"Roe": 0, "HLL": 1, "HLLC": 2}
        if name not in kinds:
            raise ValueError("Riemann solver: Roe, HLL or HLLC")
        self._chk(lib().hg_set_riemann_solver(self.h, kinds[name]))

    def set_dt_min(self, dt_min):
        """hg_set_dt_min: CFL steps below dt_min (default 0.001 s, the
        reference's swe_2D_consts.dt_min) make the stepping call raise HgError
        (HG_ERR_STATE); 0 turns the check off."""
        self._chk(lib().hg_set_dt_min(self.h, float(dt_min)))

    def set_adjoint_integrator(self, integrator):
        """hg_set_adjoint_integrator: the steps the gradient calls run and
        differentiate -- "ssprk2" (default) or "tsit5" (fixed Tsit5 steps of dt;
        an FP32C context runs them on FP32 vectors)."""
        code = {"ssprk2": 0, "tsit5": 1}[integrator]
        self._chk(lib().hg_set_adjoint_integrator(self.h, code))

    def set_adjoint_tape(self, nbytes=-1):
        """hg_set_adjoint_tape: memory for the adjoint's stage states.  -1 (the
        default): segments as long as fit in min(half the free device memory,
        a quarter of the device's), never shorter than ckpt_every; 0: exactly
        ckpt_every steps per segment; > 0: a budget in bytes.  The gradients
        do not depend on it.  Also frees the tape this context holds."""
        self._chk(lib().hg_set_adjoint_tape(self.h, int(nbytes)))

    def time_stage_kernel(self, n=10, flush_l2=True):
        ms = np.zeros(1)
        self._chk(lib().hg_time_stage_kernel(self.h, int(n), 1 if flush_l2 else 0, _d(ms)))
        return float(ms[0])

    def time_vjp_kernel(self, n=10, flush_l2=True):
        """Mean ms of the FP32C interior VJP kernel alone (hg_time_vjp_kernel)."""
        ms = np.zeros(1)
        self._chk(lib().hg_time_vjp_kernel(self.h, int(n), 1 if flush_l2 else 0, _d(ms)))
        return float(ms[0])

    def flush_l2(self):
        self._chk(lib().hg_flush_l2(self.h))

    # -- gradient ----------------------------------------------------------------
    def loss_and_grad(self, Q0, nsteps, dt, probes, obs, ckpt_every=50, want=("manning", "zb", "inletq")):
        N = self.n_cells
        Q0 = np.ascontiguousarray(Q0, dtype=np.float64)
        probes = np.ascontiguousarray(probes, dtype=np.int32)
        obs = np.ascontiguousarray(obs, dtype=np.float64)
        if obs.size != int(nsteps) * len(probes):   # the library reads nsteps x n_probe values
            raise ValueError("obs: one value per step and probe (%d x %d), got %d" % (nsteps, len(probes), obs.size))
        loss = np.zeros(1)
        gn = np.zeros(N) if "manning" in want else None
        gz = np.zeros(N) if "zb" in want else None
        gq = np.zeros(max(self.n_inletq, 1)) if "inletq" in want else None
        Qf = np.zeros(3 * N)
        self._chk(lib().hg_loss_and_grad(self.h, _d(Q0), int(nsteps), float(dt), int(ckpt_every), _i(probes),
                                         _d(obs), len(probes), _d(loss), _d(gn), _d(gz), _d(gq), _d(Qf)))
        return dict(loss=float(loss[0]), g_manning=gn, g_zb=gz, g_inletq=None if gq is None else gq[:self.n_inletq],
                    Q=Qf)

    def final_loss_and_grad(self, Q0, nsteps, dt, wse=None, u=None, v=None, zb_wse=None, ckpt_every=50,
                            want=("manning", "zb", "inletq")):
        """The final-state inversion loss of swe_2D_inversion.jl:383-431 (WSE and
        velocity misfits of the state after nsteps SSP-RK2 steps of dt) and its
        gradients (hg_final_loss_and_grad).  zb_wse None: WSE_pred = h + the
        context's zb (an active zb parameter; g_zb then has the direct term)."""
        N = self.n_cells
        arr = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        keep = [arr(a) for a in (wse, u, v, zb_wse)]
        obs = HgFinalObs(*(_d(a) for a in keep))
        parts = np.zeros(3)
        gn = np.zeros(N) if "manning" in want else None
        gz = np.zeros(N) if "zb" in want else None
        gq = np.zeros(max(self.n_inletq, 1)) if "inletq" in want else None
        Qf = np.zeros(3 * N)
        self._chk(lib().hg_final_loss_and_grad(self.h, _d(np.ascontiguousarray(Q0, dtype=np.float64)), int(nsteps),
                                               float(dt), int(ckpt_every), ctypes.byref(obs), _d(parts), _d(gn),
                                               _d(gz), _d(gq), _d(Qf)))
        return dict(loss=float(parts[0]), loss_wse=float(parts[1]), loss_uv=float(parts[2]), g_manning=gn, g_zb=gz,
                    g_inletq=None if gq is None else gq[:self.n_inletq], Q=Qf)


class PinnedBuffer:
    """Page-locked host array (float64) for timed host<->device copies."""

    def __init__(self, n):
        p = ctypes.c_void_p()
        check(lib().hg_pinned_alloc(int(n) * 8, ctypes.byref(p)))
        self.p = p
        self.array = np.ctypeslib.as_array(ctypes.cast(p, _dp), shape=(int(n),))

    def __del__(self):
        if getattr(self, "p", None):
            lib().hg_pinned_free(self.p)
            self.p = None


class SWE2DEnsemble(SWE2D):
    """Many independent problems stepped together (hg_ensemble_create).

    ``cases`` are mesh cases (as for :class:`SWE2D`); member m runs on
    ``cases[member_mesh[m]]``.  The members' cells, inlet-Q and exit-H
    boundaries are concatenated in member order (``cell_offset``,
    ``inlet_offset``, ``exit_offset``), and every :class:`SWE2D` call applies to
    the concatenation; :meth:`concat` and :meth:`split` convert between
    per-member arrays and the concatenated ones.
    """

    def __init__(self, cases, member_mesh, precision="fp64", order="hilbert", g=9.81, k_n=1.0, h_small=1.0e-3,
                 device=0):
        self._descs = [MeshDesc(c) for c in cases]
        arr = (HgMeshDesc * len(self._descs))(*[d.desc for d in self._descs])
        self._mm = np.ascontiguousarray(member_mesh, dtype=np.int32)
        e = HgEnsembleDesc(len(self._descs), arr, len(self._mm), _i(self._mm))
        self._arr = arr
        k = HgConsts(g, k_n, h_small, 0, ORDERS[order])
        h = ctypes.c_void_p()
        check(lib().hg_ensemble_create(ctypes.byref(e), ctypes.byref(k), PRECISIONS[precision], device,
                                       ctypes.byref(h)))
        self._init_handle(h, precision, h_small)
        nm = ctypes.c_int32()
        check(lib().hg_ensemble_layout(self.h, ctypes.byref(nm), None, None, None), self.h)
        self.n_members = nm.value
        self.cell_offset = np.zeros(self.n_members + 1, np.int32)
        self.inlet_offset = np.zeros(self.n_members + 1, np.int32)
        self.exit_offset = np.zeros(self.n_members + 1, np.int32)
        check(lib().hg_ensemble_layout(self.h, ctypes.byref(nm), _i(self.cell_offset), _i(self.inlet_offset),
                                       _i(self.exit_offset)), self.h)

    def steps(self, nsteps):
        """(dts [nsteps, n_members], elapsed time [n_members]): every member's
        own steps since the last upload (hg_ensemble_steps)."""
        dts = np.zeros((nsteps, self.n_members))
        t = np.zeros(self.n_members)
        self._chk(lib().hg_ensemble_steps(self.h, int(nsteps), _d(dts), _d(t)))
        return dts, t

    def concat(self, per_member, kind="cell"):
        """Concatenate per-member arrays (kind: cell, inlet, exit, state)."""
        if kind == "state":   # Q = [xi; qx; qy] per member -> the concatenated state's three blocks
            ns = np.diff(self.cell_offset)
            return np.concatenate([np.concatenate([np.asarray(q)[b * n:(b + 1) * n] for q, n in zip(per_member, ns)])
                                   for b in range(3)])
        return np.concatenate([np.asarray(a, dtype=np.float64).ravel() for a in per_member])

    def split(self, arr, kind="cell"):
        """Per-member views of a concatenated array (kind: cell, inlet, exit, state)."""
        if kind == "state":
            N = int(self.cell_offset[-1])
            return [np.concatenate([arr[b * N + a:b * N + z] for b in range(3)])
                    for a, z in zip(self.cell_offset[:-1], self.cell_offset[1:])]
        off = {"cell": self.cell_offset, "inlet": self.inlet_offset, "exit": self.exit_offset}[kind]
        return [arr[a:z] for a, z in zip(off[:-1], off[1:])]


# ---------------------------------------------------------------------------
# The reference's interface
# ---------------------------------------------------------------------------
class SWE2DExtraParameters:
    """The fields of SWE2D_Extra_Parameters (application_commons.jl:7-44) that
    the RHS reads at run time: the active parameter name and how a parameter
    vector maps onto the model."""

    def __init__(self, ctx, active_param_name="none", mat_id=None, bInPlaceODE=False):
        if active_param_name not in ("none", "ManningN", "zb", "Q"):
            raise ValueError("active_param_name must be one of none, ManningN, zb, Q "
                             "(process_model_parameters_2D.jl:2-168)")
        self.ctx = ctx
        self.active_param_name = active_param_name
        self.mat_id = None if mat_id is None else np.ascontiguousarray(mat_id, dtype=np.int32)
        self.bInPlaceODE = bInPlaceODE
        self._last = None

    def apply(self, params_vector):
        """Inject the active parameter (semi_discretize_swe_2D.jl:112-199)."""
        if self.active_param_name == "none" or params_vector is None:
            return
        p = np.asarray(params_vector, dtype=np.float64)
        if self._last is not None and self._last.shape == p.shape and np.array_equal(self._last, p):
            return
        if self.active_param_name == "ManningN":
            self.ctx.set_manning_zones(self.mat_id, p)      # ManningN_cells = p[matID + 1] (1-based)
        elif self.active_param_name == "zb":
            self.ctx.set_zb_cells(p)                        # update_bed_data (process_bed_2D.jl:46-66)
        elif self.active_param_name == "Q":
            self.ctx.set_inlet_q(p)                         # inletQ_TotalQ = params_vector
        self._last = p.copy()


def swe_2d_rhs(dQdt, Q, params_vector, t, p_extra):
    """dQ/dt of Q = [xi; q_x; q_y] (semi_discretize_swe_2D.jl:18-277).

    In-place (fills and returns ``dQdt``) when ``p_extra.bInPlaceODE``, else
    returns a new array, as the reference's two ODEFunction forms do."""
    p_extra.apply(params_vector)
    if p_extra.bInPlaceODE:
        p_extra.ctx.rhs(Q, t, out=dQdt)
        return dQdt
    return p_extra.ctx.rhs(Q, t)


def custom_ODE_solve(Q0, params_vector, p_extra, tspan, dt):
    """The reference's forward-Euler loop (custom_ODE_solvers.jl:36-95): one
    step per element of ``t_start:dt:t_end`` with its clamp; returns the saved
    states as columns, [3N, nsteps]."""
    p_extra.apply(params_vector)
    nsteps = len(np.arange(tspan[0], tspan[1] + dt * 1e-9, dt))
    _, _, saves = p_extra.ctx.integrate(Q0, nsteps, method="euler", dt=dt, save_every=1)
    return saves.T
