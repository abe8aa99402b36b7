"""ctypes wrapper around the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a CPU FP64 restatement of Hydrograd.jl's shallow-water RHS and
time stepping (hg_oracle.hpp).  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline / reference legs import this module, always as the
checker or the timed CPU baseline -- never as part of the product path.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libhg_oracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    lib.ho_create.restype = ctypes.c_void_p
    lib.ho_create.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _ip, _ip, ctypes.c_int, _ip, _ip, _ip, _ip,
                              ctypes.c_double, ctypes.c_double, ctypes.c_double]
    lib.ho_last_error.restype = ctypes.c_char_p
    lib.ho_destroy.argtypes = [ctypes.c_void_p]
    lib.ho_sizes.argtypes = [ctypes.c_void_p, _ip]
    lib.ho_mesh_arrays.argtypes = [ctypes.c_void_p, _ip, _ip, _ip, _dp, _dp, _dp, _ip, _dp]
    lib.ho_bed.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
    for name in ("ho_set_wstill", "ho_set_hstill", "ho_get_hstill", "ho_set_manning_cells", "ho_set_zb_cells"):
        getattr(lib, name).argtypes = [ctypes.c_void_p, _dp]
    lib.ho_set_inletq.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int]
    lib.ho_set_exith.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int]
    lib.ho_rhs.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int]
    lib.ho_friction.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp]
    lib.ho_cfl_dt.restype = ctypes.c_double
    lib.ho_cfl_dt.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double]
    lib.ho_rk2.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp]
    lib.ho_tsit5.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                             ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip]
    lib.ho_set_hydrograph.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp]
    lib.ho_set_riemann.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.ho_set_resistance_fn.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
    lib.ho_set_ude.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _ip, _dp, ctypes.c_int,
                               ctypes.c_double, ctypes.c_double, _dp, _dp, _dp, _dp, ctypes.c_int]
    lib.ho_resistance_cells.argtypes = [ctypes.c_void_p, _dp, _dp]
    lib.ho_manning_fn.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    lib.ho_euler_reference.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
    lib.ho_rk2_tangent.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp,
                                   ctypes.c_int, _ip, _dp, _dp, _dp, _dp, _dp, ctypes.c_int]
    lib.ho_rk2_loss.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _ip, _dp, _dp, _dp,
                                ctypes.c_int]
    lib.ho_tsit5_tangent.argtypes = lib.ho_rk2_tangent.argtypes
    lib.ho_tsit5_loss.argtypes = lib.ho_rk2_loss.argtypes
    _lib = lib
    return lib


def _d(a):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_dp)


def _i(a):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(_ip)


def manning_fn(kind, params, h, umag=None, ks=None):
    """The n functions of hg_oracle.hpp (manning_fn) at given h, Umag, ks:
    returns (n, h_ks, friction factor, Re)."""
    lib = _load()
    p = np.zeros(4)
    p[:len(params)] = params
    h = np.ascontiguousarray(h, dtype=np.float64)
    n = len(h)
    um = None if umag is None else np.ascontiguousarray(umag, dtype=np.float64)
    ks = None if ks is None else np.ascontiguousarray(ks, dtype=np.float64)
    out = [np.zeros(n) for _ in range(4)]
    lib.ho_manning_fn(int(kind), _d(p), n, _d(h), _d(um), _d(ks), *(_d(o) for o in out))
    return tuple(out)


class Oracle:
    """One case: mesh + boundary conditions + parameters, as SWE2D_Extra_Parameters holds them."""

    def __init__(self, mesh, g=9.81, k_n=1.0, h_small=1.0e-3):
        lib = _load()
        self._keep = {k: np.ascontiguousarray(v) for k, v in mesh.items() if isinstance(v, np.ndarray)}
        xyz = np.ascontiguousarray(mesh["node_xyz"], dtype=np.float64)
        x, y, z = (np.ascontiguousarray(xyz[:, i]) for i in range(3))
        self._xyz = (x, y, z)
        cn = np.ascontiguousarray(mesh["cell_nodes"], dtype=np.int32)
        cnt = np.ascontiguousarray(mesh["cell_node_count"], dtype=np.int32)
        sid = np.ascontiguousarray(mesh["string_ids"], dtype=np.int32)
        soff = np.ascontiguousarray(mesh["string_offsets"], dtype=np.int32)
        snod = np.ascontiguousarray(mesh["string_nodes"], dtype=np.int32)
        sbc = np.ascontiguousarray(mesh["string_bc"], dtype=np.int32)
        self.h = lib.ho_create(len(x), _d(x), _d(y), _d(z), len(cnt), _i(cnt), _i(cn), len(sid), _i(sid), _i(soff),
                               _i(snod), _i(sbc), g, k_n, h_small)
        if not self.h:
            raise RuntimeError("oracle: " + lib.ho_last_error().decode())
        self.lib = lib
        s = np.zeros(7, dtype=np.int32)
        lib.ho_sizes(self.h, _i(s))
        self.n_cells, self.n_faces, self.n_ghosts, self.n_inlet, self.n_exit, self.n_wall, self.n_symm = map(int, s)
        self.h_small = h_small

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ho_destroy(self.h)
            self.h = None

    def mesh_arrays(self):
        N, F = self.n_cells, self.n_faces
        out = dict(cell_faces=np.zeros(N * 8, np.int32), cell_neighbors=np.zeros(N * 8, np.int32),
                   face_is_boundary=np.zeros(F, np.int32), areas=np.zeros(N), normals=np.zeros(N * 16),
                   face_lengths=np.zeros(F), face_nodes=np.zeros(F * 2, np.int32), centroids=np.zeros(N * 2))
        self.lib.ho_mesh_arrays(self.h, _i(out["cell_faces"]), _i(out["cell_neighbors"]), _i(out["face_is_boundary"]),
                                _d(out["areas"]), _d(out["normals"]), _d(out["face_lengths"]), _i(out["face_nodes"]),
                                _d(out["centroids"]))
        return out

    def bed(self):
        N = self.n_cells
        zb, S0, zf = np.zeros(N), np.zeros(2 * N), np.zeros(self.n_faces)
        self.lib.ho_bed(self.h, _d(zb), _d(S0), _d(zf))
        return zb, S0.reshape(N, 2), zf

    def set_wstill(self, wstill):
        w = np.ascontiguousarray(np.broadcast_to(np.asarray(wstill, float), (self.n_cells,)))
        self.lib.ho_set_wstill(self.h, _d(w))

    def set_hstill(self, hstill):
        self.lib.ho_set_hstill(self.h, _d(np.asarray(hstill, float)))

    def hstill(self):
        out = np.zeros(self.n_cells)
        self.lib.ho_get_hstill(self.h, _d(out))
        return out

    def set_manning_cells(self, n):
        self.lib.ho_set_manning_cells(self.h, _d(np.ascontiguousarray(n, dtype=np.float64)))

    def set_zb_cells(self, zb):
        self.lib.ho_set_zb_cells(self.h, _d(np.ascontiguousarray(zb, dtype=np.float64)))

    def set_inlet_q(self, q):
        q = np.ascontiguousarray(np.atleast_1d(q), dtype=np.float64)
        self.lib.ho_set_inletq(self.h, _d(q), len(q))

    def set_exit_wse(self, w):
        w = np.ascontiguousarray(np.atleast_1d(w), dtype=np.float64)
        self.lib.ho_set_exith(self.h, _d(w), len(w))

    def rhs(self, Q, nthreads=1):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        out = np.zeros_like(Q)
        if self.lib.ho_rhs(self.h, _d(Q), _d(out), nthreads) != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())
        return out

    def friction(self, h, qx, qy):
        fx, fy = np.zeros(self.n_cells), np.zeros(self.n_cells)
        self.lib.ho_friction(self.h, _d(h), _d(qx), _d(qy), _d(fx), _d(fy))
        return fx, fy

    def cfl_dt(self, Q, cfl=0.4):
        return self.lib.ho_cfl_dt(self.h, _d(np.ascontiguousarray(Q, dtype=np.float64)), cfl)

    def rk2(self, Q, nsteps, dt=None, cfl=0.4, nthreads=1, return_dts=False):
        Q = np.array(Q, dtype=np.float64)
        dts = np.zeros(max(nsteps, 1))
        rc = self.lib.ho_rk2(self.h, _d(Q), nsteps, dt if dt else -1.0, cfl, nthreads, _d(dts))
        if rc != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())
        return (Q, dts[:nsteps]) if return_dts else Q

    def tsit5(self, Q, t0, t1, abstol=1e-6, reltol=1e-3, dt0=0.0, adaptive=True, max_steps=0, nthreads=1):
        """Tsit5 from t0 to t1 (hgo::tsit5); returns (Q, (accepted, rejected, evals))."""
        Q = np.array(Q, dtype=np.float64)
        st = np.zeros(3, dtype=np.int32)
        rc = self.lib.ho_tsit5(self.h, _d(Q), t0, t1, abstol, reltol, dt0, 1 if adaptive else 0, max_steps, nthreads,
                               _i(st))
        if rc != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())
        return Q, tuple(int(v) for v in st)

    def set_riemann_solver(self, name):
        """Riemann solver of the faces: "Roe" (the reference's) or "HLL" (hgo::hll_flux)."""
        kinds = {"Roe": 0, "HLL": 1}
        if name not in kinds:
            raise ValueError("Riemann solver: Roe or HLL")
        if self.lib.ho_set_riemann(self.h, kinds[name]) != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())

    def set_hydrograph(self, group, t, q):
        """Inlet-Q hydrograph of one group (hgo::hydro_at); empty t removes it."""
        t = np.ascontiguousarray(t, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        if self.lib.ho_set_hydrograph(self.h, int(group), len(t), _d(t), _d(q)) != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())

    def set_resistance_fn(self, kind, params=(0.0, 0.0, 0.0, 0.0), ks=None):
        """Manning's n as a function of the state (RES_* kinds 0-4 of hg_oracle.hpp)."""
        p = np.zeros(4)
        p[:len(params)] = params
        self._res = (p, None if ks is None else np.ascontiguousarray(ks, dtype=np.float64))
        if self.lib.ho_set_resistance_fn(self.h, int(kind), _d(p), _d(self._res[1])) != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())

    def set_ude(self, kind, in_dim, hidden, activations, params, output_bounds, h_bounds, u_bounds=(0.0, 1.0),
                ks_bounds=(0.0, 1.0), ks=None, over_batch=True):
        """UDE closure (RES_* kinds 5-7) with the network of hgo::Mlp."""
        hid = np.ascontiguousarray(hidden, dtype=np.int32)
        act = np.ascontiguousarray(activations, dtype=np.int32)
        prm = np.ascontiguousarray(params, dtype=np.float64)
        b = [np.ascontiguousarray(v, dtype=np.float64) for v in (h_bounds, u_bounds, ks_bounds)]
        ks = None if ks is None else np.ascontiguousarray(ks, dtype=np.float64)
        rc = self.lib.ho_set_ude(self.h, int(kind), int(in_dim), len(hid), _i(hid), _i(act), _d(prm), len(prm),
                                 float(output_bounds[0]), float(output_bounds[1]), _d(b[0]), _d(b[1]), _d(b[2]),
                                 _d(ks), 1 if over_batch else 0)
        if rc != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())

    def resistance_cells(self, Q):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        out = np.zeros(self.n_cells)
        self.lib.ho_resistance_cells(self.h, _d(Q), _d(out))
        return out

    def euler_reference(self, Q, nsteps, dt, nthreads=1):
        Q = np.array(Q, dtype=np.float64)
        if self.lib.ho_euler_reference(self.h, _d(Q), nsteps, dt, nthreads) != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())
        return Q

    def rk2_tangent(self, Q0, nsteps, dt, d_manning=None, d_zb=None, d_inlet=None, probes=None, obs=None,
                    nthreads=1, method="rk2"):
        """Forward-mode run of nsteps fixed-dt SSP-RK2 steps (method "rk2") or
        Tsit5 steps ("tsit5"); returns (Q, dQ[nDir,3N], loss, dloss[nDir])."""
        nd = max(a.shape[0] for a in (d_manning, d_zb, d_inlet) if a is not None)
        Q0 = np.ascontiguousarray(Q0, dtype=np.float64)
        Qo, dQo = np.zeros_like(Q0), np.zeros((nd, Q0.size))
        loss, dloss = np.zeros(1), np.zeros(nd)
        npb = 0 if probes is None else len(probes)
        fn = self.lib.ho_tsit5_tangent if method == "tsit5" else self.lib.ho_rk2_tangent
        rc = fn(self.h, _d(Q0), nsteps, dt, nd, _d(d_manning), _d(d_zb), _d(d_inlet), npb,
                _i(probes), _d(obs), _d(Qo), _d(dQo), _d(loss), _d(dloss), nthreads)
        if rc != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())
        return Qo, dQo, float(loss[0]), dloss

    def tsit5_tangent(self, Q0, nsteps, dt, **kw):
        """rk2_tangent of nsteps fixed Tsit5 steps (hgo::tsit5_fixed_step)."""
        return self.rk2_tangent(Q0, nsteps, dt, method="tsit5", **kw)

    def rk2_loss(self, Q0, nsteps, dt, probes, obs, nthreads=1, method="rk2"):
        Q0 = np.ascontiguousarray(Q0, dtype=np.float64)
        Qo, loss = np.zeros_like(Q0), np.zeros(1)
        fn = self.lib.ho_tsit5_loss if method == "tsit5" else self.lib.ho_rk2_loss
        if fn(self.h, _d(Q0), nsteps, dt, len(probes), _i(probes), _d(obs), _d(Qo), _d(loss), nthreads) != 0:
            raise RuntimeError("oracle: " + self.lib.ho_last_error().decode())
        return float(loss[0]), Qo

    def tsit5_loss(self, Q0, nsteps, dt, probes, obs, nthreads=1):
        """The probe loss of nsteps fixed Tsit5 steps and the final state."""
        return self.rk2_loss(Q0, nsteps, dt, probes, obs, nthreads, method="tsit5")
