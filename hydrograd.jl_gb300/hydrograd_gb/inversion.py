"""Parameter inversion driver: the host side of swe_2D_inversion.jl's
optimize_parameters_inversion / compute_loss_inversion, with the forward run
and its gradient on the device.

Per iteration: set the active parameter (zone Manning n, zb at cells, or inlet
Q), run hg_final_loss_and_grad (nsteps SSP-RK2 steps of dt, the final-state WSE
and velocity misfits, the checkpointed discrete adjoint), add the
parameter-only regularisers (bound loss, bed-slope loss) and their gradients,
report the iteration the way the reference's callback does, and take an
optimiser step (Optimisers.jl's Adam or Descent).

The reference differentiates a Tsit5 solve with SciMLSensitivity; here the
forward model is the device's SSP-RK2 at a fixed dt and its gradient is the
exact discrete adjoint of those steps.  The reference's per-iteration JSON
files (inversion_callback_save_iter_<n>.json: iter_number, loss_total, theta)
are written with the same names and keys; its JLD2 checkpoints (a Julia
serialisation format) become JSON files with the same contents (ITER, LOSS,
PARS) under checkpoint_inversion_iter_<n>.json.
"""
import json
import os
from dataclasses import dataclass, field

import numpy as np

EPS = np.finfo(np.float64).eps


@dataclass
class InversionSettings:
    """The inversion options of the reference's run-control JSON
    (control_settings_2D.jl inversion settings)."""
    active_param: str = "ManningN"          # "ManningN" (zone values), "zb" (cells), "Q" (inlet discharges)
    wse_loss: bool = True
    uv_loss: bool = False
    bound_loss: bool = False
    slope_loss: bool = False
    lower_bound: float = 0.0
    upper_bound: float = 1.0
    slope_upper_bound: float = 0.2
    optimizers: list = field(default_factory=lambda: ["Adam"])
    learning_rates: list = field(default_factory=lambda: [0.001])
    max_iterations: list = field(default_factory=lambda: [10])
    abs_tols: list = field(default_factory=list)   # per optimiser (control_settings_2D.jl:46-47)
    rel_tols: list = field(default_factory=list)
    save_frequency: int = 1
    save_checkpoint: bool = False
    checkpoint_frequency: int = 10

    @classmethod
    def from_run_control(cls, opts):
        """From the "inversion_options" block of a run_control.json."""
        return cls(active_param=opts["active_param_names"][0],
                   wse_loss=bool(opts["inversion_bInversion_WSE_loss"]),
                   uv_loss=bool(opts["inversion_bInversion_uv_loss"]),
                   bound_loss=bool(opts["inversion_bInversion_bound_loss"]),
                   slope_loss=bool(opts["inversion_bInversion_slope_loss"]),
                   lower_bound=float(opts["inversion_parameter_value_lower_bound"]),
                   upper_bound=float(opts["inversion_parameter_value_upper_bound"]),
                   slope_upper_bound=float(opts["inversion_parameter_slope_upper_bound"]),
                   optimizers=list(opts["inversion_optimizers"]),
                   learning_rates=[float(v) for v in opts["inversion_learning_rates"]],
                   max_iterations=[int(v) for v in opts["inversion_max_iterations"]],
                   abs_tols=[float(v) for v in opts.get("inversion_abs_tols", [])],
                   rel_tols=[float(v) for v in opts.get("inversion_rel_tols", [])],
                   save_frequency=int(opts["inversion_save_frequency"]),
                   save_checkpoint=bool(opts["inversion_save_checkpoint"]),
                   checkpoint_frequency=int(opts["inversion_checkpoint_frequency"]))


def bound_loss(p, lower, upper):
    """compute_bound_loss (swe_2D_inversion.jl:738-749) and its gradient."""
    p = np.asarray(p, dtype=np.float64)
    rng = upper - lower
    lo = np.maximum(0.0, lower - p) / rng
    up = np.maximum(0.0, p - upper) / rng
    return float(np.sum(lo * lo) + np.sum(up * up)), (-2.0 * lo + 2.0 * up) / rng


class CellGradient:
    """compute_scalar_gradients_from_cells (fvm_schemes_2D.jl:33-84): the
    Green-Gauss gradient of a cell field with face values (z_c + z_n) / 2 and
    z_n = z_c on boundary faces; linear, so its transpose gives the gradient of
    a loss of it."""

    def __init__(self, mesh_faces, cell_node_count):
        nbr = mesh_faces["nbr"]
        N = nbr.shape[0]
        valid = np.arange(8)[None, :] < np.asarray(cell_node_count)[:, None]
        self.cell = np.repeat(np.arange(N), 8).reshape(N, 8)[valid]
        nb = np.where(nbr >= 0, nbr, np.arange(N)[:, None])[valid]
        w = (mesh_faces["lengths"] / mesh_faces["areas"][:, None])[valid]
        self.nb = nb
        self.wx = mesh_faces["normals"][..., 0][valid] * w
        self.wy = mesh_faces["normals"][..., 1][valid] * w
        self.N = N

    def apply(self, z):
        zf = (z[self.cell] + z[self.nb]) / 2.0
        return (np.bincount(self.cell, self.wx * zf, self.N), np.bincount(self.cell, self.wy * zf, self.N))

    def transpose(self, gx, gy):
        t = (gx[self.cell] * self.wx + gy[self.cell] * self.wy) / 2.0
        return np.bincount(self.cell, t, self.N) + np.bincount(self.nb, t, self.N)


def slope_loss(zb, grad_op, upper):
    """calc_slope_loss (swe_2D_inversion.jl:752-772) and its gradient."""
    gx, gy = grad_op.apply(np.asarray(zb, dtype=np.float64))
    s = np.sqrt(gx ** 2 + gy ** 2 + EPS)
    val, ds = bound_loss(s, 0.0, upper)
    N = grad_op.N
    return val / N, grad_op.transpose(ds / N * gx / s, ds / N * gy / s)


class Adam:
    """Optimisers.jl's Adam(eta; beta = (0.9, 0.999), epsilon = 1e-8)."""

    def __init__(self, eta, beta=(0.9, 0.999), eps=1e-8):
        self.eta, self.beta, self.eps = eta, beta, eps
        self.m = self.v = None
        self.bt = beta

    def step(self, theta, g):
        if self.m is None:
            self.m, self.v = np.zeros_like(theta), np.zeros_like(theta)
        b1, b2 = self.beta
        self.m = b1 * self.m + (1 - b1) * g
        self.v = b2 * self.v + (1 - b2) * g * g
        dx = self.m / (1 - self.bt[0]) / (np.sqrt(self.v / (1 - self.bt[1])) + self.eps) * self.eta
        self.bt = (self.bt[0] * b1, self.bt[1] * b2)
        return theta - dx


class Descent:
    """Optimisers.jl's Descent(eta): theta - eta g."""

    def __init__(self, eta):
        self.eta = eta

    def step(self, theta, g):
        return theta - self.eta * g


def backtracking(phi, phi0, dphi0, alpha=1.0, c1=1e-4, rho_hi=0.5, rho_lo=0.1, max_iter=1000):
    """Backtracking line search with the Armijo condition phi(a) <= phi0 + c1 a
    dphi0: the first shrink from the quadratic through phi0, dphi0 and phi(a),
    the later ones from the cubic through the last two trials (Nocedal &
    Wright, Numerical Optimization, 3.5), each new step kept within
    [rho_lo, rho_hi] of the last -- the algorithm and defaults of
    LineSearches.jl's BackTracking (order 3), which the reference's LBFGS takes
    (swe_2D_inversion.jl:684-685).  Returns (a, phi(a), evaluations)."""
    a1 = a2 = alpha
    p0, p1 = phi0, phi(a2)
    n = 1
    while p1 > phi0 + c1 * a2 * dphi0 and n < max_iter:
        if n == 1:
            at = -(dphi0 * a2 * a2) / (2.0 * (p1 - phi0 - dphi0 * a2))
        else:
            div = 1.0 / (a1 * a1 * a2 * a2 * (a2 - a1))
            r1, r0 = p1 - phi0 - dphi0 * a2, p0 - phi0 - dphi0 * a1
            a = (a1 * a1 * r1 - a2 * a2 * r0) * div
            b = (-a1 ** 3 * r1 + a2 ** 3 * r0) * div
            if abs(a) <= 1e-300:
                at = dphi0 / (2.0 * b)
            else:
                at = (-b + np.sqrt(max(b * b - 3.0 * a * dphi0, 0.0))) / (3.0 * a)
        a1 = a2
        a2 = max(min(at, a2 * rho_hi), a2 * rho_lo)
        p0, p1 = p1, phi(a2)
        n += 1
    return a2, p1, n


class LBFGS:
    """Limited-memory BFGS (Nocedal & Wright, 7.2): the two-loop recursion
    over the last m (s, y) pairs with the initial inverse Hessian (s'y / y'y) I
    of the newest pair, a backtracking line search from the unit step -- the
    method and defaults of Optim.jl's LBFGS(linesearch = BackTracking()), the
    reference's choice (swe_2D_inversion.jl:684-685).  Pairs with s'y <= 0 are
    not stored.  Converged when max|g| <= g_tol or, with rel_tol, when the loss
    changes by at most rel_tol of its size.  (Restated from the published
    method; Optim.jl itself is not available to compare against.)"""

    def __init__(self, m=10, g_tol=1e-8, rel_tol=None):
        self.m, self.g_tol, self.rel_tol = m, g_tol, rel_tol
        self.S, self.Y = [], []

    def direction(self, g):
        q = g.copy()
        al = []
        for s, y in zip(reversed(self.S), reversed(self.Y)):
            rho = 1.0 / (y @ s)
            a = rho * (s @ q)
            q -= a * y
            al.append((rho, a))
        if self.S:
            q *= (self.S[-1] @ self.Y[-1]) / (self.Y[-1] @ self.Y[-1])
        for (s, y), (rho, a) in zip(zip(self.S, self.Y), reversed(al)):
            q += (a - rho * (y @ q)) * s
        return -q

    def minimize(self, fg, x0, max_iter, callback=None):
        """fg(x) -> (f, g); callback(iteration, x, f) after every iteration.
        Returns (x, f, converged)."""
        x = np.array(x0, dtype=np.float64)
        f, g = fg(x)
        cache = {}

        def phi(a, x=None, d=None):
            xa = x + a * d
            fa, ga = fg(xa)
            cache[a] = (xa, fa, ga)
            return fa
        for it in range(1, max_iter + 1):
            if np.abs(g).max() <= self.g_tol:
                return x, f, True
            d = self.direction(g)
            dphi0 = g @ d
            if dphi0 >= 0:   # not a descent direction: restart from steepest descent
                self.S.clear()
                self.Y.clear()
                d, dphi0 = -g, -(g @ g)
            cache.clear()
            a, fa, _ = backtracking(lambda t: phi(t, x, d), f, dphi0)
            xn, fn, gn = cache[a]
            s, y = xn - x, gn - g
            if s @ y > 0:
                self.S.append(s)
                self.Y.append(y)
                if len(self.S) > self.m:
                    self.S.pop(0)
                    self.Y.pop(0)
            converged = self.rel_tol is not None and abs(fn - f) <= self.rel_tol * abs(f)
            x, f, g = xn, fn, gn
            if callback:
                callback(it, x, f)
            if converged:
                return x, f, True
        return x, f, False


class Inversion:
    """One inversion problem on a device context (SWE2D): the forward model
    (Q0, nsteps SSP-RK2 steps of dt), the observations (truth fields), the
    active parameter and the settings."""

    def __init__(self, ctx, case, Q0, nsteps, dt, observed, settings, ckpt_every=50, mat_id=None, case_path=None):
        self.ctx, self.Q0, self.nsteps, self.dt = ctx, np.asarray(Q0, dtype=np.float64), int(nsteps), float(dt)
        self.obs, self.s, self.ckpt = observed, settings, int(ckpt_every)
        self.mat_id = None if mat_id is None else np.asarray(mat_id, dtype=np.int32)
        self.case_path = case_path
        self.N = ctx.n_cells
        self.grad_op = None
        if settings.slope_loss and settings.active_param == "zb":
            from .swe2d import HostMesh
            self.grad_op = CellGradient(HostMesh(case).cell_faces(), case["cell_node_count"])
        if settings.active_param not in ("ManningN", "zb", "Q"):
            raise ValueError("active_param must be ManningN, zb or Q")

    def apply(self, theta):
        """Parameter injection, as swe_2d_rhs does for the active parameter."""
        a = self.s.active_param
        if a == "ManningN":
            self.ctx.set_manning_zones(self.mat_id, theta)
        elif a == "zb":
            self.ctx.set_zb_cells(theta)
        else:
            self.ctx.set_inlet_q(theta)

    def loss_and_grad(self, theta):
        """compute_loss_inversion (swe_2D_inversion.jl:247-483) and its gradient:
        (loss_total, loss_pred, loss_pred_WSE, loss_pred_uv, loss_bound,
        loss_slope), gradient w.r.t. theta, final state."""
        s, o = self.s, self.obs
        theta = np.asarray(theta, dtype=np.float64)
        self.apply(theta)
        zb_wse = None if s.active_param == "zb" else o["zb_cell_truth"]
        want = {"ManningN": ("manning",), "zb": ("zb",), "Q": ("inletq",)}[s.active_param]
        r = self.ctx.final_loss_and_grad(self.Q0, self.nsteps, self.dt, wse=o["WSE_truth"] if s.wse_loss else None,
                                         u=o["u_truth"] if s.uv_loss else None,
                                         v=o["v_truth"] if s.uv_loss else None, zb_wse=zb_wse, ckpt_every=self.ckpt,
                                         want=want)
        if s.active_param == "ManningN":
            g = np.bincount(self.mat_id, r["g_manning"], minlength=len(theta))
        elif s.active_param == "zb":
            g = r["g_zb"].copy()
        else:
            g = r["g_inletq"].copy()
        lb = ls = 0.0
        if s.bound_loss:
            lb, gb = bound_loss(theta, s.lower_bound, s.upper_bound)
            lb /= self.N
            g += gb / self.N
        if s.slope_loss and s.active_param == "zb":
            ls, gs = slope_loss(theta, self.grad_op, s.slope_upper_bound)
            g += gs
        total = r["loss"] + lb + ls
        return (total, r["loss"], r["loss_wse"], r["loss_uv"], lb, ls), g, r["Q"]

    def _save(self, it, loss, theta, ITER, LOSS, PARS):
        if not self.case_path:
            return
        if it % self.s.save_frequency == 0:
            with open(os.path.join(self.case_path, f"inversion_callback_save_iter_{it}.json"), "w") as fh:
                json.dump({"iter_number": it, "loss_total": loss, "theta": list(map(float, theta))}, fh, indent=4)
        if self.s.save_checkpoint and it % self.s.checkpoint_frequency == 0:
            with open(os.path.join(self.case_path, f"checkpoint_inversion_iter_{it}.json"), "w") as fh:
                json.dump({"ITER": ITER, "LOSS": LOSS, "PARS": [list(map(float, p)) for p in PARS]}, fh)

    def run(self, theta0, verbose=False):
        """The optimiser sequence of optimize_parameters_inversion
        (swe_2D_inversion.jl:484-700): each optimiser runs its max_iterations
        from where the previous one stopped; max_iterations <= 0 skips it; an
        LBFGS stage that converges ends the sequence, as the reference's loop
        breaks on a successful solve.  Returns the final theta and the ITER /
        LOSS / PARS histories."""
        theta = np.array(theta0, dtype=np.float64)
        ITER, LOSS, PARS = [], [], []
        for k, (name, lr, iters) in enumerate(zip(self.s.optimizers, self.s.learning_rates, self.s.max_iterations)):
            if iters <= 0:
                continue
            if name == "LBFGS":
                rel = self.s.rel_tols[k] if k < len(self.s.rel_tols) else None

                def fg(x):
                    parts, g, _ = self.loss_and_grad(x)
                    return float(parts[0]), g

                def cb(_, x, f):
                    it = len(LOSS) + 1
                    ITER.append(it)
                    LOSS.append(float(f))
                    PARS.append(x.copy())
                    if verbose:
                        print(f"iter_number = {it}, loss_total = {f}")
                    self._save(it, float(f), x, ITER, LOSS, PARS)
                theta, _, converged = LBFGS(rel_tol=rel).minimize(fg, theta, iters, callback=cb)
                if converged:
                    break
                continue
            if name == "Adam":
                opt = Adam(lr)
            elif name == "Descent":
                opt = Descent(lr)
            else:
                raise ValueError(f"optimizer {name}: Adam, Descent and LBFGS are available")
            for _ in range(iters):
                parts, g, _ = self.loss_and_grad(theta)
                it = len(LOSS) + 1
                ITER.append(it)
                LOSS.append(float(parts[0]))
                PARS.append(theta.copy())
                if verbose:
                    print(f"iter_number = {it}, loss_total = {parts[0]}")
                self._save(it, float(parts[0]), theta, ITER, LOSS, PARS)
                theta = opt.step(theta, g)
        return dict(theta=theta, ITER=ITER, LOSS=LOSS, PARS=PARS)
