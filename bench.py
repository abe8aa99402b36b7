"""Benchmark: cell-updates/s of the SWE-2D RHS + SSP-RK2 stepping at 1M cells.

Workload: the 2 km reach on a 708 x 708 grid split into 1,002,528 jittered
triangles (hydrograd_gb.workloads.river_triangles, seed 0), 5 Manning zones,
inlet-Q 500 m^3/s, exit-H, walls; 2,000 CFL-0.4 SSP-RK2 steps.  One "step" is
one RK2 step of every cell (two fused stage passes); value = cells x steps / s.

Our arm (default): the FP32-compensated path is the headline ``value``; the
plain FP64 path, FP32C-vs-FP64 error, roofline of the stage kernel, the
end-to-end number through the C ABI with host buffers, and the CPU baseline
(the oracle, all host threads, bounded sample) are reported beside it.
--impl reference: the oracle (the reference's algorithm restated in C++,
OpenMP over cells) on this machine's host cores, on the same workload and metric.

Multi-GPU: the path does not shard in this build (replicas only): under
torchrun each rank runs its own replica; value sums the ranks' cell-updates
over the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "hydrograd.jl_gb300"))

import numpy as np  # noqa: E402

METRIC = "cell-updates/s (fwd; fwd+adjoint) at 1M cells: FP32-comp vs FP64, err≤1e-5"
UNIT = "cell-updates/s"
# Algorithmic (compulsory) bytes per cell for one stage pass: state read +
# per-cell parameters + write, plus per-face geometry phi per cell, and per
# RK2 cell-update (two stages + the stage-2 re-read of Q^n).
BYTES_STAGE = {"fp32c": (72.0, 20.0), "fp64": (96.0, 32.0)}   # (per cell, per face)
BYTES_STEP_EXTRA = {"fp32c": 24.0, "fp64": 24.0}
# The FP32C interior VJP of one stage (stage-2 form): per cell the state,
# parameter and source records (3 x 16 B), the cotangent in and out (2 x 12 B)
# and the n, S0x, S0y accumulators (3 compensated float pairs read and
# written, 48 B); per face its two slot records (2 x 16 B).
BYTES_VJP_FP32C = (120.0, 32.0)
VJP_PROFILE = "k_vjp_pipe_f32_fold_river_tri_1M.md"


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# The FP32C stage kernels hg_autotune chooses among: (name, ncu summary under profiles/)
# and the gather kernel's shapes (variant: cells per block, register budget as resident blocks per SM).
GATHER_SHAPES = {0: "256-cell tiles, 4 blocks per SM", 1: "256-cell tiles, 3 blocks per SM",
                 2: "512-cell tiles, 2 blocks per SM", 3: "128-cell tiles, 8 blocks per SM"}
STAGE_KERNELS = {0: ("k_stage_f32 (one block per tile)", "k_stage_f32_river_tri_1M.md"),
                 1: ("k_stage_pipe_f32 (persistent; the next tile and its halo prefetched by cp.async)",
                     "k_stage_pipe_f32_river_tri_1M.md"),
                 2: ("k_stage_tma_f32 (persistent; the next tile prefetched by bulk copies)", None),
                 3: ("k_stage_face_f32 (one block per 256-cell tile; each wet-wet face evaluated once)",
                     "k_stage_face_f32_river_tri_1M.md")}


def profile_traffic(precision, kernel=0, name=None):
    """Per-cell DRAM bytes of the stage kernel (or of the profile `name`) from
    the committed ncu summary, if any."""
    if name is None:
        name = STAGE_KERNELS[kernel][1] if precision == "fp32c" else "k_stage_f64_river_tri_1M.md"
    if name is None:
        return None
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        line = line.strip()
        if line.startswith("{") and '"dram_bytes_per_cell"' in line:
            d = json.loads(line)
            if d.get("precision") == precision:
                return float(d["dram_bytes_per_cell"])
    return None


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_setup(backend=None):
    """(rank, world size, local rank, torch.distributed or None) of a torchrun
    launch; NCCL on the GPUs, or the backend named (gloo: CPU tensors)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist
    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    backend = backend or os.environ.get("HG_DIST_BACKEND", "nccl")
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return rank, ws, local, dist


def _on_gpu(dist):
    return dist.get_backend() == "nccl"


def barrier(dist):
    if dist is not None:
        import torch
        t = torch.zeros(1, device="cuda" if _on_gpu(dist) else "cpu")
        dist.all_reduce(t)
        if _on_gpu(dist):
            torch.cuda.synchronize()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], device="cuda" if _on_gpu(dist) else "cpu", dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ws, units_per_rank, seconds):
    """Whole-job throughput of ws replicas: every rank processes units_per_rank
    in its own time; the job's time is the slowest rank's (max over ranks)."""
    return ws * units_per_rank / seconds


def workload_name(case, N):
    """The config.workload string of both arms (the same workload, seed and CFL rule)."""
    return f"{case['name']}: {N} jittered triangles, 2 km reach, SSP-RK2 CFL 0.4"


def make_ctx(case, precision, device):
    from hydrograd_gb import SWE2D
    ctx = SWE2D(case, precision=precision, order="hilbert", device=device)
    ctx.set_still_water(case["wstill"])
    ctx.set_manning_zones(case["mat_id"], case["manning_zones"])
    ctx.set_inlet_q(case["inlet_q"])
    ctx.set_exit_wse(case["exit_wse"])
    return ctx


def setup_oracle(case):
    from oracle.oracle import Oracle
    o = Oracle(case)
    o.set_wstill(case["wstill"])
    o.set_manning_cells(case["manning_zones"][case["mat_id"]])
    o.set_inlet_q(case["inlet_q"])
    o.set_exit_wse(case["exit_wse"])
    return o


def cpu_baseline(case, seconds=12.0):
    """The oracle's SSP-RK2 on all host threads, a bounded sample of steps."""
    o = setup_oracle(case)
    N = len(case["cell_node_count"])
    threads = os.cpu_count() or 1
    Q = case["Q0"].copy()
    dt = o.cfl_dt(Q, 0.4)
    o.rk2(Q, 1, dt=dt, nthreads=threads)            # warm-up (page-in, thread pool)
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        Q = o.rk2(Q, 1, cfl=0.4, nthreads=threads)
        steps += 1
    el = time.perf_counter() - t0
    return {"value": N * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} SSP-RK2 CFL steps of the {N}-cell workload in {el:.1f} s"}, o


def run_reference(args):
    rank, ws, _, dist = dist_setup()
    if rank != 0:
        return
    from hydrograd_gb.workloads import river_triangles
    case = river_triangles(n=args.n)
    N = len(case["cell_node_count"])
    o = setup_oracle(case)
    threads = os.cpu_count() or 1
    Q = case["Q0"].copy()
    for _ in range(args.warmup):
        Q = o.rk2(Q, 1, cfl=0.4, nthreads=threads)
    # a step is one SSP-RK2 CFL step of the whole 1M-cell workload (about 33 ms on 16 cores)
    K = args.steps
    t0 = time.perf_counter()
    Q = o.rk2(Q, K, cfl=0.4, nthreads=threads)
    el = time.perf_counter() - t0
    v = N * K / el
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": K, "warmup": args.warmup, "ms_per_step": 1e3 * el / K,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(case, N), "cells": N,
                   "sample": f"{K} steps of the 2,000-step run (one step: one RK2 step of every cell)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{K} SSP-RK2 steps of {N} cells on {threads} threads"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_hll(args, case, device):
    """The HLL Riemann solver (hg_set_riemann_solver) on the 1M-cell reach:
    FP32C forward rate over hll_steps CFL steps (L2 flushed before each, as
    the main leg), and the FP32C state against FP64 HLL's after 200 CFL steps
    each (as the main leg compares Roe's)."""
    N = len(case["cell_node_count"])
    out, final = {}, {}
    for prec in ("fp32c", "fp64"):
        c = make_ctx(case, prec, device)
        c.set_riemann_solver("HLL")
        if prec == "fp32c":
            c.upload(case["Q0"])
            c.advance_timed(args.warmup, cfl=0.4, flush_l2=True)
            c.upload(case["Q0"])
            ms = c.advance_timed(args.hll_steps, cfl=0.4, flush_l2=True)
            out["fwd"] = {"value": N * args.hll_steps / (ms * 1e-3), "steps": args.hll_steps,
                          "ms_per_step": ms / args.hll_steps}
        final[prec], _ = c.integrate(case["Q0"], 200, cfl=0.4)
        c.close()
    a, b = final["fp32c"], final["fp64"]
    out["error_fp32c_vs_fp64_state_rel_linf"] = float(np.abs(a - b).max() / np.abs(b).max())
    out["config"] = ("HLL flux (Harten-Lax-van Leer, Einfeldt wave speeds) on the 1M-cell reach, FP32C, CFL 0.4; "
                     "state error after 200 CFL steps against FP64 HLL")
    return out


def run_dry_start(args, device):
    """Configuration 2 with its written start: the 1M-cell reach dry (h =
    h_small) except a 1.5 m pool touching the inlet (river_triangles(708,
    dry_land=True)), so the pool spreads over the dry bed in moving wet/dry
    fronts.  The reference scheme diverges on a dry bed at any CFL-sized step
    (a property of its Roe wall branch and friction, pinned by
    tests/test_dry_bed.py), so the run takes a fixed step: the initial state's
    CFL step at CFL 0.01.  FP32C rate over dry_steps steps (L2 flushed before
    each), and FP32C against FP64 after the same steps: whole state and the
    cells whose wet/dry status changed (the fronts)."""
    from hydrograd_gb.workloads import river_triangles
    case = river_triangles(n=args.n, dry_land=True)
    N = len(case["cell_node_count"])
    hst = case["wstill"] - case["zb_cells"]
    K = args.dry_steps
    # The first film the scheme seeds differently in FP32C and FP64 comes
    # between steps 50 and 100 on this mesh; until then FP32C keeps to FP64
    # within the 1e-5 contract at the fronts.
    SEED_FREE = min(50, K)
    out, final, early = {"cells": N, "steps": K}, {}, {}
    for prec in ("fp32c", "fp64"):
        c = make_ctx(case, prec, device)
        if prec == "fp32c":
            c.set_dt_min(0.0)   # the CFL-0.01 step of this 1M-cell mesh is below the default dt_min (0.001 s)
            dt = float(c.integrate(case["Q0"], 1, cfl=0.01)[1][0])   # the initial state's CFL-0.01 step
            out["dt"] = dt
            c.upload(case["Q0"])
            c.advance_timed(args.warmup, dt=dt, flush_l2=True)
            c.upload(case["Q0"])
            ms = c.advance_timed(K, dt=dt, flush_l2=True)
            out["fwd"] = {"value": N * K / (ms * 1e-3), "ms_per_step": ms / K}
        final[prec], _ = c.integrate(case["Q0"], K, dt=out["dt"])
        early[prec], _ = c.integrate(case["Q0"], SEED_FREE, dt=out["dt"])
        c.close()
    a, b = final["fp32c"], final["fp64"]
    wet0 = case["Q0"][:N] + hst > 1.5e-3
    wet_a, wet_b = a[:N] + hst > 1.5e-3, b[:N] + hst > 1.5e-3
    front = np.nonzero(wet0 != wet_b)[0]
    scale = np.abs(b).max()
    blk = [max(np.abs(b[j * N:(j + 1) * N]).max(), 1e-3 * scale) for j in range(3)]
    out["wet_cells"] = [int(wet0.sum()), int(wet_b.sum())]
    out["front_cells"] = int(len(front))
    out["max_abs_q"] = float(np.abs(b[N:]).max())
    out["error_fp32c_vs_fp64"] = {
        "state_rel_linf": float(np.abs(a - b).max() / scale),
        "block_rel_linf": [float(np.abs(a[j * N:(j + 1) * N] - b[j * N:(j + 1) * N]).max() / blk[j])
                           for j in range(3)],
        "front_block_rel_linf": [float(np.abs(a[j * N:(j + 1) * N][front] - b[j * N:(j + 1) * N][front]).max()
                                       / blk[j]) if len(front) else 0.0 for j in range(3)],
        "wet_dry_decisions_differing": int((wet_a != wet_b).sum())}
    a0, b0 = early["fp32c"], early["fp64"]
    out["error_fp32c_vs_fp64_seed_free"] = {
        "steps": SEED_FREE, "state_rel_linf": float(np.abs(a0 - b0).max() / np.abs(b0).max()),
        "block_rel_linf": [float(np.abs(a0[j * N:(j + 1) * N] - b0[j * N:(j + 1) * N]).max()
                                 / max(np.abs(b0[j * N:(j + 1) * N]).max(), 1e-3 * np.abs(b0).max()))
                           for j in range(3)]}
    out["config"] = ("configuration 2 as written: 1M-cell reach dry except a 1.5 m pool at the inlet, moving "
                     "wet/dry fronts; fixed dt = the initial CFL-0.01 step (the reference scheme diverges on a dry "
                     "bed at CFL-sized steps); FP32C vs FP64 after the same steps, and over the first steps, before "
                     "the scheme seeds its first film differently in the two precisions (at the fronts it "
                     "amplifies rounding-sized differences: FP64 runs perturbed by 1e-7 per step part by 1e-2)")
    return out


def run_tsit5(args, case, device):
    """The reference's default integrator on the device (hg_integrate_tsit5:
    Tsit5 with abstol 1e-6 / reltol 1e-3, swe_2D_forward_simulation.jl:37-39)
    on the 1M-cell reach over tsit5_time simulated seconds, FP32C and FP64 (wall
    time of the call: the state is copied in and out once); then the
    discrete adjoint of fixed Tsit5 steps (hg_set_adjoint_integrator) over
    tsit5_adj_steps steps of half the initial CFL-0.4 step, FP32C and FP64,
    and the FP32C gradients against the FP64 ones."""
    from hydrograd_gb.workloads import probes_and_perturbation
    N = len(case["cell_node_count"])
    out, final, grads = {"cells": N, "simulated_seconds": args.tsit5_time}, {}, {}
    adj_dt = None
    for prec in ("fp32c", "fp64"):
        c = make_ctx(case, prec, device)
        c.integrate_tsit5(case["Q0"], 0.0, 0.05)   # warm-up
        c.synchronize()
        t0 = time.perf_counter()
        Q, st = c.integrate_tsit5(case["Q0"], 0.0, args.tsit5_time)
        el = time.perf_counter() - t0
        out[prec] = {"value": N * int(st[0]) / el, "seconds": el, "accepted": int(st[0]), "rejected": int(st[1]),
                     "rhs_evaluations": int(st[2]), "cell_rhs_per_s": N * int(st[2]) / el}
        # FP32C against FP64 on the same steps: the adaptive runs choose their
        # steps from their own error estimates, so they compare fixed steps of
        # the FP64 run's mean step over the same time
        if prec == "fp32c":
            fixed_n = int(st[0])
        final[prec], _ = c.integrate_tsit5(case["Q0"], 0.0, args.tsit5_time, dt0=args.tsit5_time / fixed_n,
                                           adaptive=False)
        if args.tsit5_adj_steps > 0:
            probes, _ = probes_and_perturbation(case, 64, inlet_share=0.5)
            if adj_dt is None:   # the same steps in both precisions
                adj_dt = 0.5 * c.integrate(case["Q0"], 1, cfl=0.4)[1][0]
            K = args.tsit5_adj_steps
            obs = np.tile((case["wstill"] - case["zb_cells"])[probes], (K, 1))
            c.set_adjoint_integrator("tsit5")
            c.loss_and_grad(case["Q0"], 2, adj_dt, probes, obs[:2])   # warm-up / allocation
            t0 = time.perf_counter()
            grads[prec] = c.loss_and_grad(case["Q0"], K, adj_dt, probes, obs, ckpt_every=K)
            el = time.perf_counter() - t0
            out["adjoint_" + prec] = {"value": N * K / el, "seconds": el, "steps": K}
        c.close()
    if len(grads) == 2:
        g32, g64 = grads["fp32c"], grads["fp64"]
        rel = lambda x, y: float(np.abs(np.asarray(x) - np.asarray(y)).max() / np.abs(np.asarray(y)).max())
        out["adjoint_error_fp32c_vs_fp64"] = {"loss_rel": rel(g32["loss"], g64["loss"]),
                                              "grad_manning_rel_linf": rel(g32["g_manning"], g64["g_manning"]),
                                              "grad_inlet_q_rel": rel(g32["g_inletq"], g64["g_inletq"]),
                                              "grad_zb_rel_linf": rel(g32["g_zb"], g64["g_zb"])}
    a, b = final["fp32c"], final["fp64"]
    out["error_fp32c_vs_fp64_state_rel_linf"] = float(np.abs(a - b).max() / np.abs(b).max())
    out["error_steps"] = fixed_n
    out["config"] = ("Tsit5 adaptive (abstol 1e-6, reltol 1e-3) over %g s of the 1M-cell reach from its release; "
                     "value = accepted steps x cells / wall second; FP32C against FP64 after the same fixed steps "
                     "(the FP32C run's step count over the same time); the fixed-step Tsit5 adjoint (probe "
                     "loss, 64 probes) at half the initial CFL-0.4 step, FP32C and FP64" % args.tsit5_time)
    return out


def run_resistance(args, case, device):
    """State-dependent resistance in every RHS evaluation:
    Manning's n = sigmoid n(h) (process_ManningN_2D.jl:102-213) and a UDE
    closure n = NN(h) (two tanh layers of 8 with batch LayerNorm,
    process_UDE.jl:3-56) on the 1M-cell reach, res_steps CFL-0.4 SSP-RK2 steps
    (L2 flushed before each), FP32C and FP64, and FP32C against FP64."""
    N = len(case["cell_node_count"])
    rng = np.random.default_rng(12)
    theta, din = [], 1
    for w in (8, 8):   # Glorot-uniform weights, small biases, LayerNorm affine terms near 1 and 0
        lim = np.sqrt(6.0 / (din + w))
        theta += [rng.uniform(-lim, lim, w * din), rng.uniform(-0.2, 0.2, w), rng.uniform(0.5, 1.5, w),
                  rng.uniform(-0.3, 0.3, w)]
        din = w
    theta += [rng.uniform(-np.sqrt(6.0 / 9.0), np.sqrt(6.0 / 9.0), 8), rng.uniform(-0.2, 0.2, 1)]
    theta = np.concatenate(theta)
    out = {"cells": N, "steps": args.res_steps}
    for kind in ("sigmoid", "ude"):
        final = {}
        for prec in ("fp32c", "fp64"):
            c = make_ctx(case, prec, device)
            if kind == "sigmoid":
                c.set_manning_function("sigmoid", [0.02, 0.06, 3.0, 0.8])
            else:
                c.set_ude("ManningN_h", [8, 8], ["tanh", "tanh"], theta, output_bounds=(0.02, 0.06),
                          h_bounds=(0.0, 4.0), layernorm_over_batch=True)
            c.upload(case["Q0"])
            c.advance_timed(args.warmup, cfl=0.4, flush_l2=True)
            c.upload(case["Q0"])
            ms = c.advance_timed(args.res_steps, cfl=0.4, flush_l2=True)
            final[prec] = c.download()
            out.setdefault(kind, {})[prec] = {"value": N * args.res_steps / (ms * 1e-3),
                                              "ms_per_step": ms / args.res_steps}
            c.close()
        a, b = final["fp32c"], final["fp64"]
        out[kind]["error_fp32c_vs_fp64_state_rel_linf"] = float(np.abs(a - b).max() / np.abs(b).max())
    out["config"] = ("sigmoid n(h) {0.02, 0.06, 3, 0.8} and a UDE n = NN(h) (8-8 tanh, batch LayerNorm, output in "
                     "[0.02, 0.06]) recomputed from every RHS evaluation's state, 1M-cell reach, SSP-RK2 CFL 0.4")
    return out


def run_config1(args, device, cpu):
    """Configuration 1 (hydrograd_gb.workloads.dam_break): 200 x 40 quads
    (8,000 cells) over 100 x 20 m, flat bed, walls, n = 0.03, h = 1.0 / 0.5 m
    either side of x = 50 m; config1_steps SSP-RK2 steps of dt = 0.01 s.  FP64
    and FP32C device rates (the steps replayed from captured CUDA graphs: at
    8,000 cells a step is launch-bound); with cpu (rank 0, unless --no-cpu),
    the oracle's rate on the host cores (the CPU baseline of this
    configuration) and both device states against the oracle's after the same
    steps."""
    from hydrograd_gb import SWE2D
    from hydrograd_gb.workloads import dam_break
    case = dam_break()
    N = len(case["cell_node_count"])
    K, dt = args.config1_steps, 0.01
    out = {"cells": N, "steps": K, "dt": dt}
    states = {}
    for prec in ("fp64", "fp32c"):
        c = SWE2D(case, precision=prec, device=device)
        c.set_still_water(case["wstill"])
        c.set_manning_zones(case["mat_id"], case["manning_zones"])
        c.upload(case["Q0"])
        c.advance(max(args.warmup, 50), dt=dt)
        c.upload(case["Q0"])
        c.synchronize()
        t0 = time.perf_counter()
        c.advance(K, dt=dt)
        c.synchronize()
        el = time.perf_counter() - t0
        states[prec] = c.download()
        out[prec] = {"value": N * K / el, "seconds": el}
        c.close()
    if cpu:
        from oracle.oracle import Oracle
        o = Oracle(case)
        o.set_wstill(case["wstill"])
        o.set_manning_cells(case["manning_zones"][case["mat_id"]])
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = o.rk2(case["Q0"], K, dt=dt, nthreads=threads)
        el = time.perf_counter() - t0
        out["cpu_oracle"] = {"value": N * K / el, "seconds": el, "cores": threads, "kind": "port"}
        # max |error| / max |state| over the whole state; and per block (xi, qx, qy) over
        # max(|block|, 1e-3 |state|) -- the dam break moves along x, so its qy block is
        # rounding noise and takes the floor
        for prec in ("fp64", "fp32c"):
            out[prec + "_vs_oracle_state_rel_linf"] = float(np.abs(states[prec] - ref).max() / np.abs(ref).max())
            out[prec + "_vs_oracle_block_rel_linf"] = [float(
                np.abs(states[prec][j * N:(j + 1) * N] - ref[j * N:(j + 1) * N]).max()
                / max(np.abs(ref[j * N:(j + 1) * N]).max(), 1e-3 * np.abs(ref).max(), 1e-300)) for j in range(3)]
    out["config"] = ("configuration 1: 200 x 40 quads (8,000 cells), flat bed, walls, n = 0.03, dam break "
                     "h = 1.0 / 0.5 m at x = 50 m, SSP-RK2 dt = 0.01 s")
    return out


def run_config5(args, device):
    """Configuration 5 (hydrograd_gb.workloads.meander_mixed): 4.0 M mixed
    cells, a meandering channel, per-cell n, the inlet hydrograph 200 -> 2,000
    m^3/s over 3,600 s.  FP32C forward over config5_steps CFL-0.4 steps (L2
    flushed before each); FP32C vs FP64 over config5_err_steps steps; the FP32C
    checkpointed forward+adjoint w.r.t. the per-cell n over config5_steps fixed
    steps, and its gradient against the FP64 adjoint's over config5_err_steps."""
    from hydrograd_gb import SWE2D
    from hydrograd_gb.workloads import Stream, meander_mixed
    t0 = time.perf_counter()
    case = meander_mixed()
    N = len(case["cell_node_count"])

    def ctx_for(prec):
        c = SWE2D(case, precision=prec, device=device)
        c.set_still_water(case["wstill"])
        c.set_manning_cells(case["manning_cells"])
        c.set_inlet_q(case["inlet_q"])
        c.set_exit_wse(case["exit_wse"])
        c.set_inlet_hydrograph(0, *case["hydrograph"])
        return c
    c32 = ctx_for("fp32c")
    setup_s = time.perf_counter() - t0
    Q0 = case["Q0"]
    c32.upload(Q0)
    c32.advance_timed(args.warmup, cfl=0.4, flush_l2=True)
    c32.upload(Q0)
    ms = c32.advance_timed(args.config5_steps, cfl=0.4, flush_l2=True)
    sim = c32.elapsed_time()
    out = {"cells": N, "quads": int((case["cell_node_count"] == 4).sum()),
           "triangles": int((case["cell_node_count"] == 3).sum()), "setup_seconds": setup_s,
           "fwd": {"value": N * args.config5_steps / (ms * 1e-3), "steps": args.config5_steps,
                   "ms_per_step": ms / args.config5_steps, "simulated_seconds": sim,
                   "inlet_q_at_end": float(np.interp(sim, *case["hydrograph"]))}}
    c64 = ctx_for("fp64")
    k = args.config5_err_steps
    a, _ = c64.integrate(Q0, k, cfl=0.4)
    b, _ = c32.integrate(Q0, k, cfl=0.4)
    out["error_fp32c_vs_fp64"] = {"steps": k, "state_rel_linf": float(max(
        np.abs(b[j * N:(j + 1) * N] - a[j * N:(j + 1) * N]).max() / np.abs(a).max() for j in range(3)))}
    # forward+adjoint w.r.t. the per-cell n: 64 probes in the wet cells, loss =
    # mean squared departure of their depths from the lake at rest
    dt = 0.5 * c64.integrate(Q0, 1, cfl=0.4)[1][0]
    rs = Stream(11)
    probes = np.unique((rs.uniform(256) * N).astype(np.int64))[:64].astype(np.int32)
    h_rest = case["wstill"] - case["zb_cells"]
    obs = np.tile(h_rest[probes], (args.config5_steps, 1))
    # warm-up at the timed size: the stage-state tape is allocated outside the timed call
    c32.loss_and_grad(Q0, args.config5_steps, dt, probes, obs, ckpt_every=50, want=("manning",))
    t0 = time.perf_counter()
    r = c32.loss_and_grad(Q0, args.config5_steps, dt, probes, obs, ckpt_every=50, want=("manning",))
    el = time.perf_counter() - t0
    out["fwd_adjoint"] = {"value": N * args.config5_steps / el, "steps": args.config5_steps, "seconds": el,
                          "checkpoint_every": 50, "probes": int(len(probes)), "gradient": "per-cell Manning n"}
    ra = c64.loss_and_grad(Q0, k, dt, probes, obs[:k], ckpt_every=50, want=("manning",))
    rb = c32.loss_and_grad(Q0, k, dt, probes, obs[:k], ckpt_every=50, want=("manning",))
    out["fwd_adjoint"]["error_fp32c_vs_fp64"] = {
        "steps": k, "grad_n_field_rel_linf": float(np.abs(rb["g_manning"] - ra["g_manning"]).max()
                                                   / np.abs(ra["g_manning"]).max()),
        "loss_rel": float(abs(rb["loss"] - ra["loss"]) / abs(ra["loss"]))}
    out["config"] = ("configuration 5: %d cells (%d quads in a core, %d jittered triangles in a band) over a "
                     "10 km reach, meandering channel 4 m deep, per-cell n U[0.02, 0.08] smoothed by a 100 m "
                     "Gaussian, inlet hydrograph 200 -> 2,000 m3/s over 3,600 s, FP32C, CFL 0.4"
                     % (N, out["quads"], out["triangles"]))
    return out


# Configuration 4: reach meshes of about these many cells, 32 members each.
ENSEMBLE_SIZES = (5000, 10000, 20000, 40000, 60000, 100000, 150000, 200000)


def run_ensemble(args, device):
    """hg_ensemble_create over 8 meshes x 32 members (about 18.7 M member-cells):
    per member zone n ~ U[0.02, 0.06] and inlet Q ~ U[100, 800]; each member
    takes its own CFL step and keeps its own clock.  FP32C forward steps, then
    one forward+adjoint (fixed dt) with 8 probes per member."""
    from hydrograd_gb import SWE2DEnsemble
    from hydrograd_gb.workloads import Stream, probes_and_perturbation, river_triangles
    meshes = [river_triangles(n=int(round((s / 2) ** 0.5))) for s in ENSEMBLE_SIZES]
    member_mesh = np.repeat(np.arange(len(meshes)), args.ens_members)
    rs = Stream(7)
    t0 = time.perf_counter()
    e = SWE2DEnsemble(meshes, member_mesh, precision="fp32c", device=device)
    setup_s = time.perf_counter() - t0
    cases = [meshes[m] for m in member_mesh]
    e.set_still_water(e.concat([c["wstill"] for c in cases]))
    mat, zones, base = [], [], 0
    for c in cases:
        mat.append(c["mat_id"] + base)
        zones.append(rs.uniform(len(c["manning_zones"]), 0.02, 0.06))
        base += len(c["manning_zones"])
    e.set_manning_zones(np.concatenate(mat).astype(np.int32), np.concatenate(zones))
    e.set_inlet_q(rs.uniform(len(cases), 100.0, 800.0))
    e.set_exit_wse(e.concat([c["exit_wse"] for c in cases], "exit"))
    Q0 = e.concat([c["Q0"] for c in cases], "state")
    N = e.n_cells
    e.upload(Q0)
    e.advance_timed(args.warmup, cfl=0.4, flush_l2=True)
    e.upload(Q0)
    ms = e.advance_timed(args.ens_steps, cfl=0.4, flush_l2=True)
    out = {"members": int(e.n_members), "meshes": [len(m["cell_node_count"]) for m in meshes], "member_cells": N,
           "setup_seconds": setup_s,
           "fwd": {"value": N * args.ens_steps / (ms * 1e-3), "steps": args.ens_steps, "ms_per_step": ms / args.ens_steps,
                   "simulated_seconds": e.elapsed_time()}}
    if args.ens_adj_steps > 0:
        dt = 0.5 * e.integrate(Q0, 1, cfl=0.4)[1][0]
        per_mesh = [probes_and_perturbation(m, 8, inlet_share=0.5)[0] for m in meshes]
        probes = np.concatenate([per_mesh[m] + e.cell_offset[i] for i, m in enumerate(member_mesh)]).astype(np.int32)
        h_rest = np.concatenate([c["wstill"] - c["zb_cells"] for c in cases])
        obs = np.tile(h_rest[probes], (args.ens_adj_steps, 1))
        e.loss_and_grad(Q0, args.ens_adj_steps, dt, probes, obs, ckpt_every=args.ens_ckpt)   # warm-up / allocation
        t0 = time.perf_counter()
        e.loss_and_grad(Q0, args.ens_adj_steps, dt, probes, obs, ckpt_every=args.ens_ckpt)
        el = time.perf_counter() - t0
        out["fwd_adjoint"] = {"value": N * args.ens_adj_steps / el, "steps": args.ens_adj_steps, "seconds": el,
                              "checkpoint_every": args.ens_ckpt, "probes": int(len(probes))}
    e.close()
    return out


def run_ours(args):
    rank, ws, local, dist = dist_setup()
    from hydrograd_gb import PinnedBuffer
    from hydrograd_gb.workloads import river_triangles
    case = river_triangles(n=args.n)
    N = len(case["cell_node_count"])
    nfaces_cell = None
    out = {}
    ctxs = {}
    for prec in ("fp32c", "fp64"):
        ctx = make_ctx(case, prec, local)
        ctxs[prec] = ctx
        nfaces_cell = ctx.n_faces / N
        steps = args.steps if prec == "fp32c" else args.steps_fp64
        # Clocks: nvidia-smi samples every 200 ms, longer than a short timed
        # region, so the sampler starts before the warm-up, which keeps the
        # GPU under the same load (graph replays of the same steps) until it
        # has a few samples, and it stops after the timed region.
        sampler = ClockSampler(local) if prec == "fp32c" else None
        if sampler:
            sampler.__enter__()
            ctx.upload(case["Q0"])
            t_load = time.perf_counter()
            while len(sampler.rows) < 4 and time.perf_counter() - t_load < 5.0:
                ctx.advance(100, cfl=0.4, graph=True)
                ctx.synchronize()
        ctx.upload(case["Q0"])
        ctx.advance_timed(args.warmup, cfl=0.4, flush_l2=True)
        ctx.upload(case["Q0"])
        barrier(dist)
        l0 = ctx.launch_count()
        ms = ctx.advance_timed(steps, cfl=0.4, flush_l2=True)
        if sampler:
            sampler.__exit__()
        launches = ctx.launch_count() - l0 - 2 * steps   # minus the L2 flushes (write + read kernel)
        ms = max_over_ranks(dist, ms)
        barrier(dist)
        out[prec] = dict(ms=ms, steps=steps, value=replica_value(ws, N * steps, ms * 1e-3), launches=launches,
                         clocks=sampler.summary() if sampler else None, state=ctx.download(),
                         sim_time=ctx.elapsed_time())
        # Continuous run without flushes (L2 kept warm), for reference.
        ctx.upload(case["Q0"])
        ctx.advance(args.warmup, cfl=0.4)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.advance(steps, cfl=0.4, graph=True)
        ctx.synchronize()
        out[prec]["warm_value"] = N * steps / (time.perf_counter() - t0)
        # Stage kernel alone (roofline).
        ctx.upload(case["Q0"])
        out[prec]["stage_ms"] = ctx.time_stage_kernel(20, True)
        if prec == "fp32c":
            out[prec]["stage_kernel"] = ctx.autotune(0)   # the kernel the autotuner chose
            out[prec]["stage_variant"] = ctx.autotune_info()[1]
    # FP32C error vs the FP64 path over the whole run (same CFL rule; the FP64
    # path itself is checked against the oracle below and by the GPU tests).
    a, b = out["fp32c"]["state"], out["fp64"]["state"]
    err = {}
    if args.steps == args.steps_fp64:
        err["fp32c_vs_fp64_state_rel_linf"] = float(max(
            np.abs(a[k * N:(k + 1) * N] - b[k * N:(k + 1) * N]).max() / max(np.abs(b).max(), 1e-300) for k in range(3)))
        err["fp32c_vs_fp64_state_rel_l2"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    # End to end through the C ABI with host (pinned) buffers: hg_integrate of
    # e2e_chunk steps per call, H2D of the state in and D2H of the state out per call.
    ctx = ctxs["fp32c"]
    host = PinnedBuffer(3 * N)
    host.array[:] = case["Q0"]
    ctx.integrate(host.array, 2, cfl=0.4)
    calls = max(1, args.steps // args.e2e_chunk)
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(calls):
        ctx.integrate(host.array, args.e2e_chunk, cfl=0.4, inplace=True)
    el = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": replica_value(ws, N * args.e2e_chunk * calls, el), "unit": UNIT,
           "h2d_bytes_per_step": 3 * N * 8 / args.e2e_chunk, "d2h_bytes_per_step": 3 * N * 8 / args.e2e_chunk,
           "calls": calls, "steps_per_call": args.e2e_chunk}
    # Forward + adjoint: hg_loss_and_grad over adj_steps fixed-dt steps (the CFL
    # step of the initial state), checkpoints every 50 steps, 64 probes.
    adj = {}
    if args.adj_steps > 0:
        from hydrograd_gb.workloads import probes_and_perturbation
        probes, _ = probes_and_perturbation(case, 64, inlet_share=0.5)
        c64 = ctxs["fp64"]
        dt_adj = 0.5 * c64.integrate(case["Q0"], 1, cfl=0.4)[1][0]
        # Observations: the probe depths of the lake at rest, so that the loss
        # measures the bore and the inflow (residuals of 0.01-1 m, well above
        # the FP32C state error, so the gradient comparison is well conditioned).
        h_rest = case["wstill"] - case["zb_cells"]
        obs = np.tile(h_rest[probes], (args.adj_steps, 1))
        grads = {}
        for prec in ("fp32c", "fp64"):
            ctx = ctxs[prec]
            ctx.loss_and_grad(case["Q0"], args.adj_steps, dt_adj, probes, obs, ckpt_every=50)   # warm-up / allocation
            barrier(dist)
            t0 = time.perf_counter()
            r = ctx.loss_and_grad(case["Q0"], args.adj_steps, dt_adj, probes, obs, ckpt_every=50)
            el = max_over_ranks(dist, time.perf_counter() - t0)
            grads[prec] = r
            adj[prec] = {"value": replica_value(ws, N * args.adj_steps, el), "seconds": el, "steps": args.adj_steps}
        g32, g64 = grads["fp32c"], grads["fp64"]
        zones = case["mat_id"]
        gz32 = np.array([g32["g_manning"][zones == z].sum() for z in range(len(case["manning_zones"]))])
        gz64 = np.array([g64["g_manning"][zones == z].sum() for z in range(len(case["manning_zones"]))])
        adj["fp32c_over_fp64_speedup"] = adj["fp32c"]["value"] / adj["fp64"]["value"]
        adj["error_fp32c_vs_fp64"] = {
            "grad_zone_n_rel": float(np.abs(gz32 - gz64).max() / np.abs(gz64).max()),
            "grad_inlet_q_rel": float(abs(g32["g_inletq"][0] - g64["g_inletq"][0]) / abs(g64["g_inletq"][0])),
            "grad_zb_field_rel_linf": float(np.abs(g32["g_zb"] - g64["g_zb"]).max() / np.abs(g64["g_zb"]).max()),
            "loss_rel": float(abs(g32["loss"] - g64["loss"]) / abs(g64["loss"])),
        }
        # The interior VJP kernel alone (roofline of the reverse sweep's dominant kernel).
        c32 = ctxs["fp32c"]
        c32.upload(case["Q0"])
        adj["vjp_ms"] = c32.time_vjp_kernel(20, True)
        adj["fp32c"]["ms_per_step"] = adj["fp32c"]["seconds"] * 1e3 / args.adj_steps
        adj["fp32c"]["reverse_over_forward"] = (adj["fp32c"]["ms_per_step"] - out["fp32c"]["ms"] / out["fp32c"]["steps"]) \
            / (out["fp32c"]["ms"] / out["fp32c"]["steps"])
        adj["config"] = (f"{args.adj_steps} fixed-dt steps (dt = half the initial CFL step), checkpoint spacing 50 "
                         "widened by the automatic stage-state tape (all steps kept where they fit in HBM), "
                         f"{len(probes)} probes (half on the pool rim, half at the inlet), loss = mean squared "
                         "departure of the probe depths from the lake at rest")
    hll = run_hll(args, case, local) if args.hll_steps > 0 else None
    ts5 = run_tsit5(args, case, local) if args.tsit5_time > 0 else None
    res = run_resistance(args, case, local) if args.res_steps > 0 else None
    dry = run_dry_start(args, local) if args.dry_steps > 0 else None
    cfg1 = run_config1(args, local, cpu=not args.no_cpu and rank == 0) if args.config1_steps > 0 else None
    cfg5 = run_config5(args, local) if args.config5_steps > 0 else None
    ens = None
    if args.ens_steps > 0:
        ens = run_ensemble(args, local)
        ens["config"] = ("configuration 4: 8 reach meshes x %d members, per-member zone n and inlet Q, "
                         "FP32C, each member on its own CFL 0.4 step, L2 flushed before every timed step"
                         % args.ens_members)
    if rank != 0:
        return
    peak, peak_kind = load_peaks()
    cell_b, face_b = BYTES_STAGE["fp32c"]
    bytes_stage = (cell_b + nfaces_cell * face_b) * N
    achieved = bytes_stage / (out["fp32c"]["stage_ms"] * 1e-3) / 1e9
    kern = out["fp32c"]["stage_kernel"]
    kname = STAGE_KERNELS[kern][0]
    variant = out["fp32c"].get("stage_variant", 0)
    if kern == 0:
        kname = kname[:-1] + "; " + GATHER_SHAPES.get(variant, "") + ")"
    # the DRAM traffic from the capture of the chosen kernel (and shape, where it has its own)
    tr = profile_traffic("fp32c", name="k_stage_f32_t128_river_tri_1M.md") if (kern == 0 and variant == 3) \
        else profile_traffic("fp32c", kern)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None if tr is None else tr * N, "kernel": kname + ", one RK2 stage pass",
            "algorithmic_bytes_per_launch": bytes_stage, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"}
    if adj and "vjp_ms" in adj:
        bytes_vjp = (BYTES_VJP_FP32C[0] + nfaces_cell * BYTES_VJP_FP32C[1]) * N
        a_vjp = bytes_vjp / (adj["vjp_ms"] * 1e-3) / 1e9
        tv = profile_traffic("fp32c", name=VJP_PROFILE)
        adj["roofline"] = {"bound": "hbm", "achieved": a_vjp, "peak": peak, "unit": "GB/s", "frac": a_vjp / peak,
                           "traffic": None if tv is None else tv * N,
                           "kernel": "k_vjp_pipe_f32 (interior VJP of one stage, boundary faces folded in)",
                           "algorithmic_bytes_per_launch": bytes_vjp,
                           "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"}
    fp64_bytes = (BYTES_STAGE["fp64"][0] + nfaces_cell * BYTES_STAGE["fp64"][1]) * N
    cpu = None
    if not args.no_cpu:
        cpu, o = cpu_baseline(case, args.cpu_seconds)
        # FP64 path vs the oracle on the full mesh, a short horizon.
        ctx64 = ctxs["fp64"]
        q_gpu, dts = ctx64.integrate(case["Q0"], args.oracle_steps, cfl=0.4)
        qo = case["Q0"].copy()
        for d in dts:
            qo = o.rk2(qo, 1, dt=float(d), nthreads=os.cpu_count() or 1)
        err["fp64_vs_oracle_state_rel_linf"] = float(max(
            np.abs(q_gpu[k * N:(k + 1) * N] - qo[k * N:(k + 1) * N]).max() / max(np.abs(qo).max(), 1e-300)
            for k in range(3)))
        err["fp64_vs_oracle_steps"] = args.oracle_steps
    f32 = out["fp32c"]
    line = {
        "metric": METRIC, "value": f32["value"], "unit": UNIT, "n_gpus": ws, "steps": f32["steps"],
        "warmup": args.warmup, "ms_per_step": f32["ms"] / f32["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (hi+lo compensated state)", "data": "synthetic",
        "config": {"workload": workload_name(case, N), "cells": N, "faces": ctxs["fp32c"].n_faces,
                   "l2": "flushed before every timed step: 256 MB written, then a different 256 MB read "
                         "(L2 left with clean lines only), outside the timed events",
                   "order": "hilbert", "parallelism": "replicas" if ws > 1 else "single GPU"},
        "fp64": {"value": out["fp64"]["value"], "ms_per_step": out["fp64"]["ms"] / out["fp64"]["steps"],
                 "steps": out["fp64"]["steps"], "stage_ms": out["fp64"]["stage_ms"],
                 "stage_gbs": fp64_bytes / (out["fp64"]["stage_ms"] * 1e-3) / 1e9,
                 "warm_value": out["fp64"]["warm_value"]},
        "fp32c_over_fp64_speedup": f32["value"] / out["fp64"]["value"],
        # like for like: the FP64 device path against the FP64 oracle on the
        # host cores (the reference arm's implementation)
        "fp64_vs_reference": None if cpu is None else out["fp64"]["value"] / cpu["value"],
        "fwd_adjoint": adj,
        "ensemble": ens,
        "hll": hll,
        "tsit5": ts5,
        "resistance": res,
        "dry_start": dry,
        "config1": cfg1,
        "config5": cfg5,
        "warm_value": f32["warm_value"], "simulated_seconds": f32["sim_time"],
        "error": err,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": f32["launches"],
        "clocks": f32["clocks"],
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=708, help="grid size: 2 n^2 triangles")
    ap.add_argument("--steps-fp64", type=int, default=None)
    ap.add_argument("--e2e-chunk", type=int, default=100)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--oracle-steps", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--adj-steps", type=int, default=100, help="steps of the forward+adjoint measurement (0: skip)")
    ap.add_argument("--ens-steps", type=int, default=1000, help="ensemble (configuration 4) forward steps (0: skip)")
    ap.add_argument("--ens-adj-steps", type=int, default=1000,
                    help="ensemble (configuration 4) forward+adjoint steps (0: skip)")
    ap.add_argument("--ens-ckpt", type=int, default=25)
    ap.add_argument("--ens-members", type=int, default=32, help="members per mesh")
    ap.add_argument("--tsit5-time", type=float, default=1.0,
                    help="simulated seconds of the Tsit5 leg on the 1M-cell reach (0: skip)")
    ap.add_argument("--tsit5-adj-steps", type=int, default=10, help="steps of the Tsit5 adjoint leg, FP32C and FP64 (0: skip)")
    ap.add_argument("--res-steps", type=int, default=200,
                    help="CFL steps of the state-dependent resistance leg (0: skip)")
    ap.add_argument("--hll-steps", type=int, default=500,
                    help="FP32C steps of the HLL-solver leg on the 1M-cell reach (0: skip)")
    ap.add_argument("--dry-steps", type=int, default=2000,
                    help="steps of the dry-start leg (configuration 2's written dry-pool start; 0: skip)")
    ap.add_argument("--config1-steps", type=int, default=1000,
                    help="configuration 1 (8,000-cell dam break) steps at dt = 0.01 s (0: skip)")
    ap.add_argument("--config5-steps", type=int, default=5000,
                    help="configuration 5 (4 M mixed cells, hydrograph) forward and forward+adjoint steps (0: skip)")
    ap.add_argument("--config5-err-steps", type=int, default=200,
                    help="configuration 5 steps of the FP32C-vs-FP64 state and gradient comparison")
    ap.add_argument("--profile-stage", default=None, choices=["fp32c", "fp64"],
                    help="only run the stage kernel a few times (a small case for ncu captures)")
    ap.add_argument("--profile-adjoint", default=None, choices=["fp32c", "fp64"],
                    help="only run one short forward+adjoint (a small case for ncu captures)")
    ap.add_argument("--profile-adj-steps", type=int, default=4, help="steps of the --profile-adjoint run")
    ap.add_argument("--profile-adj-ckpt", type=int, default=2, help="checkpoint spacing of the --profile-adjoint run")
    args = ap.parse_args()
    if args.steps_fp64 is None:
        args.steps_fp64 = args.steps
    args.warmup = max(args.warmup, 3)
    if args.profile_stage:
        profile_stage(args)
    elif args.profile_adjoint:
        profile_adjoint(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


def profile_stage(args):
    """Workload state after `warmup` CFL steps, then 3 stage-kernel launches
    (each after an L2 flush): launches 1-2 of k_stage_* are warm-up, 3 is the one to capture."""
    from hydrograd_gb.workloads import river_triangles
    case = river_triangles(n=args.n)
    ctx = make_ctx(case, args.profile_stage, 0)
    ctx.upload(case["Q0"])
    ctx.advance(args.warmup, cfl=0.4, graph=False)
    ctx.synchronize()
    ms = ctx.time_stage_kernel(3, True)
    print(json.dumps({"precision": args.profile_stage, "cells": len(case["cell_node_count"]), "stage_ms": ms}))


def profile_adjoint(args):
    """One forward+adjoint of --profile-adj-steps fixed-dt steps (default 4,
    checkpoints every --profile-adj-ckpt, default 2) on the workload: with the
    defaults, 8 VJP launches after the 4 + 4 forward stage pairs."""
    from hydrograd_gb.workloads import probes_and_perturbation, river_triangles
    case = river_triangles(n=args.n)
    ctx = make_ctx(case, args.profile_adjoint, 0)
    probes, _ = probes_and_perturbation(case, 64)
    dt = 0.5 * ctx.integrate(case["Q0"], 1, cfl=0.4)[1][0]
    K = args.profile_adj_steps
    obs = np.tile(case["Q0"][probes], (K, 1))
    t0 = time.perf_counter()
    r = ctx.loss_and_grad(case["Q0"], K, dt, probes, obs, ckpt_every=args.profile_adj_ckpt)
    print(json.dumps({"precision": args.profile_adjoint, "cells": len(case["cell_node_count"]), "loss": r["loss"],
                      "seconds": time.perf_counter() - t0}))


if __name__ == "__main__":
    main()
