"""Benchmark of the DG residual path on one GB300 (or N independent replicas, one per GPU).

Workload: 3D compressible Euler isentropic vortex (strength 5, axis along z, free stream (1,1,1,0,1)) on the periodic
box [-5,5]^2 x [0,2.5] with 32x32x8 HEX elements, p = 3 (GLL solution / GL cubature), Roe-Pike flux.  One step is one
SSP-RK3 time step = 3 residual evaluations over all 2,621,440 DOF.  Unit: DOF/s = n_DOF * residual evaluations / s.

Arms:
  (default)          the GPU path through the C ABI (dpg_gpu_rk_step on device-resident state; e2e through
                     dpg_gpu_rk_step_host with pinned host buffers, copies inside the timed region);
  --impl reference   the CPU oracle (the reference's algorithm restated in serial C), one process per host core,
                     each step one residual evaluation of the full mesh per process.
Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DG residual DOF/s split-prec vs FP64 at equal L2 err; implicit solve time vs plain"
UNIT = "DOF/s"
WORKLOAD = dict(d=3, p=3, n_elem=(32, 32, 8), lo=(-5.0, -5.0, 0.0), hi=(5.0, 5.0, 2.5))
WORKLOAD_NAME = "3D Euler isentropic vortex, periodic [-5,5]^2x[0,2.5], 32x32x8 HEX, p=3, Roe-Pike, one SSP-RK3 step"
L2_BYTES = 129 * 1024 * 1024


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _sync_ranks(ws: int, device: str = "cuda"):
    """Device synchronisation and, with several ranks, a barrier: both sides of every timed region."""
    import torch
    if device == "cuda":
        torch.cuda.synchronize()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(vals, ws: int, device: str = "cuda"):
    """Element-wise maximum of a list of floats over the ranks (the slowest replica sets the time)."""
    if ws == 1:
        return [float(v) for v in vals]
    import torch
    import torch.distributed as dist
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def _aggregate_rate(ws: int, n_dof: int, evals: int, seconds: float) -> float:
    """Whole-job DOF/s: every replica evaluates its own copy of the workload (weak scaling)."""
    return ws * n_dof * evals / seconds


def _prec_arg(s: str):
    import dpgsolver_gb300 as dg
    if s == "fp64":
        return dg.PREC_FP64, 0, "f64"
    if s == "bf16x3":
        return dg.PREC_BF16X3, 0, "bf16x3"
    if s == "tf32x3":
        return dg.PREC_TF32X3, 0, "tf32x3"
    if s.startswith("sliced"):
        tail = s[len("sliced"):].lstrip(":")
        n = int(tail) if tail else 7
        return dg.PREC_BF16_SLICED, n, f"bf16-sliced{n}"
    raise SystemExit(f"unknown --prec {s}")


# ------------------------------------------------------------------------------------------------------------
# CPU legs: the oracle on its own set-up (never the library: neither arm below imports dpgsolver_gb300 for it)
# ------------------------------------------------------------------------------------------------------------
def _cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def _oracle(threads: int):
    from oracle import Oracle, Problem, build_oracle
    build_oracle()
    return Oracle(Problem(**WORKLOAD), threads=threads)


def _cfl_dt(u, n_vol: int, n_var: int, cfl: float = 0.4) -> float:
    """dt = CFL h / (max(|V| + c) (2p + 1)) over the solution nodes of the state u (the library's cfl_dt)."""
    import numpy as np
    d, p = WORKLOAD["d"], WORKLOAD["p"]
    w = u.reshape(n_vol, n_var, -1)
    rho, m, E = w[:, 0], w[:, 1:1 + d], w[:, d + 1]
    V2 = np.sum((m / rho[:, None]) ** 2, axis=1)
    pres = 0.4 * (E - 0.5 * rho * V2)
    smax = float(np.max(np.sqrt(V2) + np.sqrt(1.4 * pres / rho)))
    h = (WORKLOAD["hi"][0] - WORKLOAD["lo"][0]) / WORKLOAD["n_elem"][0]
    return cfl * h / (smax * (2 * p + 1))


def cpu_baseline_port(n_warm: int = 1, n_eval: int = 5) -> dict:
    """The oracle (serial C restatement of compute_rhs_dg) on one core: median of n_eval residual evaluations of
    the full workload after n_warm untimed ones."""
    orc = _oracle(1)
    u = orc.initial_solution()
    for _ in range(n_warm):
        orc.compute_rhs(u)
    times = []
    for _ in range(n_eval):
        t0 = time.perf_counter()
        orc.compute_rhs(u)
        times.append(time.perf_counter() - t0)
    med = statistics.median(times)
    return {"value": orc.n_dof / med, "unit": UNIT, "cores": 1, "kind": "port", "cpu": _cpu_model(),
            "sample": f"median of {n_eval} FP64 residual evaluations (after {n_warm} untimed) of the full "
                      f"32x32x8 HEX p=3 mesh by the oracle (serial C restatement of compute_rhs_dg), 1 thread",
            "seconds_per_residual": times}


def run_reference(args):
    """--impl reference: the reference's CPU algorithm (the oracle port: compute_rhs_dg, time_step_ssp_rk_33 with
    the positivity limiter) on all host threads, on the same workload; one step = one SSP-RK3 step of the full mesh.
    Under torchrun only rank 0 runs; the other ranks return without work."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    t_wall = time.time()
    orc = _oracle(threads)
    u = orc.initial_solution()
    dt = _cfl_dt(u, orc.n_vol, orc.layout["n_var"])
    for _ in range(args.warmup):
        orc.rk_step(u, dt, 1)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.rk_step(u, dt, 1)
        times.append(time.perf_counter() - t0)
    value = orc.n_dof * 3 * args.steps / sum(times)
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * sum(times) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded analytic initial state)",
        "config": {"workload": WORKLOAD_NAME, "n_dof": orc.n_dof, "residual_evals_per_step": 3, "dt": dt},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "cpu": _cpu_model(),
                         "sample": f"{args.steps} SSP-RK3 steps (3 residual evaluations + positivity limiter each) of "
                                   f"the full mesh by the oracle on {threads} host threads, after {args.warmup} "
                                   f"untimed steps"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.time() - t_wall,
    }
    print(json.dumps(out), flush=True)


def _against_oracle(dg, np, sim, ctx, mode, n_slices, tiles_used, dt, n_steps):
    """The split path and the FP64 form on the GPU against the FP64 oracle from the same initial state (the
    oracle's own), step by step over n_steps SSP-RK3 steps: per step the state difference of each form and the
    difference of the split residual evaluated at the oracle's state; every 10 steps the L2 errors of the three
    against the exact solution.  "Equal L2 error" is read on the L2 norm of the whole error vector (all
    variables) relative to the oracle's, at every sample; per variable the line reports the largest relative
    difference among the variables whose exact error is not rounding noise (the vortex's w-momentum is exactly
    zero: its L2 error, ~1e-15, is rounding alone)."""
    orc = _oracle(os.cpu_count() or 1)
    u0 = orc.initial_solution()
    ctx.upload(u0)
    c64 = dg.GpuContext(sim)
    c64.upload(u0)
    cres = dg.GpuContext(sim)
    cres.set_precision(mode, n_slices)
    cres.set_tiles(**tiles_used)
    uo = u0.copy()
    rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    per_step, l2 = [], []
    t0 = time.perf_counter()
    for s in range(1, n_steps + 1):
        cres.upload(uo)
        cres.compute_rhs()
        _, r_or = orc.compute_rhs(uo)
        r_rel = rel(cres.rhs(), r_or)
        orc.rk_step(uo, dt, 1)
        ctx.rk_step(dt, 1)
        c64.rk_step(dt, 1)
        us, u64 = ctx.download(), c64.download()
        per_step.append({"step": s, "residual_rel_diff_split": r_rel, "state_rel_diff_split": rel(us, uo),
                         "state_rel_diff_fp64": rel(u64, uo)})
        if s % 10 == 0 or s == n_steps:
            eo, es, e6 = orc.l2_error(uo, s * dt), orc.l2_error(us, s * dt), orc.l2_error(u64, s * dt)
            no = float(np.sqrt(np.sum(eo ** 2)))
            l2.append({"step": s, "oracle": [float(x) for x in eo], "split": [float(x) for x in es],
                       "fp64": [float(x) for x in e6],
                       "total_rel_diff_split": abs(float(np.sqrt(np.sum(es ** 2))) - no) / no,
                       "total_rel_diff_fp64": abs(float(np.sqrt(np.sum(e6 ** 2))) - no) / no,
                       "per_variable_rel_diff_split": [float(x) for x in np.abs(es - eo) / eo],
                       "per_variable_rel_diff_fp64": [float(x) for x in np.abs(e6 - eo) / eo]})
    c64.close()
    cres.close()
    last = l2[-1]
    return {"steps": n_steps, "dt": dt, "seconds": time.perf_counter() - t0,
            "max_residual_rel_diff_split": max(p["residual_rel_diff_split"] for p in per_step),
            "max_state_rel_diff_split": max(p["state_rel_diff_split"] for p in per_step),
            "max_state_rel_diff_fp64": max(p["state_rel_diff_fp64"] for p in per_step),
            "l2_total_rel_diff_split": last["total_rel_diff_split"],
            "l2_total_rel_diff_fp64": last["total_rel_diff_fp64"],
            "l2_total_rel_diff_split_max": max(e["total_rel_diff_split"] for e in l2),
            "l2_total_rel_diff_fp64_max": max(e["total_rel_diff_fp64"] for e in l2),
            "l2_nonzero_variable_rel_diff_split_max": max(
                max(x for x, o in zip(e["per_variable_rel_diff_split"], e["oracle"]) if o > 1e-12) for e in l2),
            "l2_nonzero_variable_rel_diff_fp64_max": max(
                max(x for x, o in zip(e["per_variable_rel_diff_fp64"], e["oracle"]) if o > 1e-12) for e in l2),
            "equal_l2_within_1e-10": bool(max(e["total_rel_diff_split"] for e in l2) <= 1e-10),
            "l2_every_10_steps": l2, "per_step": per_step}


# ------------------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------------------
def run_gpu(args):
    import ctypes as C

    import numpy as np
    import torch

    import dpgsolver_gb300 as dg

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    mode, n_slices, dtype_name = _prec_arg(args.prec)

    sim = dg.Simulation(dg.Config(**WORKLOAD))
    n_dof = sim.n_dof
    ctx = dg.GpuContext(sim)
    ctx.set_precision(mode, n_slices)
    # block configuration of the split kernels: the autotuner's pick on the initial state (outside the timed
    # region; it times whole residual evaluations), or the one given on the command line
    tiles = None
    if mode != dg.PREC_FP64:
        tiles = {"wave_rule": ctx.tiles()}
        if args.tiles:
            eb, share, warps = (int(t) for t in args.tiles.split(","))
            ctx.set_tiles(eb, share, warps)
            tiles["source"] = "command line"
        else:
            t0 = time.perf_counter()
            _, tune_ms = ctx.autotune(10)
            tiles.update(source="autotuner", tune_seconds=time.perf_counter() - t0, tuned_ms_per_residual=tune_ms)
        tiles["used"] = ctx.tiles()
    h = 10.0 / WORKLOAD["n_elem"][0]
    dt = sim.cfl_dt(0.4, h)
    lib = dg.load_library()
    stream_ev = lib  # kernels run on the context stream; timing below uses the library's event timer

    # L2 flush buffer (> L2) written between timed steps
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        ctx.rk_step(dt, 1)
    torch.cuda.synchronize()

    # device-time of each step with CUDA events recorded on the context stream
    step_ms = _time_steps(lib, ctx, dt, args.steps, flush)
    clocks_sampler = ClockSampler(local)
    clocks_sampler.start()
    _sync_ranks(ws)
    step_ms = _time_steps(lib, ctx, dt, args.steps, flush)
    _sync_ranks(ws)
    clocks = clocks_sampler.stop()
    t_dev = sum(step_ms) / 1000.0

    # e2e: host buffers (pinned), H2D + steps + D2H inside the timed region, through dpg_gpu_rk_step_host
    host = torch.empty(n_dof, dtype=torch.float64, pin_memory=True).numpy()
    host[:] = sim.sol_coef()
    ctx.rk_step_host(host, dt, 1)
    _sync_ranks(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.rk_step_host(host, dt, 1)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    _sync_ranks(ws)

    # per-kernel device times (events on the context stream) for the roofline
    kt = ctx.kernel_times(5)

    # the FP64 form of the same step on the same GPU (its speed), and both forms against the FP64 oracle
    fp64 = None
    oracle_cmp = None
    if mode != dg.PREC_FP64:
        c64 = dg.GpuContext(sim)
        c64.rk_step(dt, 1)
        fp64_ms = [_one_step_ms(lib, c64, dt) for _ in range(3)]
        fp64 = {"value": n_dof * 3 / (min(fp64_ms) / 1000.0), "unit": UNIT, "ms_per_step": min(fp64_ms),
                "kernel_ms": c64.kernel_times(2)}
        c64.close()
        if args.oracle_steps > 0 and rank == 0:
            oracle_cmp = _against_oracle(dg, np, sim, ctx, mode, n_slices, ctx.tiles(), dt, args.oracle_steps)

    implicit = _implicit_comparison(dg, np) if (args.implicit and rank == 0) else None
    implicit_euler = _implicit_comparison_euler(dg, np) if (args.implicit and rank == 0) else None
    ns_line = _navier_stokes_residual(dg, np, lib) if (args.implicit and rank == 0) else None
    implicit_full = _implicit_full_size(dg) if (args.implicit and args.implicit_full and rank == 0) else None
    tri_line = _advection_tri(dg, np, lib) if (args.implicit and rank == 0) else None
    tet_line = _advection_tet(dg, np, lib) if (args.implicit and rank == 0) else None
    euler_tet_line = _euler_tet(dg, np, lib) if (args.implicit and rank == 0) else None

    t_max, e2e_max = _max_over_ranks([t_dev, t_e2e], ws)
    if ws > 1:
        _sync_ranks(ws)
    if rank != 0:
        return

    evals = 3 * args.steps
    value = _aggregate_rate(ws, n_dof, evals, t_max)
    e2e_value = _aggregate_rate(ws, n_dof, evals, e2e_max)
    peaks, peak_kind = _peaks()
    roof = _roofline(sim, kt, mode, peaks, peak_kind)
    cpu = cpu_baseline_port() if (not args.no_cpu_baseline and ws == 1) else None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype_name, "data": "synthetic (seeded analytic initial state)",
        "config": {"workload": WORKLOAD_NAME, "n_dof": n_dof, "residual_evals_per_step": 3,
                   "precision": dtype_name, "l2": "flushed between timed steps (256 MiB write)",
                   "parallelism": f"replicas x{ws}", "tiles": tiles},
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n_dof * 8, "d2h_bytes_per_step": n_dof * 8},
        "gpu_launches": (3 * 3 + (3 if "positivity" in kt else 0)) * args.steps,   # per RK stage: 3 + limiter
        "kernel_ms": kt,
        "fp64_form": fp64,
        "speedup_vs_fp64_form": (value / ws / fp64["value"]) if fp64 else None,
        "against_oracle": oracle_cmp,
        "implicit": implicit,
        "implicit_euler_periodic": implicit_euler,
        "navier_stokes_residual": ns_line,
        "implicit_full": implicit_full,
        "advection_tri": tri_line,
        "advection_tet": tet_line,
        "euler_tet": euler_tet_line,
    }
    print(json.dumps(out), flush=True)


TC = dict(d=2, p=3, mesh="annulus", lo=(1.0, 0.0, 0.0), hi=(2.0, 0.0, 0.0), pde="navier_stokes", mu=5e-3, Pr=0.72,
          omega=0.5, test_case="taylor_couette", bc=("noslip_all_rotating", "noslip_adiabatic"))


def _implicit_comparison(dg, np, n_elem=(16, 32)):
    """Second half of the metric: time to the steady state ||F||_inf <= 1e-10 of the 2D Navier-Stokes flow between
    rotating cylinders (radii 1 and 2, inner wall speed 0.5, mu = 5e-3 (Re = 100 on the inner radius), Pr = 0.72, BR2 +
    Roe-Pike, curved QUADs p = 3) by matrix-free Newton-GMRES with pseudo-transient continuation, from the uniform-
    pressure Taylor-Couette state, with:
      "plain": the reference's settings for this case -- local pseudo time steps by CFL ramping from cfl_initial
               10 (navier_stokes/steady/taylor_couette/test_case.data) and the default linear solver, GMRES(60),
               rtol 1e-4, ILU (petsc_options_gmres_default.txt) -- with the block ILU(0) of the element-block
               matrix in volume order, factorised on 4 contiguous subdomains (as PETSc's block-Jacobi / ILU on
               several processes);
      "block_jacobi": exact element blocks (tangent probing + batched LU), GMRES(500), rtol 1e-3;
      "learned": the learned block inverse (2 x 256 hidden ReLU MLP on the tensor cores, trained on the block-Jacobi
               run's element blocks), same GMRES settings, falling back to block-Jacobi when GMRES misses 10x rtol.
    Times are the library's own wall clock of each solve; the network's training is reported apart."""
    sim = dg.Simulation(dg.Config(**TC, n_elem=(n_elem[0], n_elem[1], 1)))
    ctx = dg.GpuContext(sim)
    u0 = sim.sol_coef()
    kw = dict(dtau0=0.1, gmres_restart=500, max_gmres=1500, gmres_rtol=1e-3, max_newton=60)
    plain_kw = dict(cfl_initial=10.0, gmres_restart=60, max_gmres=600, gmres_rtol=1e-4, max_newton=60,
                    ilu_order=dg.api.ILU_ORDER_VOLUME, ilu_parts=4)

    def solve(precond, settings, **extra):
        ctx.upload(u0)
        try:
            st = ctx.newton_solve(precond, tol=1e-10, **{**settings, **extra})
            return {"converged": True, "newton": st.newton_iterations, "gmres": st.gmres_iterations,
                    "seconds": st.seconds, "assembly_seconds": st.assembly_seconds, "residual": st.residual_final,
                    "fallback_steps": st.fallback_steps}
        except dg.DpgError as e:
            return {"converged": False, "status": e.status}

    plain = solve(dg.PRECOND_BLOCK_ILU, plain_kw)
    ctx.mlp_enable(hidden=256, capacity=sim.n_vol * kw["max_newton"], seed=1)
    bj = solve(dg.PRECOND_BLOCK_JACOBI, kw, collect_blocks=1)
    samples = ctx.mlp_samples()
    t0 = time.perf_counter()
    loss = ctx.mlp_train(epochs=40, batch=512, lr=1e-3)
    train_s = time.perf_counter() - t0
    learned = solve(dg.PRECOND_MLP, kw)
    learned.update(train_seconds=train_s, samples=samples, final_loss=loss)
    ratio = (learned["seconds"] / plain["seconds"]) if learned.get("converged") and plain.get("converged") else None
    ratio_bj = (learned["seconds"] / bj["seconds"]) if learned.get("converged") and bj.get("converged") else None
    return {"problem": f"2D Navier-Stokes Taylor-Couette annulus {n_elem[0]}x{n_elem[1]} curved QUADs p=3 "
                       f"({sim.n_dof} DOF), BR2 + Roe-Pike, ||F||_inf <= 1e-10",
            "settings": {"plain": {**plain_kw, "preconditioner": "block ILU(0), volume order, 4 subdomains",
                                   "pseudo_time": "local CFL ramping"},
                         "block_jacobi_and_learned": kw},
            "plain": plain, "block_jacobi": bj, "learned": learned,
            "learned_over_plain_time": ratio, "learned_over_block_jacobi_time": ratio_bj}


def _implicit_full_size(dg):
    """The Navier-Stokes configuration at full size (64 x 128 curved QUADs p = 3, 524,288 DOF) from the
    uniform-pressure state to ||F||_inf <= 1e-10: block ILU(0) on 16 subdomains of the volume order, GMRES(300),
    rtol 1e-4, local CFL ramping from 10.  Block-Jacobi and the learned inverse do not converge at this size
    (restarted GMRES stagnates once the pseudo time steps grow)."""
    sim = dg.Simulation(dg.Config(**TC, n_elem=(64, 128, 1)))
    ctx = dg.GpuContext(sim)
    ctx.upload(sim.sol_coef())
    kw = dict(cfl_initial=10.0, gmres_restart=300, max_gmres=1500, gmres_rtol=1e-4, max_newton=60,
              ilu_order=dg.api.ILU_ORDER_VOLUME, ilu_parts=16)
    try:
        st = ctx.newton_solve(dg.PRECOND_BLOCK_ILU, tol=1e-10, **kw)
        res = {"converged": True, "newton": st.newton_iterations, "gmres": st.gmres_iterations, "seconds": st.seconds,
               "assembly_seconds": st.assembly_seconds, "residual": st.residual_final}
    except dg.DpgError as e:
        res = {"converged": False, "status": e.status}
    return {"problem": f"2D Navier-Stokes Taylor-Couette annulus 64x128 curved QUADs p=3 ({sim.n_dof} DOF), "
                       "||F||_inf <= 1e-10", "settings": kw, "block_ilu": res}


def _implicit_comparison_euler(dg, np):
    """Second half of the metric: time to a steady state with matrix-free Newton-GMRES (pseudo-transient
    continuation) with the reference's default linear solver ("plain": GMRES(60), rtol 1e-4, block ILU(0)), with
    block-Jacobi, and with the learned block inverse trained on the block-Jacobi run's element blocks.  Problem: 2D Euler on a periodic 8x8 QUAD p=2 mesh, a uniform stream
    with velocity (0.6, 0.3) as the manufactured root (its residual is subtracted as a forcing), started from the
    root plus a seeded perturbation with zero totals; converged when ||F||_inf <= 1e-10.  Jacobian products and element blocks come from the analytic
    linearisation (tangents); "block_jacobi_fd" repeats the block-Jacobi solve with finite differences instead.
    Times are the library's own wall-clock of each solve."""
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(8, 8, 1), test_case="free_stream",
                                  vortex=(5.0, 0.0, 0.0, 1.0, 0.6, 0.3, 0.0, 1.0)))
    ctx = dg.GpuContext(sim)
    u_star = sim.sol_coef()
    ctx.upload(u_star)
    ctx.compute_rhs()
    forcing = ctx.rhs()
    r = np.random.default_rng(7).standard_normal(u_star.shape).reshape(sim.n_vol, -1)
    d = 1e-2 * (r - np.roll(r, 1, axis=0))          # element differences: zero totals on the uniform mesh
    u0 = u_star + d.ravel()

    def solve(precond, **kw):
        ctx.upload(u0)
        try:
            st = ctx.newton_solve(precond, tol=1e-10, forcing=forcing, dtau0=10.0, **kw)
            return {"converged": True, "newton": st.newton_iterations, "gmres": st.gmres_iterations,
                    "seconds": st.seconds, "residual": st.residual_final, "fallback_steps": st.fallback_steps}
        except dg.DpgError as e:
            return {"converged": False, "status": e.status}

    ctx.mlp_enable(hidden=256, capacity=16 * sim.n_vol, seed=1)
    bj = solve(dg.PRECOND_BLOCK_JACOBI, max_newton=40, collect_blocks=1)
    bj_fd = solve(dg.PRECOND_BLOCK_JACOBI, max_newton=40, jacobian=dg.JACOBIAN_FD)
    t0 = time.perf_counter()
    ctx.mlp_train(epochs=300, batch=64, lr=1e-3)
    train_s = time.perf_counter() - t0
    learned = solve(dg.PRECOND_MLP, max_newton=40)
    learned["train_seconds"] = train_s
    plain = solve(dg.PRECOND_BLOCK_ILU, max_newton=40, gmres_restart=60, max_gmres=600, gmres_rtol=1e-4)
    ratio = (learned["seconds"] / plain["seconds"]) if learned.get("converged") and plain.get("converged") else None
    ratio_bj = (learned["seconds"] / bj["seconds"]) if learned.get("converged") and bj.get("converged") else None
    return {"problem": "2D Euler free stream (0.6, 0.3) + zero-total perturbation, periodic 8x8 QUAD p=2, "
                       "||F||_inf <= 1e-10", "plain": plain, "block_jacobi": bj, "block_jacobi_fd": bj_fd,
            "learned": learned,
            "learned_over_plain_time": ratio,
            "learned_over_block_jacobi_time": ratio_bj}   # solve times; the network's training is reported apart


def _navier_stokes_residual(dg, np, lib):
    """The Navier-Stokes configuration at full size (64 x 128 curved QUADs, p = 3, 524,288 DOF): FP64 residual
    throughput of the general chain and its parity with the oracle (all host threads) at a perturbed state."""
    sim = dg.Simulation(dg.Config(**TC, n_elem=(64, 128, 1)))
    ctx = dg.GpuContext(sim)
    from oracle import Oracle
    orc = Oracle(sim, threads=os.cpu_count() or 1)
    u = orc.initial_solution() * (1.0 + 1e-3 * np.random.default_rng(2).standard_normal(sim.n_dof))
    ctx.upload(u)
    ctx.compute_rhs()
    _, r_ref = orc.compute_rhs(u)
    rel = float(np.max(np.abs(ctx.rhs() - r_ref)) / np.max(np.abs(r_ref)))
    kt = ctx.kernel_times(10)
    ms = kt["residual"]
    t0 = time.perf_counter()
    orc.compute_rhs(u)
    cpu_s = time.perf_counter() - t0
    return {"workload": "2D Navier-Stokes Taylor-Couette annulus 64x128 curved QUADs p=3, BR2 + Roe-Pike, FP64",
            "n_dof": sim.n_dof, "ms_per_residual": ms, "dof_per_s": sim.n_dof / (ms * 1e-3),
            "launches_per_residual": lib.dpg_gpu_launches_per_rhs(ctx.handle),
            "rel_diff_vs_oracle": rel, "oracle_dof_per_s": sim.n_dof / cpu_s, "oracle_threads": os.cpu_count()}


def _advection_tri(dg, np, lib):
    """The advection configuration's element type and mesh: 2D linear advection, velocity (1, 0.5), upwind flux, on a
    periodic unit square of 64 x 64 cells split into 8,192 triangles with vertices jittered by up to 0.1 h (seeded).
    One uniform order per run, p = 1..4, and the configuration itself: each triangle's order drawn uniformly from
    {1, 2, 3, 4} (seeded), all orders in each of the three launches of a residual.  FP64 residual throughput (CUDA
    events on the library stream) and parity with the oracle's own set-up (all host threads); at one order per mesh
    also the split-precision modes' parity and the S = 7 residual time."""
    from oracle import Oracle
    rows = []
    for p in (1, 2, 3, 4, "1-4"):
        mixed = p == "1-4"
        cfg = dg.Config(d=2, p=1 if mixed else p, p_max=4 if mixed else 0, p_seed=5, n_elem=(64, 64, 1),
                        element="tri", pde="advection", num_flux="upwind", test_case="advection_sine",
                        lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=11, b_adv=(1.0, 0.5, 0.0))
        sim = dg.Simulation(cfg)
        ctx = dg.GpuContext(sim)
        orc = Oracle(cfg, threads=os.cpu_count() or 1)
        u = orc.initial_solution()
        ctx.upload(u)
        ctx.compute_rhs()
        _, r_ref = orc.compute_rhs(u)
        rel = float(np.max(np.abs(ctx.rhs() - r_ref)) / np.max(np.abs(r_ref)))
        kt = ctx.kernel_times(20)
        ms = sum(v for k, v in kt.items() if k != "positivity")
        t0 = time.perf_counter()
        orc.compute_rhs(u)
        cpu_s = time.perf_counter() - t0
        row = {"p": p, "n_dof": sim.n_dof, "ms_per_residual": ms, "dof_per_s": sim.n_dof / (ms * 1e-3),
               "rel_diff_vs_oracle": rel, "oracle_dof_per_s": sim.n_dof / cpu_s}
        if not mixed:   # the split modes (one order per mesh): residual parity, and the S = 7 residual time
            split = {}
            for name, mode, ns in (("bf16_sliced7", dg.PREC_BF16_SLICED, 7), ("tf32x3", dg.PREC_TF32X3, 0),
                                   ("bf16x3", dg.PREC_BF16X3, 0)):
                ctx.set_precision(mode, ns)
                ctx.upload(u)
                ctx.compute_rhs()
                entry = {"rel_diff_vs_oracle": float(np.max(np.abs(ctx.rhs() - r_ref)) / np.max(np.abs(r_ref)))}
                if name == "bf16_sliced7":
                    kt = ctx.kernel_times(20)
                    ms7 = sum(v for k, v in kt.items() if k != "positivity")
                    entry.update({"ms_per_residual": ms7, "dof_per_s": sim.n_dof / (ms7 * 1e-3)})
                split[name] = entry
            ctx.set_precision(dg.PREC_FP64, 0)
            row["split"] = split
        rows.append(row)
        ctx.close()
    return {"workload": "2D linear advection, 64x64 cells split into 8192 jittered TRIs, upwind, FP64 (and the split "
                        "modes at one order per mesh); uniform p and p drawn per element from {1,2,3,4} (p = '1-4')",
            "oracle_threads": os.cpu_count(), "per_order": rows}


def _advection_tet(dg, np, lib):
    """Tetrahedra at the size of the mixed 3D configuration: 3D linear advection, velocity (1, 0.5, 0.25), upwind
    flux, a periodic unit cube of 32^3 cells split into 196,608 tetrahedra with vertices jittered by up to 0.1 h
    (seeded); orders drawn per element from {1, 2, 3, 4} (FP64, `kernels_hp.cu`), and one order p = 2 in FP64 and
    in split precision (S = 7).  Residual time by CUDA events on the library stream; parity with the oracle's own
    TET set-up (all host threads) on the same problem at 12^3 cells (the oracle's symmetrised face rules make its
    set-up of the full mesh take minutes)."""
    from oracle import Oracle
    rows = []
    for p, p_max in ((1, 4), (2, 0)):
        row = {"p": "1-4" if p_max else p}
        for n, timed in ((12, False), (32, True)):
            cfg = dg.Config(d=3, p=p, p_max=p_max, p_seed=3, n_elem=(n, n, n), element="tet", pde="advection",
                            num_flux="upwind", test_case="advection_sine", lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1,
                            seed=2, b_adv=(1.0, 0.5, 0.25))
            sim = dg.Simulation(cfg)
            ctx = dg.GpuContext(sim)
            if timed:
                row.update(n_vol=sim.n_vol, n_dof=sim.n_dof)
                u = sim.sol_coef()
            else:
                orc = Oracle(cfg, threads=os.cpu_count() or 1)
                u = orc.initial_solution()
                _, r_ref = orc.compute_rhs(u)
            modes = [("fp64", dg.PREC_FP64, 0)] + ([] if p_max else [("bf16_sliced7", dg.PREC_BF16_SLICED, 7)])
            for name, mode, ns in modes:
                ctx.set_precision(mode, ns)
                ctx.upload(u)
                ctx.compute_rhs()
                entry = row.setdefault(name, {})
                if timed:
                    kt = ctx.kernel_times(10)
                    ms = sum(v for k, v in kt.items() if k != "positivity")
                    entry.update(ms_per_residual=ms, dof_per_s=sim.n_dof / (ms * 1e-3))
                else:
                    entry["rel_diff_vs_oracle_12cubed"] = float(np.max(np.abs(ctx.rhs() - r_ref)) / np.max(np.abs(r_ref)))
            ctx.close()
        rows.append(row)
    return {"workload": "3D linear advection, 32^3 cells split into 196608 jittered TETs, upwind; orders 1..4 per "
                        "element (FP64) and p = 2 (FP64, split S = 7)", "oracle_threads": os.cpu_count(),
            "rows": rows}


def _euler_tet(dg, np, lib):
    """The Euler equations on tetrahedra at the size of the mixed 3D configuration: periodic isentropic vortex (axis
    along z, strength 5) on [-5,5]^2 x [0,2.5] meshed by 32^3 cells split into 196,608 tetrahedra with vertices
    jittered by up to 0.1 h, Roe-Pike flux, p = 2 and 3, FP64 and split precision (S = 7), and orders drawn per
    element from 1..4 (FP64, every order in each launch, the limiter per order group).  Per residual: the CUDA-event
    times of its kernels plus the dense positivity limiter of one RK stage; parity with the oracle's own set-up (the
    reference's Witherden-Vincent rules, all host threads) at 8^3 cells."""
    import json as _json, itertools as _it
    from oracle import Oracle, Problem
    gold = _json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                                        "reference_goldens.json")))["wv_rules"]

    def wv(kind, st):
        g = gold[kind][str(st)]
        a = np.array([list(q) + [w] for b, w in zip(g["bary"], g["w"]) for q in sorted(set(_it.permutations(b)))])
        a[:, -1] /= a[:, -1].sum()
        return a
    rows = []
    for p, p_max in ((2, 0), (3, 0), (1, 4)):
        row = {"p": f"{p}-{p_max}" if p_max else p}
        for n, timed in ((8, False), (32, True)):
            c = dict(d=3, p=p, p_max=p_max, p_seed=3, n_elem=(n, n, n), element="tet", pde="euler",
                     num_flux="Roe-Pike", test_case="isentropic_vortex", lo=(-5, -5, 0), hi=(5, 5, 2.5), jitter=0.1,
                     seed=2)
            sim = dg.Simulation(dg.Config(**c))
            ctx = dg.GpuContext(sim)
            u = sim.sol_coef()
            if timed:
                row.update(n_vol=sim.n_vol, n_dof=sim.n_dof)
            elif p_max:   # orders 1..4: the oracle on the library's set-up (no WV rule of strength 8 is derived)
                orc = Oracle(data_model=lib.dpg_sim_view(sim.handle), threads=os.cpu_count() or 1)
                _, r_ref = orc.compute_rhs(u)
            else:
                orc = Oracle(Problem(**c, vol_rules={p: wv("tet", 2 * p)}, face_rules={p: wv("tri", 2 * p)}),
                             threads=os.cpu_count() or 1)
                _, r_ref = orc.compute_rhs(u)
            modes = [("fp64", dg.PREC_FP64, 0)] + ([] if p_max else [("bf16_sliced7", dg.PREC_BF16_SLICED, 7)])
            for name, mode, ns in modes:
                ctx.set_precision(mode, ns)
                ctx.upload(u)
                ctx.compute_rhs()
                entry = row.setdefault(name, {})
                if timed:
                    kt = ctx.kernel_times(10)
                    ms = sum(kt.values())
                    entry.update(ms_per_residual_with_limiter=ms, kernels_ms=kt, dof_per_s=sim.n_dof / (ms * 1e-3))
                else:
                    entry["rel_diff_vs_oracle_8cubed"] = float(np.max(np.abs(ctx.rhs() - r_ref)) / np.max(np.abs(r_ref)))
            ctx.close()
        rows.append(row)
    return {"workload": "3D Euler isentropic vortex, 32^3 cells split into 196608 jittered TETs, Roe-Pike; p = 2, 3 "
                        "(FP64, split S = 7) and orders 1..4 per element (FP64); each residual with the positivity "
                        "limiter of one RK stage",
            "oracle_threads": os.cpu_count(), "rows": rows}


def _time_steps(lib, ctx, dt, n, flush):
    import torch
    # Events on torch's current stream cannot see the library's stream, so time each step by synchronising the
    # library stream (rk_step returns after reading back the norm) and measuring device time with the library's
    # own event timer on its stream.
    ms = []
    for _ in range(n):
        flush.zero_()
        torch.cuda.synchronize()
        ms.append(_one_step_ms(lib, ctx, dt))
    return ms


def _one_step_ms(lib, ctx, dt):
    import ctypes as C
    out = C.c_double()
    rc = lib.dpg_gpu_time_rk_steps(ctx.handle, dt, 1, C.byref(out))
    if rc != 0:
        raise RuntimeError(f"dpg_gpu_time_rk_steps failed: {rc}")
    return out.value


# Algorithmic bytes per element of each kernel of one residual evaluation (the compute_rhs form timed by
# kernel_times: no RK stage update), from the operand sizes of the workload: n_s solution nodes, n_c volume
# cubature nodes, n_fl local faces with n_fc face nodes each, NV variables, d dimensions.  Each face's numerical
# flux is computed once (the face kernel is counted per element through n_fl / 2 faces per element).
def _bytes_per_element(sim, split):
    d, NV = sim.d, sim.n_var
    n_s, n_c, n_fc = sim.n_s, sim.n_c, sim.n_fc
    n_fl = 2 * d
    nfq = n_fl * n_fc
    faces_per_elem = n_fl / 2
    face = faces_per_elem * n_fc * (2 * NV * 8 + d * 8 + 8 + 4 + NV * 8)   # two traces, normal, |J_f|, nc_fc; nnf
    if split:
        # traces, normals and |J_f| as FP32 pairs (8 bytes per value); the flux written to both elements' lift rows
        interp = n_s * NV * 8 + d * d * 8 + nfq * NV * 8 + d * n_c * NV * 8 + NV * 4   # U; metrics; traces; fr; bounds
        face = faces_per_elem * (n_fc * (2 * NV * 8 + d * 8 + 8 + 4 + 2 * NV * 8) + 8 + 2 * NV * 4)   # + sides; bounds
        lift = (nfq + d * n_c) * NV * 8 + NV * 32 + 8 + n_s * NV * 8   # lift operand row; 8 bound slots; 1/detJ; rhs
        return {"trace": interp, "face": face, "volume": lift, "positivity": n_s * NV * 8}
    trace = n_s * NV * 8 + nfq * NV * 8
    volume = n_s * NV * 8 + n_s * NV * 8 + d * d * 8 + 8 + nfq * NV * 8 + n_fl * 4
    # positivity limiter of an RK stage: reads the state; writes only the volumes it corrects (none on this workload)
    return {"trace": trace, "face": face, "volume": volume, "positivity": n_s * NV * 8}


_KERNEL_NAMES = {True: {"trace": "ks_interp", "face": "ks_face", "volume": "ks_lift", "positivity": "k_positivity"},
                 False: {"trace": "k_trace", "face": "k_face", "volume": "k_volume", "positivity": "k_positivity"}}


def _ncu_traffic():
    """DRAM bytes per element of each kernel from the committed ncu summary of this workload (one capture of
    dram__bytes_read.sum + dram__bytes_write.sum per launch, divided by the elements of the captured case)."""
    path = os.path.join(ROOT, "profiles", "launch_list_split_hex_p3_32x32x8.md")   # both forms were captured
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("dram_bytes_per_element:"):
                    return {k: float(v) for k, v in (t.split("=") for t in line.split(":", 1)[1].split())}
    except OSError:
        pass
    return None


def _algorithmic_per_residual(sim):
    """Algorithmic work of one residual evaluation in the reference's dense formulation.
    Bytes: the compulsory FP64 state traffic (sol_coef read + rhs write, 16 B per DOF) plus the geometry as the
    reference stores it (metrics_vc: n_c d^2 doubles per volume; normals_fc and jacobian_det_fc: n_fc (d + 1)
    doubles per face); the operators, read once per (element type, order), are negligible.
    Flops: interpolation, d weak derivatives and m_inv per volume, 2 n_c n_s n_var (1 + d) + 2 n_s^2 n_var, plus
    per face and side the trace interpolation and the lift, 2 n_fc n_s n_var + 2 n_s n_fc n_eq (pointwise fluxes
    excluded)."""
    d, NV, n_s, n_c, n_fc = sim.d, sim.n_var, sim.n_s, sim.n_c, sim.n_fc
    bytes_ = sim.n_dof * 16 + sim.n_vol * n_c * d * d * 8 + sim.n_face * n_fc * (d + 1) * 8
    flops = sim.n_vol * (2 * n_c * n_s * NV * (1 + d) + 2 * n_s * n_s * NV) + sim.n_face * 2 * (4 * n_fc * n_s * NV)
    return bytes_, flops


def _roofline(sim, kt, mode, peaks, peak_kind):
    """HBM roofline of one residual evaluation (its three launches: interpolation, face flux, lift): achieved =
    the algorithmic bytes of a residual / the summed CUDA-event durations of those launches on the library stream;
    traffic = their DRAM bytes per residual from the committed ncu summary (scaled per element), or null.  Every
    kernel is listed with its own time and the bytes this design moves through it ("design_bytes": intermediates
    included), which explain the gap."""
    import dpgsolver_gb300 as dg
    split = mode != dg.PREC_FP64
    n_vol = sim.n_vol
    per_elem = _bytes_per_element(sim, split)
    traffic = _ncu_traffic()
    names = _KERNEL_NAMES[split]
    kernels = {}
    for k, ms in kt.items():
        des = per_elem[k] * n_vol
        kernels[names[k]] = {"ms": ms, "design_bytes": des, "design_gbs": des / (ms * 1e-3) / 1e9,
                             "traffic": (traffic[names[k]] * n_vol) if traffic and names[k] in traffic else None}
    res_keys = [k for k in ("trace", "face", "volume") if k in kt]
    t_res = sum(kt[k] for k in res_keys) * 1e-3
    alg, flops = _algorithmic_per_residual(sim)
    ach = alg / t_res / 1e9
    tr = [kernels[names[k]]["traffic"] for k in res_keys]
    return {"bound": "hbm", "kernel": "residual (" + " + ".join(names[k] for k in res_keys) + ")",
            "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": ach / peaks["hbm_gbs"],
            "peak_source": f"hbm_gbs of {peak_kind}", "traffic": (sum(tr) if all(x is not None for x in tr) else None),
            "algorithmic_bytes_per_launch": alg, "residual_ms": t_res * 1e3,
            "fp64_equivalent_tflops": flops / t_res / 1e12, "algorithmic_flops_per_residual": flops,
            "kernels": kernels}


def run_case(case: str):
    """Small runs of one kernel family for profiler captures (see --case)."""
    import numpy as np
    import dpgsolver_gb300 as dg
    if case in ("ns", "ns_full", "ilu", "ilu_full"):
        full = case in ("ns_full", "ilu_full")
        sim = dg.Simulation(dg.Config(**TC, n_elem=(64, 128, 1) if full else (16, 32, 1)))
        ctx = dg.GpuContext(sim)
        ctx.upload(sim.sol_coef())
        if case in ("ns", "ns_full"):
            for _ in range(5):
                ctx.compute_rhs()
        else:
            try:
                ctx.newton_solve(dg.PRECOND_BLOCK_ILU, tol=1e-10, dtau0=0.1, max_newton=1 if full else 2,
                                 gmres_restart=300 if full else 60, max_gmres=120, gmres_rtol=1e-12 if full else 1e-4,
                                 ilu_parts=16 if full else 4)
            except dg.DpgError as e:
                if e.status != dg.api.DPG_ERR_NOT_CONVERGED:
                    raise
    elif case == "hp":
        sim = dg.Simulation(dg.Config(d=2, p=1, p_max=4, p_seed=5, n_elem=(64, 64, 1), element="tri",
                                      pde="advection", num_flux="upwind", test_case="advection_sine", lo=(0, 0, 0),
                                      hi=(1, 1, 1), jitter=0.1, seed=11, b_adv=(1.0, 0.5, 0.0)))
        ctx = dg.GpuContext(sim)
        ctx.upload(sim.sol_coef())
        for _ in range(5):
            ctx.compute_rhs()
    elif case == "euler_tet":   # 32^3 cells x 6 TETs, p = 3 Euler (157 MB state, larger than L2): stage + limiter
        sim = dg.Simulation(dg.Config(d=3, p=3, n_elem=(32, 32, 32), element="tet", pde="euler", num_flux="Roe-Pike",
                                      test_case="isentropic_vortex", lo=(-5, -5, 0), hi=(5, 5, 2.5), jitter=0.1,
                                      seed=2))
        ctx = dg.GpuContext(sim)
        ctx.upload(sim.sol_coef())
        ctx.rk_step(1e-4, 2)
    else:
        sim = dg.Simulation(dg.Config(**dict(TC, p=2), n_elem=(3, 12, 1)))
        ctx = dg.GpuContext(sim)
        ctx.upload(sim.sol_coef())
        ctx.mlp_enable(hidden=256, capacity=36 * 40, seed=1)
        try:
            ctx.newton_solve(dg.PRECOND_BLOCK_JACOBI, tol=1e-10, dtau0=1.0, max_newton=40, collect_blocks=1)
        except dg.DpgError as e:
            if e.status != dg.api.DPG_ERR_NOT_CONVERGED:
                raise
        ctx.mlp_train(epochs=2, batch=128, lr=1e-3)
    lib = dg.load_library()
    print(json.dumps({"case": case, "n_dof": sim.n_dof}), flush=True)
    del ctx, lib


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--prec", default="sliced7")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--oracle-steps", type=int, default=100,
                    help="SSP-RK3 steps of the split path and the FP64 form compared with the FP64 oracle (0: none)")
    ap.add_argument("--no-implicit", dest="implicit", action="store_false",
                    help="skip the implicit-solver comparison (profiling runs)")
    ap.add_argument("--tiles", default=None,
                    help="EB,SHARE,WARPS: use this split-kernel block configuration instead of the autotuner's "
                         "(profiling runs: the tuner's own timing launches stay out of the capture)")
    ap.add_argument("--n-elem", default=None,
                    help="profiling only: NX,NY,NZ HEX elements instead of the 32x32x8 workload (no bench line use)")
    ap.add_argument("--no-implicit-full", dest="implicit_full", action="store_false",
                    help="skip the Navier-Stokes configuration at its full size (64 x 128, p = 3) solved to 1e-10 with "
                         "the block ILU and GMRES(300) (about 1.5 minutes; the `implicit_full` key of the line)")
    ap.add_argument("--case", default=None, choices=["ns", "ns_full", "ilu", "ilu_full", "mlp", "hp", "euler_tet"],
                    help="profiling only: run a small case of one implicit-path kernel family and exit (no bench "
                         "line): ns = 5 FP64 Navier-Stokes residuals of the 16x32 p=3 annulus (ns_full: of the "
                         "64x128 one); ilu = 2 Newton steps, block ILU on 4 subdomains (ilu_full: 1 Newton step "
                         "with GMRES(300), 120 iterations, 16 subdomains, on the 64x128 annulus) "
                         "with the block ILU on it; mlp = 2 epochs of MLP training on block-Jacobi blocks of a "
                         "3x12 p=2 annulus; hp = 5 FP64 residuals of the mixed-order advection mesh (8192 TRIs, "
                         "p uniform in 1..4)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.n_elem:
        nx, ny, nz = (int(t) for t in args.n_elem.split(","))
        WORKLOAD["n_elem"] = (nx, ny, nz)
    if args.case:
        import __graft_entry__
        __graft_entry__.build()
        run_case(args.case)
    elif args.impl == "reference":
        run_reference(args)      # the oracle only: the library is neither built nor loaded in this arm
    else:
        import __graft_entry__
        __graft_entry__.build()
        run_gpu(args)


if __name__ == "__main__":
    main()
