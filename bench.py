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
# CPU oracle timing (cpu_baseline leg and the reference arm)
# ------------------------------------------------------------------------------------------------------------
def _oracle_worker(args):
    n_eval, q = args
    import dpgsolver_gb300 as dg
    from oracle import Oracle
    sim = dg.Simulation(dg.Config(**WORKLOAD))
    orc = Oracle(sim)
    sol = sim.sol_coef()
    times = []
    for _ in range(n_eval):
        t0 = time.perf_counter()
        orc.compute_rhs(sol)
        times.append(time.perf_counter() - t0)
    return sim.n_dof, times


def cpu_oracle_rate(n_proc: int, n_eval: int):
    """Aggregate DOF/s of n_proc independent oracle processes, each timing n_eval residual evaluations."""
    ctx = mp.get_context("spawn")
    with ctx.Pool(n_proc) as pool:
        res = pool.map(_oracle_worker, [(n_eval, None)] * n_proc)
    n_dof = res[0][0]
    # each process: n_eval residuals; aggregate over processes that ran concurrently
    per_proc = [n_dof * len(t) / sum(t) for _, t in res]
    return sum(per_proc), [t for _, t in res]


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    n_proc = os.cpu_count() or 1
    steps, warm = args.steps, args.warmup
    t0 = time.time()
    rate, times = cpu_oracle_rate(n_proc, warm + steps)
    # drop the warm-up evaluations of every process
    import dpgsolver_gb300 as dg
    n_dof = dg.Simulation(dg.Config(**WORKLOAD)).n_dof
    per_proc = [n_dof * steps / sum(t[warm:]) for t in times]
    value = sum(per_proc)
    ms = 1000.0 * max(sum(t[warm:]) for t in times) / steps
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": steps,
        "warmup": warm, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded analytic initial state)",
        "config": {"workload": WORKLOAD_NAME + " (reference arm: one residual evaluation per step per process)",
                   "n_dof": n_dof, "processes": n_proc},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": n_proc, "kind": "port",
                         "sample": f"{n_proc} independent processes x {steps} FP64 residual evaluations of the full "
                                   f"mesh (serial C restatement of compute_rhs_dg)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.time() - t0,
    }
    print(json.dumps(out), flush=True)


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

    # the FP64 form of the same step on the same GPU, and the split-vs-FP64 state difference after 10 steps
    fp64 = None
    if mode != dg.PREC_FP64:
        u0 = sim.sol_coef()
        ctx.upload(u0)
        ctx.rk_step(dt, 10)
        u_split = ctx.download()
        ctx.set_precision(dg.PREC_FP64, 0)
        ctx.upload(u0)
        ctx.rk_step(dt, 10)
        u_fp64 = ctx.download()
        fp64_ms = [_one_step_ms(lib, ctx, dt) for _ in range(3)]
        fp64_rate = n_dof * 3 / (min(fp64_ms) / 1000.0)
        # L2 errors against the exact (advected) vortex after the 10 steps, per variable, both forms
        sim.set_sol_coef(u_split)
        l2_split = sim.l2_error(10 * dt)
        sim.set_sol_coef(u_fp64)
        l2_fp64 = sim.l2_error(10 * dt)
        sim.set_sol_coef(u0)
        fp64 = {"value": fp64_rate, "unit": UNIT, "ms_per_step": min(fp64_ms),
                "state_rel_diff_after_10_steps": float(np.max(np.abs(u_split - u_fp64)) / np.max(np.abs(u_fp64))),
                "l2_error_after_10_steps": {"split": [float(x) for x in l2_split], "fp64": [float(x) for x in l2_fp64],
                                            # relative to the largest variable error (a variable whose exact
                                            # solution is constant has an L2 error at rounding level)
                                            "max_rel_diff": float(np.max(np.abs(l2_split - l2_fp64)) / np.max(l2_fp64))}}
        kt64 = ctx.kernel_times(2)
        fp64["kernel_ms"] = kt64

    implicit = _implicit_comparison(dg, np) if (args.implicit and rank == 0) else None

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
    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        rate, _ = cpu_oracle_rate(1, 2)
        cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "2 FP64 residual evaluations of the full 32x32x8 HEX p=3 mesh by the serial C oracle, 1 core"}
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
        "implicit": implicit,
    }
    print(json.dumps(out), flush=True)


def _implicit_comparison(dg, np):
    """Second half of the metric: time to a steady state with matrix-free Newton-GMRES (pseudo-transient
    continuation) without a preconditioner ("plain"), with block-Jacobi, and with the learned block inverse trained
    on the block-Jacobi run's element blocks.  Problem: 2D Euler on a periodic 8x8 QUAD p=2 mesh, a uniform stream
    with velocity (0.6, 0.3) as the manufactured root (its residual is subtracted as a forcing), started from the
    root plus a seeded perturbation with zero totals; converged when ||F||_inf <= 1e-10.  The plain solve gets the
    Newton budget of the block-Jacobi solve.  Jacobian products and element blocks come from the analytic
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

    ctx.mlp_enable(hidden=128, capacity=16 * sim.n_vol, seed=1)
    bj = solve(dg.PRECOND_BLOCK_JACOBI, max_newton=40, collect_blocks=1)
    bj_fd = solve(dg.PRECOND_BLOCK_JACOBI, max_newton=40, jacobian=dg.JACOBIAN_FD)
    t0 = time.perf_counter()
    ctx.mlp_train(epochs=300, batch=64, lr=1e-3)
    train_s = time.perf_counter() - t0
    learned = solve(dg.PRECOND_MLP, max_newton=40)
    learned["train_seconds"] = train_s
    t0 = time.perf_counter()
    plain = solve(dg.PRECOND_NONE, max_newton=bj.get("newton", 40), max_gmres=1000)
    plain.setdefault("seconds", time.perf_counter() - t0)
    ratio = (learned["seconds"] / plain["seconds"]) if learned.get("converged") and plain.get("converged") else None
    ratio_bj = (learned["seconds"] / bj["seconds"]) if learned.get("converged") and bj.get("converged") else None
    return {"problem": "2D Euler free stream (0.6, 0.3) + zero-total perturbation, periodic 8x8 QUAD p=2, "
                       "||F||_inf <= 1e-10", "plain": plain, "block_jacobi": bj, "block_jacobi_fd": bj_fd,
            "learned": learned,
            "learned_over_plain_time": ratio,
            "learned_over_block_jacobi_time": ratio_bj}   # solve times; the network's training is reported apart


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


def _roofline(sim, kt, mode, peaks, peak_kind):
    """HBM roofline of the dominant kernel (largest device time of one residual evaluation), with every kernel's
    figures beside it.  achieved = algorithmic bytes per launch / the launch's CUDA-event duration on the library
    stream; traffic = DRAM bytes per launch from the ncu summary (scaled per element), or null."""
    import dpgsolver_gb300 as dg
    split = mode != dg.PREC_FP64
    n_vol = sim.n_vol
    per_elem = _bytes_per_element(sim, split)
    traffic = _ncu_traffic()
    names = _KERNEL_NAMES[split]
    kernels = {}
    for k, ms in kt.items():
        alg = per_elem[k] * n_vol
        ach = alg / (ms * 1e-3) / 1e9
        kernels[names[k]] = {"ms": ms, "algorithmic_bytes": alg, "achieved_gbs": ach, "frac": ach / peaks["hbm_gbs"],
                             "traffic": (traffic[names[k]] * n_vol) if traffic and names[k] in traffic else None}
    dom = max(kt, key=lambda k: kt[k])
    kd = kernels[names[dom]]
    return {"bound": "hbm", "kernel": names[dom], "achieved": kd["achieved_gbs"], "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": kd["frac"], "peak_source": f"hbm_gbs of {peak_kind}", "traffic": kd["traffic"],
            "algorithmic_bytes_per_launch": kd["algorithmic_bytes"], "kernels": kernels}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--prec", default="sliced7")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-implicit", dest="implicit", action="store_false",
                    help="skip the implicit-solver comparison (profiling runs)")
    ap.add_argument("--tiles", default=None,
                    help="EB,SHARE,WARPS: use this split-kernel block configuration instead of the autotuner's "
                         "(profiling runs: the tuner's own timing launches stay out of the capture)")
    ap.add_argument("--n-elem", default=None,
                    help="profiling only: NX,NY,NZ HEX elements instead of the 32x32x8 workload (no bench line use)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.n_elem:
        nx, ny, nz = (int(t) for t in args.n_elem.split(","))
        WORKLOAD["n_elem"] = (nx, ny, nz)
    import __graft_entry__
    __graft_entry__.build()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
