"""Benchmark: batched uneven Heston MCS instances on one GB300 (grid-point-steps/s).

Workload (one "step"): one pass of the batched ADI path over 4096 uneven Heston call
instances drawn from numpy PCG64(20261203): kappa~U[0.5,5], theta~U[0.01,0.1],
sigma~U[0.1,1], rho~U[-0.95,0], r~U[0,0.05], T~U[0.25,2], K~U[80,120],
Nx in {64..256}, Ny in {32..128}, 100-400 steps each; modified Craig-Sneyd, FP64, one
persistent kernel, graph-launched.  value = sum(Nx*Ny*steps) / device time per step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--mode fwd|fwdadj]

Under torchrun (N > 1) every rank runs its own batch (seed + rank): weak scaling, no
collective on the data path; rank 0 prints the JSON line (max time over ranks).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 20261203
METRIC = "grid-point-steps/s, batched fwd+adjoint vs plain path, FP64 \u22641e-10 rel err"
BYTES_PER_GPS_FWD = {"dr": 40, "cs": 96, "mcs": 96, "hv": 96}  # algorithmic bytes per grid-point-step (FP64)
# Figures of one ncu capture each of the batched kernels on the 1024-instance, 40-step case
# (--count 1024 --max-time-steps 40; forward: --mode fwd; forward + adjoint: --mode fwdadj
# --workspace-gb 12, whose plan recomputes a fraction CAPTURE_RF = 0.4898 of the steps), per
# grid-point-step, scaled to a launch by the grid-point-steps it processes.  Forward + adjoint
# is one forward pass, the recomputation of every checkpoint segment but the last (a fraction rf
# of the steps) and the adjoint steps, so a figure X of it is X_FWD * (1 + rf) + X_ADJ, with X_ADJ
# what the forward + adjoint capture (at rf = CAPTURE_RF) leaves after its forward passes.
CAPTURE_RF = 0.4898
# DRAM bytes read + written (dram__bytes_read.sum + dram__bytes_write.sum): k_batch_forward,
# k_batch_fwdadj
DRAM_BYTES_FWD = 339.1
CAPTURE_DRAM_FWDADJ = 1026.9
DRAM_BYTES_ADJ = CAPTURE_DRAM_FWDADJ - DRAM_BYTES_FWD * (1.0 + CAPTURE_RF)
# FP64 instructions, thread level (smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum)
FP64_INSTR_FWD = 32.07
CAPTURE_FWDADJ = 139.30
FP64_INSTR_ADJ = CAPTURE_FWDADJ - FP64_INSTR_FWD * (1.0 + CAPTURE_RF)


# Adjoint workspace cap of the timed batch, as a fraction of the device memory (the library's
# default is a quarter; a larger cap stores more stage values and recomputes fewer steps)
WS_FRACTION = 0.8


def per_gps(fwd, adj, mode, rf):
    """A per-grid-point-step figure of the run: the forward kernel's, or forward + adjoint at the
    run's recomputed fraction rf."""
    return fwd if mode == 0 else fwd * (1.0 + rf) + adj


def fp64_rate(lib):
    """The FP64 pipe's rate measured on this device now (lss_diag_fp64_rate: thread-level DFMA/s,
    eight independent chains per thread, four 256-thread CTAs per SM, best of three launches)."""
    import ctypes

    from linear_system_solvers_gb300 import _lib as L

    r = ctypes.c_double()
    L.check(lib.lss_diag_fp64_rate(ctypes.byref(r), None))
    return r.value


def recompute_fraction(problems, intervals=None):
    """Grid-point-step weighted fraction of the steps the adjoint recomputes (every checkpoint
    segment but the last); `intervals`: the checkpoint interval of every instance
    (lss_adi_batch_checkpoints), default ceil(sqrt(steps))."""
    import math

    num = den = 0.0
    for k, p in enumerate(problems):
        steps = p.nt - 1
        c = int(intervals[k]) if intervals is not None else max(1, math.ceil(math.sqrt(steps)))
        nseg = (steps + c - 1) // c
        w = p.nx * p.ny
        num += w * (nseg - 1) * c
        den += w * steps
    return num / den if den else 0.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--mode", default="auto", choices=["auto", "fwd", "fwdadj"])
    ap.add_argument("--cpu-sample", type=int, default=32, help="instances timed on the host cores")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain per-instance device path")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of the timed batch's sample")
    ap.add_argument("--no-genuine-mcs", action="store_true",
                    help="skip timing the batch once more with a genuine modified Craig-Sneyd weight (zeta = 1/3)")
    ap.add_argument("--strong", action="store_true",
                    help="under torchrun: split one batch over the ranks by cost (strong scaling) instead of one "
                         "batch per rank (weak scaling)")
    ap.add_argument("--workspace-gb", type=float, default=None,
                    help="cap of the forward + adjoint workspace in GB (default: WS_FRACTION of the device memory; "
                         "0 = the library default, a quarter of it)")
    ap.add_argument("--checkpoint-every", type=int, default=0,
                    help="fixed checkpoint interval of the adjoint (0 = planned from the workspace cap)")
    ap.add_argument("--max-time-steps", type=int, default=0,
                    help="cap every instance's time loop (a smaller workload for profiler captures; 0 = no cap)")
    ap.add_argument("--configs", default="", help="comma list of configurations to measure instead of the batched "
                    "headline: c1, c2, c4, c5, c5sabr, sabr_r, mcsz, euler, batch32, heat1d (one JSON line each)")
    return ap.parse_args()


# ------------------------------------------------------------------------------------------
# CPU baseline (the oracle: C restatement of the reference's host Thomas-LU ADI path)
# ------------------------------------------------------------------------------------------
def _cpu_one(kw):
    from oracle import oracle as O

    p = O.Problem(**kw)
    t0 = time.perf_counter()
    O.solve(p, "f64")
    return time.perf_counter() - t0, p.nx * p.ny * (p.nt - 1)


def _cpu_ref_one(kw):
    from oracle import oracle as O

    p = O.Problem(**kw)
    _, secs = O.run_reference(p, "f64")
    return secs, p.nx * p.ny * (p.nt - 1)


def cap_time_steps(problems, cap):
    if cap > 0:
        for p in problems:
            p.nt = min(p.nt, cap + 1)
    return problems


def cpu_sample(problems, m):
    """Stratified bounded sample: every (count // m)-th instance of the batch."""
    step = max(1, len(problems) // m)
    return problems[::step][:m]


def oracle_kwargs(p):
    import dataclasses

    return p.pde_fields()


def run_cpu_baseline(problems, m, cores, kind, max_steps=None):
    """Time `m` instances of the batch on `cores` host processes; with `max_steps` each
    instance's backward time loop stops after that many steps (the per-step work of an
    instance is the same at every step, so the rate is that of the full loop)."""
    from oracle import oracle as O

    O.build()
    sample = [oracle_kwargs(p) for p in cpu_sample(problems, m)]
    if max_steps is not None:
        for kw in sample:
            kw["nt"] = min(kw["nt"], max_steps + 1)
    cores = max(1, min(cores, len(sample)))
    sample.sort(key=lambda kw: -kw["nx"] * kw["ny"] * kw["nt"])  # largest first: the pool's tail stays short
    fn = _cpu_ref_one if kind == "reference" else _cpu_one
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(fn, sample, chunksize=1)
    wall = time.perf_counter() - t0
    gps = sum(r[1] for r in res)
    return {"value": gps / wall, "unit": "grid-point-steps/s", "cores": cores, "kind": kind,
            "sample": f"{len(sample)} of the batch's instances (every {max(1, len(problems) // m)}-th), "
                      f"{'full time loops' if max_steps is None else f'first {max_steps} steps of each time loop'}, "
                      f"{gps:.3e} grid-point-steps in {wall:.1f} s wall on {cores} host threads",
            "single_core_gps": gps / sum(r[0] for r in res)}


def reference_kind():
    from oracle import oracle as O

    if not O.reference_available() and os.path.exists(os.path.join(ROOT, "oracle", "_ref", "src", ".patched")):
        # rebuild the reference driver for this host from the patched copy that travelled here
        try:
            subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True, timeout=900,
                           capture_output=True)
        except Exception:
            pass
    if O.reference_available():
        try:
            O.run_reference(O.Problem(nx=8, ny=8, nt=3), "f64")
            return "reference"
        except Exception:
            pass
    return "port"


# ------------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sms, maxes, reasons = [], [], set()
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                maxes.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxes), "reasons": sorted(reasons),
                "samples": len(sms)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------------------------------
def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    from linear_system_solvers_gb300.batch import draw_batch, grid_point_steps

    if args.configs:
        if rank == 0:
            run_configs(args)
        return

    if args.impl == "reference":
        # the reference's own CPU path on the host cores; rank 0 only
        if rank != 0:
            return
        problems = draw_batch(args.count, seed=SEED)
        kind = reference_kind()
        cores = os.cpu_count() or 1
        # the compiled reference is ~50x slower than the port: four instances per host thread, each
        # on its full grid but only the first 25 steps of its time loop (5-10 s per step)
        if kind == "port":
            m, max_steps = args.cpu_sample, None
        else:
            m, max_steps = 4 * cores, 25
        for _ in range(args.warmup):
            run_cpu_baseline(problems, max(2, m // 4), cores, kind, max_steps=10)
        vals = [run_cpu_baseline(problems, m, cores, kind, max_steps=max_steps) for _ in range(max(1, args.steps))]
        v = statistics.median(x["value"] for x in vals)
        cb = dict(vals[0])
        cb["value"] = v
        out = {"metric": METRIC, "value": v, "unit": "grid-point-steps/s", "impl": "reference",
               "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
               "scaling": "none", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": {"workload": f"batched MCS Heston, {args.count} uneven instances (seed {SEED}); "
                                      f"each step times a bounded sample of the batch's instances on the host cores",
                          "global_batch": args.count},
               "cpu_baseline": cb,
               "e2e": {"value": v, "unit": "grid-point-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
               "note": "the reference has no adjoint: this is its forward rate; a value with five parameter "
                       "gradients by central bump-and-revalue costs it 11 forward solves per instance"}
        print(json.dumps(out))
        return

    import numpy as np
    import torch

    import linear_system_solvers_gb300 as lss
    from linear_system_solvers_gb300 import _lib as L

    problems_all = draw_batch(args.count, seed=SEED)
    cap_time_steps(problems_all, args.max_time_steps)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # spawn-context pool before the first GPU call
        cpu = run_cpu_baseline(problems_all, args.cpu_sample, os.cpu_count() or 1, "port")

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from linear_system_solvers_gb300.sharding import max_over_ranks, rank_seed, shard_lpt, sum_over_ranks

    if args.strong:
        # one batch, cost-balanced shards (every rank draws the same batch and takes its own share)
        problems = [problems_all[k] for k in shard_lpt(problems_all, world)[rank]]
    else:
        problems = problems_all if rank == 0 else cap_time_steps(draw_batch(args.count, seed=rank_seed(SEED, rank)),
                                                                 args.max_time_steps)
    gps = grid_point_steps(problems)

    lib = L.load()
    fp64_peak = fp64_rate(lib)
    batch = lss.BatchSolver(problems, precision="f64")
    # the batch has the GPU to itself: give the adjoint workspace most of it (fewer recomputed steps)
    ws_cap = (WS_FRACTION * torch.cuda.get_device_properties(0).total_memory if args.workspace_gb is None
              else args.workspace_gb * 1e9)
    batch.set_workspace(ws_cap, args.checkpoint_every)
    mode = 0
    if args.mode in ("auto", "fwdadj"):
        try:
            batch.run(mode=1)
            torch.cuda.synchronize()
            mode = 1
        except L.LssError as e:
            if args.mode == "fwdadj":
                raise
            if e.code != L.EUNSUPPORTED:
                raise
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    # lines-per-CTA autotuner (its timed runs double as warm-up)
    with torch.cuda.stream(stream):
        threads = batch.autotune(mode=mode, stream=sptr)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            batch.run(mode=mode, stream=sptr, graph=True)
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            e0.record(stream)
            for _ in range(args.steps):
                batch.run(mode=mode, stream=sptr, graph=True)
            e1.record(stream)
            barrier()
        ms = e0.elapsed_time(e1) / args.steps
    launches = batch.launch_count() * args.steps
    values, grads, status = batch.results()

    # end to end through the C-ABI with host buffers (payoff grids in, values/grads out)
    total_n = sum(p.nx * p.ny for p in problems)
    pay_src = build_payoffs(problems, torch.empty(total_n, dtype=torch.float64, pin_memory=True).numpy())
    vals_h = torch.empty(len(problems), dtype=torch.float64, pin_memory=True).numpy()
    grads_h = torch.empty((len(problems), 5), dtype=torch.float64, pin_memory=True).numpy()
    with torch.cuda.stream(stream):
        batch.run_host(mode, vals_h, grads_h if mode == 1 else None, payoffs=pay_src, stream=sptr)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            batch.run_host(mode, vals_h, grads_h if mode == 1 else None, payoffs=pay_src, stream=sptr)
        barrier()
        e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_ok = bool(np.allclose(vals_h, values, rtol=1e-12, atol=1e-12))

    t_max, e2e_s = max_over_ranks([ms, e2e_s], device="cuda")
    (gps_all,) = sum_over_ranks([float(gps)], device="cuda")  # every rank's batch or shard
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    value = gps_all / (t_max * 1e-3)
    bpg = BYTES_PER_GPS_FWD["mcs"] * (1 if mode == 0 else 10.0 / 3.0)
    rf = recompute_fraction(problems, batch.checkpoints()) if mode == 1 else 0.0
    fp64_per_gps = per_gps(FP64_INSTR_FWD, FP64_INSTR_ADJ, mode, rf)
    dram_per_gps = per_gps(DRAM_BYTES_FWD, DRAM_BYTES_ADJ, mode, rf)
    peak, peak_kind = measured_peaks()
    achieved = gps * bpg / (ms * 1e-3) / 1e9
    out = {
        "metric": METRIC,
        "value": value, "unit": "grid-point-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max, "higher_is_better": True, "scaling": "strong" if args.strong else "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"batched modified Craig-Sneyd Heston calls, {len(problems)} uneven instances per GPU "
                               f"(seed {SEED}), Nx 64-256, Ny 32-128, "
                               f"{f'100-400 steps capped at {args.max_time_steps}' if args.max_time_steps else '100-400 steps'}, "
                               f"{'forward + adjoint' if mode == 1 else 'forward'}, one persistent kernel per step, "
                               "graph-launched",
                   "global_batch": len(problems_all) if args.strong else len(problems) * world,
                   "grid_point_steps_per_gpu": gps,
                   "threads_per_instance": threads,
                   "l2": f"inputs larger than L2 (line tables {total_n * 23 * 8 / 1e9:.1f} GB streamed every step)",
                   "parallelism": (f"instance sharding x{world} ({'one batch split by cost' if args.strong else 'a batch per rank'})"
                                   if world > 1 else "single GPU")},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": dram_per_gps * gps, "traffic_unit": "bytes per launch",
                     "traffic_source": "ncu dram__bytes_read+write of the 1024-instance 40-step captures, per "
                                       "grid-point-step (forward + adjoint: forward x (1 + recomputed fraction) + "
                                       "adjoint), times this launch's grid-point-steps", "peak_source": peak_kind,
                     "algorithmic_bytes_per_grid_point_step": bpg,
                     "note": f"the FP64 pipe ({2 * fp64_peak / 1e12:.3f} TFLOP/s of DFMA measured in this run) "
                             "binds before HBM on GB300"},
        "fp64_pipe": {"instructions_per_grid_point_step": fp64_per_gps, "recomputed_fraction": rf,
                      "achieved": gps * fp64_per_gps / (ms * 1e-3), "peak": fp64_peak,
                      "peak_source": "lss_diag_fp64_rate, measured in this run",
                      "unit": "FP64 instructions/s", "frac": gps * fp64_per_gps / (ms * 1e-3) / fp64_peak,
                      "note": "the binding resource of this path; instruction counts from ncu (forward + adjoint: "
                              "forward x (1 + recomputed fraction) + adjoint), peak from a DFMA probe"},
        "e2e": {"value": gps_all / e2e_s, "unit": "grid-point-steps/s", "h2d_bytes_per_step": int(total_n * 8),
                "d2h_bytes_per_step": int(len(problems) * 8 * (6 if mode == 1 else 1)), "matches_device_values": e2e_ok},
        "adjoint_workspace": ({"cap_gb": ws_cap / 1e9, "held_gb": batch.workspace_bytes() / 1e9,
                               "recomputed_fraction": rf,
                               "how": "lss_adi_batch_set_workspace (library default: a quarter of the device memory)"}
                              if mode == 1 else None),
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "nonfinite_instances": int(np.count_nonzero(status)),
    }
    if cpu is not None:
        out["cpu_baseline"] = cpu
    if world == 1 and not args.no_parity:
        out["parity"] = headline_parity(batch, problems, mode, values, grads)
    if world == 1 and not args.no_plain:
        out["plain_path"] = time_plain_path(lss, problems, stream, value, mode)
    if world == 1 and mode == 1 and not args.no_genuine_mcs:
        batch.close()  # its workspace, before the next batch takes its own
        out["genuine_mcs"] = time_genuine_mcs(lss, problems, ws_cap, stream)
    print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


# ------------------------------------------------------------------------------------------
# single-instance configurations (measured with --configs; parity against the oracle)
# ------------------------------------------------------------------------------------------
CONFIG1 = dict(model="heston", kappa=1.5, theta_v=0.04, sigma=0.3, rho=-0.9, rate=0.02, strike=100.0, maturity=1.0,
               s_lo=0.0, s_hi=200.0, v_lo=0.0, v_hi=1.2, nx=100, ny=50, nt=201, scheme="dr", eval_s=100.0,
               eval_v=0.04)
NU_K100 = dict(nonuniform=True, acc_point=100.0, alpha_scale=10.0, beta_scale=24.0)


def _rel_err(a, ref):
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    if not np.all(np.isfinite(ref)):
        return float("nan")
    den = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return float(np.max(np.abs(a - ref) / den))


def _time_solver(solver, reps):
    import torch

    solver.solve(graph=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        surf, val = solver.solve(graph=True)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps, surf, val


def run_configs(args):
    import dataclasses

    import numpy as np
    import torch

    import linear_system_solvers_gb300 as lss
    from oracle import oracle as O

    O.build()
    torch.cuda.set_device(0)
    wanted = [c.strip() for c in args.configs.split(",") if c.strip()]

    def oracle_problem(p, nt=None):
        kw = p.pde_fields()
        if nt is not None:
            kw["nt"] = nt
        return O.Problem(**kw)

    def case(name, p, fp, reps, oracle_nt=None):
        gps = p.nx * p.ny * (p.nt - 1)
        s = lss.ImplicitHestonSolver(p, precision=fp, arith="fast")
        secs, surf, val = _time_solver(s, reps)
        rec = {"config": name, "precision": fp, "scheme": p.scheme, "grid": [p.nx, p.ny, p.nt - 1],
               "device_gps": gps / secs, "device_seconds": secs, "value": val, "path": "wide (kernel per stage, graph)"}
        # parity against the oracle (full run, or the first oracle_nt - 1 steps for the largest grids)
        if oracle_nt is not None:
            p_short = dataclasses.replace(p, nt=oracle_nt)
            surf = lss.ImplicitHestonSolver(p_short, precision=fp, arith="fast").solve()[0]
            op = oracle_problem(p, oracle_nt)
            rec["parity_steps"] = oracle_nt - 1
        else:
            op = oracle_problem(p)
        t0 = time.perf_counter()
        ref64 = O.solve(op, "f64")
        cpu_s = time.perf_counter() - t0
        rec["cpu_oracle_gps_1core"] = op.nx * op.ny * (op.nt - 1) / cpu_s
        rec["rel_err_vs_fp64_oracle"] = _rel_err(surf, ref64)
        rec["oracle_unstable"] = bool((not np.all(np.isfinite(ref64))) or np.abs(ref64).max() > 10 * p.s_hi)
        if fp == "f32":
            rec["rel_err_reference_fp32_vs_fp64"] = _rel_err(O.solve(op, "f32"), ref64)
        print(json.dumps(rec), flush=True)

    if "c1" in wanted:
        p = lss.HestonProblem(**CONFIG1)
        case("config1 DR 100x50x200", p, "f64", 20)
        # FP32 following the FP64 problem (grid, remaps and tables built in double, rounded once)
        case("config1 DR 100x50x200 FP32 with FP64 tables", dataclasses.replace(p, fp64_tables=True), "f32", 20)
        ref = lss.ImplicitHestonSolver(p, precision="f64", arith="reference")
        secs, surf, _ = _time_solver(ref, 5)
        print(json.dumps({"config": "config1 DR 100x50x200", "path": "reference-order plain kernels (bitwise)",
                          "device_gps": p.nx * p.ny * (p.nt - 1) / secs,
                          "bitwise_equal_oracle": bool(np.array_equal(surf, O.solve(oracle_problem(p), "f64")))}),
              flush=True)
    if "c2" in wanted:
        for scheme in ("cs", "mcs", "hv"):
            for fp in ("f64", "f32"):
                p = lss.HestonProblem(**dict(CONFIG1, scheme=scheme, nx=400, ny=200, nt=501, **NU_K100))
                case(f"config2 {scheme.upper()} 400x200x500", p, fp, 2)
            # stable companion (rho = 0) on the same grid, FP64 and FP32 with FP64 tables
            p = lss.HestonProblem(**dict(CONFIG1, scheme=scheme, rho=0.0, nx=400, ny=200, nt=501, **NU_K100))
            case(f"config2 {scheme.upper()} 400x200x500 rho=0 companion", p, "f64", 2)
            case(f"config2 {scheme.upper()} 400x200x500 rho=0 companion FP32 with FP64 tables",
                 dataclasses.replace(p, fp64_tables=True), "f32", 2)
        # MCS with a genuine weight (zeta = 1/3 != theta = 1/2: the full MCS stencil)
        p = lss.HestonProblem(**dict(CONFIG1, scheme="mcs", zeta=1.0 / 3.0, nx=400, ny=200, nt=501, **NU_K100))
        case("config2 MCS(zeta=1/3) 400x200x500", p, "f64", 2)
    if "c4" in wanted:
        run_config4()
    if "c5" in wanted:
        # --max-time-steps caps the time loop (profiler captures of the large-grid kernels)
        nt5 = min(1001, args.max_time_steps + 1) if args.max_time_steps else 1001
        for fp in ("f64", "f32"):
            p = lss.HestonProblem(**dict(CONFIG1, scheme="hv", nx=4096, ny=2048, nt=nt5, **NU_K100))
            case(f"config5 HV 4096x2048x{nt5 - 1}", p, fp, 1, oracle_nt=min(11, nt5))
    if "euler" in wanted:
        # explicit Euler (explicit_solvers::general_heston_equation): 200 x 100, 8000 steps, T = 0.25
        p = lss.HestonProblem(**dict(CONFIG1, scheme="euler", nx=200, ny=100, nt=8001, maturity=0.25))
        op = oracle_problem(p)
        t0 = time.perf_counter()
        want = O.solve(op, "f64")
        cpu_s = time.perf_counter() - t0
        gps = p.nx * p.ny * (p.nt - 1)
        for arith in ("reference", "fast"):
            sv = lss.ImplicitHestonSolver(p, precision="f64", arith=arith)
            secs, surf, val = _time_solver(sv, 3)
            rec = {"config": "explicit Euler 200x100x8000", "arith": arith, "device_gps": gps / secs,
                   "device_seconds": secs, "value": val, "path": "kernel per step, graph",
                   "cpu_oracle_gps_1core": gps / cpu_s}
            if arith == "reference":
                rec["bitwise_equal_oracle"] = bool(np.array_equal(surf, want))
            else:
                rec["rel_err_vs_fp64_oracle"] = _rel_err(surf, want)
            print(json.dumps(rec), flush=True)
        if O.reference_available():
            ref_p = oracle_problem(p, 201)
            _, ref_s = O.run_reference(ref_p, "f64")
            print(json.dumps({"config": "explicit Euler 200x100x8000", "path": "reference host Euler (compiled), "
                              "first 200 steps", "cpu_reference_gps_1core": p.nx * p.ny * 200 / ref_s}), flush=True)
    if "batch32" in wanted:
        # the headline batch in FP32, forward (the adjoint is FP64 only)
        from linear_system_solvers_gb300.batch import draw_batch, grid_point_steps

        probs = draw_batch(4096, seed=SEED)
        b = lss.BatchSolver(probs, precision="f32")
        threads = b.autotune(mode=0)
        b.run(0, graph=True)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            b.run(0, graph=True)
        e1.record()
        torch.cuda.synchronize()
        secs = e0.elapsed_time(e1) / 3e3
        gps = grid_point_steps(probs)
        print(json.dumps({"config": "batched MCS FP32 forward, 4096 uneven instances (seed 20261203)",
                          "device_gps": gps / secs, "device_seconds": secs, "threads_per_instance": threads,
                          "hbm_gbs_at_48_B": gps * 48 / secs / 1e9,
                          "nonfinite_instances": int(np.count_nonzero(b.results()[2]))}), flush=True)
    if "mcsz" in wanted:
        # the batch of the headline with a genuine modified Craig-Sneyd weight (zeta = 1/3 != theta):
        # the full MCS stencil, forward and forward + adjoint
        from linear_system_solvers_gb300.batch import draw_batch, grid_point_steps

        probs = draw_batch(4096, seed=SEED)
        for p in probs:
            p.zeta = 1.0 / 3.0
        b = lss.BatchSolver(probs, precision="f64")
        for mode in (0, 1):
            threads = b.autotune(mode=mode)
            b.run(mode, graph=True)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            b.run(mode, graph=True)
            e1.record()
            torch.cuda.synchronize()
            secs = e0.elapsed_time(e1) / 1e3
            status = b.results()[2]
            print(json.dumps({"config": "batched MCS zeta=1/3, 4096 uneven instances (seed 20261203)",
                              "mode": ["forward", "forward + adjoint"][mode], "device_gps": grid_point_steps(probs) / secs,
                              "device_seconds": secs, "threads_per_instance": threads,
                              "nonfinite_instances": int(np.count_nonzero(status))}), flush=True)
    if "heat1d" in wanted:
        run_heat1d()
    for key, rate, nt, fd_names in (("c5sabr", 0.0, 801, ("sigma", "rho")),
                                    ("sabr_r", 0.03, 201, ("sigma", "rho", "rate"))):
        if key not in wanted:
            continue
        # c5sabr: config 5's SABR problem (r unspecified there: 0, coefficients constant in time);
        # sabr_r: the reference's own SABR rate r = 0.03, whose D(t) = exp(-r (T - t)) makes the
        # coefficients time-dependent (the S-line tables are rebuilt before every step)
        p = lss.HestonProblem(model="sabr", sigma=0.4, rho=-0.3, sabr_beta=0.5, rate=rate, strike=0.05, maturity=2.0,
                              s_lo=0.0, s_hi=0.2, v_lo=0.0, v_hi=1.0, nx=2048, ny=1024, nt=nt, scheme="dr",
                              nonuniform=True, acc_point=0.05, alpha_scale=10.0, beta_scale=24.0, eval_s=0.05,
                              eval_v=0.2)
        label = f"config5 SABR DR 2048x1024x{nt - 1}" + (f" r={rate}" if rate else "")
        case(label, p, "f64", 1, oracle_nt=11)
        # forward + adjoint: dV/d(nu, rho, r) and dV/d(payoff) in one backward pass; checked against
        # Richardson central differences (relative bumps 1e-4, 5e-5: the sensitivities are ~1e-2 of
        # the value) of the device forward, thread-per-line solves
        s = lss.ImplicitHestonSolver(p, precision="f64", arith="fast")
        s.adjoint(want_payoff_grad=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        val, grads, _ = s.adjoint()
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0

        def fwd(q):
            q = dataclasses.replace(q, line_per_thread=True)
            return lss.ImplicitHestonSolver(q, precision="f64", arith="fast").solve()[1]

        errs = {}
        for name in fd_names:
            idx = {"sigma": 2, "rho": 3, "rate": 4}[name]
            base = getattr(p, name)
            cd = []
            # r = 0.03: a relative bump of 1e-4 moves r by 3e-6, where the forward's rounding noise
            # (~1e-12 of V) is ~1e-6 of the difference; 1e-3 / 5e-4 keep it below 1e-7
            for rel in ((1e-3, 5e-4) if name == "rate" else (1e-4, 5e-5)):
                h = rel * abs(base)
                cd.append((fwd(dataclasses.replace(p, **{name: base + h})) -
                           fwd(dataclasses.replace(p, **{name: base - h}))) / (2 * h))
            fd = (4.0 * cd[1] - cd[0]) / 3.0
            errs[name] = abs(grads[idx] - fd) / max(abs(fd), 1e-3 * abs(val))
        print(json.dumps({"config": label + " forward + adjoint", "device_gps_fwd_adj":
                          p.nx * p.ny * (p.nt - 1) / secs, "device_seconds": secs, "value": val,
                          "dV_dnu": grads[2], "dV_drho": grads[3], "dV_dr": grads[4],
                          "rel_err_vs_device_fd": errs,
                          "fd": "Richardson central, relative bumps 1e-4 / 5e-5 (r: 1e-3 / 5e-4), device forward"}),
              flush=True)


def _oracle_value(args):
    """Bump-and-revalue leg: V(eval_s, eval_v) from the oracle surface (bilinear in S, v)."""
    import numpy as np

    from oracle import oracle as O

    kw, s0, v0 = args
    p = O.Problem(**kw)
    surf = O.solve(p, "f64")
    x, y = O.grid(p, "f64")
    i = max(0, min(len(x) - 2, int(np.searchsorted(x, s0, side="right")) - 1))
    j = max(0, min(len(y) - 2, int(np.searchsorted(y, v0, side="right")) - 1))
    wx = min(1.0, max(0.0, (s0 - x[i]) / (x[i + 1] - x[i])))
    wy = min(1.0, max(0.0, (v0 - y[j]) / (y[j + 1] - y[j])))
    return float((1 - wx) * (1 - wy) * surf[i, j] + wx * (1 - wy) * surf[i + 1, j] + (1 - wx) * wy * surf[i, j + 1]
                 + wx * wy * surf[i + 1, j + 1])


# 1-D implicit heat / Black-Scholes batch (lss_heat1d.h): bytes and FP64 operations per
# point-step of the factorised kernel k_h1_fast (forward: WB, WD, M, U[t+1] loads, Y store;
# backward: Y, G loads, U store; 4 + 1 FP64 operations)
HEAT1D_BYTES_PER_PS = {"f64": 64.0, "f32": 32.0}
HEAT1D_SEED = 20261205


def run_heat1d(count=65536, sample=48):
    """Batched 1-D Black-Scholes (draw_black_scholes: n 128-512, 99-999 steps, CN, sinh grid at K):
    device throughput of both arithmetics and precisions, end to end through run_host, parity on
    a sample against the oracle, CPU baselines (oracle and the compiled reference) on a sample."""
    import numpy as np
    import torch

    import linear_system_solvers_gb300 as lss
    from oracle import oracle as O

    torch.cuda.set_device(0)
    qs = lss.draw_black_scholes(count, seed=HEAT1D_SEED)
    ps = float(sum(q.n * (q.nt - 1) for q in qs))
    peak, peak_kind = measured_peaks()
    rng = np.random.default_rng(1)
    idx = sorted(rng.choice(count, size=sample, replace=False).tolist())

    def oproblem(q):
        return O.Heat1DProblem(model="bs", sigma=q.sigma, rate=q.rate, strike=q.strike, put=q.put, x_lo=q.s_lo,
                               x_hi=q.s_hi, t_lo=0.0, t_hi=q.maturity, n=q.n, nt=q.nt, theta_scheme=q.theta_scheme,
                               nonuniform=q.nonuniform, acc_point=q.acc_point, alpha_scale=q.alpha_scale,
                               forward=False)

    t0 = time.perf_counter()
    wants = {i: O.solve_1d(oproblem(qs[i]), "f64") for i in idx}
    cpu_s = time.perf_counter() - t0
    cpu_ps = sum(qs[i].n * (qs[i].nt - 1) for i in idx)
    for fp in ("f64", "f32"):
        for arith in ("fast", "reference"):
            t0 = time.perf_counter()
            b = lss.black_scholes_batch(qs, fp, arith)
            create_s = time.perf_counter() - t0
            b.run()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            reps = 3
            with ClockSampler(0) as clk:
                e0.record()
                for _ in range(reps):
                    b.run()
                e1.record()
                torch.cuda.synchronize()
            secs = e0.elapsed_time(e1) / 1e3 / reps
            # end to end: new terminal conditions from pinned host memory, values back
            init = np.concatenate([np.maximum(0.0, b.grid(i).astype(np.float64) - qs[i].strike) for i in range(count)])
            init_t = torch.from_numpy(init.astype(np.float64 if fp == "f64" else np.float32)).pin_memory()
            init_np = init_t.numpy()
            b.run_host(init_np)
            t0 = time.perf_counter()
            for _ in range(reps):
                vals, st = b.run_host(init_np)
            e2e_s = (time.perf_counter() - t0) / reps
            errs = [_rel_err(b.solution(i), wants[i]) for i in idx]
            rec = {"config": f"batched 1-D Black-Scholes, {count} uneven calls (seed {HEAT1D_SEED})",
                   "precision": fp, "arith": arith, "device_point_steps_per_s": ps / secs, "device_seconds": secs,
                   "e2e": {"value": ps / e2e_s, "unit": "point-steps/s", "h2d_bytes_per_step": int(init_np.nbytes),
                           "d2h_bytes_per_step": int(count * (8 + 4))},
                   "create_seconds": create_s, "gpu_launches_per_run": b.launch_count(),
                   "nonfinite_instances": int(np.count_nonzero(st)),
                   "max_rel_err_vs_fp64_oracle_sample": float(max(errs)), "sample": sample,
                   "clocks": clk.summary()}
            if arith == "fast":
                gbs = ps * HEAT1D_BYTES_PER_PS[fp] / secs / 1e9
                rec["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                                   "peak_source": peak_kind, "bytes_per_point_step": HEAT1D_BYTES_PER_PS[fp]}
                if fp == "f64":
                    from linear_system_solvers_gb300 import _lib as L

                    fpk = fp64_rate(L.load())
                    rec["fp64_pipe"] = {"fp64_ops_per_point_step": 5, "achieved_ops_per_s": 5 * ps / secs,
                                        "peak": fpk, "peak_source": "lss_diag_fp64_rate, measured in this run",
                                        "frac": 5 * ps / secs / fpk}
            else:
                eq = [bool(np.array_equal(b.solution(i), O.solve_1d(oproblem(qs[i]), fp))) for i in idx[:16]]
                rec["bitwise_equal_oracle_sample"] = f"{sum(eq)}/{len(eq)}"
            print(json.dumps(rec), flush=True)
            del b
    base = {"config": "batched 1-D Black-Scholes CPU baselines", "oracle_point_steps_per_s_1core": cpu_ps / cpu_s,
            "sample": f"{sample} instances of the batch, full time loops"}
    if O.reference_1d_available():
        t0 = time.perf_counter()
        ref_ps = 0
        for i in idx[:16]:
            _, sec = O.run_reference_1d(oproblem(qs[i]), "f64")
            ref_ps += qs[i].n * (qs[i].nt - 1) / sec
        base["reference_point_steps_per_s_1core"] = ref_ps / 16
        base["reference_sample"] = "16 instances, compiled reference host Thomas LU, solver time only"
    print(json.dumps(base), flush=True)


def run_config4(count=1024, sample=16):
    """Config 4: adjoint of 1024 uneven MCS instances (seed 20261204); gradients of a stable
    16-instance sample against central finite differences (relative bump 1e-5) of the CPU
    oracle, which is bit-exact with the reference's Thomas-LU path."""
    import numpy as np
    import torch

    import linear_system_solvers_gb300 as lss
    from linear_system_solvers_gb300.batch import draw_batch, grid_point_steps

    probs = draw_batch(count, seed=20261204)
    b = lss.BatchSolver(probs, precision="f64")
    threads = b.autotune(mode=1)
    b.run(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.run(1)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    vals, grads, status = b.results()
    names = ("kappa", "theta_v", "sigma", "rho", "rate")
    picked = []
    for k, p in enumerate(probs):
        surf = b.surface(k)
        if np.all(np.isfinite(surf)) and np.abs(surf).max() <= 10 * p.s_hi:
            picked.append(k)
        if len(picked) == sample:
            break
    # central differences at the relative bump 1e-5 (as specified) and, Richardson-extrapolated
    # (error O(h^4)), at 1e-3 / 5e-4: above the rounding noise of small sensitivities (with
    # r ~ 1e-3 a relative bump of 1e-5 moves r by 1e-8 and the difference is mostly rounding)
    bumps = (1e-5, 1e-3, 5e-4)
    jobs = []
    for k in picked:
        p = probs[k]
        kw = oracle_kwargs(p)
        for name in names:
            for rel in bumps:
                h = rel * abs(kw[name])
                for sgn in (+1, -1):
                    q = dict(kw)
                    q[name] = kw[name] + sgn * h
                    jobs.append((q, p.eval_s, p.eval_v))
    ctx = mp.get_context("spawn")
    with ctx.Pool(os.cpu_count() or 1) as pool:
        fdv = pool.map(_oracle_value, jobs, chunksize=1)
    worst = worst_rich = 0.0
    q = 0
    for k in picked:
        p = probs[k]
        kw = oracle_kwargs(p)
        for c, name in enumerate(names):
            h = 1e-5 * abs(kw[name])
            fd = (fdv[q] - fdv[q + 1]) / (2 * h)
            H = 1e-3 * abs(kw[name])
            fd_h = (fdv[q + 2] - fdv[q + 3]) / (2 * H)
            fd_h2 = (fdv[q + 4] - fdv[q + 5]) / H
            q += 6
            rich = (4.0 * fd_h2 - fd_h) / 3.0
            den = max(abs(rich), 1e-3 * abs(vals[k]))
            worst = max(worst, abs(grads[k, c] - fd) / den)
            worst_rich = max(worst_rich, abs(grads[k, c] - rich) / den)
    print(json.dumps({"config": "config4 adjoint, 1024 uneven MCS instances (seed 20261204)",
                      "device_gps_fwd_adj": grid_point_steps(probs) / secs, "device_seconds": secs,
                      "threads_per_instance": threads, "nonfinite_instances": int(np.count_nonzero(status)),
                      "fd_sample_instances": len(picked),
                      "max_rel_err_grad_vs_reference_fd": worst,
                      "max_rel_err_grad_vs_reference_fd_richardson": worst_rich,
                      "fd": "central, relative bump 1e-5 (plain); Richardson from 1e-3 / 5e-4; CPU oracle"}),
          flush=True)


def _oracle_surface(kw):
    """FP64 oracle surface of one instance (the reference's host Thomas-LU path, restated) and its
    spread: the largest relative change of the surface when the terminal condition is scaled by
    1 + 1e-15, i.e. how far the reference scheme itself amplifies a rounding-sized perturbation."""
    import numpy as np

    from oracle import oracle as O

    op = O.Problem(**kw)
    ref = O.solve(op, "f64")
    x, _ = O.grid(op, "f64")
    pay = np.repeat(np.maximum(x - kw["strike"], 0.0)[:, None], kw["ny"], axis=1) * (1.0 + 1e-15)
    alt = O.solve(op, "f64", payoff=pay)
    if not (np.all(np.isfinite(ref)) and np.all(np.isfinite(alt))):
        return ref, float("inf")
    den = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return ref, float(np.max(np.abs(alt - ref) / den))


def stratified_sample(problems, m=64):
    """Indices of `m` instances covering every (Nx, Ny) bucket: one per bucket in batch order,
    then a second per bucket, and so on."""
    buckets = {}
    for k, p in enumerate(problems):
        buckets.setdefault((p.nx, p.ny), []).append(k)
    keys = sorted(buckets)
    out, depth = [], 0
    while len(out) < min(m, len(problems)):
        added = False
        for key in keys:
            if depth < len(buckets[key]) and len(out) < m:
                out.append(buckets[key][depth])
                added = True
        if not added:
            break
        depth += 1
    return sorted(out)


def headline_parity(batch, problems, mode, values, grads, m=64, grad_members=4):
    """Parity of the timed batch: the final surfaces of a stratified sample (every Nx x Ny bucket,
    full time loops) against the FP64 oracle, relative error with the denominator
    max(|V|, 1e-3 max|V|).  A call is bounded by S, so an oracle surface with max|V| above S_max
    by more than 0.1 % (or not finite) is a growing mode of the reference scheme itself: such members are counted
    apart, with their error stated beside the oracle's own spread (how far a 1e-15 relative change
    of the terminal condition moves the reference's surface).  The bounded members are held to
    1e-10.  Mode 1: the gradients of the cheapest bounded members against Richardson-extrapolated
    central differences of the oracle (relative bumps 1e-3 / 5e-4, tolerance 1e-6), and the plain
    central difference at the relative bump 1e-5 for reference."""
    import numpy as np

    idx = stratified_sample(problems, m)
    kws = [oracle_kwargs(problems[k]) for k in idx]
    order = sorted(range(len(idx)), key=lambda q: -kws[q]["nx"] * kws[q]["ny"] * kws[q]["nt"])
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(min(len(idx), os.cpu_count() or 1)) as pool:
        res = pool.map(_oracle_surface, [kws[q] for q in order], chunksize=1)
    refs = [None] * len(idx)
    for q, r in zip(order, res):
        refs[q] = r
    stable_err, stable = 0.0, []
    growing = []
    for q, k in enumerate(idx):
        ref, spread = refs[q]
        got = batch.surface(k)
        finite = bool(np.all(np.isfinite(ref)))
        err = float("nan")
        if finite:
            den = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
            err = float(np.max(np.abs(got - ref) / den))
        if finite and float(np.abs(ref).max()) <= problems[k].s_hi * 1.001:
            stable_err = max(stable_err, err)
            stable.append(k)
        else:
            growing.append((k, err, spread, float(np.abs(ref).max()) if finite else float("inf")))
    g_err = [e for _, e, _, _ in growing if e == e]
    g_ratio = [e / sp for _, e, sp, _ in growing if e == e and 0.0 < sp < float("inf")]
    out = {"sample": f"{len(idx)} instances of the timed batch covering all "
                     f"{len({(p.nx, p.ny) for p in problems})} Nx x Ny buckets, full time loops, FP64 oracle "
                     f"(C restatement of the reference's host Thomas-LU ADI, pinned bit-exact to the compiled reference)",
           "bounded_instances": len(stable), "max_rel_err_vs_fp64_oracle": stable_err, "tolerance": 1e-10,
           "bounded_max_oracle_spread": max((refs[idx.index(k)][1] for k in stable), default=0.0),
           "growing_instances": len(growing),
           "growing_max_rel_err": max(g_err) if g_err else None,
           "growing_max_err_over_oracle_spread": max(g_ratio) if g_ratio else None,
           "rel_err": "max over grid points of |V - V_ref| / max(|V_ref|, 1e-3 max|V_ref|)",
           "growing": "max|V| > S_max or not finite in the reference scheme itself (a call is bounded by S); the "
                      "oracle spread is the relative change of its surface under a 1e-15 relative change of the "
                      "terminal condition"}
    if mode == 1 and stable:
        names = ("kappa", "theta_v", "sigma", "rho", "rate")
        members = sorted(stable, key=lambda k: problems[k].nx * problems[k].ny * problems[k].nt)[:grad_members]
        jobs = []
        for k in members:
            p = problems[k]
            kw = oracle_kwargs(p)
            for name in names:
                for rel in (1e-5, 1e-3, 5e-4):
                    h = rel * abs(kw[name])
                    for sgn in (+1, -1):
                        qkw = dict(kw)
                        qkw[name] = kw[name] + sgn * h
                        jobs.append((qkw, p.eval_s, p.eval_v))
        with ctx.Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
            fdv = pool.map(_oracle_value, jobs, chunksize=1)
        worst = worst_rich = 0.0
        q = 0
        for k in members:
            kw = oracle_kwargs(problems[k])
            for c, name in enumerate(names):
                fd = (fdv[q] - fdv[q + 1]) / (2 * 1e-5 * abs(kw[name]))
                H = 1e-3 * abs(kw[name])
                rich = (4.0 * (fdv[q + 4] - fdv[q + 5]) / H - (fdv[q + 2] - fdv[q + 3]) / (2 * H)) / 3.0
                q += 6
                den = max(abs(rich), 1e-3 * abs(values[k]))
                worst = max(worst, abs(grads[k, c] - fd) / den)
                worst_rich = max(worst_rich, abs(grads[k, c] - rich) / den)
        out["gradients"] = {"members": [int(k) for k in members],
                            "max_rel_err_vs_oracle_richardson_fd": worst_rich, "tolerance": 1e-6,
                            "max_rel_err_vs_oracle_central_fd_1e-5": worst,
                            "fd": "oracle bump-and-revalue of dV/d(kappa, theta, sigma, rho, r); Richardson from "
                                  "relative bumps 1e-3 / 5e-4; denominator max(|FD|, 1e-3 |V|)"}
    out["oracle_seconds"] = time.perf_counter() - t0
    return out


def time_genuine_mcs(lss, problems, ws_cap, stream):
    """The timed batch once more with a genuine modified Craig-Sneyd weight: zeta = 1/3 instead of
    theta = 1/2 (at zeta = theta the scheme is Craig-Sneyd's and runs its stencil), forward +
    adjoint at the same workspace cap, one timed launch after the autotuner's and a warm-up."""
    import numpy as np
    import torch

    from linear_system_solvers_gb300.batch import grid_point_steps

    probs = [dataclasses.replace(p, zeta=1.0 / 3.0) for p in problems]
    b = lss.BatchSolver(probs, precision="f64")
    b.set_workspace(ws_cap, 0)
    sptr = stream.cuda_stream
    with torch.cuda.stream(stream):
        threads = b.autotune(mode=1, stream=sptr)
        b.run(mode=1, stream=sptr, graph=True)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(mode=1, stream=sptr, graph=True)
        e1.record(stream)
        torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1e3
    status = b.results()[2]
    rf = recompute_fraction(probs, b.checkpoints())
    b.close()
    return {"value": grid_point_steps(probs) / secs, "unit": "grid-point-steps/s", "zeta": 1.0 / 3.0,
            "threads_per_instance": threads, "recomputed_fraction": rf, "seconds": secs,
            "nonfinite_instances": int(np.count_nonzero(status)),
            "note": "the same batch with the full MCS stencil (zeta != theta), forward + adjoint; instances that "
                    "diverge in the reference scheme itself stay non-finite"}


def time_plain_path(lss, problems, stream, batched_value, mode, m=64):
    """The plain device path (one instance per launch sequence, kernel per sweep, FMA
    arithmetic) on a bounded sample of the same batch, for the batched/plain ratio."""
    import torch

    sample = cpu_sample(problems, m)
    solvers = [lss.ImplicitHestonSolver(p, precision="f64", arith="fast") for p in sample]
    gps = sum(p.nx * p.ny * (p.nt - 1) for p in sample)
    sptr = stream.cuda_stream
    with torch.cuda.stream(stream):
        for s in solvers[:4]:
            s.solve(graph=True, stream=sptr)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s in solvers:
            s.solve(graph=True, stream=sptr)
        e1.record(stream)
        torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) * 1e-3
    plain = gps / secs
    out = {"value": plain, "unit": "grid-point-steps/s", "sample_instances": len(sample),
           "how": "lss_adi_forward_graph per instance (forward only; kernel per stage over the whole GPU, "
                  "graph replay), host copies per instance",
           "batched_over_plain": batched_value / plain}
    if mode == 1:
        # like for like: forward + adjoint through lss_adi_adjoint, one instance per call, each on
        # the whole GPU (kernel per stage, partitioned line solves) rather than one CTA
        import dataclasses

        sub = cpu_sample(problems, 16)
        adj = [lss.ImplicitHestonSolver(dataclasses.replace(p, wide_adjoint=True), precision="f64", arith="fast")
               for p in sub]
        gps_a = sum(p.nx * p.ny * (p.nt - 1) for p in sub)
        adj[0].adjoint(stream=sptr)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in adj:
            s.adjoint(stream=sptr)
        torch.cuda.synchronize()
        plain_a = gps_a / (time.perf_counter() - t0)
        out = {"value": plain_a, "unit": "grid-point-steps/s", "sample_instances": len(sub),
               "how": "lss_adi_adjoint per instance with LSS_ADI_OPT_WIDE_ADJOINT (forward + adjoint, the same "
                      "work as the batched run, each instance on the whole GPU: kernel per stage, partitioned "
                      "line solves, autotuned chunks)",
               "batched_over_plain": batched_value / plain_a, "forward_only": out}
    return out


def build_payoffs(problems, buf):
    """Terminal conditions max(0, S - K) of every instance on its sinh grid, concatenated."""
    import numpy as np

    off = 0
    for p in problems:
        n = p.nx * p.ny
        x = grid_x(p)
        buf[off:off + n] = np.repeat(np.maximum(x - p.strike, 0.0), p.ny)
        off += n
    return buf


def grid_x(p):
    """S grid of the reference's sinh map (double), same formula as the library's host set-up."""
    import numpy as np

    lo, hi, pt = p.s_lo, p.s_hi, p.acc_point
    alpha = (pt - lo) / p.alpha_scale if p.nonuniform else hi - lo
    c0 = np.arcsinh((hi - pt) / alpha)
    c1 = np.arcsinh((lo - pt) / alpha)
    z = (1.0 / (p.nx - 1)) * np.arange(p.nx)
    return pt + alpha * np.sinh(c0 * z + c1 * (1.0 - z))


if __name__ == "__main__":
    main()
