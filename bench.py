#!/usr/bin/env python
"""Benchmark of the QMS per-step hot path: DOF-timesteps/s on one GB300.

Workload (default): the 256^3 moving-conductor case (aluminium plate
200x200x10, sigma 3.5e7 S/m, in Bz = 10 mT + 0.1 T/m z-gradient; the frame
ramps to -10 m/s along x in the first step; dt = 1e-5 s).  n_dims =
67,700,225 unknowns (~50.7 M edge A + ~17 M node V).  A "step" is one
backward-Euler step: RHS, FP64-refined solve to ||D^-1 r|| <= 2e-13 ||x||.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
    python bench.py --impl reference ...     # the reference algorithm on the host cores

value   = n_dims * K / (device time of K steps), inputs resident in HBM.
e2e     = the same metric through the public Python API per step (qms_step
          with the step's velocity/field from host memory + read-back of the
          H slice the reference dumps every step).
roofline: the inner solver's matrix-free FP32 operator: algorithmic bytes / CUDA-event
          time of its launches in a second pass of as many steps with the profile's
          events on (the timed pass runs without them).
cpu_baseline: the CPU oracle (C restatement of the reference assembly with
          OpenMP + SuperLU direct solve reused across steps, as PARDISO phase 33)
          on a bounded sample: the same workload at a reduced grid.
"""
from __future__ import annotations

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

METRIC = "DOF-timesteps/s at 256^3, mixed vs FP64 GPU at rel L2<=1e-8; p99 request latency"
UNIT = "DOF-timesteps/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=33,
                    help="timed steps; 33 = one period of the residual chain (32 chained steps and one "
                         "FP64 re-anchor)")
    ap.add_argument("--warmup", type=int, default=20,
                    help="untimed steps; the first ~15 steps of a run adapt the FGMRES replay length and "
                         "build up the extrapolated start (4 solutions)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--cpu-size", type=int, default=0, help="grid of the CPU sample (0: auto)")
    ap.add_argument("--cpu-steps", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the plain FP64 GPU solver leg (its timing and the per-step comparison)")
    ap.add_argument("--workload", default="moving_plate_256", choices=WORKLOADS)
    ap.add_argument("--serving-requests", type=int, default=24,
                    help="requests of the serving sample reported beside the line (0: none)")
    ap.add_argument("--serving-steps", type=int, default=10)
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="steps of the kernel-timing pass (0: as many as the timed steps)")
    ap.add_argument("--fp64-steps", type=int, default=0,
                    help="steps of the FP64 leg (0: the warm-up and timed steps; fewer for grids whose FP64 "
                         "solve takes seconds per step)")
    ap.add_argument("--check-every", type=int, default=None)
    ap.add_argument("--set", action="append", default=[], metavar="FIELD=VALUE",
                    help="override a qms_desc field of the timed solver (e.g. gmres_m=24, mg_alpha=1.8)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, val in zip(names, r[5:9]):
                    if val.lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel):
    """Per-launch DRAM traffic of `kernel` from the committed ncu summary (bytes per unknown), or None."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------
def cpu_sample(size, steps, threads=None):
    """Time the reference algorithm (oracle) on the moving-plate workload at a reduced grid."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import qms_oracle as o
    from alpineqms_gb300 import workloads
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field
    inp, geom = workloads.moving_plate(size, nt=steps + 1, plate=(int(size * 200 / 256), int(size * 200 / 256), 10),
                                       h=256e-3 / size)
    c = o.materials(inp.xs, inp.ys, inp.zs, geom, inp.props_table())
    n = inp.n_dims
    sched = VelocitySchedule(inp.traj, inp.dt)
    B, G = scaled_field(inp.B, inp.G, None, 0.0)
    d = (inp.dx, inp.dy, inp.dz)
    ia, ja, a, b = o.assemble(inp.xs, inp.ys, inp.zs, *d, c, False, inp.dt, sched.steady(), B, G)
    ds = o.DirectSolver()
    ds.factor(ia, ja, a, n)
    x = ds.solve(b)
    # step 1: the velocity changes, the reference refactors (phase 23) -- not timed
    v = sched.step(1)
    ia, ja, a, b = o.assemble(inp.xs, inp.ys, inp.zs, *d, c, True, inp.dt, v, B, G, x)
    ds.factor(ia, ja, a, n)
    x = ds.solve(b)
    t0 = time.perf_counter()
    for k in range(2, steps + 2):       # constant velocity: phase 33 (back-substitution) steps
        v = sched.step(k)
        ia, ja, a, b = o.assemble(inp.xs, inp.ys, inp.zs, *d, c, True, inp.dt, v, B, G, x)
        x = ds.solve(b)
        o.hfield(inp.xs, inp.ys, inp.zs, *d, c, x)
    dtm = time.perf_counter() - t0
    return {"value": n * steps / dtm, "unit": UNIT, "cores": o.num_threads(), "kind": "port",
            "sample": (f"moving plate at {size}^3 (n_dims {n}, h = {256 / size:.2f} mm): {steps} constant-velocity "
                       f"steps of C assembly ({o.num_threads()} OpenMP threads) + SuperLU back-substitution "
                       f"(1 thread, factor reused as PARDISO phase 33) + H; the reference's direct solver "
                       f"cannot hold 256^3 (nnz 1.43e9, its own nnz guard stops it above 100^3)"),
            "seconds": dtm}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    size = args.cpu_size or 20
    # exactly the requested number of timed steps; the factorisation (PARDISO phases 11/22) and
    # the magnetostatic init inside cpu_sample stay outside the timed region
    steps = args.cpu_steps or max(args.steps, 1)
    cb = cpu_sample(size, steps)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * cb["seconds"] / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "moving_plate_256", "sample_grid": [size] * 3},
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def aggregate_replicas(ms_local, units_local, dist=None, device="cpu"):
    """Whole-job timing of N independent replicas: the max of the per-rank times and the
    sum of the units (DOF-timesteps) all ranks processed.  No data-path collective."""
    if dist is None:
        return float(ms_local), float(units_local)
    import torch
    mx = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    sm = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return float(mx.item()), float(sm.item())


WORKLOADS = ("moving_plate_256", "inclusions_96", "laminated_core", "plain_block_32")


def make_workload(args, nt):
    from alpineqms_gb300 import workloads
    if args.workload == "moving_plate_256":
        return workloads.moving_plate(args.size, nt=nt)
    if args.workload == "inclusions_96":
        return workloads.inclusions_96(nt=nt)
    if args.workload == "laminated_core":
        return workloads.laminated_core(nt=nt)
    return workloads.plain_block_32(nt=nt)


class Run:
    """One solver handle driven through a workload's steps: steady init, then transient steps
    with the velocity of trajectory type 1 and the (possibly AC) background field of each step."""

    def __init__(self, inp, geom, desc):
        from alpineqms_gb300.solver import QMSSolver
        from alpineqms_gb300.trajectory import VelocitySchedule
        self.inp = inp
        self.s = QMSSolver(desc)
        self.s.set_geometry_f64(geom, inp.props_table())
        self.sched = VelocitySchedule(inp.traj, inp.dt)
        self.counter = 0

    def field(self, k):
        from alpineqms_gb300.trajectory import scaled_field
        return scaled_field(self.inp.B, self.inp.G, self.inp.excitation, k * self.inp.dt)

    def steady(self):
        B, G = self.field(0)
        return self.s.steady(self.sched.steady(), B, G)

    def args_of_next(self):
        k = self.counter + 1
        B, G = self.field(k)
        return self.sched.step(k), B, G

    def step(self):
        v, B, G = self.args_of_next()
        self.counter += 1
        return self.s.step(v, B, G)

    def close(self):
        self.s.close()


def timed_steps(run, k, ext):
    """k steps bracketed by CUDA events on the library's stream (inputs resident)."""
    import torch
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(ext)
    its = [run.step() for _ in range(k)]
    ev1.record(ext)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), its


def run_gpu(args):
    import numpy as np
    import torch
    from alpineqms_gb300 import compare
    from alpineqms_gb300.solver import default_desc

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    W, K = args.warmup, args.steps
    inp, geom = make_workload(args, W + 2 * K + 4)
    kw = {}
    if args.check_every:
        kw["check_every"] = args.check_every
    for item in args.set:
        key, _, val = item.partition("=")
        kw[key] = float(val) if any(ch in val for ch in ".eE") else int(val)

    def desc_of(precision, **extra):
        return default_desc(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, inp.dt, precision=precision,
                            device=local, **{**kw, **extra})

    desc = desc_of(args.precision)

    # -- 1. device-timed pass: W untimed steps, then K steps between CUDA events
    run = Run(inp, geom, desc)
    n = run.s.n
    t0 = time.perf_counter()
    st0 = run.steady()
    steady_s = time.perf_counter() - t0
    for _ in range(W):
        run.step()
    ext = torch.cuda.ExternalStream(run.s.stream_ptr())
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    clocks.start()
    torch.cuda.nvtx.range_push("timed_steps")     # lets a profiler capture exactly these steps
    ms_local, iters = timed_steps(run, K, ext)
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    ms, units = aggregate_replicas(ms_local, n * K, dist, "cuda")
    if dist:
        dist.barrier()
    value = units / (ms / 1e3)
    run.close()

    # -- 2. end to end through the public API, on the same steps in the same solver states: a
    # fresh handle replays the steady init and the W warm-up steps, then per step the velocity
    # and field scalars come from pinned host memory and the H slice (what the reference dumps
    # every step) is read back
    e2e = None
    run = Run(inp, geom, desc)
    run.steady()
    for _ in range(W):
        run.step()
    if not args.no_e2e:
        hostbuf = torch.empty(15, dtype=torch.float64).pin_memory()
        slice_bytes = 3 * inp.slice_shape()[0] * inp.slice_shape()[1] * 8
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(K):
            v, B, G = run.args_of_next()
            hostbuf[:3] = torch.tensor(v, dtype=torch.float64)
            hostbuf[3:6] = torch.from_numpy(np.asarray(B, np.float64))
            hostbuf[6:15] = torch.from_numpy(np.asarray(G, np.float64).reshape(9))
            hv = hostbuf.numpy()
            run.s.step(hv[:3], hv[3:6], hv[6:15])
            run.counter += 1
            run.s.slices(inp.slice_axis, inp.slice_index)
        torch.cuda.synchronize()
        e2e_ms, e2e_units = aggregate_replicas(1e3 * (time.perf_counter() - t1), n * K, dist, "cuda")
        e2e = {"value": e2e_units / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": 15 * 8,
               "d2h_bytes_per_step": slice_bytes,
               "steps": "the same steps (%d..%d) as the device-timed pass, from the same states" % (W + 1, W + K)}
    else:
        for _ in range(K):
            run.step()

    # -- 3. kernel timings: K more steps with the profile on (CUDA events around every operator,
    # V-cycle and level-0 A-block sweep, recorded into the replayed graphs; two untimed steps
    # first capture the graphs that carry them).  The event records cost time of their own, so
    # this pass is timed apart from the one above and its step time is reported beside it.
    run.s.profile_enable(True)
    for _ in range(2):
        run.step()
    torch.cuda.synchronize()
    run.s.profile_enable(True)          # counts from here
    ext = torch.cuda.ExternalStream(run.s.stream_ptr())
    KP = args.profile_steps if args.profile_steps > 0 else K
    # (a profiler's per-kernel list can capture this range: kernels inside the conditional
    # nodes of the whole-step graphs cannot be profiled one by one, and this pass runs the
    # per-cycle graphs instead)
    torch.cuda.nvtx.range_push("profiled_steps")
    prof_ms, _ = timed_steps(run, KP, ext)
    torch.cuda.nvtx.range_pop()
    prof = run.s.profile()
    run.s.profile_enable(False)
    prof_ms_per_step = prof_ms / KP
    run.close()

    # -- 4. the plain FP64 GPU solver (the same algorithm with every inner component in FP64, the
    # same tolerance) over the same steps, in lockstep with a fresh mixed-precision run: each
    # FP64 step starts from the mixed run's previous solution, its K steps after the same W
    # warm-up are timed between CUDA events on its own stream, and after every step (outside
    # the timed events) the two solutions of that step are compared block by block
    fp64 = accuracy = None
    if rank == 0 and not args.no_fp64 and args.precision == "mixed":
        esig = compare.edge_sigma(inp, geom)
        fixer = compare.GaugeFixer(inp, geom, esig)
        # the FP64 solver's Krylov basis shrinks when both solvers would not fit the device at once
        from alpineqms_gb300.solver import device_bytes
        free_b = torch.cuda.mem_get_info()[0]
        d64 = desc_of("fp64")
        while d64.gmres_m > 8 and device_bytes(desc) + device_bytes(d64) > 0.92 * free_b:
            d64 = desc_of("fp64", gmres_m=d64.gmres_m - 4)
        rm = Run(inp, geom, desc)
        r64 = Run(inp, geom, d64)
        ext64 = torch.cuda.ExternalStream(r64.s.stream_ptr())
        rm.steady()
        r64.steady()
        per_step = []
        t64 = 0.0
        it64 = []
        xm_prev = rm.s.get_state()
        n64 = args.fp64_steps if args.fp64_steps > 0 else W + K
        w64 = min(W, max(n64 - 1, 0))            # untimed FP64 steps before its timed ones
        for k in range(1, n64 + 1):
            rm.step()
            r64.s.set_state(xm_prev)
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(ext64)
            s64 = r64.step()
            ev1.record(ext64)
            torch.cuda.synchronize()
            if k > w64:
                t64 += ev0.elapsed_time(ev1)
                it64.append({"outer": s64["outer"], "inner": s64["inner"]})
            xm, xd = rm.s.get_state(), r64.s.get_state()
            cmp = compare.compare_states(inp, geom, xm, xd, rm.s.fields(), r64.s.fields(), fixer, esig)
            cmp["step"] = k
            per_step.append(cmp)
            xm_prev = xm
        rm.close()
        r64.close()
        k64 = len(it64)
        fp64 = {"value": n * k64 / (t64 / 1e3), "unit": UNIT, "ms_per_step": t64 / k64, "steps": k64,
                "warmup": w64, "tol": desc.tol, "gmres_m": d64.gmres_m, "iters": it64,
                "from": "each step from the mixed run's previous solution",
                "mixed_over_fp64": value / (n * k64 / (t64 / 1e3))}
        keys = ("A", "V_gauge_fixed", "J", "H")
        worst = {q: max(r[q] for r in per_step) for q in keys}
        accuracy = {"vs": "plain FP64 GPU solver at the same tolerance, every step from the same start state "
                          "(the mixed run's previous solution)",
                    "max_rel_l2": worst, "max_rel_l2_V_raw": max(r["V_raw"] for r in per_step),
                    "pass_1e-8": all(worst[q] <= 1e-8 for q in ("A", "V_gauge_fixed", "H")),
                    "V_gauge": "V on the nodes with a conducting edge, each floating body's mean removed (%d "
                               "nodes, %d floating bodies)" % (fixer.nodes.size, int(fixer.floating.sum())),
                    "H": "B / mu at the cell centres (the dumped field)",
                    "per_step": per_step}

    peak, peak_kind = measured_peak()
    # The roofline kernel is the largest single kernel of a step: the level-0 Jacobi sweep on
    # the three A blocks (mg0_tiled<T, 1, 1>).  Algorithmic bytes per launch: x and b read, x
    # written (3 p n_A) and one material byte per cell.
    kms, kbytes, klaunch = prof["mg0a_ms"], prof["mg0a_bytes"], prof["mg0a_launches"]
    achieved = kbytes / (kms / 1e3) / 1e9 if kms > 0 else 0.0
    p = 4 if args.precision == "mixed" else 8
    tr = ncu_traffic("mg0_tiled_f32_a" if p == 4 else "mg0_tiled_f64_a")
    n_a = n - (inp.xs + 1) * (inp.ys + 1) * (inp.zs + 1)
    roofline = {"bound": "hbm", "kernel": "mg0_tiled<%s,1,1> (level-0 Jacobi sweep, A blocks, TMA)" %
                                          ("float" if p == 4 else "double"),
                "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6800 GB/s",
                "traffic": (tr * n_a if tr else None), "launches": klaunch,
                "avg_launch_us": 1e3 * kms / max(klaunch, 1),
                "algorithmic_bytes_per_launch": kbytes / max(klaunch, 1),
                "algorithmic_bytes_def": "3 p n_A + cells (x and b read, x written; one material byte per cell)",
                "share_of_step": kms / (prof_ms_per_step * KP) if prof_ms_per_step > 0 else None,
                "timed_pass": "kernel timings from a later pass of as many steps with CUDA events around the "
                              "timed launches (%.2f ms per step there)" % prof_ms_per_step,
                "other_kernels_ms": {"op32": prof["op32_ms"], "op64": prof["op64_ms"], "vcycles": prof["mg_ms"],
                                     "refinement_residual": prof["resid_ms"]}}
    if prof["op32_launches"] > 0:
        roofline["inner_stencil_fp32"] = {"launches": prof["op32_launches"],
                                          "achieved_gbs": prof["op32_bytes"] / (prof["op32_ms"] / 1e3) / 1e9}

    # -- 5. the serving half of the metric: a sample of the seeded request stream (the first
    # requests of the 512-request stream, fewer steps each) through the native serving object,
    # with its per-step and per-request latency percentiles
    serving = None
    if rank == 0 and args.serving_requests > 0 and args.precision == "mixed":
        from alpineqms_gb300 import serving as srv_mod
        reqs, gaps = srv_mod.poisson_stream(args.serving_requests, 0.05, nt=args.serving_steps)
        t0 = time.perf_counter()
        with srv_mod.NativeServer(150 << 30, 16, device=local) as srv:
            res = srv.serve(reqs, gaps)
            wall = time.perf_counter() - t0
            rep = srv_mod.latency_report(res, wall)
            st_ = srv.stats()
        serving = {"sample": "the first %d requests of the seeded 512-request stream (48^3..128^3, 8-32 "
                             "random ellipsoids, Poisson arrivals 50 ms mean gap), %d steps each, 16 resident, "
                             "150 GB budget" % (args.serving_requests, args.serving_steps),
                   "completed": rep["completed"], "failed": rep["failed"],
                   "step_p50_ms": st_["step_p50_ms"], "step_p99_ms": st_["step_p99_ms"],
                   "request_p50_s": rep["request_p50_s"], "request_p99_s": rep["request_p99_s"],
                   "dof_timesteps_per_s": rep["dof_timesteps_per_s"], "wall_s": wall}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_sample(args.cpu_size or 20, args.cpu_steps or 5)
        except Exception as e:  # the baseline is a report, never the product path
            cpu = {"error": repr(e)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
                "warmup": W, "ms_per_step": ms / K, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
                "config": {"workload": args.workload if args.workload != "moving_plate_256" or args.size == 256
                           else "moving_plate_%d" % args.size,
                           "grid": [inp.xs, inp.ys, inp.zs], "dof": n,
                           "dt": inp.dt, "precision": args.precision, "tol": desc.tol,
                           "solver": {"krylov": "fgmres" if desc.krylov == 0 else "bicgstab",
                                      "gmres_m": desc.gmres_m, "mg_sweeps": desc.mg_sweeps,
                                      "mg_omega": desc.mg_omega, "mg_alpha": desc.mg_alpha,
                                      "mg_coupling": "lower block-triangular" if desc.mg_coupling == 1
                                      else "block-diagonal", "extrapolate": desc.extrapolate, "start_ls": desc.start_ls,
                                      "residual": "FP64 anchor + double-float" if args.precision == "mixed"
                                      else "FP64"},
                           "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                           "l2": "inputs larger than L2 (one FP32 vector = %.0f MB)" % (n * 4 / 1e6)},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": prof["launches"],
                "fp64": fp64, "accuracy": accuracy, "serving": serving,
                "clocks": clk, "steady_s": steady_s,
                "steady_iters": {"outer": st0["outer"], "inner": st0["inner"]},
                "step_iters": [{"outer": q["outer"], "inner": q["inner"], "r0": q["r0"], "r": q["r"]}
                               for q in iters]}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
