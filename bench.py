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
    ap.add_argument("--no-accuracy", action="store_true", help="skip the mixed-vs-FP64 step comparison")
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


def edge_current(inp, geom, x):
    """sigma_edge * dV/dh on every x-, y- and z-edge (sigma_edge the mean of the four cells
    around the edge): how V enters the A rows.  Used to compare potentials up to the
    floating constant of isolated conductors."""
    import numpy as np
    xs, ys, zs = inp.xs, inp.ys, inp.zs
    Nx, Ny, Nz = xs + 1, ys + 1, zs + 1
    oV = 4 * Nx * Ny * Nz - Ny * Nz - Nx * Nz - Nx * Ny - Nx * Ny * Nz
    V = np.asarray(x[oV:]).reshape((Nx, Ny, Nz), order="F")
    g = np.asarray(geom).reshape((xs, ys, zs), order="F")
    table = inp.props_table()
    lut = {int(r[0]): r[4:7] for r in table}
    sig = np.zeros((3, xs, ys, zs))
    for mid, sv in lut.items():
        m = g == mid
        for a in range(3):
            sig[a][m] = sv[a]
    out = []
    for a, (d, n) in enumerate(((inp.dx, xs), (inp.dy, ys), (inp.dz, zs))):
        s = np.pad(sig[a], 1)                   # cells with a zero halo
        # edge along axis a from node p: the four cells sharing it (other two indices p-1, p)
        if a == 0:
            se = 0.25 * (s[1:-1, :-1, :-1] + s[1:-1, 1:, :-1] + s[1:-1, :-1, 1:] + s[1:-1, 1:, 1:])
            dv = (V[1:] - V[:-1]) / d
        elif a == 1:
            se = 0.25 * (s[:-1, 1:-1, :-1] + s[1:, 1:-1, :-1] + s[:-1, 1:-1, 1:] + s[1:, 1:-1, 1:])
            dv = (V[:, 1:] - V[:, :-1]) / d
        else:
            se = 0.25 * (s[:-1, :-1, 1:-1] + s[1:, :-1, 1:-1] + s[:-1, 1:, 1:-1] + s[1:, 1:, 1:-1])
            dv = (V[:, :, 1:] - V[:, :, :-1]) / d
        # the reference forms edge conductivities only for node indices 2..size (F:258-269)
        mask = np.zeros(se.shape, bool)
        mask[1:xs if a != 0 else xs, 1:ys if a != 1 else ys, 1:zs if a != 2 else zs] = True
        if a == 0:
            mask[0] = False
        elif a == 1:
            mask[:, 0] = False
        else:
            mask[:, :, 0] = False
        out.append((np.where(mask, se, 0.0) * dv).ravel(order="F"))
    return np.concatenate(out)


# ---------------------------------------------------------------------------
def run_gpu(args):
    import numpy as np
    import torch
    from alpineqms_gb300 import workloads
    from alpineqms_gb300.solver import QMSSolver, default_desc
    from alpineqms_gb300.trajectory import VelocitySchedule, scaled_field

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    inp, geom = workloads.moving_plate(args.size, nt=args.steps + args.warmup + 1)
    kw = {}
    if args.check_every:
        kw["check_every"] = args.check_every
    for item in args.set:
        key, _, val = item.partition("=")
        kw[key] = float(val) if any(ch in val for ch in ".eE") else int(val)
    desc = default_desc(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, inp.dt, precision=args.precision,
                        device=local, **kw)
    solver = QMSSolver(desc)
    solver.set_geometry_f64(geom, inp.props_table())
    n = solver.n
    sched = VelocitySchedule(inp.traj, inp.dt)
    B, G = scaled_field(inp.B, inp.G, inp.excitation, 0.0)
    t0 = time.perf_counter()
    st0 = solver.steady(sched.steady(), B, G)
    steady_s = time.perf_counter() - t0
    counter = 0
    for _ in range(args.warmup):
        counter += 1
        solver.step(sched.step(counter), B, G)

    ext = torch.cuda.ExternalStream(solver.stream_ptr())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    iters = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0.record(ext)
    for _ in range(args.steps):
        counter += 1
        iters.append(solver.step(sched.step(counter), B, G))
    ev1.record(ext)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms, units = aggregate_replicas(ev0.elapsed_time(ev1), n * args.steps, dist, "cuda")
    if dist:
        dist.barrier()
    value = units / (ms / 1e3)

    # Kernel timings: as many steps again with the profile on (CUDA events around every operator
    # and V-cycle launch, recorded into the replayed graphs; two untimed steps first capture the
    # graphs that carry them).  The event records cost time of their own, so this pass is timed
    # apart from the one above and its step time is reported beside it.
    solver.profile_enable(True)
    for _ in range(2):
        counter += 1
        solver.step(sched.step(counter), B, G)
    torch.cuda.synchronize()
    solver.profile_enable(True)          # counts from here
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev2.record(ext)
    piters = []
    for _ in range(args.steps):
        counter += 1
        piters.append(solver.step(sched.step(counter), B, G))
    ev3.record(ext)
    torch.cuda.synchronize()
    prof = solver.profile()
    solver.profile_enable(False)
    prof_ms_per_step = ev2.elapsed_time(ev3) / args.steps

    # end to end through the public API: per step the velocity / field scalars come from
    # pinned host memory and the H slice (what the reference dumps every step) is read back
    e2e = None
    if not args.no_e2e:
        hostbuf = torch.empty(15, dtype=torch.float64).pin_memory()
        slice_bytes = 3 * inp.slice_shape()[0] * inp.slice_shape()[1] * 8
        # two untimed steps capture the graphs without the profile's event records
        for _ in range(2):
            counter += 1
            solver.step(sched.step(counter), B, G)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(args.steps):
            counter += 1
            v = sched.step(counter)
            hostbuf[:3] = torch.tensor(v, dtype=torch.float64)
            hostbuf[3:6] = torch.from_numpy(np.asarray(B))
            hostbuf[6:15] = torch.from_numpy(np.asarray(G))
            hv = hostbuf.numpy()
            solver.step(hv[:3], hv[3:6], hv[6:15])
            solver.slices(inp.slice_axis, inp.slice_index)
        torch.cuda.synchronize()
        e2e_ms, e2e_units = aggregate_replicas(1e3 * (time.perf_counter() - t1), n * args.steps, dist, "cuda")
        e2e = {"value": e2e_units / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": 15 * 8,
               "d2h_bytes_per_step": slice_bytes}

    # Accuracy at the bench workload: one more step in both precisions from the same state,
    # compared per unknown block (A, V) and on H, the field the reference dumps.
    accuracy = None
    if not args.no_accuracy and rank == 0 and args.precision == "mixed":
        x_prev = solver.get_state()
        counter += 1
        v = sched.step(counter)
        stm = solver.step(v, B, G)
        xm = solver.get_state()
        hm = [h.copy() for h in solver.fields()]
        # the solver's own final residual (double-float, or from the Arnoldi relation) against
        # the exact FP64 residual of the same state
        r_exact = solver.residual_norm(True, v)
        # the FP64 reference step is solved well below the mixed solver's tolerance, so the
        # difference measures the mixed solver's error rather than the reference's
        s64 = QMSSolver(default_desc(inp.xs, inp.ys, inp.zs, inp.dx, inp.dy, inp.dz, inp.dt, precision="fp64",
                                     device=local, tol=1e-14, max_outer=60))
        s64.set_geometry_f64(geom, inp.props_table())
        s64.set_state(x_prev)
        st64 = s64.step(v, B, G)
        xd = s64.get_state()
        hd = s64.fields()
        oV = n - (inp.xs + 1) * (inp.ys + 1) * (inp.zs + 1)

        def rel(a, b):
            nb = float(np.linalg.norm(b))
            return float(np.linalg.norm(a - b)) / nb if nb > 0 else float(np.linalg.norm(a))
        jm, jd = edge_current(inp, geom, xm), edge_current(inp, geom, xd)
        accuracy = {"vs": "fp64 GPU solver (tol 1e-14), same start state, one step", "step": counter,
                    "rel_l2_A": rel(xm[:oV], xd[:oV]), "rel_l2_J": rel(jm, jd),
                    "rel_l2_H": rel(np.concatenate([h.ravel() for h in hm]), np.concatenate([h.ravel() for h in hd])),
                    "rel_l2_V_raw": rel(xm[oV:], xd[oV:]),
                    "note": "V enters through sigma grad V (J); an isolated conductor's potential carries an "
                            "arbitrary constant that no residual sees",
                    "fp64_iters": {"outer": st64["outer"], "inner": st64["inner"]},
                    "final_residual": {"reported": stm["r"], "fp64": r_exact, "tol": desc.tol}}
        accuracy["pass_1e-8"] = all(accuracy[k] <= 1e-8 for k in ("rel_l2_A", "rel_l2_J", "rel_l2_H"))
        s64.close()

    peak, peak_kind = measured_peak()
    # The roofline kernel is the inner solver's stencil (the TMA-staged operator on the padded
    # layout): algorithmic bytes 2 p n + cells per launch (x and y, one material byte per cell).
    inner = "fp32" if args.precision == "mixed" else "fp64"
    kms = prof["op32_ms"] if inner == "fp32" else prof["op64_ms"]
    kbytes = prof["op32_bytes"] if inner == "fp32" else prof["op64_bytes"]
    klaunch = prof["op32_launches"] if inner == "fp32" else prof["op64_launches"]
    kern = "qk_op_pl<float> (inner stencil, TMA)" if inner == "fp32" else "qk_op_pl<double> (inner stencil, TMA)"
    achieved = kbytes / (kms / 1e3) / 1e9 if kms > 0 else 0.0
    tr = ncu_traffic("qk_op_pl_f32" if inner == "fp32" else "qk_op_pl_f64")
    roofline = {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6800 GB/s",
                "traffic": (tr * n if tr else None), "launches": klaunch,
                "avg_launch_us": 1e3 * kms / max(klaunch, 1),
                "algorithmic_bytes_per_launch": kbytes / max(klaunch, 1),
                "algorithmic_bytes_def": "2 p n_dims + cells (x, y, one material byte per cell)",
                "share_of_step": kms / (prof_ms_per_step * args.steps) if prof_ms_per_step > 0 else None,
                "timed_pass": "the kernel timings come from a second pass of as many steps with CUDA events "
                              "around every operator / V-cycle launch (%.2f ms per step there)" % prof_ms_per_step,
                "op32_ms": prof["op32_ms"], "op64_ms": prof["op64_ms"], "mg_ms": prof["mg_ms"],
                "mg_cycles": prof["mg_cycles"]}
    if prof["resid_launches"] > 0:
        # the refinement residuals: the FP64 anchor (bound by GB300's FP64 rate), the double-float
        # ones from the anchor, and the chained step start
        roofline["refinement_residual"] = {"launches": prof["resid_launches"], "ms": prof["resid_ms"],
                                     "avg_launch_us": 1e3 * prof["resid_ms"] / prof["resid_launches"],
                                     "achieved_gbs": prof["resid_bytes"] / (prof["resid_ms"] / 1e3) / 1e9
                                     if prof["resid_ms"] > 0 else None}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_sample(args.cpu_size or 20, args.cpu_steps or 5)
        except Exception as e:  # the baseline is a report, never the product path
            cpu = {"error": repr(e)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
                "config": {"workload": "moving_plate_256", "grid": [inp.xs, inp.ys, inp.zs], "dof": n,
                           "dt": inp.dt, "precision": args.precision, "tol": desc.tol,
                           "solver": {"krylov": "fgmres" if desc.krylov == 0 else "bicgstab",
                                      "gmres_m": desc.gmres_m, "mg_sweeps": desc.mg_sweeps,
                                      "mg_omega": desc.mg_omega, "mg_alpha": desc.mg_alpha,
                                      "mg_coupling": "lower block-triangular" if desc.mg_coupling == 1
                                      else "block-diagonal", "extrapolate": desc.extrapolate,
                                      "residual": "FP64 anchor + double-float" if args.precision == "mixed"
                                      else "FP64"},
                           "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                           "l2": "inputs larger than L2 (one FP32 vector = %.0f MB)" % (n * 4 / 1e6)},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": prof["launches"],
                "accuracy": accuracy,
                "clocks": clk, "steady_s": steady_s,
                "steady_iters": {"outer": st0["outer"], "inner": st0["inner"]},
                "step_iters": [{"outer": s["outer"], "inner": s["inner"], "r0": s["r0"], "r": s["r"]}
                               for s in iters]}
        print(json.dumps(line))
    solver.close()
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
