"""Benchmark of the channel-flow hot path on one GB300 (or N replicas).

Workload (the reference's metric is quoted on it: 128^3 plain FP64):
a 128 x 128 x 128 channel, 2*pi*h x 2h x pi*h, tanh wall stretching
(gamma 2.0), seeded laminar-plus-noise state at Mach 0.5.  One step is one
right-hand-side evaluation of the reference's per-step sequence: x halo,
wall and periodic ghosts, Filter (ADM sensor), Flux_X/Y/Z_limiter and
Viscous_terms, all FP64.  ``value`` = cells x steps / time (Mcell-updates/s
per RHS) with every input resident in HBM; ``e2e`` = the same through the
C-ABI on registered HOST arrays, with the state uploaded and the face fluxes
and viscous terms (the RHS) downloaded every step.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl gb300|reference]

``--impl reference`` times the CPU implementation of the same steps (the C
restatement of the reference routines in oracle/, OpenMP on all host
cores), on rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

GRID = (128, 128, 128)
GAMMA = 2.0
SEED = 2800
FILTER_ARGS = (0.007, 1.0, 0.0)        # Roe_criterion, E_high, E_low (main.cpp:55-57)
# algorithmic bytes per cell of each routine, FP64: arrays of the routine's
# signature read and written once (Filter 7+3, limited fluxes 16/17 + 5,
# viscous 36 + 4 arrays of 8 bytes)
ALG_BYTES = {"Filter": 80, "Flux_X_limiter": 168, "Flux_Y_limiter": 176, "Flux_Z_limiter": 176,
             "Viscous_terms": 320, "Dual_time_stepping": 2680}
# routines eligible as "the dominant kernel" of the roofline: the single
# launches of Flux_X/Y_limiter and Flux_Z_limiter, whose interior-face
# launch (the step's longest single launch) is timed together with its two
# short companions (z weights, edge faces: about 5 % of the routine)
ROOF_KERNELS = {"Flux_X_limiter": "k_flux<0,true,double>", "Flux_Y_limiter": "k_flux<1,true,double>",
                "Flux_Z_limiter": "k_flux<2,true,double,ZP=1> (+ k_flux_zweights, k_flux<2,true,double,ZP=2>)"}
# DRAM bytes per cell measured by ncu (dram__bytes_read.sum + write.sum of one
# launch on the 96^3 case divided by its cells) and FP64-pipe activity
NCU_TRAFFIC_PER_CELL = {"Flux_X_limiter": (76.687360e6 + 11.400192e6) / (96 * 96 * 96),
                        "Flux_Y_limiter": (76.323328e6 + 11.568640e6) / (96 * 96 * 96),
                        "Flux_Z_limiter": (81.8e6 + 12.1e6) / (96 * 96 * 93)}
NCU_FP64_PIPE_PCT = {"Flux_X_limiter": 87.6, "Flux_Y_limiter": 87.3, "Flux_Z_limiter": 87.4}
# floating-point operations per interior cell of the routine's algorithm:
# the exact count of the oracle's restatement on the seeded 64x48x32 case
# (tests/golden/flop_counts.json, made by tests/golden/make_flop_counts.py)
ALG_FLOPS_PER_CELL = {"Flux_X_limiter": 1001.5, "Flux_Y_limiter": 998.3, "Flux_Z_limiter": 1023.7}
FP64_NOMINAL_TFLOPS = 1.25   # GB300 FP64 (non-tensor), nominal
LU_SUBITERATIONS = 10   # LU-SGS sub-iterations of one physical step of the fixed-count schedule
L2_BYTES = 129 * 2 ** 20


def fp64_peak(torch, blocks=152 * 8, iters=4096, reps=5):
    """Measured FP64 rate of this GPU: sixteen independent FMA chains per
    thread (cf_fp64_peak_probe), CUDA events around `reps` launches after
    one warm-up; TFLOP/s (an FMA counted as two operations)."""
    from channel_flow_gb300 import _lib
    lib = _lib.load()
    out = torch.zeros(blocks, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    _lib.check(lib, None, lib.cf_fp64_peak_probe(s.cuda_stream, blocks, iters, out.data_ptr()))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        _lib.check(lib, None, lib.cf_fp64_peak_probe(s.cuda_stream, blocks, iters, out.data_ptr()))
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    return 2.0 * 16 * 256 * iters * blocks / (ms * 1e-3) / 1e12, ms


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# --------------------------------------------------------------------------
# workload

LU_SCHEDULE = None   # --lu-schedule


def new_context(cf, g, **kw):
    """A context with the bench's sweep schedule (--lu-schedule)."""
    ctx = cf.Context(g, **kw)
    if LU_SCHEDULE:
        ctx.set_lu_schedule(LU_SCHEDULE)
    return ctx


def make_host_workload(g):
    """numpy arrays of the benchmark channel (host, set-up only)."""
    from channel_flow_gb300 import synthetic as syn
    cm = syn.flat_metrics(g, GAMMA, "cell")
    J = cm["J"]
    U = syn.channel_state(g, J, seed=SEED, mach=0.5, noise=0.05, jitter=0.01, gamma=GAMMA)
    Yp = syn.y_points(g, gamma=GAMMA)
    return {"U": U, "J": J, "cm": [cm[n] for n in syn.METRIC_NAMES], "Yp": Yp}


class DeviceWorkload:
    def __init__(self, ctx, g, host, torch):
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        z = lambda: torch.zeros(g.shape, dtype=torch.float64, device="cuda")
        self.U = [dev(a) for a in host["U"]]
        self.J = dev(host["J"])
        self.cm = [dev(a) for a in host["cm"]]
        self.Yp = dev(host["Yp"])
        # face metrics from the GPU Jacobian_u/v/w routines (flat walls)
        self.fu = [z() for _ in range(10)]
        self.fv = [z() for _ in range(10)]
        self.fw = [z() for _ in range(10)]
        ctx.Jacobian_u(*self.fu)
        ctx.Jacobian_v(*self.fv, self.J, *self.cm)
        ctx.Jacobian_w(*self.fw)
        self.Ep = [z() for _ in range(3)]
        self.Fx = [z() for _ in range(5)]
        self.Fy = [z() for _ in range(5)]
        self.Fz = [z() for _ in range(5)]
        self.vF = [z() for _ in range(4)]
        self.LL = [z() for _ in range(4)]
        self.ML = [z() for _ in range(4)]
        self.NL = [z() for _ in range(4)]
        torch.cuda.synchronize()

    def outputs(self):
        return self.Fx + self.Fy + self.Fz + self.vF


def rhs_calls(ctx, w, ptr):
    """The per-step routine calls as (name, function, args) with the
    pointer arguments resolved once; `ptr` maps a field to what the C-ABI
    gets (a device pointer, or a registered host array's address)."""
    lib, h = ctx.lib, ctx.h
    U = [ptr(x) for x in w.U]
    J = ptr(w.J)
    cm = [ptr(x) for x in w.cm]
    fu, fv, fw = ([ptr(x) for x in s] for s in (w.fu, w.fv, w.fw))
    Ep = [ptr(x) for x in w.Ep]
    F = {"x": [ptr(x) for x in w.Fx], "y": [ptr(x) for x in w.Fy], "z": [ptr(x) for x in w.Fz]}
    vF = [ptr(x) for x in w.vF]
    none10 = [None] * 10
    from channel_flow_gb300 import _lib
    visc = U + vF + [J] + cm + fu + fv + fw + [None] * 6 + [ptr(x) for x in w.LL] + [None] * 6 + \
        [ptr(x) for x in w.ML] + [None] * 6 + [ptr(x) for x in w.NL]
    visc_arr = _lib.ptr_array(visc)
    calls = [
        ("X_periodic", lib.cf_X_periodic, (h, 0, *U)),
        ("Y_boundary_condition", lib.cf_Y_boundary_condition, (h, 0, *U, J)),
        ("Z_boundary_condition", lib.cf_Z_boundary_condition, (h, 0, *U, J)),
        ("Filter", lib.cf_Filter, (h, 0, *FILTER_ARGS, *U, ptr(w.Yp), *Ep, J)),
        ("Flux_X_limiter", lib.cf_Flux_X_limiter, (h, 0, *U, *none10, J, *fu, *F["x"], Ep[0])),
        ("Flux_Y_limiter", lib.cf_Flux_Y_limiter, (h, 0, *U, *none10, J, *fv, *F["y"], Ep[1])),
        ("Flux_Z_limiter", lib.cf_Flux_Z_limiter, (h, 0, *U, *none10, J, *fw, *F["z"], Ep[2])),
        ("Viscous_terms", lib.cf_Viscous_terms, (h, 0, visc_arr)),
    ]
    return calls


# kernels launched per RHS step: x halo 1, y wall 1, z periodic 1, Filter
# (1 coefficients + 2 x 6 fused levels + 2 energy + 3 ghost fills + 3
# thresholds = 21), fluxes (FP64: x, y, z weights, z interior, z edges = 5;
# FP32: an FP32 copy of U and J before each of the three, z in two parts =
# 7), viscous (primitives, three face sets, divergence = 5)
LAUNCHES_PER_STEP = {"fp64": 1 + 1 + 1 + 21 + 5 + 5, "fp64_exact": 1 + 1 + 1 + 21 + 5 + 5,
                     "fp32": 1 + 1 + 1 + 21 + 7 + 5}


def run_calls(ctx, calls):
    from channel_flow_gb300 import _lib
    for name, fn, args in calls:
        rc = fn(*args)
        if rc:
            _lib.check(ctx.lib, ctx.h, rc)


# --------------------------------------------------------------------------
# clocks

class ClockSampler:
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        busy = [s for s in sm if smax and s > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# CPU arm (C restatement of the reference routines)

def cpu_rhs_port(g, host, faces):
    """One RHS on the host cores with the C oracle (same routine sequence)."""
    from oracle.cforacle import Port
    port = Port()
    U = [a.copy() for a in host["U"]]
    J, cm, Yp = host["J"], host["cm"], host["Yp"]
    z = lambda: np.zeros(g.shape)
    Ep = [z() for _ in range(3)]
    F = [[z() for _ in range(5)] for _ in range(3)]
    scratch = [z() for _ in range(10)]
    vF = [z() for _ in range(4)]
    vs = [z() for _ in range(30)]

    def step():
        port.x_periodic(g, U)
        port.Y_boundary_condition(g, U + [J])
        port.Z_boundary_condition(g, U + [J])
        port.Filter(g, *FILTER_ARGS, U + [Yp] + Ep + [J])
        for d, name in enumerate(("Flux_X_limiter", "Flux_Y_limiter", "Flux_Z_limiter")):
            port.flux(name, g, U + scratch + [J] + faces[d] + F[d] + [Ep[d]])
        port.Viscous_terms(g, U + vF + [J] + cm + faces[0] + faces[1] + faces[2] + vs)
    return step


# the C restatement against the reference's own routine sources built by
# the oracle recipe, one 128^3 RHS on the same 8 x86 cores (the reference
# does not build on the Arm GPU host): restatement time / reference time
PORT_OVER_REFERENCE = {"time_ratio": 0.80, "restatement_s": [1.01, 1.33], "reference_s": [1.26, 1.67],
                       "where": "x86, 8 threads, 128^3 RHS (Filter + limited fluxes + Viscous_terms)"}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def host_faces(g, host):
    """face metrics on the host (C oracle of Jacobian_u/v/w, same gamma)"""
    from oracle.cforacle import Port
    port = Port()
    faces = []
    for w in ("u", "v", "w"):
        arrs = [np.zeros(g.shape) for _ in range(10)]
        extra = [host["J"]] + host["cm"] if w == "v" else []
        port.Jacobian_face(w, g, GAMMA, arrs + extra)
        faces.append(arrs)
    return faces


def time_cpu(g, host, steps, warmup):
    faces = host_faces(g, host)
    step = cpu_rhs_port(g, host, faces)
    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = time.perf_counter() - t0
    return g.cells * steps / dt / 1e6, dt / steps


# --------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp64_exact", "fp32"])
    ap.add_argument("--grid", default="x".join(map(str, GRID)))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-large", action="store_true", help="skip the 256x192x192 secondary measurement")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-guess physical-step comparison")
    ap.add_argument("--no-wavy", action="store_true", help="skip the 512x256x384 wavy-wall measurement")
    ap.add_argument("--step", default="rhs",
                    choices=["rhs", "lusgs", "mlp", "physical", "northstar", "guess", "schedule"],
                    help="rhs: the benchmark (one RHS per step); lusgs: time Dual_time_stepping alone "
                         "(one LU-SGS pseudo-iteration per step, for profiling); mlp: the learned guess's "
                         "tensor-core GEMMs on --mlp-rows feature rows; physical: whole physical steps "
                         "(cf_step, sub-iterations to the 1e-6 tolerance, extrapolated start) of the "
                         "configuration 2/3 physics, for profiling; northstar: the FP64 against mixed+learned "
                         "physical-step comparison alone; guess: the learned guess's kernels on --grid after a "
                         "short harvest, for profiling; schedule: a configuration's fixed schedule (--config) "
                         "in FP64 and FP32 with the profiles compared")
    ap.add_argument("--mlp-rows", type=int, default=2097152, help="rows (cells) of the --step mlp GEMMs")
    ap.add_argument("--config", default="0", choices=sorted(SCHEDULES),
                    help="--step schedule: which configuration's fixed schedule to run")
    ap.add_argument("--schedule-steps", type=int, default=0, help="--step schedule: steps (0 = the configuration's)")
    ap.add_argument("--compare-steps", type=int, default=0,
                    help="--step schedule: run FP64 for this many steps only and compare there (0 = all)")
    ap.add_argument("--dt-factor", type=float, default=1.0, help="--step schedule: time step / (0.005 h/U_b)")
    ap.add_argument("--lu-schedule", default=None, choices=["wavefront", "pencil", "planes"],
                    help="sweep schedule of Dual_time_stepping (default: the library's)")
    args = ap.parse_args()
    dims = tuple(int(x) for x in args.grid.split("x"))
    global LU_SCHEDULE
    LU_SCHEDULE = args.lu_schedule

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    from channel_flow_gb300 import synthetic as syn
    g = syn.channel_grid(*dims)
    workload = f"rhs_{dims[0]}x{dims[1]}x{dims[2]}_{args.precision}"
    cfg = {"workload": workload, "grid": list(dims), "cells": g.cells,
           "domain": "2*pi*h x 2h x pi*h, tanh stretching gamma 2.0, Mach 0.5, laminar + 5% noise",
           "step": "x halo + wall/periodic ghosts + Filter + Flux_X/Y/Z_limiter + Viscous_terms",
           "precision": args.precision,
           "l2": "working set of a step about 1.5 GB (> 129 MB L2); no flush needed"}

    if args.impl == "reference":
        if rank != 0:
            return 0
        host = make_host_workload(g)
        value, sec = time_cpu(g, host, max(1, args.steps), max(0, min(args.warmup, 1)))
        cores = cpu_threads()
        sample = f"{args.steps} RHS evaluations of the {dims[0]}x{dims[1]}x{dims[2]} workload (C restatement, OpenMP)"
        line = {"impl": "reference", "metric": "Mcell-updates/s per RHS", "value": value,
                "unit": "Mcell-updates/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": cfg,
                "cpu_baseline": {"value": value, "unit": "Mcell-updates/s", "cores": cores, "kind": "port",
                                 "sample": sample, "port_over_reference": PORT_OVER_REFERENCE},
                "e2e": {"value": value, "unit": "Mcell-updates/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch
    import channel_flow_gb300 as cf

    if args.step == "mlp":
        torch.cuda.set_device(local)
        r = mlp_gemms(torch, args.mlp_rows, max(2, args.steps), max(1, args.warmup))
        if rank == 0:
            print(json.dumps(r))
        return 0
    if args.step == "guess":
        torch.cuda.set_device(local)
        from channel_flow_gb300 import mlp, stepper
        g, ctx, w, dt = northstar_case(torch, dims, "fp32")
        st = stepper.Stepper(ctx, stepper.fields_from_workload(w, torch, g), deltaT=dt, **NS_STEP)
        hist = [[u.clone() for u in st.f["U"]]]
        for _ in range(5):
            st.step(None)
            hist.append([u.clone() for u in st.f["U"]])
        net = mlp.LearnedGuess(capacity=g.cells, seed=0, lr=2e-3, batch=min(g.cells, 131072))
        net.train(g, hist, epochs=2, batch=min(g.cells, 131072))
        r = guess_breakdown(torch, net, g, hist[-3:], st.f["U_"], reps=max(1, args.steps))
        ctx.close()
        print(json.dumps({"step": "guess", "grid": list(dims), "ms": r}))
        return 0
    if args.step == "schedule":
        torch.cuda.set_device(local)
        with solver_stream(torch):
            r = schedule_run(torch, args.config, steps=args.schedule_steps or None,
                             compare_steps=args.compare_steps or None, dt_factor=args.dt_factor)
        if rank == 0:
            print(json.dumps({"step": "schedule", **r}))
        return 0
    if args.step == "northstar":
        torch.cuda.set_device(local)
        with solver_stream(torch):
            r = physical_step_to_tolerance(torch)
        if rank == 0:
            print(json.dumps({"step": "northstar", "physical_step_to_tolerance": r}))
        return 0
    if args.step == "physical":
        torch.cuda.set_device(local)
        with solver_stream(torch):
            r = physical_steps(torch, g, args.precision, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps(r))
        return 0

    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    host = make_host_workload(g)
    ctx = new_context(cf, g, precision=args.precision, gamma=GAMMA)
    w = DeviceWorkload(ctx, g, host, torch)
    calls = rhs_calls(ctx, w, lambda x: x.data_ptr())
    stream = torch.cuda.current_stream()

    # warm-up (allocates the scratch on the first call)
    for _ in range(max(args.warmup, 3)):
        run_calls(ctx, calls)
    torch.cuda.synchronize()
    if args.step == "lusgs":
        r = pseudo_iteration(ctx, g, w, calls, stream, torch, max(2, args.steps))
        print(json.dumps({"step": "lusgs", "metric": "ms per Dual_time_stepping", "value": r["dual_time_lusgs_ms"],
                          "unit": "ms", "higher_is_better": False, "config": cfg, "detail": r}))
        ctx.close()
        return 0

    # timed region: K steps, events around every routine for the roofline
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        total_ms, per_routine = timed_steps(ctx, calls, args.steps, stream, torch)
    total_ms, value = replica_value(torch, dist, total_ms, g.cells, args.steps, world)
    ms_per_step = total_ms / args.steps

    # roofline of the dominant single kernel (the slowest limited flux) with
    # the byte model; traffic = ncu DRAM bytes per cell x cells
    hbm, peak_kind = peaks()
    try:
        fp64_pk, fp64_ms = fp64_peak(torch)
        fp64_kind = f"measured: FP64 FMA chains (cf_fp64_peak_probe), {fp64_ms:.2f} ms per launch"
    except Exception as exc:   # reported, with the nominal figure in its place
        fp64_pk, fp64_kind = FP64_NOMINAL_TFLOPS, f"nominal (probe failed: {exc})"
    dom = max(ROOF_KERNELS, key=lambda nm: per_routine[nm])
    achieved = ALG_BYTES[dom] * g.cells / (per_routine[dom] * 1e-3) / 1e9
    traffic = NCU_TRAFFIC_PER_CELL.get(dom)
    roof = {"bound": "hbm", "kernel": ROOF_KERNELS[dom], "routine": dom, "achieved": achieved, "peak": hbm,
            "unit": "GB/s", "frac": achieved / hbm, "peak_kind": peak_kind,
            "alg_bytes_per_cell": ALG_BYTES[dom], "launch_ms": per_routine[dom],
            "traffic": traffic * g.cells if traffic else None,
            "traffic_source": "ncu dram bytes of one launch at 96^3 scaled by cells" if traffic else None,
            "fp64_pipe_active_pct": NCU_FP64_PIPE_PCT.get(dom),
            "fp64": {"alg_flops_per_cell": ALG_FLOPS_PER_CELL[dom],
                     "achieved_tflops": ALG_FLOPS_PER_CELL[dom] * g.cells / (per_routine[dom] * 1e-3) / 1e12,
                     "peak_tflops": fp64_pk, "peak_kind": fp64_kind, "nominal_tflops": FP64_NOMINAL_TFLOPS,
                     "frac": ALG_FLOPS_PER_CELL[dom] * g.cells / (per_routine[dom] * 1e-3) / 1e12 / fp64_pk},
            "per_routine_ms": {k: round(v, 4) for k, v in per_routine.items()},
            "note": "FP64 on GB300 (1/64 of FP32 rate) is FP64-pipe bound (ncu: 84-88% pipe busy, "
                    "DRAM 1%): fp64.frac (the oracle's exact flop count per cell over the launch time, "
                    "against the FP64 rate measured in this run by FMA chains) is the binding roofline; "
                    "the HBM fraction is the byte-model figure"}

    # secondary measurements on the same workload: FP32 kernels, and one
    # dual-time pseudo-iteration (RHS + hyperplane LU-SGS) per precision
    extra = {}
    try:
        extra = secondary(ctx, g, w, calls, stream, torch, args)
    except Exception as exc:
        extra = {"error": repr(exc)}

    # e2e through the C-ABI with registered host arrays
    e2e = None
    try:
        e2e = measure_e2e(ctx, g, host, w, torch, args.steps)
    except Exception as exc:  # reported, not hidden
        e2e = {"error": str(exc)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            csteps = 2 if g.cells >= 2_000_000 else 4
            cval, csec = time_cpu(g, host, csteps, 0)
            cpu = {"value": cval, "unit": "Mcell-updates/s", "cores": cpu_threads(), "kind": "port",
                   "port_over_reference": PORT_OVER_REFERENCE,
                   "sample": f"{csteps} RHS evaluations of the full workload on the host cores "
                             f"(C restatement of the reference routines, OpenMP), {csec:.2f} s each"}
        except Exception as exc:
            cpu = {"error": str(exc)}

    if rank == 0:
        line = {"metric": "Mcell-updates/s per RHS", "value": value, "unit": "Mcell-updates/s",
                "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.precision != "fp32" else "f32", "data": "synthetic",
                "config": cfg, "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "secondary": extra,
                "clocks": clocks.summary(), "gpu_launches": LAUNCHES_PER_STEP[args.precision] * args.steps,
                "parallelism": "replicas" if world > 1 else "single"}
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def timed_steps(ctx, calls, steps, stream, torch):
    """K steps bracketed by CUDA events on the context's stream, with an
    event between every two routine calls; returns (total ms, ms per routine)."""
    from channel_flow_gb300 import _lib
    names = [c[0] for c in calls]
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(calls) + 1)] for _ in range(steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for s in range(steps):
        for n, (name, fn, a) in enumerate(calls):
            ev[s][n].record(stream)
            rc = fn(*a)
            if rc:
                _lib.check(ctx.lib, ctx.h, rc)
        ev[s][len(calls)].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    per = {nm: 0.0 for nm in names}
    for s in range(steps):
        for n, nm in enumerate(names):
            per[nm] += ev[s][n].elapsed_time(ev[s][n + 1]) / steps
    return t_start.elapsed_time(t_end), per


def pseudo_iteration(ctx, g, w, calls, stream, torch, steps):
    """RHS and Dual_time_stepping timings of one context, in its current
    precision; the state is restored between the LU-SGS calls."""
    from channel_flow_gb300 import _lib
    z = lambda: torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    U0 = [u.clone() for u in w.U]
    Un = [u.clone() for u in w.U]
    Uq = [u.clone() for u in w.U]
    lu = [z() for _ in range(20)]          # MR, NR, NL, Residual
    arrays = w.U + Un + Uq + [w.J] + w.cm + w.Fx + w.Fy + w.Fz + w.vF + lu
    ptrs = _lib.ptr_array([a.data_ptr() for a in arrays])
    er = np.zeros(5)
    e = [er[n:].ctypes.data for n in range(5)]
    dt = 0.00000005
    for _ in range(2):
        run_calls(ctx, calls)
    torch.cuda.synchronize()
    tot, per = timed_steps(ctx, calls, steps, stream, torch)
    rhs_ms = tot / steps
    lu_ms = []
    for it in range(3):
        for u, u0 in zip(w.U, U0):
            u.copy_(u0)
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        rc = ctx.lib.cf_Dual_time_stepping(ctx.h, 0, dt, *e, None, None, ptrs)
        t1.record(stream)
        torch.cuda.synchronize()
        _lib.check(ctx.lib, ctx.h, rc)
        if it > 0:
            lu_ms.append(t0.elapsed_time(t1))
    for u, u0 in zip(w.U, U0):
        u.copy_(u0)
    del Un, Uq, lu, arrays
    dts = sum(lu_ms) / len(lu_ms)
    return {"rhs_ms": rhs_ms, "rhs_mcell_updates_per_s": g.cells / (rhs_ms * 1e-3) / 1e6,
            "dual_time_lusgs_ms": dts, "pseudo_iteration_ms": rhs_ms + dts,
            "physical_step_s": LU_SUBITERATIONS * (rhs_ms + dts) * 1e-3,
            "per_routine_ms": {k: round(v, 4) for k, v in per.items()}}


# rows 10..16 of the Statistic accumulators: sums of U, V, W, UU, VV, WW, UV
# per wall-normal row (Statistic.cpp:1053-1068)
STAT_ROWS = {"U": 10, "V": 11, "W": 12, "UU": 13, "VV": 14, "WW": 15, "UV": 16}


def stat_profiles(acc, g, steps):
    """Mean velocity and Reynolds-stress profiles (interior rows) from the
    Statistic accumulators of `steps` steps: the sums over x, z and steps
    divided by their count, as the st files hold them (Statistic.cpp:1102),
    and the stresses <u'u'> = <UU> - <U>^2 and so on."""
    Ym = g.Y_out + 4
    n = float(g.X_out) * g.Z_out * steps
    row = lambda name: acc[STAT_ROWS[name] * Ym + 2: STAT_ROWS[name] * Ym + g.ny + 1] / n
    U, V, W = row("U"), row("V"), row("W")
    return {"U": U, "V": V, "W": W, "uu": row("UU") - U * U, "vv": row("VV") - V * V,
            "ww": row("WW") - W * W, "uv": row("UV") - U * V}


# Physics of the physical-step comparison (configurations 2 and 3): Mach
# 0.5, bulk Reynolds number 5600 on the full height 2h, limited MUSCL-5 +
# Roe with the ADM sensor, seeded laminar state with wall-damped +-5 %
# velocity noise.  The reference's face-state scaling of the limited fluxes
# diverges (scheme "consistent": see cf_set_scheme); the sensor is
# evaluated once per physical step ("per_step": re-evaluated every
# sub-iteration its on/off switch holds the residual near 4e-3 of its
# maximum, so no tolerance below that is reached); the time step is 1/4 of
# 0.005 h/U_b (at 0.005 and 0.0025 h/U_b, wall-normal acoustic CFL 6.5 and
# 3.3 at 256 x 192 x 192, the dual-time LU-SGS iteration diverges).
NS_MACH, NS_RE, NS_DT_FACTOR = 0.5, 5600.0, 0.25
NS_STEP = dict(max_iterations=200, tolerance=1e-6, limiter=True, filter="per_step")


def northstar_case(torch, dims, precision):
    """Context (consistent scheme) and device workload of the configuration
    2/3 channel on grid dims; returns (grid, ctx, workload, deltaT)."""
    import channel_flow_gb300 as cf
    from channel_flow_gb300 import synthetic as syn
    g = syn.channel_physics(syn.channel_grid(*dims), NS_MACH, NS_RE)
    cm = syn.flat_metrics(g, GAMMA, "cell")
    J = cm["J"]
    host = {"U": syn.channel_state(g, J, seed=SEED, mach=NS_MACH, noise=0.05, jitter=0.01, gamma=GAMMA,
                                   wall_damped=True),
            "J": J, "cm": [cm[n] for n in syn.METRIC_NAMES], "Yp": syn.y_points(g, gamma=GAMMA)}
    ctx = new_context(cf, g, precision=precision, gamma=GAMMA, scheme="consistent")
    w = DeviceWorkload(ctx, g, host, torch)
    return g, ctx, w, syn.time_step(g, NS_MACH) * NS_DT_FACTOR


def replica_value(torch, dist, total_ms, cells, steps, world):
    """Whole-job throughput of `world` independent replicas: the slowest
    rank's time (max over ranks when a process group is given) and
    cells x steps x world cell updates in that time, in Mcell-updates/s."""
    if dist is not None:
        t = torch.tensor([float(total_ms)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, cells * steps * world / (total_ms * 1e-3) / 1e6


def solver_stream(torch):
    """The physical steps run on a stream of the highest priority: cf_step's
    Statistic (its own stream, the least priority) then fills what the
    solver's kernels leave of the SMs instead of taking SMs from them."""
    return torch.cuda.stream(torch.cuda.Stream(priority=-1))


def physical_steps(torch, g, precision, steps, warmup):
    """`warmup` then `steps` timed physical steps (cf_step to the tolerance
    1e-6 from the extrapolated start, Statistic every step) of the
    configuration 2/3 physics on grid g: CUDA event time per step and per
    sub-iteration.  The timed steps are bracketed by cudaProfilerStart/Stop."""
    import tempfile
    from channel_flow_gb300 import stepper
    g, ctx, w, dt = northstar_case(torch, (g.X_out, g.Y_out, g.Z_out), precision)
    tmp = tempfile.TemporaryDirectory()       # the Statistic's Shear_stress.dat
    ctx.set_output_dir(tmp.name)
    st = stepper.Stepper(ctx, stepper.fields_from_workload(w, torch, g), deltaT=dt, **NS_STEP)
    st.kw["statistic_step"] = 1 << 30          # Statistic accumulates every step, as in the comparison
    for n in range(max(warmup, 3)):
        st.step("extrapolate" if n >= 2 else None)
    its = []
    # the timed steps alone for a profiler started with --profile-from-start
    # off; timed as one region that ends after the last step's Statistic
    # (each step's Statistic runs beside the next step)
    ctx.statistic_flush()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        its.append(st.step("extrapolate")[0])
    ctx.statistic_flush()
    e1.record()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    total = e0.elapsed_time(e1)
    ctx.close()
    tmp.cleanup()
    return {"step": "physical", "grid": [g.X_out, g.Y_out, g.Z_out], "precision": precision,
            "subiterations": its, "ms_total": total, "ms_per_step": total / max(1, steps),
            "ms_per_subiteration": total / max(1, sum(its))}


# The configurations' fixed schedules: 10 LU-SGS sub-iterations per step
# (the tolerance test never met), limited MUSCL-5 + Roe with the consistent
# face-state scaling and the Filter at every sub-iteration, Mach 0.5,
# seeded laminar state with wall-damped +-5 % velocity noise; Statistic
# accumulates every step.  Config 4 has the wavy lower wall (0.05 h, wavelength
# pi h) with the metrics of cf_wavy_metrics.
SCHEDULES = {
    "0": {"dims": (64, 64, 64), "re": 2800.0, "wavy": False, "steps": 100},
    "2": {"dims": (256, 192, 192), "re": 5600.0, "wavy": False, "steps": 1000},
    "4": {"dims": (512, 256, 384), "re": 11000.0, "wavy": True, "steps": 500},
}


def schedule_case(torch, key, precision, dt_factor):
    """Context (consistent scheme), device workload and time step of
    schedule `key`."""
    import channel_flow_gb300 as cf
    from channel_flow_gb300 import synthetic as syn
    spec = SCHEDULES[key]
    g = syn.channel_physics(syn.channel_grid(*spec["dims"]), 0.5, spec["re"])
    ctx = new_context(cf, g, precision=precision, gamma=GAMMA, scheme="consistent")
    if spec["wavy"]:
        w, _ = wavy_workload(ctx, g, torch, wall_damped=True)
    else:
        cm = syn.flat_metrics(g, GAMMA, "cell")
        host = {"U": syn.channel_state(g, cm["J"], seed=SEED, mach=0.5, noise=0.05, jitter=0.01, gamma=GAMMA,
                                       wall_damped=True),
                "J": cm["J"], "cm": [cm[n] for n in syn.METRIC_NAMES], "Yp": syn.y_points(g, gamma=GAMMA)}
        w = DeviceWorkload(ctx, g, host, torch)
        del host
    return g, ctx, w, syn.time_step(g, 0.5) * dt_factor


def schedule_run(torch, key, steps=None, compare_steps=None, precisions=("fp64", "fp32"), dt_factor=1.0):
    """Run schedule `key` for `steps` physical steps per precision (the
    FP64 run for `compare_steps` only, when given): CUDA-event time per
    step, and at the FP64 run's last step the FP32 run's mean-velocity and
    Reynolds-stress profiles and state against the FP64 run's (the FP64 GPU
    path is the FP64 oracle: it equals the C restatement to 1e-12 per
    routine and bit for bit in its no-FMA build)."""
    import tempfile
    from channel_flow_gb300 import stepper
    spec = SCHEDULES[key]
    steps = steps or spec["steps"]
    out = {"config": key, "grid": list(spec["dims"]), "re_bulk_2h": spec["re"], "mach": 0.5,
           "wavy_wall": spec["wavy"], "subiterations_per_step": LU_SUBITERATIONS, "dt_factor": dt_factor,
           "scheme": "limited MUSCL-5 + Roe (consistent face-state scaling), Viscous_terms, Filter every "
                     "sub-iteration, Dual_time_stepping; Statistic every step"}
    ref = None
    for prec in precisions:
        n_steps = compare_steps if (prec == "fp64" and compare_steps) else steps
        g, ctx, w, dt = schedule_case(torch, key, prec, dt_factor)
        out["deltaT_s"] = dt
        tmp = tempfile.TemporaryDirectory()
        ctx.set_output_dir(tmp.name)
        st = stepper.Stepper(ctx, stepper.fields_from_workload(w, torch, g), deltaT=dt,
                             max_iterations=LU_SUBITERATIONS, tolerance=0.0, limiter=True, filter=True,
                             statistic_step=1 << 30)
        ctx.statistic_reset()
        done, r, at_cmp = 0, {"steps": n_steps}, None
        cmp_at = compare_steps or steps
        # one timed region over the steps, ending after the last step's
        # Statistic (each step's Statistic runs beside the next step)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        try:
            for n in range(1, n_steps + 1):
                st.step(None)
                done = n
                if n == cmp_at:
                    at_cmp = (stat_profiles(ctx.statistic_read(), g, n), [u.clone() for u in st.f["U"]])
            ctx.statistic_flush()
        except Exception as exc:     # a diverged run is reported with its step
            r["failed_at_step"] = done + 1
            r["error"] = str(exc)
        e1.record()
        torch.cuda.synchronize()
        total = e0.elapsed_time(e1)
        r["s_per_step_mean"] = total / done * 1e-3 if done else None
        r["s_total"] = total * 1e-3
        r["ms_per_subiteration"] = total / done / LU_SUBITERATIONS if done else None
        if at_cmp is not None:
            prof, state = at_cmp
            r["profiles_at_step"] = cmp_at
            r["U_centre_over_Ub"] = float(np.max(prof["U"])) / syn_bulk_velocity(g)
            if ref is None:
                ref = at_cmp
            else:
                umax = max(float(np.max(np.abs(ref[0]["U"]))), 1e-300)
                r["profile_max_rel_err_vs_fp64"] = {
                    k: float(np.max(np.abs(prof[k] - ref[0][k]))) /
                    (umax if k in ("U", "V", "W") else max(float(np.max(np.abs(ref[0][k]))), 1e-300))
                    for k in prof}
                r["state_max_rel_err_vs_fp64"] = [
                    float((state[v] - ref[1][v]).abs().max()) / max(float(ref[1][v].abs().max()), 1e-300)
                    for v in range(5)]
        out[prec] = r
        ctx.close()
        tmp.cleanup()
        del st, w
        torch.cuda.empty_cache()
    return out


def syn_bulk_velocity(g):
    from channel_flow_gb300 import synthetic as syn
    return syn.bulk_velocity(g, 0.5)


def physical_step_to_tolerance(torch, dims=(256, 192, 192), harvest=48, evals=4, epochs=200, batch=131072,
                               online=0, learned_cap=20):
    """Wall time per physical step at equal pseudo-time tolerance on the
    configuration 2/3 channel: plain FP64 (the reference's start from U^n,
    every kernel FP64) against the mixed FP32 path with the plain start,
    with the quadratic extrapolation and with the learned guess.

    The sub-iterations of every mode run until er_n / max er_n < 1e-6 for
    n = 1..4 (main.cpp:387-406; er_n are sums of squared primitive updates,
    Dual_time_stepping.cpp:1318-1361) or 200 iterations.  `harvest` steps of
    the mixed path from the seeded state (each from U^n: on this oscillating
    transient the quadratic extrapolation overshoots, and a start that far
    off can make the sub-iterations diverge) give the training windows and
    the common start (the last three levels and the residual maxima).  Every mode then runs
    `evals` timed steps from that start with Statistic accumulating; its
    mean velocity and Reynolds-stress profiles and its final state are
    compared with those of the FP64 run.  The learned mode also runs capped
    at `learned_cap` sub-iterations (the configuration-3 limit), reported
    with the residual it reached.  The learned mode's timed steps include
    its online update when `online` > 0; its initial training is reported
    apart."""
    import tempfile
    from channel_flow_gb300 import mlp, stepper
    g, ctx, w, dt = northstar_case(torch, dims, "fp32")
    tmp = tempfile.TemporaryDirectory()
    ctx.set_output_dir(tmp.name)
    st = stepper.Stepper(ctx, stepper.fields_from_workload(w, torch, g), deltaT=dt, **NS_STEP)
    hist = [[u.clone() for u in st.f["U"]]]
    harvest_its = []
    t0 = time.perf_counter()
    for n in range(harvest):
        harvest_its.append(st.step(None)[0])
        hist.append([u.clone() for u in st.f["U"]])
    torch.cuda.synchronize()
    harvest_s = time.perf_counter() - t0
    E = ctx.step_scale()
    start = hist[-3:]
    t0 = time.perf_counter()
    net = mlp.LearnedGuess(capacity=g.cells, seed=0, lr=2e-3, batch=batch)
    losses = net.train(g, hist, epochs=epochs, batch=batch)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del hist
    out = {"grid": list(dims),
           "scheme": "limited MUSCL-5 + Roe (consistent face-state scaling) + Viscous_terms + Dual_time_stepping, "
                     "Filter once per physical step",
           "physics": {"mach": NS_MACH, "re_bulk_2h": NS_RE, "mu": g.mu_L, "body_force": g.f,
                       "deltaT_s": dt, "deltaT_h_over_Ub": 0.005 * NS_DT_FACTOR,
                       "initial": "laminar parabola + wall-damped +-5% u,v,w noise, +-1% rho,T jitter"},
           "tolerance": NS_STEP["tolerance"], "max_iterations": NS_STEP["max_iterations"],
           "harvest": {"steps": harvest, "subiterations": harvest_its, "s": harvest_s},
           "timed_steps": evals,
           "training": {"s": train_s, "adam_steps": len(losses), "batch_cells": batch,
                        "loss_first_last": [losses[0], losses[-1]], "held_out": net.validation},
           "online_adam_steps": online}
    out["guess_breakdown_ms"] = guess_breakdown(torch, net, g, start, st.f["U_"])
    ref = None
    modes = (("fp64", "fp64", None, None), ("fp32", "fp32", None, None),
             ("fp32+extrapolate", "fp32", "extrapolate", None), ("fp32+learned", "fp32", net, None),
             (f"fp32+learned_cap{learned_cap}", "fp32", net, learned_cap))
    for mode, prec, guess, cap in modes:
        ctx.set_precision(prec)
        st.restore(start, step=harvest)
        st.online = {"adam_steps": online, "batch": batch} if guess is net and online else None
        st.kw["max_iterations"] = cap or NS_STEP["max_iterations"]
        ctx.step_scale(E)
        ctx.statistic_reset()
        st.kw["statistic_step"] = 1 << 30
        its, last = [], []
        # the timed steps as one region that ends after the last step's
        # Statistic (each step's Statistic runs beside the next step)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(evals):
            it, er, q = st.step(guess)
            its.append(it)
            last.append(float(max(er[:4])))
        ctx.statistic_flush()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / evals
        st.kw["max_iterations"] = NS_STEP["max_iterations"]
        prof = stat_profiles(ctx.statistic_read(), g, evals)
        final = [u.clone() for u in st.f["U"]]
        r = {"subiterations": its, "ms_per_step": round(ms, 3),
             "s_per_step_mean": ms * 1e-3, "final_max_er_over_E": last}
        if ref is None:
            ref = (prof, final)
        else:
            r["speedup_vs_fp64"] = out["fp64"]["s_per_step_mean"] / r["s_per_step_mean"]
            # mean velocities against the largest mean streamwise velocity
            # (V and W average to about zero), stresses against their own
            # largest magnitude
            umax = max(float(np.max(np.abs(ref[0]["U"]))), 1e-300)
            r["profile_max_rel_err"] = {
                k: float(np.max(np.abs(prof[k] - ref[0][k]))) /
                (umax if k in ("U", "V", "W") else max(float(np.max(np.abs(ref[0][k]))), 1e-300)) for k in prof}
            # state error relative to the change over the timed steps
            r["state_err_over_change"] = max(
                float((final[v] - ref[1][v]).abs().max()) / max(float((ref[1][v] - start[-1][v]).abs().max()), 1e-300)
                for v in range(5))
        out[mode] = r
    if net.updates:
        out["fp32+learned"]["online_held_out"] = [u["err_over_extrapolation_raw"] for u in net.updates]
    ctx.close()
    tmp.cleanup()
    return out


def guess_breakdown(torch, net, g, levels, out, reps=5):
    """CUDA-event time of each part of one learned guess on all cells:
    the device-side feature scales, the feature rows, the three forward
    GEMMs and the guess itself (mean of `reps` after one untimed call),
    and of the whole guess; with the fitted predictor coefficients."""
    from channel_flow_gb300 import mlp
    un, u1, u2 = levels[2], levels[1], levels[0]
    Mpad = (g.cells + 255) // 256 * 256
    b1, b2, b3 = net.view("b1"), net.view("b2"), net.view("b3")
    a15 = (mlp.C.c_void_p * 15)(*[t.data_ptr() for t in list(un) + list(u1) + list(u2)])
    o5 = (mlp.C.c_void_p * 5)(*[t.data_ptr() for t in out])
    parts = [
        ("scales", lambda: net.set_scale_device(g, un, u1, u2)),
        ("features", lambda: net.load_features(g, un, u1, u2)),
        ("gemm_L1", lambda: net.gemm(net.X, net.W1b, Mpad, mlp.H, mlp.K1, mlp.EPI_SILU, b1, net.H1, None, mlp.H)),
        ("gemm_L2", lambda: net.gemm(net.H1, net.W2b, Mpad, mlp.H, mlp.H, mlp.EPI_SILU, b2, net.H2, None, mlp.H)),
        ("gemm_L3", lambda: net.gemm(net.H2, net.W3b, Mpad, mlp.N3, mlp.H, mlp.EPI_BIAS, b3, net.Y, None, mlp.N3)),
        ("apply", lambda: net._ok(net.lib.cf_mlp_apply(net._s(), g.X_out, g.Y_out, g.Z_out, a15, net.coef.ctypes.data,
                                                       net.scale.data_ptr(), net.ogain.data_ptr(), net.Y.data_ptr(),
                                                       o5), "cf_mlp_apply")),
        ("guess_total", lambda: net.guess(g, un, u1, u2, out)),
    ]
    res = {}
    for name, fn in parts:
        fn()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        res[name] = e0.elapsed_time(e1) / reps
    res["predictor_coef_a_b"] = [round(float(x), 4) for x in net.coef]
    return res


def mlp_gemms(torch, rows, steps=5, warmup=2):
    """The learned guess's six tcgen05 GEMMs (forward: features x W1,
    H1 x W2, H2 x W3; backward: the activation gradients and the weight
    gradients, whose reduction dimension is the rows) on `rows` random
    feature rows: CUDA-event time per GEMM and its TFLOP/s (2 M N K per
    product) against the measured BF16 peak."""
    from channel_flow_gb300 import mlp
    net = mlp.LearnedGuess(capacity=rows, seed=0, batch=rows)
    M = net.cap
    gen = torch.Generator(device="cuda")
    gen.manual_seed(SEED)
    net.X.copy_(torch.randn(M, mlp.K1, generator=gen, device="cuda").to(torch.bfloat16))
    net.T.copy_(torch.randn(M, mlp.N3, generator=gen, device="cuda"))
    H, K1, N3, K3 = mlp.H, mlp.K1, mlp.N3, mlp.K3
    b1, b2, b3 = net.view("b1"), net.view("b2"), net.view("b3")
    g = net.g
    prods = [
        ("fwd_L1", lambda: net.gemm(net.X, net.W1b, M, H, K1, mlp.EPI_SILU, b1, net.H1, net.Z1, H), M, H, K1),
        ("fwd_L2", lambda: net.gemm(net.H1, net.W2b, M, H, H, mlp.EPI_SILU, b2, net.H2, net.Z2, H), M, H, H),
        ("fwd_L3", lambda: net.gemm(net.H2, net.W3b, M, N3, H, mlp.EPI_BIAS, b3, net.Y, None, N3), M, N3, H),
        ("bwd_dH2", lambda: net.gemm(net.dY, net.W3p, M, H, K3, mlp.EPI_F32, None, net.dH, None, H), M, H, K3),
        ("bwd_dH1", lambda: net.gemm(net.dZ2, net.W2T, M, H, H, mlp.EPI_F32, None, net.dH, None, H), M, H, H),
        ("bwd_dW1", lambda: net.gemm_wgrad(net.dZ1T, net.XT, H, K1, M, net.view("W1", g)), H, K1, M),
    ]
    # one full training step first, so that every operand holds data
    net.step(M, M)
    out = {"rows": M, "peak_bf16_tflops": None, "gemms": {}}
    pk = ROOT / "MEASURED_PEAKS.json"
    peak = float(json.loads(pk.read_text())["bf16_tflops"]) if pk.exists() else 1900.0
    out["peak_bf16_tflops"] = peak
    for name, fn, m, n, k in prods:
        for _ in range(warmup):
            fn()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        tf = 2.0 * m * n * k / (ms * 1e-3) / 1e12
        out["gemms"][name] = {"M": m, "N": n, "K": k, "ms": ms, "tflops": tf, "frac_of_peak": tf / peak}
    net.check_device()
    # the guess on all rows: features are not timed here; forward = the three products
    out["forward_ms"] = sum(out["gemms"][k]["ms"] for k in ("fwd_L1", "fwd_L2", "fwd_L3"))
    del net
    torch.cuda.empty_cache()
    return out


def wavy_workload(ctx, g, torch, amplitude_over_h=0.05, wavelength_over_h=math.pi, wall_damped=False):
    """The benchmark channel with a wavy lower wall (amplitude 0.05 h,
    wavelength pi h: two waves over 2 pi h) and the conservative metrics of
    cf_wavy_metrics; seeded laminar-plus-noise state at Mach 0.5."""
    from channel_flow_gb300 import synthetic as syn, wavy
    wall = wavy.wall_for(g, amplitude_over_h, wavelength_over_h, stretching=GAMMA, conservative=True)
    m = wavy.channel_metrics(g, wall)
    J = m["J"].cpu().numpy()
    host = {"U": syn.channel_state(g, J, seed=SEED, mach=0.5, noise=0.05, jitter=0.01, gamma=GAMMA,
                                   wall_damped=wall_damped), "J": J,
            "cm": [t.cpu().numpy() for t in m["cm"]], "Yp": m["Yp"].cpu().numpy()}
    w = DeviceWorkload(ctx, g, host, torch)
    del host
    for dst, src in ((w.fu, m["fu"]), (w.fv, m["fv"]), (w.fw, m["fw"])):
        for a, b in zip(dst, src):
            a.copy_(b)
    del m
    torch.cuda.synchronize()
    return w, wall


def secondary(ctx, g, w, calls, stream, torch, args):
    """Per precision: the RHS and one dual-time pseudo-iteration (RHS +
    hyperplane LU-SGS) on the benchmark grid, and on the 256 x 192 x 192
    mixed-precision channel (9.4 M cells)."""
    import channel_flow_gb300 as cf
    from channel_flow_gb300 import synthetic as syn
    out = {}
    steps = max(2, min(args.steps, 5))
    prec0 = ctx.precision
    key = "x".join(str(v) for v in (g.X_out, g.Y_out, g.Z_out))
    out[key] = {}
    for prec in ("fp64", "fp32"):
        ctx.set_precision(prec)
        out[key][prec] = pseudo_iteration(ctx, g, w, calls, stream, torch, steps)
    ctx.set_precision(prec0)
    if (g.X_out, g.Y_out, g.Z_out) != (256, 192, 192) and not args.no_large:
        g2 = syn.channel_grid(256, 192, 192)
        ctx2 = new_context(cf, g2, precision="fp64", gamma=GAMMA)
        w2 = DeviceWorkload(ctx2, g2, make_host_workload(g2), torch)
        calls2 = rhs_calls(ctx2, w2, lambda x: x.data_ptr())
        out["256x192x192"] = {}
        for prec in ("fp64", "fp32"):
            ctx2.set_precision(prec)
            out["256x192x192"][prec] = pseudo_iteration(ctx2, g2, w2, calls2, stream, torch, 3)
        ctx2.close()
        del w2, calls2
        torch.cuda.empty_cache()
    if not args.no_large and not args.no_wavy:
        # the 50 M-cell channel with a wavy lower wall (metrics from cf_wavy_metrics)
        try:
            g3 = syn.channel_grid(512, 256, 384)
            ctx3 = new_context(cf, g3, precision="fp64", gamma=GAMMA)
            w3, wall = wavy_workload(ctx3, g3, torch)
            calls3 = rhs_calls(ctx3, w3, lambda x: x.data_ptr())
            r = {"wall": {"amplitude_over_h": 0.05, "wavelength_over_h": math.pi, "metrics": "conservative"}}
            for prec in ("fp64", "fp32"):
                ctx3.set_precision(prec)
                r[prec] = pseudo_iteration(ctx3, g3, w3, calls3, stream, torch, 2)
            out["512x256x384_wavy"] = r
            ctx3.close()
            del w3, calls3
        except Exception as exc:
            out["512x256x384_wavy"] = {"error": repr(exc)}
        torch.cuda.empty_cache()
    for k, v in out.items():
        if "fp64" in v and "fp32" in v:
            v["physical_step_fp64_over_fp32"] = v["fp64"]["physical_step_s"] / v["fp32"]["physical_step_s"]
    if not args.no_learned:
        try:
            out["mlp_gemm"] = mlp_gemms(torch, 2097152)
        except Exception as exc:
            out["mlp_gemm"] = {"error": repr(exc)}
    if not args.no_large and not args.no_learned:
        try:
            with solver_stream(torch):
                out["physical_step_to_tolerance"] = physical_step_to_tolerance(torch)
        except Exception as exc:
            out["physical_step_to_tolerance"] = {"error": repr(exc)}
    out["note"] = ("per grid: physical step = 10 LU-SGS sub-iterations x (RHS + Dual_time_stepping), the "
                   "reference's limited scheme with the filter; FP32 = flux/viscous/filter/LU-SGS sweeps in FP32, "
                   "FP64 state accumulating the FP32 changes, BDF2 differences and norms FP64.  "
                   "physical_step_to_tolerance: steps run to the pseudo-time tolerance instead, with and without "
                   "the learned initial guess")
    return out


def measure_e2e(ctx, g, host, w, torch, steps):
    """Same steps through the C-ABI with HOST arrays registered as device
    mirrors: every step uploads its state (U1_..U5_) and downloads its RHS
    (inF of the three directions and vF).  Two registered sets of those
    arrays alternate, so step n+1's upload (on an H2D stream) and step n-1's
    download (on a D2H stream) run while step n's routines run on the
    context's stream; CUDA events order the three streams.  The static
    inputs (J, Y_point, metrics) are uploaded once before the timed region."""
    n = ctx.field_count
    pinned = lambda: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy().reshape(g.shape)
    shared = type("H", (), {})()
    shared.J, shared.Yp = pinned(), pinned()
    shared.J[...] = host["J"]
    shared.Yp[...] = host["Yp"]
    shared.cm = [pinned() for _ in range(9)]
    for a, src in zip(shared.cm, host["cm"]):
        a[...] = src
    for attr in ("fu", "fv", "fw"):
        arrs = [pinned() for _ in range(10)]
        for a, d in zip(arrs, getattr(w, attr)):
            a[...] = d.cpu().numpy()
        setattr(shared, attr, arrs)
    for attr, cnt in (("Ep", 3), ("LL", 4), ("ML", 4), ("NL", 4)):
        setattr(shared, attr, [pinned() for _ in range(cnt)])
    every = [shared.J, shared.Yp] + shared.cm + shared.fu + shared.fv + shared.fw + shared.Ep + shared.LL + \
        shared.ML + shared.NL
    sets = []
    for _ in range(2):
        hw = type("H", (), {})()
        for attr in ("J", "Yp", "cm", "fu", "fv", "fw", "Ep", "LL", "ML", "NL"):
            setattr(hw, attr, getattr(shared, attr))
        hw.U = [pinned() for _ in range(5)]
        for a, src in zip(hw.U, host["U"]):
            a[...] = src
        for attr, cnt in (("Fx", 5), ("Fy", 5), ("Fz", 5), ("vF", 4)):
            setattr(hw, attr, [pinned() for _ in range(cnt)])
        hw.outs = hw.Fx + hw.Fy + hw.Fz + hw.vF
        every += hw.U + hw.outs
        sets.append(hw)
    for a in every:
        ctx.register(a)
    for a in every:
        ctx.upload(a)       # set-up: static inputs resident on the device
    ctx.synchronize()
    for hw in sets:
        hw.calls = rhs_calls(ctx, hw, lambda x: x.ctypes.data)
    comp = torch.cuda.current_stream()
    h2d, d2h = torch.cuda.Stream(), torch.cuda.Stream()
    ev = lambda: [torch.cuda.Event(), torch.cuda.Event()]
    uploaded, computed, downloaded = ev(), ev(), ev()
    for e in computed + downloaded:
        e.record(comp)

    def step(k):
        s, hw = k % 2, sets[k % 2]
        h2d.wait_event(computed[s])          # step k-2's routines have read (and ghost-filled) U of set s
        for a in hw.U:
            ctx.upload_async(a, h2d.cuda_stream)
        uploaded[s].record(h2d)
        comp.wait_event(uploaded[s])
        comp.wait_event(downloaded[s])       # step k-2's RHS of set s has reached the host
        run_calls(ctx, hw.calls)
        computed[s].record(comp)
        d2h.wait_event(computed[s])
        for a in hw.outs:
            ctx.download_async(a, d2h.cuda_stream)
        downloaded[s].record(d2h)

    for k in range(2):
        step(k)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        step(k)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    # the downloaded RHS equals the device-resident path's on the same inputs
    for d, src in zip(w.U, host["U"]):
        d.copy_(torch.from_numpy(np.ascontiguousarray(src)).to(d.device))
    run_calls(ctx, rhs_calls(ctx, w, lambda x: x.data_ptr()))
    torch.cuda.synchronize()
    last = sets[(steps - 1) % 2]
    match = all(np.array_equal(a, d.cpu().numpy(), equal_nan=True)
                for a, d in zip(last.outs, list(w.Fx) + list(w.Fy) + list(w.Fz) + list(w.vF)))
    for a in every:
        ctx.lib.cf_unregister(ctx.h, a.ctypes.data)
    field_bytes = n * 8
    return {"value": g.cells * steps / dt / 1e6, "unit": "Mcell-updates/s",
            "h2d_bytes_per_step": 5 * field_bytes, "d2h_bytes_per_step": len(sets[0].outs) * field_bytes,
            "ms_per_step": dt / steps * 1e3, "rhs_matches_device_path": bool(match),
            "path": "C-ABI, registered pinned host arrays; two sets alternate so the copies of steps n-1 and "
                    "n+1 overlap the routines of step n (host wall clock, all streams synchronised at both ends)"}


if __name__ == "__main__":
    sys.exit(main())
