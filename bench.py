#!/usr/bin/env python3
"""Benchmark of the GB300 IBM-DEM particle hot path.

One step = the particle side of one fluid step on a frozen synthetic fluid
field: restore the field, 5 multi-direct-forcing iterations (interpolation,
direct forcing, deterministic spreading, post-guess), the per-body force and
torque reduction, then one DEM sub-step (contact forces, rigid-body update,
marker motion, cell/contact/periodic-image list rebuild, delta weights and the
spread plan).  Metric: particle-steps/s, a particle being one rigid sphere;
marker-steps/s is reported beside it.

Default workload: a triply periodic 256x256x512 grid (h = 1) with 2048 spheres
of diameter 12h (452 Fibonacci markers each, 925,696 markers), seeded random
sequential addition, body velocities N(0, 0.01), and a 64-mode divergence-free
Fourier field of amplitude 0.05; dt = 1e-3.  The working set (fields, weights,
spread plan) is several GB, far larger than L2, so no flush is needed between
steps.

  python bench.py [--gpus N --steps K --warmup W]       this library on the GPU
  python bench.py --impl reference [...]                 the CPU restatement of the
                                                         reference on the host cores
Under torchrun each rank advances its own replica on its own GPU (no data-path
exchange: the cases are independent), timing is the max over ranks, and rank 0
prints one JSON line.
"""
import argparse
import json
import os

# more hardware work queues, so that independent cases' streams do not share one
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ibm-dem_gb300"))

WORKLOADS = {
    # name: (nx, ny, nz, bodies, diameter, modes)
    "resolved-2048-spheres-256x256x512": (256, 256, 512, 2048, 12.0, 64),
    "resolved-64-spheres-128cube": (128, 128, 128, 64, 16.0, 32),
    "resolved-512-spheres-256cube": (256, 256, 256, 512, 12.0, 64),
}
# unresolved CFD-DEM: name -> (fluid cells per axis, particles)
UNRESOLVED_WORKLOADS = {"unresolved-1048576-particles-128cube": (128, 1_048_576)}
DEFAULT_WORKLOAD = "resolved-2048-spheres-256x256x512"
METRIC = "particle-steps/s (contact+IBM) on 1 GB300, batched vs plain; p50/p99 serve latency"


# DRAM bytes (read + write) per local marker and launch of the main kernels, from
# one ncu capture of the 512-sphere 256^3 case; the benchmark workload has the
# same per-marker structure, so traffic scales with markers.
DRAM_BYTES_PER_MARKER = {"interp": 1189.0, "spread": 1781.0, "weights": 530.0}


def max_over_ranks(x):
    """Max of a float over all ranks (the slowest replica sets the job time)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS) + sorted(UNRESOLVED_WORKLOADS))
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--batch-cases", type=int, default=256, help="cases of the batched mix (0 = skip)")
    ap.add_argument("--batch-steps", type=int, default=100, help="steps per case of the batched mix")
    ap.add_argument("--batch-mode", choices=["auto", "own", "shared"], default="auto",
                    help="batched forcing loops: the autotuner's choice, each member's own launches, or shared "
                         "launches for all members")
    ap.add_argument("--serve-requests", type=int, default=512, help="requests of the served stream (0 = skip)")
    ap.add_argument("--serve-plain-requests", type=int, default=128,
                    help="the first this many requests also run on the plain one-at-a-time path")
    ap.add_argument("--serve-steps", type=int, default=100)
    ap.add_argument("--unresolved-particles", type=int, default=1_048_576,
                    help="particles of the unresolved CFD-DEM case (0 = skip)")
    ap.add_argument("--unresolved-steps", type=int, default=100)
    ap.add_argument("--fluid-steps", type=int, default=20,
                    help="steps of the GPU fluid stencils on the default grid (0 = skip)")
    ap.add_argument("--serve-work-limit", type=int, default=2_000_000,
                    help="markers the running requests may hold together (0 = no limit)")
    return ap.parse_args()


def make_case(workload, seed, field_device):
    from ibmdem import scenario

    nx, ny, nz, nb, d, modes = WORKLOADS[workload]
    return scenario.resolved_case(nx, ny, nz, nb, d, seed=seed, n_modes=modes, amp=0.05, vel_std=0.01,
                                  field_device=field_device)


def config_of(workload, nparts):
    nx, ny, nz, nb, d, modes = WORKLOADS[workload]
    return {"workload": workload, "grid": [nx, ny, nz], "bodies": nb, "diameter_h": d, "markers": int(nparts),
            "fourier_modes": modes, "mdf_iterations": 5, "dem_substeps": 1, "dt": 1e-3,
            "boundary": "triply periodic", "l2": "working set several GB > 129 MB L2 (no flush needed)"}


class ClockSampler:
    """SM clock, power and clock-event reasons sampled during the timed region:
    NVML through ctypes every 10 ms on the device whose PCI bus id CUDA reports
    (so a short timed region still gets samples), or nvidia-smi every 200 ms
    where NVML cannot be loaded.  Only reads; no setting is changed."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # clock-event reason bits of nvml.h
    REASONS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.p = None
        self.nvml = None
        self.rows = []
        self.source = None

    def _nvml_open(self):
        import ctypes
        import threading

        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        dev = ctypes.c_void_p()
        bus = None
        try:
            import torch

            pr = torch.cuda.get_device_properties(self.idx)
            bus = "%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
        except Exception:
            bus = None
        if bus is None or lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(dev)) != 0:
            if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.idx), ctypes.byref(dev)) != 0:
                lib.nvmlShutdown()
                raise RuntimeError("no NVML handle")
        reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        cmax = ctypes.c_uint()
        lib.nvmlDeviceGetMaxClockInfo(dev, ctypes.c_int(1), ctypes.byref(cmax))
        self.max_mhz = float(cmax.value)
        self.stop = threading.Event()

        def run():
            clk, rs, pw = ctypes.c_uint(), ctypes.c_ulonglong(), ctypes.c_uint()
            while not self.stop.is_set():
                ok = lib.nvmlDeviceGetClockInfo(dev, ctypes.c_int(1), ctypes.byref(clk)) == 0
                ok = ok and reasons_fn(dev, ctypes.byref(rs)) == 0
                if lib.nvmlDeviceGetPowerUsage(dev, ctypes.byref(pw)) != 0:
                    pw.value = 0
                if ok:
                    self.rows.append((float(clk.value), int(rs.value), pw.value / 1000.0))
                self.stop.wait(0.01)

        self.nvml = (lib, threading.Thread(target=run, daemon=True))
        self.nvml[1].start()
        self.source = "nvml, 10 ms"

    def __enter__(self):
        try:
            self._nvml_open()
        except Exception:
            self.nvml = None
            try:
                self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                           "--format=csv,noheader,nounits", "-lms", "200"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
                self.source = "nvidia-smi, 200 ms"
            except Exception:
                self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.nvml:
            lib, th = self.nvml
            self.stop.set()
            th.join(timeout=5)
            lib.nvmlShutdown()
        if self.p:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        if self.nvml is not None:
            if not self.rows:
                return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["unsampled"], "samples": 0,
                        "source": self.source}
            reasons = sorted(n for n, bit in self.REASONS.items() if any(r[1] & bit for r in self.rows))
            return {"sm_mhz": statistics.median(r[0] for r in self.rows), "sm_max_mhz": self.max_mhz,
                    "sm_min_mhz": min(r[0] for r in self.rows), "reasons": reasons, "samples": len(self.rows),
                    "power_w_max": max(r[2] for r in self.rows), "source": self.source}
        rows = []
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": float(rows[0][2]),
                "reasons": sorted(reasons), "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit()),
                "source": self.source}


def cpu_baseline(case_data, steps):
    """The CPU restatement of the reference on this host's cores (all threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    p, parts, bodies, field = case_data
    r = O.OracleCase(p, parts, bodies, field)
    r.InitializationDEM()
    t0 = time.perf_counter()
    r.step(steps)
    dt = time.perf_counter() - t0
    nb = len(bodies)
    r.close()
    return {"value": nb * steps / dt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full step(s) of the same {len(parts)}-marker case, OpenMP over the marker loops",
            "seconds": dt, "marker_steps_per_s": len(parts) * steps / dt}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    if args.workload in UNRESOLVED_WORKLOADS:
        return run_reference_unresolved(args, O, threads)
    p, parts, bodies, field = make_case(args.workload, args.seed, "cpu")
    r = O.OracleCase(p, parts, bodies, field)
    r.InitializationDEM()
    # bounded sample: one warm-up step, then as many of the requested steps as
    # fit in about two minutes of host time
    t0 = time.perf_counter()
    r.step(min(args.warmup, 1))
    per = max(time.perf_counter() - t0, 1e-3)
    k = max(1, min(args.steps, int(120.0 / per)))
    t0 = time.perf_counter()
    r.step(k)
    dt = time.perf_counter() - t0
    nb = len(bodies)
    val = nb * k / dt
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": k, "steps_requested": args.steps, "warmup": min(args.warmup, 1), "ms_per_step": dt / k * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(args.workload, len(parts)),
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{k} full step(s) of the {len(parts)}-marker case (CPU restatement, "
                                       f"OpenMP over marker loops)"},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "marker_steps_per_s": len(parts) * k / dt}
    print(json.dumps(line), flush=True)
    return 0


def run_reference_unresolved(args, O, threads):
    from ibmdem import scenario

    ncell, n = UNRESOLVED_WORKLOADS[args.workload]
    p, parts, field = scenario.unresolved_case(ncell, n, seed=args.seed, n_modes=32, bed_spacing=0.9)
    r = O.OracleUnresolved(p, parts, field)
    t0 = time.perf_counter()
    r.step(min(args.warmup, 1))
    per = max(time.perf_counter() - t0, 1e-3)
    k = max(1, min(args.steps, int(120.0 / per)))
    t0 = time.perf_counter()
    r.step(k)
    dt = time.perf_counter() - t0
    r.close()
    val = n * k / dt
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": k, "steps_requested": args.steps, "warmup": min(args.warmup, 1), "ms_per_step": dt / k * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "fluid_cells": [ncell] * 3, "particles": n},
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{k} step(s) of the {n}-particle case (CPU restatement, OpenMP)"},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def algorithmic(counters):
    """Per launch of the main kernels: the compulsory HBM bytes of the hot-path
    scope table, the bytes the implementation moves with its own intermediates
    (stored weights, the spread plan), and the FP64 instructions it issues.

    Units: M local markers, NP markers with their periodic images, U touched
    grid nodes summed over the three velocity components, C spread
    contributions.  Compulsory bytes: interpolation with its weights (a7+a8,
    one launch = one forcing iteration, all three components) M (48 x,v + 24
    fdrag read + 48 fdrag,vgap written) + 8 U field gathers; spreading with the
    post-guess (a10+a11) NP (24 x + 24 fdrag + 8 vol) + 24 U (the old forcing
    and u read, u and f written); the weights kernel and the plan fill have no
    row of their own there (their outputs are intermediates of a7/a10): their
    compulsory bytes are the positions and cells they read.

    FP64 instructions issued (DADD, DMUL, DFMA, square-root steps), counted
    from the kernels' operations and checked against ncu's
    sm__sass_thread_inst_executed_op_fp64_pred_on on the 512-sphere case:
    interpolation 60 per marker and component (27 products, 26 sums, the
    velocity gap, the division by dt as 4 operations, the fdrag update and
    fdrag*vol); spreading 2 per contribution less the first subtraction of
    each node (an integer sign flip), plus 3 per node for the post-guess;
    weights FP64_WEIGHTS_PER_PARCEL per parcel (ncu's count: 18 one-axis
    kernels with a square root and an exact /3 each, 108 products, and the
    window's coordinates)."""
    M = counters["npLocal"]
    NP = counters["np"]
    C = counters["contributions"]
    U = counters["nodes_u"] + counters["nodes_v"] + counters["nodes_w"]
    # per launch; the two weight launches (locals, then images) as one
    return {
        "interp": {"compulsory": M * 120 + 8 * U,
                   "moved": M * (81 * 8 + 16 + 8 + 3 * 5 * 8) + 8 * U,
                   "fp64": M * 3 * 60, "per_step": 5},
        "spread": {"compulsory": NP * 56 + 24 * U,
                   "moved": C * (4 + 8) + NP * 24 + U * (4 + 4 + 16 + 16 + 8),
                   "fp64": 2 * C - U + 3 * U, "per_step": 5},
        "weights": {"compulsory": NP * (24 + 4),
                    "moved": NP * (24 + 4 + 84 * 8 + 16 + 4),
                    "fp64": NP * FP64_WEIGHTS_PER_PARCEL, "per_step": 1},
        "plan": {"compulsory": NP * (24 + 4),
                 "moved": C * 12 + NP * (4 + 16) * 2 + U * 12,
                 "fp64": 0, "per_step": 1},
    }


# FP64 instructions per parcel of the delta-weight kernel (ncu's
# sm__sass_thread_inst_executed_op_fp64_pred_on over the two launches of a step
# of the 64-sphere case, divided by its 57,216 parcels)
FP64_WEIGHTS_PER_PARCEL = 506


def kernel_rows(alg, phases, hbm_peak, fp64_peak, npLocal):
    """One roofline row per main kernel from its CUDA-event time per launch."""
    rows = {}
    for k, a in alg.items():
        tot, n = phases.get(k, (0.0, 0))
        if not n:
            continue
        # the weights phase counts its two launches (locals, images) separately
        n = n // 2 if k == "weights" else n
        s = tot / n / 1e3
        gbs = a["compulsory"] / s / 1e9
        per_marker = DRAM_BYTES_PER_MARKER.get(k)
        traffic = per_marker * npLocal if per_marker else None
        fp = a["fp64"] / s / 1e9
        row = {"ms_per_launch": tot / n, "launches": n, "compulsory_bytes": a["compulsory"],
               "compulsory_gbs": gbs, "hbm_frac": gbs / hbm_peak, "moved_bytes": a["moved"],
               "moved_gbs": a["moved"] / s / 1e9, "traffic": traffic,
               "waste_ratio": traffic / a["compulsory"] if traffic else None,
               "fp64_issued": a["fp64"], "fp64_gops": fp,
               "fp64_frac": fp / fp64_peak if fp64_peak and a["fp64"] else None}
        row["bound"] = "fp64" if (row["fp64_frac"] or 0) > row["hbm_frac"] else (
            "issue" if k == "plan" else "hbm")
        rows[k] = row
    return rows


def percentile(xs, q):
    import numpy as np

    return float(np.percentile(np.asarray(xs, dtype=float), q)) if len(xs) else None


def run_batched(args, device, stream):
    """Batched mix (256 independent cases of uneven size): the plain path
    advances the cases one after another with ibmdem_step (each case's step a
    replay of its own captured graph, the library's default); the batched path
    advances all of them with one CUDA graph launch per step, its shape picked
    by the autotuner.  Both time the same steps of the same cases, host launch
    overhead included (wall clock, synchronised).  The plain path kernel by
    kernel (step graphs off) is timed too, over batch_steps // 5 steps."""
    import torch
    from ibmdem import api, scenario

    mix = scenario.batched_mix(args.batch_cases, seed=args.seed, n_modes=32, field_device="cuda")
    nbodies = sum(len(c[2]) for c in mix)
    nmark = sum(len(c[1]) for c in mix)
    cases = []
    for p, parts, bodies, field in mix:
        c = api.Case(p, parts, bodies, field, device=device, stream=stream)
        c.InitializationDEM()
        cases.append(c)
    del mix
    k = args.batch_steps
    for c in cases:
        c.step(1)
    torch.cuda.synchronize()
    l0 = sum(c.launches for c in cases)
    t0 = time.perf_counter()
    for c in cases:
        c.step(k)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    plain_launch = sum(c.launches for c in cases) - l0
    # the same cases kernel by kernel on their stream (step graphs off)
    kk = max(1, k // 5)
    for c in cases:
        c.set_step_graphs(False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for c in cases:
        c.step(kk)
    torch.cuda.synchronize()
    plain_kbk_s = time.perf_counter() - t0
    for c in cases:
        c.set_step_graphs(True)
        c.synchronize()
    b = api.Batch(cases, device=device)
    lanes = b.autotune(trial_steps=2)
    if args.batch_mode != "auto":
        b.set_fused(args.batch_mode == "shared")
    _, fused, interp_block = b.config()
    b.step(1)
    b.synchronize()
    l0 = sum(c.launches for c in cases)
    t0 = time.perf_counter()
    b.step(k)
    b.synchronize()
    batch_s = time.perf_counter() - t0
    batch_launch = sum(c.launches for c in cases) - l0
    b.close()
    for c in cases:
        c.close()
    return {"value": nbodies * k / batch_s, "unit": "particle-steps/s", "plain_value": nbodies * k / plain_s,
            "ratio_vs_plain": plain_s / batch_s, "steps": k, "cases": len(cases), "bodies": nbodies,
            "plain_kernel_by_kernel_value": nbodies * kk / plain_kbk_s,
            "ratio_vs_plain_kernel_by_kernel": (plain_kbk_s / kk) / (batch_s / k),
            "markers": nmark, "lanes": lanes, "shared_forcing_launches": bool(fused), "interp_block": interp_block,
            "ms_per_step": batch_s / k * 1e3, "plain_ms_per_step": plain_s / k * 1e3,
            "gpu_launches": batch_launch, "plain_gpu_launches": plain_launch, "graph_launches": k,
            "workload": f"{len(cases)} cases: grid in {{32,64,96,128}}^3, d in {{8,12,16}}h, bodies log-uniform "
                        f"8..512 capped at 25% solid fraction, 32-mode Fourier field, seed {args.seed}+i",
            "timing": "wall clock around the steps, synchronised on both sides"}


def run_served(args, device, stream):
    """Served stream: Poisson arrivals at 200 requests/s of settling and shear
    cases (16..2048 bodies on 64^3..256^3 grids), each advancing serve_steps
    steps, admitted by an 80 GB device-memory budget and run concurrently by the
    library's request server.  The plain path runs the first
    serve_plain_requests of the same requests one at a time in arrival order
    (the whole stream would take minutes more); its throughput is theirs, and
    its latencies follow from their measured service times and arrivals."""
    import numpy as np
    from ibmdem import api, scenario

    reqs = scenario.serve_requests(args.serve_requests, seed=args.seed)
    steps = args.serve_steps
    budget = 80 * 10 ** 9
    # plain: one case at a time, in arrival order
    plain_reqs = reqs[:max(1, min(len(reqs), args.serve_plain_requests))]
    service = []
    for r in plain_reqs:
        p, parts, bodies, field = r["case"]
        if field is None:
            field = [np.zeros(api.field_shape(np.array(p, dtype=api.PARAMS))) for _ in range(3)]
        t0 = time.perf_counter()
        c = api.Case(p, parts, bodies, field, device=device, stream=stream)
        c.InitializationDEM()
        c.step(steps)
        c.get_bodies()
        c.close()
        service.append(time.perf_counter() - t0)
    done, plain_lat = 0.0, []
    for r, sv in zip(plain_reqs, service):
        done = max(done, r["arrival"]) + sv
        plain_lat.append(done - r["arrival"])
    plain_span = done - plain_reqs[0]["arrival"]
    # the same one-at-a-time service with the served arm's admission order:
    # at each completion the arrived request with the fewest marker-steps
    work = [len(r["case"][1]) * steps for r in plain_reqs]
    t, left, plain_lat_lw = 0.0, list(range(len(plain_reqs))), []
    while left:
        arrived = [q for q in left if plain_reqs[q]["arrival"] <= t]
        if not arrived:
            t = min(plain_reqs[q]["arrival"] for q in left)
            continue
        q = min(arrived, key=lambda x: (work[x], x))
        t += service[q]
        plain_lat_lw.append(t - plain_reqs[q]["arrival"])
        left.remove(q)
    plain_body_steps = sum(len(r["case"][2]) for r in plain_reqs) * steps
    # served
    srv = api.Server(budget, max_active=64, device=device, work_limit=args.serve_work_limit)
    srv.set_policy(api.Server.LEAST_WORK)
    ids = []
    t0 = time.perf_counter()
    i = 0
    peak = 0
    while True:
        now = time.perf_counter() - t0
        while i < len(reqs) and reqs[i]["arrival"] <= now:
            p, parts, bodies, field = reqs[i]["case"]
            ids.append(srv.submit(p, parts, bodies, field, nsteps=steps))
            i += 1
        pending = srv.poll()
        peak = max(peak, srv.memory()[0])
        if i == len(reqs) and pending == 0:
            break
        if pending == 0:
            time.sleep(max(0.0, min(1e-3, reqs[i]["arrival"] - now)))
    span = time.perf_counter() - t0 - reqs[0]["arrival"]
    lat, failed = [], 0
    for rid in ids:
        st, latency, _ = srv.state(rid)
        if st == api.Server.DONE:
            lat.append(latency)
        else:
            failed += 1
        srv.release(rid)
    srv.close()
    body_steps = sum(len(r["case"][2]) for r in reqs) * steps
    value, plain_value = body_steps / span, plain_body_steps / plain_span
    return {"value": value, "unit": "particle-steps/s", "p50_s": percentile(lat, 50),
            "p99_s": percentile(lat, 99), "plain_value": plain_value,
            "plain_p50_s": percentile(plain_lat, 50), "plain_p99_s": percentile(plain_lat, 99),
            "plain_least_work_p50_s": percentile(plain_lat_lw, 50), "plain_least_work_p99_s": percentile(plain_lat_lw, 99),
            "policy": "least work (marker-steps) first among the queued requests that fit; plain_p50_s/p99 in "
                      "arrival order, plain_least_work_* with the same order as the served arm",
            "ratio_vs_plain": value / plain_value, "requests": len(reqs), "plain_requests": len(plain_reqs),
            "plain_note": "plain value and latencies over the first plain_requests requests of the same stream",
            "failed": failed,
            "steps_per_request": steps, "rate_per_s": 200.0,
            "bodies": sum(len(r["case"][2]) for r in reqs), "markers": sum(len(r["case"][1]) for r in reqs),
            "hbm_budget_bytes": budget, "peak_bytes_admitted": peak, "max_active": 64,
            "work_limit_markers": args.serve_work_limit,
            "workload": "Poisson arrivals (200/s, seed %d) of settling (fluid at rest, gravity) and shear "
                        "(Kolmogorov u_x = 0.05 sin(2 pi z/L)) cases, 16..2048 bodies d = 12h on the smallest of "
                        "64..256^3 holding them at <= 20%% solid fraction" % args.seed,
            "latency": "completion - arrival, host clock"}


def run_unresolved(args, device, stream, cpu=True):
    """Unresolved CFD-DEM: 1,048,576 polydisperse point particles on a 128^3 periodic
    fluid grid (packed bed plus gas region, upward flow 0.5 with a 5% Fourier
    perturbation), Gaussian volume fraction, drag of CalculateDragForce, contacts
    with Coulomb friction and tangential history.  Device-timed steps; the CPU
    restatement times one step of the same case on all host threads."""
    import torch
    from ibmdem import api, scenario

    n = args.unresolved_particles
    p, parts, field = scenario.unresolved_case(128, n, seed=args.seed, n_modes=32, field_device="cuda",
                                               bed_spacing=0.9)
    g = api.Unresolved(p, parts, field, device=device, stream=stream)
    g.step(3)
    g.synchronize()
    k = args.unresolved_steps
    l0 = g.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.step(k)
    e1.record(stream)
    torch.cuda.synchronize()
    g.synchronize()
    ms = e0.elapsed_time(e1)
    launches = g.launches - l0
    st, partner, _ = g.get_contacts()
    g.close()
    out = {"value": n * k / (ms / 1e3), "unit": "particle-steps/s", "steps": k, "ms_per_step": ms / k,
           "particles": n, "contacts_last_step": int(len(partner)), "gpu_launches": launches,
           "workload": "128^3 periodic fluid cells (h = 1 mm), d ~ U[0.8,1.2] x 0.25 h, 75%% in a packed bed "
                       "(jittered lattice of 0.9 x the largest diameter from z = 0, so neighbours start in contact), "
                       "25%% in the gas region, upward flow 0.5 m/s + 5%% 32-mode "
                       "Fourier perturbation, Gaussian volume fraction (sigma = 3 d, 5^3 cells), Di Felice drag "
                       "(CalculateDragForce), spring-dashpot with Coulomb friction (mu = 0.3, kt = 2/7 kn), "
                       "dt = 1e-5 s, seed %d" % args.seed,
           "timing": "CUDA events on the launching stream"}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        O.build()
        threads = os.cpu_count() or 1
        O.set_threads(threads)
        r = O.OracleUnresolved(p, parts, field)
        t0 = time.perf_counter()
        r.step(1)
        dt = time.perf_counter() - t0
        r.close()
        out["cpu_baseline"] = {"value": n / dt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                               "sample": "1 step of the same case (CPU restatement, OpenMP)", "seconds": dt}
    return out


# algorithmic bytes per interior node of the fluid stencil kernels (FP64 fields
# streamed once; the stencil neighbours come through L1/L2)
FLUID_BYTES = {
    # u,v,w, P, fx..fz, uold..wold, RHSul..wl read; the guess, Px..Pz, RHSul..wl written;
    # then the guess copied into u,v,w
    "guess": 13 * 8 + 9 * 8 + 6 * 8,
    # u,v,w read, velDiv written; P, Pcorr read, P written; u,v,w, P, Px..Pz read and
    # u,v,w written, then u,v,w read and omega written; the bulk sums and shift
    "other": 4 * 8 + 3 * 8 + 7 * 8 + 3 * 8 + 6 * 8 + 3 * 8 + 6 * 8,
}
# FP64 operations per interior node of VelocityGuess with unit spacing: 18 flux
# products (2 adds, 3 multiplies), 9 differences, 9 Laplacians (2 adds, 2
# multiplies), 3 gradients (a subtraction and a division), 3 right-hand sides
# (7 adds) and 3 updates (7 operations)
FLUID_GUESS_FP64_REF = 18 * 5 + 9 + 9 * 4 + 3 * 2 + 3 * 7 + 3 * 7
# FP64 instructions the guess kernel issues per interior node (ncu's
# sm__sass_thread_inst_executed_op_fp64_pred_on on the 128^3 grid: 371.2 M over
# 2,097,152 nodes; fewer than the statements' FLUID_GUESS_FP64_REF because exact
# scalings and identity coefficients are not issued, compares included)
FLUID_GUESS_FP64 = 177
# the Poisson kernels issue this many FP64 instructions per operation that
# poisson_counts counts (ncu on the 128^3 grid: 187.0 M issued against 155.8 M)
POISSON_ISSUED_PER_COUNTED = 1.2006


def poisson_counts(n, walls):
    """HBM bytes and FP64 operations of one PoissonSolver on an n grid (nx, ny,
    nz) with the walled axes doubled to ne: the ordered sum and the x forward
    read velDiv (two real rows per complex transform, nh = ne_x/2 + 1 columns
    kept), the y forward and the z solve read and write the half-spectrum grid,
    the y inverse covers the original z, the x inverse reads the original rows
    and writes Pcorr.  Per line of N points: an odd first stage 4 adds per
    pair, a first radix-4 stage 16 adds per 4 points, the other radix-4 stages
    3 complex products of 4 operations and 16 adds per 4 points; the spectrum
    split 8 per column, the eigenvalue scaling 5 per point."""
    import math
    ne = [2 * m if w else m for m, w in zip(n, walls)]
    nh = ne[0] // 2 + 1

    def line(N):
        lg = int(math.log2(N))
        if lg % 2:
            return (N // 2) * 4 + (N // 4) * 28 * ((lg - 1) // 2)
        return (N // 4) * 16 + (N // 4) * 28 * (lg // 2 - 1)

    nint = n[0] * n[1] * n[2]
    grid = nh * ne[1] * ne[2]
    pairs_f = (ne[1] * ne[2] + 1) // 2
    pairs_i = (n[1] * n[2] + 1) // 2
    nbytes = (nint * 8 * 2 + grid * 16 + grid * 32 * 2 + nh * ne[1] * n[2] * 32 + nh * n[1] * n[2] * 16
              + nint * 8)
    ops = (pairs_f * line(ne[0]) + pairs_f * nh * 8 + nh * ne[2] * line(ne[1]) + 2 * nh * ne[1] * line(ne[2])
           + grid * 5 + nh * n[2] * line(ne[1]) + pairs_i * line(ne[0]))
    return nbytes, ops


def run_fluid(args, device, stream, cpu=True):
    """The fluid step of FirstOrderForwardEuler around the Poisson solve on the GPU
    (fluid.F90:251-326 without SetPressureVector/PoissonSolver): uold = u,
    VelocityGuess(1,0,1), ModifyBulkVelocity (u and w switched, the reference's
    initialization), VelocityDivergence, PressureCorrection with a resident
    Pcorr, VelocityCorrection, each followed by FillGhostRegionForFluid and
    Boundary, on the default grid with the workload's Fourier field.
    Device-timed; the CPU restatement times one step on all host threads."""
    import torch
    import numpy as np
    from ibmdem import api

    p, parts, bodies, field = make_case(args.workload, args.seed, "cuda")
    g = api.Case(p, parts, bodies, field, device=device, stream=stream)
    g.set_fluid_params(1e-6, 0.0, 0.0, 0.0)

    def halo():
        g.FillGhostRegionForFluid()
        g.Boundary()

    def fstep():
        g.StoreOldVelocity()
        g.VelocityGuess(1.0, 0.0, 1.0)
        halo()
        g.ModifyBulkVelocity(1, 0, 1, 0.1, 0.0, 0.0)
        halo()
        g.VelocityDivergence(1.0)
        halo()
        g.PressureCorrection(None)
        halo()
        g.VelocityCorrection(1.0)
        halo()

    for _ in range(3):
        fstep()
    g.synchronize()
    k = args.fluid_steps
    g.timing(True)
    g.phase_times(reset=True)
    l0 = g.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(k):
        fstep()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = g.launches - l0
    ph = g.phase_times(reset=True)
    # the Poisson solve alone: velDiv of the last step in, Pcorr out
    for _ in range(3):
        g.PoissonSolver()
    g.synchronize()
    kp = max(5, k // 2)
    e0.record(stream)
    for _ in range(kp):
        g.PoissonSolver()
    e1.record(stream)
    torch.cuda.synchronize()
    pois_ms = e0.elapsed_time(e1) / kp

    # the whole fluid step of FirstOrderForwardEuler on the device: the
    # stencils with the Poisson solve between the divergence and the correction
    def full_step():
        g.StoreOldVelocity()
        g.VelocityGuess(1.0, 0.0, 1.0)
        halo()
        g.ModifyBulkVelocity(1, 0, 1, 0.1, 0.0, 0.0)
        halo()
        g.VelocityDivergence(1.0)
        halo()
        g.PoissonSolver()
        g.PressureCorrection(None)
        halo()
        g.VelocityCorrection(1.0)
        halo()

    for _ in range(3):
        full_step()
    g.synchronize()
    e0.record(stream)
    for _ in range(kp):
        full_step()
    e1.record(stream)
    torch.cuda.synchronize()
    full_ms = e0.elapsed_time(e1) / kp

    # the reference's whole time step on the device (FirstOrderForwardEuler,
    # fluid.F90:251-326, then CloudEvolutionMS): the forcing loop on the live
    # fields, the fluid update with the Poisson solve, the bodies
    def coupled_step():
        g.StoreOldVelocity()
        g.MultiDirectForcing()
        g.VelocityGuess(1.0, 0.0, 1.0)
        halo()
        g.ModifyBulkVelocity(1, 0, 1, 0.1, 0.0, 0.0)
        halo()
        g.VelocityDivergence(1.0)
        halo()
        g.PoissonSolver()
        g.PressureCorrection(None)
        halo()
        g.VelocityCorrection(1.0)
        halo()
        g.CloudEvolutionMS()

    # InitializationDEM's lists and weights (CloudEvolutionMS rebuilds them after every step)
    g.RebuildAllListOrNot()
    g.UpdateLocalCellWeightListDEM()
    g.UpdateGhostCellWeightListDEM()
    for _ in range(3):
        coupled_step()
    g.synchronize()
    e0.record(stream)
    for _ in range(kp):
        coupled_step()
    e1.record(stream)
    torch.cuda.synchronize()
    coupled_ms = e0.elapsed_time(e1) / kp
    nbodies = int(len(bodies))
    g.close()
    nint = int(p["nx"]) * int(p["ny"]) * int(p["nz"])
    phases = {name: {"ms_per_step": ph[name][0] / k} for name in ("fluid_guess", "fluid_halo", "fluid_other")}
    guess_ms = phases["fluid_guess"]["ms_per_step"]
    hbm_peak, peak_kind = measured_peaks()
    fp64_peak = api.fp64_rate(device)
    out = {"value": nint * k / (ms / 1e3), "unit": "interior node-steps/s", "steps": k, "ms_per_step": ms / k,
           "interior_nodes": nint, "gpu_launches": launches, "phases": phases,
           "roofline": {"kernel": "fluid_guess", "bound": "fp64",
                        "algorithmic_bytes_per_step": nint * FLUID_BYTES["guess"],
                        "hbm_achieved_gbs": nint * FLUID_BYTES["guess"] / (guess_ms / 1e3) / 1e9,
                        "hbm_peak_gbs": hbm_peak, "hbm_peak_kind": peak_kind,
                        "fp64_ops_per_node": FLUID_GUESS_FP64,
                        "fp64_ops_note": "FP64 instructions the kernel issues (ncu count); the reference's "
                                         "statements have %d" % FLUID_GUESS_FP64_REF,
                        "fp64_achieved_gops": nint * FLUID_GUESS_FP64 / (guess_ms / 1e3) / 1e9,
                        "fp64_peak_gops": fp64_peak,
                        "fp64_frac": nint * FLUID_GUESS_FP64 / (guess_ms / 1e3) / 1e9 / fp64_peak if fp64_peak else None},
           "workload": "%s grid, the workload's Fourier field, visc 1e-6, bulk velocity (u: 0.1, w: 0) switched on "
                       "as in the reference's initialization; the Poisson solve (PETSc) is outside, Pcorr resident"
                       % "x".join(str(int(p[a])) for a in ("nx", "ny", "nz")),
           "timing": "CUDA events on the launching stream"}
    dims = [int(p[a]) for a in ("nx", "ny", "nz")]
    pb, pops = poisson_counts(dims, [int(p["bType"][2 * d]) == 1 for d in range(3)])
    out["poisson"] = {
        "ms_per_solve": pois_ms, "solves": kp, "value": nint / (pois_ms / 1e3), "unit": "interior node-solves/s",
        "method": "direct FFT solve of the reference's pinned 7-point system (FP64, hand-written radix-4 lines in "
                  "shared memory, real rows paired into complex x transforms, half spectrum along y and z; 8 launches)",
        "roofline": {"bound": "fp64", "fp64_ops_per_solve": pops,
                     "fp64_achieved_gops": pops / (pois_ms / 1e3) / 1e9, "fp64_peak_gops": fp64_peak,
                     "fp64_frac": pops / (pois_ms / 1e3) / 1e9 / fp64_peak if fp64_peak else None,
                     "fp64_issued_frac": pops * POISSON_ISSUED_PER_COUNTED / (pois_ms / 1e3) / 1e9 / fp64_peak
                     if fp64_peak else None,
                     "fp64_note": "fp64_frac counts the transforms' operations (poisson_counts); the kernels issue "
                                  "%.2f times as many FP64 instructions (ncu, 128^3), fp64_issued_frac" %
                                  POISSON_ISSUED_PER_COUNTED,
                     "hbm_bytes_per_solve": pb, "hbm_achieved_gbs": pb / (pois_ms / 1e3) / 1e9,
                     "hbm_peak_gbs": hbm_peak},
        "cpu_baseline": None,
        "cpu_baseline_note": "the reference solves with PETSc GMRES + hypre, which cannot be built here",
        "full_fluid_step_ms": full_ms,
        "full_fluid_step_note": "the fluid step above with the Poisson solve between the divergence and the pressure "
                                "correction: the whole FirstOrderForwardEuler fluid update on the device",
        "coupled_step_ms": coupled_ms,
        "coupled_value": nbodies / (coupled_ms / 1e3), "coupled_unit": "particle-steps/s",
        "coupled_note": "the reference's whole time step on the device with no host copy: uold, the 5-iteration "
                        "forcing loop on the live fields, the guess, the bulk shift, the divergence, the Poisson "
                        "solve, the corrections with their halo fills, then CloudEvolutionMS; %d spheres" % nbodies}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        O.build()
        threads = os.cpu_count() or 1
        O.set_threads(threads)
        r = O.OracleFluid(p)
        r.set_fluid_params(1e-6, 0.0, 0.0, 0.0)
        from ibmdem.records import FLUID
        host = [np.ascontiguousarray(f.cpu().numpy() if hasattr(f, "cpu") else f) for f in field]
        for name, a in zip(("u", "v", "w"), host):
            r.set_field(FLUID[name], a)
        t0 = time.perf_counter()
        r.StoreOldVelocity()
        r.VelocityGuess(1.0, 0.0, 1.0)
        for call in (lambda: r.ModifyBulkVelocity(1, 0, 1, 0.1, 0.0, 0.0), lambda: r.VelocityDivergence(1.0),
                     r.PressureCorrection, lambda: r.VelocityCorrection(1.0), None):
            r.FillGhostRegionForFluid()
            r.Boundary()
            if call is not None:
                call()
        dt = time.perf_counter() - t0
        r.close()
        out["cpu_baseline"] = {"value": nint / dt, "unit": "interior node-steps/s", "cores": threads, "kind": "port",
                               "sample": "1 step of the same grid and field (CPU restatement; VelocityGuess, the "
                                         "divergence and the corrections with OpenMP, the halo fills serial)",
                               "seconds": dt}
    return out


def unresolved_algorithmic(n, nint, contacts):
    """Compulsory bytes and FP64 instructions per launch of the unresolved kernels."""
    return {
        # each stamp (25 partial products + 5 gx) read once, cell starts, alphaf written
        "alpha": {"bytes": n * 30 * 8 + nint * (4 + 8), "fp64": n * 125 * 2},
        # particle state read and written, 3 x 8 face values + 8 fractions gathered, fdrag/alphaf written
        "drag": {"bytes": n * (2 * 16 * 8 + 32 * 8 + 4 * 8), "fp64": n * 330},
        # per pair: both particles' x, v, omega, m, r, the old and new displacement, the two terms
        "contacts": {"bytes": contacts * (2 * 11 * 8 + 2 * 24 + 48) + n * 6 * 8, "fp64": contacts * 150},
        "stamps": {"bytes": n * (5 * 8 + 32 * 8), "fp64": n * 220},
    }


def run_unresolved_main(args, world, rank, local):
    """bench.py --workload unresolved-...: the unresolved step as the headline line."""
    import numpy as np
    import torch
    from ibmdem import api, scenario

    ncell, n = UNRESOLVED_WORKLOADS[args.workload]
    fp64_peak = api.fp64_rate(local)
    p, parts, field = scenario.unresolved_case(ncell, n, seed=args.seed + rank, n_modes=32, field_device="cuda",
                                               bed_spacing=0.9)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        O.build()
        threads = os.cpu_count() or 1
        O.set_threads(threads)
        r = O.OracleUnresolved(p, parts, field)
        t0 = time.perf_counter()
        r.step(1)
        dt = time.perf_counter() - t0
        r.close()
        cpu = {"value": n / dt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": "1 step of the same case (CPU restatement, OpenMP)", "seconds": dt}
    stream = torch.cuda.Stream()
    g = api.Unresolved(p, parts, field, device=local, stream=stream)
    g.step(args.warmup)
    g.synchronize()
    g.timing(True)
    g.phase_times(reset=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = g.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        g.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    g.synchronize()
    ms = e0.elapsed_time(e1)
    launches = g.launches - l0
    phases = g.phase_times(reset=True)
    g.timing(False)
    ms_max = max_over_ranks(ms)
    value = world * n * args.steps / (ms_max / 1e3)
    _, partner, _ = g.get_contacts()
    # end to end: host fluid in, step, fluid fraction out (what a coupled fluid solver exchanges)
    shape = g.shape
    hin = [torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    for a, b in zip(hin, field):
        a[...] = b
    hout = torch.empty(g.nint, dtype=torch.float64, pin_memory=True).numpy()
    import ctypes

    def e2e_step():
        g._chk(g.lib.ibmdem_unresolved_set_fluid(g.h, *[a.ctypes.data for a in hin]), "set_fluid")
        g.step(1)
        g._chk(g.lib.ibmdem_unresolved_get_volume_fraction(g.h, hout.ctypes.data), "get_volume_fraction")

    e2e_val = None
    if args.e2e_steps > 0:
        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        e2e_val = world * n * args.e2e_steps / max_over_ranks(time.perf_counter() - t0)
    g.close()
    if rank == 0:
        hbm_peak, peak_kind = measured_peaks()
        alg = unresolved_algorithmic(n, g.nint, len(partner))
        dom = max(alg, key=lambda k: phases.get(k, (0, 0))[0])
        tot, cnt = phases[dom]
        ms_launch = tot / max(cnt, 1)
        achieved = alg[dom]["bytes"] / (ms_launch / 1e3) / 1e9
        fp64_gops = alg[dom]["fp64"] / (ms_launch / 1e3) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "fluid_cells": [ncell] * 3, "particles": n,
                       "contacts_last_step": int(len(partner)), "dt": float(p["dt"]),
                       "l2": "working set several GB > 129 MB L2 (no flush needed)"},
            "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "peak_kind": peak_kind, "traffic": None,
                         "algorithmic_bytes_per_launch": alg[dom]["bytes"], "ms_per_launch": ms_launch,
                         "fp64": {"achieved_gops": fp64_gops, "peak_gops": fp64_peak,
                                  "peak_kind": "measured live (ibmdem_measure_fp64_rate)",
                                  "frac": fp64_gops / fp64_peak, "instr_per_launch": alg[dom]["fp64"]}},
            "phases": {k: {"ms_total": round(t, 3), "launches": c, "ms_per_launch": t / c}
                       for k, (t, c) in phases.items() if c},
            "e2e": {"value": e2e_val, "unit": "particle-steps/s", "h2d_bytes_per_step": 3 * int(np.prod(shape)) * 8,
                    "d2h_bytes_per_step": g.nint * 8, "steps": args.e2e_steps,
                    "path": "ibmdem_unresolved_set_fluid(host u,v,w) + ibmdem_unresolved_step + "
                            "ibmdem_unresolved_get_volume_fraction, pinned host buffers"},
            "gpu_launches": launches, "clocks": clk.summary(),
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if not torch.cuda.is_available():
        print(json.dumps({"error": "no CUDA device"}))
        return 1
    torch.cuda.set_device(local)
    from ibmdem import api

    api.load()
    if args.workload in UNRESOLVED_WORKLOADS:
        rc = run_unresolved_main(args, world, rank, local)
        if world > 1:
            torch.distributed.destroy_process_group()
        return rc
    fp64_peak = api.fp64_rate(local)
    p, parts, bodies, field = make_case(args.workload, args.seed + rank, "cuda")
    # CPU baseline on the same case (OpenMP threads in this process; no fork)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline((p, parts, bodies, field), args.cpu_steps)
    stream = torch.cuda.Stream()
    case = api.Case(p, parts, bodies, field, device=local, stream=stream)
    nb, nm = len(bodies), len(parts)
    case.InitializationDEM()
    case.step(max(args.warmup - 1, 0))
    # list sizes for the algorithmic bytes (this builds the plan that the next
    # step would build first), then the last warm-up step
    counters = case.counters()
    case.step(1)
    case.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = case.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            case.step(1)
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    case.synchronize()
    ms = e0.elapsed_time(e1)
    launches = case.launches - launches0
    # per-phase times: a second pass of the same steps with CUDA events around
    # every phase (kept out of the timed pass above)
    case.timing(True)
    case.phase_times(reset=True)
    for _ in range(args.steps):
        case.step(1)
    case.synchronize()
    phases = case.phase_times(reset=True)
    case.timing(False)
    ms_phased = sum(t for t, _ in phases.values())
    ms_max = max_over_ranks(ms)
    value = world * nb * args.steps / (ms_max / 1e3)

    # end to end through the C ABI: host field in, fluid + forcing + bodies out
    shape = case.shape
    pin = lambda: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
    hin = [pin() for _ in range(3)]
    for a, b in zip(hin, field):
        a[...] = b
    hout = [pin() for _ in range(6)]
    import numpy as np
    from ibmdem.records import MULTISPHERE

    hb = np.zeros(nb, MULTISPHERE)
    import ctypes

    copy_stream = torch.cuda.Stream()
    hf = [pin() for _ in range(3)]  # the caller's fx, fy, fz
    for a in hf:
        a[...] = 0.0

    def e2e_step_sparse():
        # the coupled sequence of a caller that keeps its fields: fluid in,
        # multi-direct forcing, the changed nodes of u,v,w and the forcing back
        # into the caller's arrays while the bodies and lists advance, bodies out
        case._chk(case.lib.ibmdem_set_fluid_async(case.h, *[a.ctypes.data for a in hin]), "set_fluid_async")
        case.MultiDirectForcing()
        case._chk(case.lib.ibmdem_update_fluid_async(case.h, *[a.ctypes.data for a in hin + hf],
                                                     ctypes.c_void_p(copy_stream.cuda_stream)), "update_fluid_async")
        case.CloudEvolutionMS()
        n = ctypes.c_int32()
        case._chk(case.lib.ibmdem_get_bodies(case.h, hb.ctypes.data, nb, ctypes.byref(n)), "get_bodies")
        case._chk(case.lib.ibmdem_update_fluid_wait(case.h), "update_fluid_wait")

    def e2e_step():
        # the coupled sequence: fluid in, multi-direct forcing, the corrected
        # fluid and forcing out (six whole fields) while the bodies and lists
        # advance, bodies out
        case._chk(case.lib.ibmdem_set_fluid_async(case.h, *[a.ctypes.data for a in hin]), "set_fluid_async")
        case.MultiDirectForcing()
        case._chk(case.lib.ibmdem_get_fluid_async(case.h, *[a.ctypes.data for a in hout],
                                                  ctypes.c_void_p(copy_stream.cuda_stream)), "get_fluid_async")
        case.CloudEvolutionMS()
        n = ctypes.c_int32()
        case._chk(case.lib.ibmdem_get_bodies(case.h, hb.ctypes.data, nb, ctypes.byref(n)), "get_bodies")
        copy_stream.synchronize()

    def timed(fn):
        fn()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            fn()
        return world * nb * args.e2e_steps / max_over_ranks(time.perf_counter() - t0)

    e2e_val = e2e_sparse = None
    upd_bytes = ctypes.c_int64()
    if args.e2e_steps > 0:
        e2e_val = timed(e2e_step)
        e2e_sparse = timed(e2e_step_sparse)
        case.lib.ibmdem_update_fluid_bytes(case.h, ctypes.byref(upd_bytes))
    fbytes = int(np.prod(shape)) * 8

    if rank == 0:
        hbm_peak, peak_kind = measured_peaks()
        alg = algorithmic(counters)
        per_phase = {}
        for k, (tot, n) in phases.items():
            if n:
                per_phase[k] = {"ms_total": round(tot, 3), "launches": n, "ms_per_launch": tot / n}
        rows = kernel_rows(alg, phases, hbm_peak, fp64_peak, counters["npLocal"])
        # dominant kernel: the one with the largest share of the timed region
        dom = max(rows, key=lambda k: phases.get(k, (0, 0))[0])
        r = rows[dom]
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(args.workload, nm),
            "marker_steps_per_s": world * nm * args.steps / (ms_max / 1e3),
            "roofline": {"kernel": dom, "bound": r["bound"], "achieved": r["compulsory_gbs"], "peak": hbm_peak,
                         "unit": "GB/s", "frac": r["hbm_frac"], "peak_kind": peak_kind + " (hbm_gbs)",
                         "traffic": r["traffic"], "algorithmic_bytes_per_launch": r["compulsory_bytes"],
                         "bytes_note": "compulsory bytes of the hot-path scope table; the kernel also moves its "
                                       "own intermediates (moved_bytes: the spread plan, the stored weights)",
                         "waste_ratio": r["waste_ratio"], "ms_per_launch": r["ms_per_launch"],
                         "fp64": {"achieved_gops": r["fp64_gops"], "peak_gops": fp64_peak,
                                  "peak_kind": "measured live (ibmdem_measure_fp64_rate: DFMA issue rate)",
                                  "frac": r["fp64_frac"], "instr_per_launch": r["fp64_issued"],
                                  "instr_note": "FP64 instructions the kernel issues"},
                         "kernels": rows},
            "phases": per_phase,
            "phases_note": "a second pass of the same steps with CUDA events around every phase: "
                           "ms_per_step_phased %.3f" % (ms_phased / args.steps),
            "e2e": {"value": e2e_val, "unit": "particle-steps/s", "h2d_bytes_per_step": 3 * fbytes,
                    "d2h_bytes_per_step": 6 * fbytes + nb * MULTISPHERE.itemsize, "steps": args.e2e_steps,
                    "path": "ibmdem_set_fluid_async(host u,v,w; each component's forcing loop starts when it "
                            "has arrived) + ibmdem_MultiDirectForcing (by component) + "
                            "ibmdem_get_fluid_async(u,v,w,fx,fy,fz; each component leaves when done) + "
                            "ibmdem_CloudEvolutionMS + "
                            "ibmdem_get_bodies, pinned host buffers",
                    "sparse_readout": {
                        "value": e2e_sparse, "d2h_bytes_per_step": int(upd_bytes.value) + nb * MULTISPHERE.itemsize,
                        "path": "the same with ibmdem_update_fluid_async: the touched nodes' u and f written into "
                                "the caller's own arrays by host threads (slower here: the touched nodes cover most "
                                "cache lines of the arrays, so the scatter moves more host memory than the copy)"}},
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "counters": counters,
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
    case.close()
    if rank == 0 and world == 1:
        legs = [("batched", args.batch_cases > 0, lambda: run_batched(args, local, stream)),
                ("served", args.serve_requests > 0, lambda: run_served(args, local, stream)),
                ("unresolved", args.unresolved_particles > 0,
                 lambda: run_unresolved(args, local, stream, cpu=not args.no_cpu_baseline)),
                ("fluid", args.fluid_steps > 0, lambda: run_fluid(args, local, stream, cpu=not args.no_cpu_baseline))]
        for name, on, leg in legs:
            if on:
                t_leg = time.perf_counter()
                line[name] = leg()
                line[name]["wall_s"] = round(time.perf_counter() - t_leg, 1)  # the whole leg, set-up included
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
