#!/usr/bin/env python
"""Benchmark of the FLUE hot path on GB300: 5-loop F_munu + B^2 forward +
backward (the su(3) gradient of B^2) on a 32^3 x 64 lattice.

One "step" = one call of flue_magnetic_force on a device-resident FP32 field
(reconstruct-12 by default): lines -> F and B^2 -> line cotangents -> link
gradient.  ``value`` is sites/s = n_ranks * V / (max over ranks of the
device time per step).  The same step in FP64 (complex128), the FP32 error
against FP64, the end-to-end call through the host-buffer C ABI
(flue_magnetic_force_c: H2D of the field, kernels, D2H of the gradient) and
the CPU baseline (the oracle's OpenMP restatement of the reference's
magnetic(), forward only -- the reference has no backward) are reported on
the same JSON line.

Synthetic data: links exp(i eps H), H = sum_a c_a lambda_a / 2, c_a ~ N(0,1)
from numpy PCG64(seed), eps = 0.3, reunitarised (FixSU3Matrix).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Multi-GPU (torchrun): every rank runs an independent replica on its own
field (the path has no cross-field exchange): weak scaling.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sites/s 5-loop Fmunu+B^2 fwd+bwd @32^3x64: FP32 vs FP64 GPU, ≤1e-6 rel, %HBM"
# algorithmic bytes per site of one fwd+bwd (3 spatial links read for the
# forward, read again for the backward, a 4-direction gradient written in U's
# dtype): FP64 1440, FP32-18 720, FP32-r12 576
ALG_BYTES = {"c128": 1440, "c64": 720, "r12": 576}
# matrix products per site of one fwd+bwd as this implementation structures it:
# lines 6, forward 3 planes x 28 leaves x 3, line cotangents 3 dirs x (96+64+64),
# link cotangents 3 x 7; 198 flop per 3x3 complex product (27 cmul + 18 cadd)
PRODUCTS_PER_SITE = {"lines": 6, "fwd": 252, "linecot": 672, "linkcot": 21}
FLOP_PER_PRODUCT = 198


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--prec", choices=["r12", "c64"], default="r12")
    p.add_argument("--dims", default="64,32,32,32", help="NT,NX,NY,NZ")
    p.add_argument("--eps", type=float, default=0.3)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--fp64-steps", type=int, default=3)
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="target length of the CPU sample")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--ensemble", action="store_true",
                   help="also time the 96-field ensemble (plaquette/Polyakov/B^2 in one graph-captured launch)")
    p.add_argument("--propagator", action="store_true",
                   help="instead of the headline step, time the scalar gluon propagator (FFT pipeline) per precision")
    p.add_argument("--observables", action="store_true",
                   help="instead of the headline step, time every observable entry point (FP64 and FP32-r12)")
    return p.parse_args()


# algorithmic bytes per site (links that must be read once + outputs written
# once) and products per site, per observable, for (c128, r12)
OBS_COST = {
    # name: (links read per site, output matrices per site, products per site)
    "plaquette (6 planes)": (4, 0, 6 * 2.2),
    "polyakov": (1, 0, 1.0),
    "wmunu 2x2 (1 plane)": (2, 0, 9.0),
    "wmunu table R,T<=8 (1 plane)": (2, 0, 14.0 + 64 * 3),
    "genericpath 8 steps (every site)": (2, 1, 7.0),
    "clover F (1 plane)": (2, 1, 12.0 + 1),
    "5-loop F (1 plane)": (2, 1, 84.0 + 4),
    "magnetic B^2 forward": (3, 0, 252.0 + 6),
    "B^2 forward+backward": (3, 7, 951.0),
    "plaquette action + force": (4, 4, 4 * 3 * 4.0),
    "Wilson-flow RK3 step": (4, 4, 3 * (48.0 + 12)),
}


def observables_bench(dims, steps):
    """Device time of one call of every observable at `dims`, FP64 (c128) and
    FP32 (r12), with achieved bandwidth (algorithmic bytes / time) and FLOP rate."""
    import torch

    from flue_gb300 import flow, forces, generate, gluonCalc as G
    from flue_gb300.field import GaugeField

    nt, nx, ny, nz = dims
    V = nt * nx * ny * nz
    f64 = generate.random_field(dims, 0.3, 1, device="cuda")
    fields = {"c128": f64, "r12": GaugeField.from_array(f64, prec="r12"), "c64": GaugeField.from_array(f64, prec="c64")}
    link_b = {"c128": 144, "r12": 48, "c64": 72}
    mat_b = {"c128": 144, "r12": 72, "c64": 72}
    path = [2, 2, 3, 3, -2, -2, -3, -3]

    def calls(f):
        return {
            "plaquette (6 planes)": lambda: G.plaquette(f, 1, 4, 4),
            "polyakov": lambda: G.polyakov(f),
            "wmunu 2x2 (1 plane)": lambda: G.wmunu(f, 2, 3, 2, 2),
            "wmunu table R,T<=8 (1 plane)": lambda: G.wmunu_table(f, 2, 3, 8, 8),
            "genericpath 8 steps (every site)": lambda: G.genericpath_all(f, path),
            "clover F (1 plane)": lambda: G.cloverloopmunucoord(f, 3, 2),
            "5-loop F (1 plane)": lambda: G.loop5munucoord(f, 3, 2),
            "magnetic B^2 forward": lambda: G.magnetic(f),
            "B^2 forward+backward": lambda: forces.magnetic_force(f),
            "plaquette action + force": lambda: forces.plaquette_force(f),
            "Wilson-flow RK3 step": (lambda: flow.wflow_step(f, 0.01)) if f.prec != "r12" else None,
        }

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    rows = []
    for prec in ("c128", "c64", "r12"):
        f = fields[prec]
        for name, fn in calls(f).items():
            if fn is None:
                continue
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            n = steps if name not in ("B^2 forward+backward",) or prec != "c128" else max(1, steps // 5)
            e0.record()
            for _ in range(n):
                fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / n
            lr, mo, pr = OBS_COST[name]
            byt = V * (lr * link_b[prec] + mo * mat_b[prec])
            rows.append({"observable": name, "prec": prec, "ms": ms, "sites_per_s": V / (ms * 1e-3),
                         "alg_GBps": byt / (ms * 1e-3) / 1e9, "hbm_frac": byt / (ms * 1e-3) / 1e9 / peaks.get("hbm_gbs", 6800.0),
                         "TFLOPs": V * pr * 198 / (ms * 1e-3) / 1e12})
    return {"lattice": list(dims), "sites": V, "rows": rows,
            "note": "ms includes the host round trip of scalar results (tiny) and per-call launches; bytes are "
                    "algorithmic (links read once, outputs written once)"}


def propagator_bench(dims, steps):
    """Scalar gluon propagator D(q) on every momentum of `dims` (device-resident
    field, FP64 output): ms per call and sites/s for c128 (FP64 transforms),
    c64 and r12 (FP32 transforms).  `alg_bytes_per_site` = links read once +
    D written once; `pipeline_bytes_per_site` = that plus the 32 colour fields
    written, read by the time transform, its half spectrum written, read and
    written by the (x,y,z) transform and read twice by the sum (the +-q reads)."""
    import torch

    from flue_gb300 import generate, gluonProp
    from flue_gb300.field import GaugeField

    nt, nx, ny, nz = dims
    V = nt * nx * ny * nz
    f64 = generate.random_field(dims, 0.3, 1, device="cuda")
    fields = {"c128": f64, "c64": GaugeField.from_array(f64, prec="c64"), "r12": GaugeField.from_array(f64, prec="r12")}
    link_b = {"c128": 144, "c64": 72, "r12": 48}
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    rows = []
    for prec, f in fields.items():
        es = 8 if prec == "c128" else 4
        spec = 32 * (nt // 2 + 1) / nt * 2 * es  # half spectrum bytes per site
        alg = 4 * link_b[prec] + 8
        pipe = alg + 32 * es * 2 + spec * 4
        for _ in range(3):
            gluonProp.scalar_gluon_prop(f)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            gluonProp.scalar_gluon_prop(f)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        rows.append({"prec": prec, "ms": ms, "sites_per_s": V / (ms * 1e-3), "alg_bytes_per_site": alg,
                     "pipeline_bytes_per_site": round(pipe, 1), "alg_GBps": alg * V / (ms * 1e-3) / 1e9,
                     "pipeline_GBps": pipe * V / (ms * 1e-3) / 1e9,
                     "pipeline_hbm_frac": pipe * V / (ms * 1e-3) / 1e9 / hbm})
    return {"metric": "scalar gluon propagator D(q), all momenta", "lattice": list(dims), "sites": V,
            "hbm_peak_gbs": hbm, "steps": steps, "rows": rows}


def bench_config(args, dims, n_replicas):
    """The workload description shared by both arms of the benchmark."""
    nt, nx, ny, nz = dims
    return {"workload": f"5-loop F_munu + B^2 forward + backward (su(3) gradient), {nx}^3x{nt}",
            "lattice": [nt, nx, ny, nz], "sites": nt * nx * ny * nz, "field_format": args.prec, "eps": args.eps,
            "seed": args.seed, "global_batch": n_replicas, "parallelism": f"replicas x{n_replicas}",
            "l2": "inputs and intermediates larger than L2 (field 0.4-0.6 GB, 9 GB DRAM traffic per step)"}


def ensemble_bench(steps: int):
    """96 fields: L in {16,24,32} x T in {32,48,64}, 8 each, plus 24 at 24^3x48,
    eps = 0.4, per-field seeds (GPU Philox); FP32 (c64) and FP64 (c128)."""
    import torch

    from flue_gb300 import ensemble as E, generate
    from flue_gb300.field import GaugeField

    dims = [(t, l, l, l) for l in (16, 24, 32) for t in (32, 48, 64) for _ in range(8)] + [(48, 24, 24, 24)] * 24
    sites = sum(d[0] * d[1] ** 3 for d in dims)
    t0 = time.perf_counter()
    f64 = [generate.random_field_philox(d, 0.4, 5000 + i, prec="c128") for i, d in enumerate(dims)]
    f32 = [GaugeField.from_array(f, prec="c64") for f in f64]
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    out = {"fields": len(dims), "sites": sites, "gen_s": gen_s}
    cands = [(t, b, m) for t in (4, 16, 32) for b in (128, 256) for m in (1, 3)]
    cfg = E.autotune(f32, candidates=cands, reps=1)
    b2s = {}
    from flue_gb300 import _lib

    L = _lib.load()
    runs = (("fp32", f32, steps, "persistent"), ("fp64", f64, 1, "persistent"), ("fp32_pipeline", f32, steps, "pipeline"),
            ("fp64_pipeline", f64, 1, "pipeline"))
    for name, fs, nrep, mode in runs:
        if mode == "pipeline":
            ens = E.Ensemble(fs, mode="pipeline")
        else:
            ens = E.Ensemble(fs, tile=cfg[0], block=cfg[1], blocks_per_sm=cfg[2])
        ens.capture()
        ens.launch()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = L.flue_kernel_launches()
        e0.record()
        for _ in range(nrep):
            ens.launch()
        e1.record()
        torch.cuda.synchronize()
        nl = (L.flue_kernel_launches() - n0) // nrep
        ms = e0.elapsed_time(e1) / nrep
        b2 = ens.out[:, 4].cpu().numpy()
        b2s[name] = b2
        out[name] = {"mode": mode, "ms_per_eval": ms, "sites_per_s": sites / (ms * 1e-3),
                     "fields_per_s": len(dims) / (ms * 1e-3), "b2_first": float(b2[0]), "kernels_per_eval": int(nl)}
        if mode == "persistent":
            out[name].update({"items": ens.items,
                              "config": {"tile_cols": cfg[0], "block": cfg[1], "blocks_per_sm": cfg[2]}})
        ens.close()
    out["b2_rel_pipeline_persistent_fp64_max"] = float(
        max(abs(a - b) / abs(b) for a, b in zip(b2s["fp64_pipeline"], b2s["fp64"])))
    out["b2_rel_fp32_fp64_max"] = float(max(abs(a - b) / abs(b) for a, b in zip(b2s["fp32"], b2s["fp64"])))
    return out


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.15)
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch

    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(dims, eps, seed, target_s):
    """The oracle's OpenMP magnetic() on a bounded sample: repeated passes over
    the first time slices of the benchmark field (built on the host)."""
    import oracle

    U = host_slab(dims, eps, seed)
    nts = U.shape[0]
    V3 = dims[1] * dims[2] * dims[3]
    t0 = time.perf_counter()
    oracle.magnetic_slab(U, 1, nts)
    one = max(time.perf_counter() - t0, 1e-3)
    reps = int(max(1, round(target_s / one)))
    t0 = time.perf_counter()
    for _ in range(reps):
        oracle.magnetic_slab(U, 1, nts)
    dt = time.perf_counter() - t0
    return {"value": reps * nts * V3 / dt, "unit": "sites/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"oracle magnetic() forward (B^2 only; the reference has no backward), OpenMP, {reps} passes "
                      f"over time slices 1..{nts} of the {dims[1]}^3x{dims[0]} field ({reps * nts * V3} sites, "
                      f"{dt:.2f} s)"}


# time slices of the field that the CPU legs generate and time: B^2 uses only
# the spatial planes, so time slices are independent and the first nts slices
# of the full seeded field are the field random_field((nts, NX, NY, NZ))
CPU_SLICES = 8


def host_slab(dims, eps, seed, nts=CPU_SLICES):
    """The first `nts` time slices of the benchmark field, built on the host
    with numpy only (the Gell-Mann coefficients are drawn in (t,x,y,z,mu,a)
    order, so these slices are bitwise those of the full field's host
    construction).  Touches neither the GPU nor this repository's library."""
    from flue_gb300 import generate

    nt, nx, ny, nz = dims
    return generate.random_field((min(nt, nts), nx, ny, nz), eps, seed)


def run_reference(args, dims, ws, rank):
    """--impl reference: the reference's algorithm (oracle port of wloops.F90
    magnetic(), forward only) on the host cores; rank 0 only.  The field is
    built on the host (numpy) and the arm never loads the CUDA library."""
    if rank != 0:
        return
    import oracle

    oracle.build()
    nt, nx, ny, nz = dims
    U = host_slab(dims, args.eps, args.seed)
    nts = U.shape[0]
    V3 = nx * ny * nz
    t0 = time.perf_counter()
    oracle.magnetic_slab(U, 1, nts)
    one = max(time.perf_counter() - t0, 1e-3)
    per_step_s = max(1.0, min(20.0, 120.0 / max(1, args.steps + args.warmup)))
    reps = int(max(1, round(per_step_s / one)))
    for _ in range(args.warmup):
        oracle.magnetic_slab(U, 1, nts)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for _ in range(reps):
            oracle.magnetic_slab(U, 1, nts)
    dt = (time.perf_counter() - t0) / args.steps
    val = reps * nts * V3 / dt
    line = {"metric": METRIC, "value": val, "unit": "sites/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args, dims, 1),
            "impl": "reference",
            "cpu_baseline": {"value": val, "unit": "sites/s", "cores": oracle.num_threads(), "kind": "port",
                             "sample": f"per step: {reps} x magnetic() over time slices 1..{nts} of the field "
                                       f"({reps * nts * V3} sites, built on the host with numpy), forward only "
                                       "(the reference has no backward); Fortran reference not buildable here, "
                                       "C restatement of src/wloops.F90 timed instead"},
            "e2e": {"value": val, "unit": "sites/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# DRAM bytes (read + write) per site of one device step, from an ncu capture of this bench
# (16 time slabs at 32^3x64, reconstruct-12) with --cache-control none: no cache flush
# between the kernels, so the write-backs of the intermediates (lines, F, line
# cotangents) count where they happen.  ncu's default flush before every kernel writes
# them back outside any kernel and the per-kernel sum then reads 3886.5 B/site.
TRAFFIC_PER_SITE = {("r12", (64, 32, 32, 32)): 4358.6}


def step_traffic(prec, dims):
    b = TRAFFIC_PER_SITE.get((prec, tuple(dims)))
    return None if b is None else b * dims[0] * dims[1] * dims[2] * dims[3]


def main():
    args = parse()
    dims = tuple(int(v) for v in args.dims.split(","))
    nt, nx, ny, nz = dims
    V = nt * nx * ny * nz
    if args.impl == "reference":
        ws = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        run_reference(args, dims, ws, rank)
        return
    if args.propagator:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps(propagator_bench(dims, max(3, min(args.steps, 20)))), flush=True)
        return
    if args.observables:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps(observables_bench(dims, max(3, min(args.steps, 20)))), flush=True)
        return

    import numpy as np
    import torch

    from flue_gb300 import _lib, generate
    from flue_gb300.field import GaugeField, _ptr, workspace

    wsz, rank, local = dist_setup(args)
    L = _lib.load()
    dev = torch.device("cuda", local if wsz > 1 else 0)
    stream = torch.cuda.current_stream()
    sh = ctypes.c_void_p(stream.cuda_stream)

    # --- fields (per rank: its own replica, seed offset by rank) ---
    f64 = generate.random_field(dims, args.eps, args.seed + rank, device=dev)
    f32 = GaugeField.from_array(f64, prec=args.prec)

    def prep(f):
        w = workspace(_lib.OP_MAGNETIC_FORCE, f).clone()
        out = torch.empty(1, dtype=torch.float64, device=dev)
        force = torch.empty((3, 3, 4, nz, ny, nx, nt), dtype=f.compute_dtype, device=dev)
        return f.descriptor(), w, out, force

    d32, w32, b32, g32 = prep(f32)

    def step32():
        rc = L.flue_magnetic_force(ctypes.byref(d32), _ptr(b32), _ptr(g32), _lib.FORCE_LIE, _ptr(w32), w32.numel(), sh)
        if rc:
            raise RuntimeError(L.flue_last_error_detail().decode())

    for _ in range(args.warmup):
        step32()
    torch.cuda.synchronize()
    barrier(wsz)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        n_launch0 = L.flue_kernel_launches()
        e0.record()
        for _ in range(args.steps):
            step32()
        e1.record()
        n_launches = L.flue_kernel_launches() - n_launch0
        torch.cuda.synchronize()
    barrier(wsz)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(wsz, ms)
    value = wsz * V / (ms * 1e-3)

    # --- per-stage timing of one step (CUDA events between the launches; with
    # stage timing on, the library runs the step as one pass over the lattice,
    # not as time slabs on several streams) ---
    L.flue_stage_timing(1)
    stage_ms = {k: 0.0 for k in ("lines", "fwd", "linecot", "linkcot")}
    nrep = min(10, args.steps)
    for _ in range(nrep):
        step32()
        buf = (ctypes.c_double * 8)()
        n = ctypes.c_int()
        L.flue_stage_times(buf, 8, ctypes.byref(n))
        for k, name in enumerate(("lines", "fwd", "linecot", "linkcot")[: n.value]):
            stage_ms[name] += buf[k] / nrep
    L.flue_stage_timing(0)
    torch.cuda.synchronize()

    # --- forward only: B^2 without the gradient, the reference's magnetic()
    # (src/wloops.F90:479-544) -- what the reference arm times ---
    def fwd32():
        rc = L.flue_magnetic(ctypes.byref(d32), _ptr(b32), _ptr(w32), w32.numel(), sh)
        if rc:
            raise RuntimeError(L.flue_last_error_detail().decode())

    for _ in range(2):
        fwd32()
    torch.cuda.synchronize()
    nfwd = max(3, min(args.steps, 20))
    e0.record()
    for _ in range(nfwd):
        fwd32()
    e1.record()
    torch.cuda.synchronize()
    ms_fwd = max_over_ranks(wsz, e0.elapsed_time(e1) / nfwd)

    # --- FP64 (complex128) GPU kernels: the denominator of the FP32 speed-up ---
    d64, w64, b64, g64 = prep(f64)

    def step64():
        rc = L.flue_magnetic_force(ctypes.byref(d64), _ptr(b64), _ptr(g64), _lib.FORCE_LIE, _ptr(w64), w64.numel(), sh)
        if rc:
            raise RuntimeError(L.flue_last_error_detail().decode())

    step64()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.fp64_steps):
        step64()
    e1.record()
    torch.cuda.synchronize()
    ms64 = max_over_ranks(wsz, e0.elapsed_time(e1) / args.fp64_steps)
    value64 = wsz * V / (ms64 * 1e-3)

    # FP64 forward only: the reference's magnetic() at the reference's own
    # precision -- the like-for-like GPU counterpart of the CPU figures
    def fwd64():
        rc = L.flue_magnetic(ctypes.byref(d64), _ptr(b64), _ptr(w64), w64.numel(), sh)
        if rc:
            raise RuntimeError(L.flue_last_error_detail().decode())

    fwd64()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.fp64_steps):
        fwd64()
    e1.record()
    torch.cuda.synchronize()
    ms_fwd64 = max_over_ranks(wsz, e0.elapsed_time(e1) / args.fp64_steps)

    # --- FP32 error against the FP64 result on the same field ---
    step32()
    torch.cuda.synchronize()
    B32, B64 = b32.item(), b64.item()
    rel_b = abs(B32 - B64) / abs(B64)
    gdiff = torch.linalg.vector_norm((g32.to(torch.complex128) - g64).flatten()).item()
    gnorm = torch.linalg.vector_norm(g64.flatten()).item()
    rel_g = gdiff / gnorm
    gmax = ((g32.to(torch.complex128) - g64).abs().max() / g64.abs().max()).item()
    del w64, g64
    torch.cuda.empty_cache()

    # --- end to end through the host-buffer C ABI (pinned host buffers): the
    # field in the reference's own data type (complex128, Fortran order, as
    # its readers produce it) in, FP32 compute in the bench precision, the
    # complex128 gradient out; and the same with a complex64 host field ---
    prec_code = {"r12": _lib.R12, "c64": _lib.C64}[args.prec]
    hb = ctypes.c_double()

    def e2e_leg(host_dtype, dtype_code):
        host_in = f64.to_tensor(host_dtype).permute(6, 5, 4, 3, 2, 1, 0).contiguous().cpu().pin_memory()
        host_grad = torch.empty_like(host_in).pin_memory()

        def e2e_step():
            rc = L.flue_magnetic_force_c(ctypes.c_void_p(host_in.data_ptr()), dtype_code, nt, nx, ny, nz, prec_code,
                                         _lib.FORCE_LIE, ctypes.byref(hb), ctypes.c_void_p(host_grad.data_ptr()))
            if rc:
                raise RuntimeError(L.flue_last_error_detail().decode())

        for _ in range(3):
            e2e_step()
        barrier(wsz)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        e2e_s = max_over_ranks(wsz, (time.perf_counter() - t0) / args.e2e_steps)
        L.flue_release_host_cache()
        nbytes = host_in.numel() * host_in.element_size()
        del host_in, host_grad
        return e2e_s, nbytes

    e2e_s, h2d = e2e_leg(torch.complex128, _lib.C128)
    e2e_val = wsz * V / e2e_s
    e2e64_s, h2d64 = e2e_leg(torch.complex64, _lib.C64)

    def link_bytes(esz):
        # what crosses the host link per call: B^2 reads the spatial links
        # (their stored rows: 2 of 3 for reconstruct-12) and writes the
        # spatial gradient; host threads write the zero time-direction part
        rows = 2 if args.prec == "r12" else 3
        return {"h2d": 3 * rows * 3 * V * esz, "d2h": 27 * V * esz,
                "note": "spatial links (stored rows) in, spatial gradient out; the zero time-direction gradient "
                        "is written into the caller's buffer by host threads"}

    # --- CPU baseline (rank 0, N = 1 only) ---
    cpu = None
    cpu_b2 = None
    if rank == 0 and wsz == 1 and not args.no_cpu:
        import oracle

        oracle.build()
        cpu = cpu_baseline(dims, args.eps, args.seed, args.cpu_seconds)

    # --- roofline ---
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    alg_bytes = ALG_BYTES[args.prec] * V
    achieved_gbs = alg_bytes / (ms * 1e-3) / 1e9 / wsz * wsz  # per GPU
    achieved_gbs = ALG_BYTES[args.prec] * V / (ms * 1e-3) / 1e9
    clk = clk.summary()
    sm_mhz = clk["sm_mhz"] or 1900.0
    # FP32 CUDA-core peak at the sampled clock: SMs x 128 lanes x 2 flop
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak_tflops = sm_count * 128 * 2 * sm_mhz * 1e6 / 1e12
    lc_ms = stage_ms["linecot"] or ms
    lc_flops = PRODUCTS_PER_SITE["linecot"] * FLOP_PER_PRODUCT * V
    lc_tflops = lc_flops / (lc_ms * 1e-3) / 1e12
    step_flops = sum(PRODUCTS_PER_SITE.values()) * FLOP_PER_PRODUCT * V
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "sites/s",
        "n_gpus": wsz,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": bench_config(args, dims, wsz),
        "fp64": {"value": value64, "unit": "sites/s", "ms_per_step": ms64, "steps": args.fp64_steps},
        "fp32_over_fp64": value / value64,
        "fp32_error_vs_fp64": {"b2_rel": rel_b, "grad_rel_l2": rel_g, "grad_rel_max": gmax, "b2_fp64": B64},
        "stages_ms": stage_ms,
        "forward_only": {"value": wsz * V / (ms_fwd * 1e-3), "unit": "sites/s", "ms_per_step": ms_fwd,
                         "steps": nfwd, "what": "flue_magnetic: B^2 without the gradient (the reference's magnetic)"},
        "forward_only_fp64": {"value": wsz * V / (ms_fwd64 * 1e-3), "unit": "sites/s", "ms_per_step": ms_fwd64,
                              "steps": args.fp64_steps,
                              "what": "flue_magnetic on the complex128 field: the reference's magnetic() at its own "
                                      "precision, the same work as the CPU figures"},
        "gpu_launches": int(n_launches),
        "e2e": {"value": e2e_val, "unit": "sites/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d + 8,
                "s_per_step": e2e_s, "host_link_bytes_per_step": link_bytes(16),
                "api": f"flue_magnetic_force_c (host complex128 field in, {args.prec} FP32 compute, host complex128 "
                       "gradient out)"},
        "e2e_c64": {"value": wsz * V / e2e64_s, "unit": "sites/s", "h2d_bytes_per_step": h2d64,
                    "d2h_bytes_per_step": h2d64 + 8, "s_per_step": e2e64_s, "host_link_bytes_per_step": link_bytes(8),
                    "api": f"flue_magnetic_force_c (host complex64 field in, {args.prec} FP32 compute, host "
                           "complex64 gradient out)"},
        "roofline": {"bound": "hbm", "kernel": "whole fwd+bwd step (metric's %HBM)", "achieved": achieved_gbs,
                     "peak": hbm_peak, "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
                     "traffic": step_traffic(args.prec, dims),
                     "peak_source": peak_src, "alg_bytes_per_site": ALG_BYTES[args.prec]},
        "compute_roofline": {"bound": "fp32_cuda_core", "kernel": "k_linecot (line cotangents)",
                             "achieved": lc_tflops, "peak": fp32_peak_tflops, "unit": "TFLOP/s",
                             "frac": lc_tflops / fp32_peak_tflops,
                             "step_tflops": step_flops / (ms * 1e-3) / 1e12,
                             "peak_basis": f"{sm_count} SM x 128 FP32 lanes x 2 flop x median sampled SM clock"},
        "sm_count": sm_count,
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    if args.ensemble and rank == 0:
        del f64, f32, d32, w32, g32
        torch.cuda.empty_cache()
        line["ensemble"] = ensemble_bench(max(3, min(args.steps, 10)))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if wsz > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
