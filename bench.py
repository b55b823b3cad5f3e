#!/usr/bin/env python
"""Benchmark of the GB300-native OpenCFD-EC2D pseudo-time-marching core.

Workload (one GPU): the laminar flat plate -- 2-block 193x97 H-grid (two
97x97 blocks, 18,432 cells), first cell 1e-4 with ratio 1.1, M 0.3,
Re 1e4, adiabatic wall, AUSM+ with MUSCL (van Albada), 3-level V-cycle with
LU-SGS smoothing.  A "step" is one main-loop iteration (one V-cycle).
Metric: cell-updates/s = fine cells x iterations / time (coarse-level work is
not counted as extra updates), plus the time to a 1e-8 drop of the
continuity RMS residual from the freestream start.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) each rank runs an independent replica (the path has no
data exchange); value = all ranks' cell-updates / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "opencfd-ec2d_gb300")
for _p in (PKG, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "time-to-1e-8 residual drop/case & cell-updates/s, learned+batched vs plain"
UNIT = "cell-updates/s"
WORKLOAD = ("laminar flat plate, 2-block 193x97 H-grid (18432 cells), M 0.3, Re 1e4, adiabatic wall, "
            "AUSM+ + MUSCL van Albada, 3-level V-cycle with LU-SGS smoothing, FP64")
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0

# Algorithmic bytes per unit (cell or face of the fine level) of each kernel,
# laminar Navier-Stokes, NV = 4 (8-byte words read once + written once):
#   k_prim    read U(4), write d,u,v,T,p,c, mu, mu_t                  = 12 w
#   k_flux_i  read d,u,v,p,T, mu, mu_t, x1, y1, s, n1, n2; write F(4) = 16 w
#   k_flux_j  same as k_flux_i                                        = 16 w
#   k_res     read Fi(4), Fj(4), vol, si, sj, ni1, ni2, nj1, nj2,
#             d, u, v, c, mu, mu_t; write Res(4), Lci, Lcj, Lvi, Lvj, dt = 30 w
#   k_lusgs   read Res(4), U(4), dt, vol, Lci, Lcj, Lvi, Lvj, si, sj,
#             ni1, ni2, nj1, nj2; dU written, re-read and rewritten (12) = 32 w
#   k_add_du  read U(4), dU(4), write U(4)                            = 12 w
BYTES_PER_UNIT = {"k_prim": 96, "k_flux_i": 128, "k_flux_j": 128, "k_res": 240, "k_lusgs": 256, "k_add_du": 96}


def peaks():
    try:
        with open(PEAKS) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1])); mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].strip() == "Active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_case():
    from ec2d import cases
    p, blocks = cases.laminar_flat_plate(97, 97, num_mesh=3)
    return p, blocks


def fine_cells(blocks):
    return sum(b.ncell for b in blocks)


def cpu_port_rate(p, blocks, seconds=12.0, threads=None):
    """Cell-updates/s of the CPU port (C++ restatement of the reference, the
    only CPU implementation runnable here) on all host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    threads = threads or os.cpu_count()
    os.environ.setdefault("OMP_WAIT_POLICY", "passive")
    orc = oracle.Oracle(p, blocks, threads=threads)
    orc.init_flow()
    orc.step(2)
    t0 = time.perf_counter(); orc.step(1); t1 = time.perf_counter() - t0
    n = max(1, min(2000, int(seconds / max(t1, 1e-6))))
    t0 = time.perf_counter(); orc.step(n); dt = time.perf_counter() - t0
    return fine_cells(blocks) * n / dt, threads, n, dt


def run_reference(args, rank, world):
    """--impl reference: the CPU restatement of the reference timed on the
    host cores (no Fortran compiler exists here or on the GPU machine, so the
    reference itself cannot run; the port is its stand-in)."""
    if rank != 0:
        return
    p, blocks = build_case()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    os.environ.setdefault("OMP_WAIT_POLICY", "passive")
    threads = os.cpu_count()
    orc = oracle.Oracle(p, blocks, threads=threads)
    orc.init_flow()
    orc.step(max(1, args.warmup))
    t0 = time.perf_counter()
    orc.step(args.steps)
    dt = time.perf_counter() - t0
    cells = fine_cells(blocks)
    v = cells * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": cells, "step": "one 3-level V-cycle"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} V-cycles after {args.warmup} warm-up cycles"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_to_drop(g, cells, cap_s=30.0, check=25, target=1e-8):
    """Iterations and wall time from the freestream start until the
    continuity RMS residual drops below target x its first-iteration value."""
    g.init_flow()
    g.sync()
    t0 = time.perf_counter()
    g.step(1)
    r0 = g.norms()[1][0]
    it, r = 1, r0
    while r > target * r0 and time.perf_counter() - t0 < cap_s:
        g.step(check)
        it += check
        r = g.norms()[1][0]
    dt = time.perf_counter() - t0
    return {"iterations": it, "seconds": dt, "drop": r / r0, "reached": bool(r <= target * r0),
            "cell_updates_per_s": cells * it / dt}


def run_gb300(args, rank, world):
    import numpy as np
    import torch
    from ec2d import gpu

    dev = int(os.environ.get("LOCAL_RANK", "0")) if world > 1 else 0
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    p, blocks = build_case()
    cells = fine_cells(blocks)
    g = gpu.Solver([(p, blocks)], device=dev)
    g.init_flow()
    stream = torch.cuda.ExternalStream(g.stream_handle())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    for _ in range(max(3, args.warmup)):
        g.step(1)
    g.sync()

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-timed region: K V-cycles, L2 flushed before each ----------
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    n0 = g.launch_count()
    barrier()
    with ClockSampler(dev) as clk:
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ev[k][0].record(stream)
            g.step(1)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    barrier()
    launches = (g.launch_count() - n0) // args.steps
    ms = sum(a.elapsed_time(b) for a, b in ev)
    clocks = clk.summary()
    if dist is not None:
        t = torch.tensor([ms], device=f"cuda:{dev}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = cells * args.steps * world / (ms / 1e3)

    # ---- per-kernel event timing (same K cycles, separate pass) -----------
    g.kernel_timing(True)
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        g.step(1)
    kt = g.kernel_times()
    g.kernel_timing(False)
    hbm, peak_kind = peaks()
    best = max(kt.items(), key=lambda kv: kv[1][2])
    (kname, klev), (kcalls, knk, kms) = best
    lv_cells = sum(((b.nx - 1) // (2 ** (klev - 1))) * ((b.ny - 1) // (2 ** (klev - 1))) for b in blocks)
    if kname in ("k_flux_i",):
        units = sum(((b.nx - 1) // 2 ** (klev - 1) + 1) * ((b.ny - 1) // 2 ** (klev - 1)) for b in blocks)
    elif kname in ("k_flux_j",):
        units = sum(((b.nx - 1) // 2 ** (klev - 1)) * ((b.ny - 1) // 2 ** (klev - 1) + 1) for b in blocks)
    else:
        units = lv_cells
    bpu = BYTES_PER_UNIT.get(kname, 0)
    avg_ms = kms / kcalls
    achieved = bpu * units / (avg_ms / 1e3) / 1e9 if bpu else None
    roofline = {"bound": "hbm", "kernel": f"{kname} (mesh {klev})", "achieved": achieved, "peak": hbm,
                "unit": "GB/s", "frac": (achieved / hbm) if achieved else None, "traffic": None,
                "peak_source": f"{peak_kind} hbm_gbs", "avg_launch_us": avg_ms * 1e3,
                "bytes_per_launch": bpu * units,
                "share_of_step": kms / sum(v[2] for v in kt.values()),
                "kernels": {f"{n}@{l}": {"calls": c, "ms_total": round(m, 4)} for (n, l), (c, _, m) in
                            sorted(kt.items(), key=lambda kv: -kv[1][2])[:12]}}

    # ---- end to end through the C-ABI with host buffers --------------------
    nbl = len(blocks)
    host = []
    h2d = 0
    for b in range(1, nbl + 1):
        U = g.download_U(1, 1, b)
        pin = torch.empty(U.size, dtype=torch.float64, pin_memory=True)
        arr = pin.numpy().reshape(U.shape, order="F")
        arr[...] = U
        host.append((pin, arr))
        h2d += U.nbytes
    d2h = 12 * 8 + 4 * 4
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        for b in range(1, nbl + 1):
            g.upload_U(1, 1, b, host[b - 1][1])
        g.step(1)
        g.norms(1, 1)
    t_e2e = time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([t_e2e], device=f"cuda:{dev}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    e2e = {"value": cells * args.steps * world / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}

    ttd = time_to_drop(g, cells, cap_s=args.drop_cap) if args.drop_cap > 0 else None
    cl, cd, cm = g.forces(1)

    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            rate, thr, n, dt = cpu_port_rate(p, blocks, seconds=args.cpu_seconds)
            cpu = {"value": rate, "unit": UNIT, "cores": thr, "kind": "port",
                   "sample": f"{n} V-cycles of the same workload ({dt:.1f} s) on the C++ restatement"}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "cells": cells, "step": "one 3-level V-cycle",
                           "l2": "flushed before every timed step (512 MiB write)", "parallelism": f"replicas{world}"},
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
                "gpu_launches": launches * args.steps, "launches_per_step": launches,
                "time_to_drop": ttd, "forces": {"cl": cl, "cd": cd, "cm": cm}}
        print(json.dumps(line), flush=True)
    g.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--drop-cap", type=float, default=30.0)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gb300(args, rank, world)


if __name__ == "__main__":
    main()
