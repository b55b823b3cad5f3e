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
#   k_residual_tile  the residual stage in one kernel: read U(4), 7 metrics,
#             x1, y1 (viscous inverse Jacobians counted as the metrics);
#             write Res(4), Lci, Lcj, Lvi, Lvj, dt                    = 22 w
BYTES_PER_UNIT = {"k_prim": 96, "k_flux_i": 128, "k_flux_j": 128, "k_res": 240, "k_lusgs": 256, "k_add_du": 96,
                  "k_residual_tile": 176}


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


def thread_counts():
    n = os.cpu_count() or 1
    return sorted({t for t in (1, 2, 4, 8, n) if t <= n}), n


def best_threads(oracle, p, blocks, trials=4, fast=False):
    """Thread count at which a CPU build runs this workload fastest.  On the
    18,432-cell flat plate its OpenMP regions are short, so all host cores
    are not the fastest setting (measured on the 16-core Arm host: 7.5 ms
    per V-cycle on 4 threads, 12.5 ms on 16)."""
    best = None
    for th in thread_counts()[0]:
        orc = oracle.Oracle(p, blocks, threads=th, fast=fast)
        orc.init_flow()
        orc.step(2)
        t0 = time.perf_counter(); orc.step(trials); dt = time.perf_counter() - t0
        if best is None or dt < best[1]:
            best = (th, dt)
    return best[0]


def cpu_port_rates(p, blocks, seconds=16.0):
    """Cell-updates/s of the CPU timing port (the C++ restatement of the
    reference built -O3 with FMA contraction, the stand-in for gfortran -O3
    -fopenmp on the reference, whose Fortran cannot be compiled here) on 1
    thread, on every host core, and on the counts between; each count runs
    for about seconds / (number of counts).  Returns the fastest count's
    rate, that count, and the rate of every count."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    counts, ncores = thread_counts()
    per = seconds / len(counts)
    by, best = {}, None
    for th in counts:
        orc = oracle.Oracle(p, blocks, threads=th, fast=True)
        orc.init_flow()
        orc.step(2)
        t0 = time.perf_counter(); orc.step(2); t1 = (time.perf_counter() - t0) / 2
        n = max(5, min(2000, int(per / max(t1, 1e-6))))
        t0 = time.perf_counter(); orc.step(n); dt = time.perf_counter() - t0
        rate = fine_cells(blocks) * n / dt
        by[str(th)] = {"value": rate, "seconds_per_step": dt / n, "steps": n}
        if best is None or rate > best[1]:
            best = (th, rate)
    return best[1], best[0], by, ncores


def parity_record(p, blocks, gpu_hist, gpu_iters, gpu_forces, gpu_cf, mixed_forces=None, check=25, target=1e-8):
    """The oracle (parity build, FP64, separately rounded like the reference)
    run from the freestream start to the same residual drop, checked every
    `check` V-cycles as the GPU run was: V-cycle counts, the differences of
    CL, CD, CM and of every wall face's skin friction, and the largest
    relative difference of the Res_rms(1) histories at the common checks."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    th = best_threads(oracle, p, blocks)
    orc = oracle.Oracle(p, blocks, threads=th)
    orc.init_flow()
    t0 = time.perf_counter()
    orc.step(1)
    r0 = orc.norms()[1][0]
    hist, it = [r0], 1
    while hist[-1] > target * r0 and it < 4 * gpu_iters:
        orc.step(check)
        it += check
        hist.append(orc.norms()[1][0])
    secs = time.perf_counter() - t0
    cl, cd, cm = orc.forces()
    cf, _ = orc.wall_cf(2, 2)
    n = min(len(hist), len(gpu_hist))
    h_o, h_g = np.array(hist[:n]), np.array(gpu_hist[:n])
    rec = {"oracle": "C++ restatement of the reference, parity build (-O2, no FMA contraction)",
           "oracle_threads": th, "oracle_seconds": secs, "target": target, "check_every": check,
           "iterations_oracle": it, "iterations_gpu": gpu_iters,
           "forces_oracle": {"cl": cl, "cd": cd, "cm": cm},
           "dcl": gpu_forces[0] - cl, "dcd": gpu_forces[1] - cd, "dcm": gpu_forces[2] - cm,
           "max_dcf": float(np.max(np.abs(np.asarray(gpu_cf) - cf))), "max_cf": float(np.max(np.abs(cf))),
           "history_max_rel": float(np.max(np.abs(h_g - h_o) / h_o)), "history_points": n,
           "bar": "|dCL|, |dCD|, |dCM| <= 1e-6 and Res_rms(1) history within 1e-6 relative"}
    rec["within_1e-6"] = bool(max(abs(rec["dcl"]), abs(rec["dcd"]), abs(rec["dcm"])) <= 1e-6
                              and rec["history_max_rel"] <= 1e-6 and it == gpu_iters)
    if mixed_forces is not None:
        rec["mixed_vs_oracle"] = {"dcl": mixed_forces[0] - cl, "dcd": mixed_forces[1] - cd,
                                  "dcm": mixed_forces[2] - cm}
    return rec


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path on the host cores.  No
    Fortran compiler exists here or on the GPU host, so the reference itself
    cannot run; its stand-in is the C++ restatement built like gfortran -O3
    -fopenmp would build it (the timing port), at its fastest thread count,
    with the 1-thread and all-core rates beside it."""
    if rank != 0:
        return
    p, blocks = build_case()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cells = fine_cells(blocks)
    best, threads, by, ncores = cpu_port_rates(p, blocks, seconds=args.cpu_seconds)
    orc = oracle.Oracle(p, blocks, threads=threads, fast=True)
    orc.init_flow()
    orc.step(max(1, args.warmup))
    t0 = time.perf_counter()
    orc.step(args.steps)
    dt = time.perf_counter() - t0
    v = cells * args.steps / dt
    ttd = None
    if args.drop_cap > 0:
        # the same freestream-start drop as the GPU arm, bounded by 2x the cap
        cap = 2.0 * args.drop_cap
        orc.init_flow()
        t0 = time.perf_counter()
        orc.step(1)
        r0 = orc.norms()[1][0]
        it, r = 1, r0
        while r > 1e-8 * r0 and time.perf_counter() - t0 < cap:
            orc.step(25)
            it += 25
            r = orc.norms()[1][0]
        tdrop = time.perf_counter() - t0
        cl, cd, cm = orc.forces()
        ttd = {"fp64": {"target": 1e-8, "iterations": it, "seconds": tdrop, "drop": r / r0,
                        "reached": bool(r <= 1e-8 * r0), "cap_s": cap, "forces": {"cl": cl, "cd": cd, "cm": cm}}}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": cells, "step": "one 3-level V-cycle"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port-O3",
                             "host_cores": ncores, "by_cores": by,
                             "sample": f"{args.steps} V-cycles after {args.warmup} warm-up cycles, "
                                       f"{threads} of {ncores} host threads (fastest count)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "time_to_drop": ttd}
    print(json.dumps(line), flush=True)


def time_to_drop(g, cells, cap_s=60.0, target=1e-8, check=25):
    """Iterations and wall time from the freestream start until the
    continuity RMS residual drops below target x its first-iteration value,
    through the library's own iterate-to-drop call (ec2d_run_to_drop)."""
    g.init_flow()
    g.sync()
    t0 = time.perf_counter()
    it, ratio, _ = g.run_to_drop(drop=target, max_seconds=cap_s, check_every=check)
    dt = time.perf_counter() - t0
    return {"target": target, "iterations": it, "seconds": dt, "drop": ratio, "reached": bool(ratio <= target),
            "cell_updates_per_s": cells * it / dt, "cap_s": cap_s}


# DRAM bytes per launch of the dominant kernel on this workload, from one
# ncu capture of the default wavefront (k_lusgs_sweep_quad<1, 8>) on the fine
# level (dram__bytes_read.sum + dram__bytes_write.sum, caches flushed before
# the launch; the run is in the profiling summaries of the repo)
PROFILED_TRAFFIC = {("k_lusgs", 1): 7426816.0}
# FP64 work per fine cell of one laminar residual evaluation (k_prim,
# k_flux_i, k_flux_j, k_res; AUSM+, MUSCL van Albada, primitive
# reconstruction) on the 4.19 M-cell grid, from one ncu capture of those
# kernels (thread instructions executed / cells): FLOPs = dadd + dmul +
# 2 dfma, instructions = dadd + dmul + dfma.  Every FP64 instruction takes
# one issue slot of the FP64 pipe, whose rate is half the FMA FLOP rate.
FP64_PER_CELL_RESIDUAL = {"chain": (966.1, 689.9), "tile": (None, None)}
SWEEP_PLANES = lambda blocks, lev: 2 * max((b.nx - 1) // 2 ** (lev - 1) + (b.ny - 1) // 2 ** (lev - 1) - 1
                                         for b in blocks)


def timed_steps(torch, g, stream, flush, steps):
    """K steps, each bracketed by CUDA events on the solver's stream, with a
    512 MiB L2 flush before each.  Returns total ms and launches per step."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    n0 = g.launch_count()
    for k in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        ev[k][0].record(stream)
        g.step(1)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev), (g.launch_count() - n0) // steps


def kernel_table(g, torch, flush, steps):
    """Per-kernel CUDA-event times of `steps` steps (launched one by one)."""
    g.kernel_timing(True)
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        g.step(1)
    kt = g.kernel_times()
    g.kernel_timing(False)
    return kt


def merge_lusgs(kt):
    """With kernel timing on, the FP64 wavefront's record builder and sweep
    are timed apart (k_lusgs_prep, k_lusgs_sweep); fold them back into the
    k_lusgs stage in place and return the sweep's (calls, ms) per level."""
    sweep = {}
    for (name, lev) in list(kt):
        if name == "k_lusgs_sweep":
            c, nk, ms = kt.pop((name, lev))
            pc, pnk, pms = kt.pop(("k_lusgs_prep", lev), (0, 0, 0.0))
            sweep[lev] = (c, ms)
            kt[("k_lusgs", lev)] = (c, nk + pnk, ms + pms)
    return sweep


def residual_hbm(torch, gpu, dev, reps=10, forms=("chain", "tile"), grid=(2049, 1025), transfer_reps=10):
    """Residual evaluation (Comput_Residual_one_mesh) on a grid far larger
    than L2: 2 blocks of 2049x1025 nodes (4.19 M cells; `grid` sets another
    size, e.g. a small one for instruction counts), laminar flat-plate
    physics, a perturbed state, in both forms: the four-kernel chain through
    HBM planes and the one kernel over shared-memory tiles.  Achieved =
    algorithmic bytes of the residual (176 B per cell: read U, 7 metrics, x1,
    y1; write Res, dt and the 4 spectral radii) / CUDA-event time of the whole
    residual stage; the FP64 roofline beside it (the bound on this part) from
    the FP64 instructions each form executes per cell."""
    import numpy as np
    from ec2d import cases, grids
    p, _ = cases.laminar_flat_plate(33, 33, num_mesh=1)
    blocks = grids.flat_plate(grid[0], grid[1], first=1.0e-4, ratio=1.0065)
    cells = fine_cells(blocks)
    g = gpu.Solver([(p, blocks)], device=dev)
    g.init_flow()
    rng = np.random.default_rng(7)
    for b in range(1, len(blocks) + 1):
        U = g.download_U(1, 1, b)
        U *= 1.0 + 0.01 * rng.standard_normal(U.shape[1:])[None]
        g.upload_U(1, 1, b, U)
    g.bc()
    hbm, kind = peaks()
    try:
        fp64_peak = gpu.measure_fp64_peak()
    except Exception:
        fp64_peak = None
    out = {"cells": cells, "grid": f"2 x {grid[0]}x{grid[1]} (flat plate, {cells / 1e6:.2f} M cells)",
           "algorithmic_bytes_per_cell": 176,
           "peak_gbs": hbm, "peak_source": f"{kind} hbm_gbs", "fp64_peak_tflops": fp64_peak,
           "fp64_peak_source": "measured in this run (ec2d_measure_fp64_peak: FMA chains on every SM)"}
    for form in forms:
        g.tile_residual(1 if form == "tile" else 0)
        for _ in range(2):
            g.residual()
        g.sync()
        g.kernel_timing(True)
        for _ in range(reps):
            g.residual()
        kt = g.kernel_times()
        g.kernel_timing(False)
        total_ms = sum(v[2] for v in kt.values()) / reps
        achieved = 176.0 * cells / (total_ms / 1e3) / 1e9
        per = {}
        for (name, lev), (calls, _, ms) in kt.items():
            bpu = BYTES_PER_UNIT.get(name)
            t = ms / calls
            per[name] = {"us": round(t * 1e3, 1), "gbs": round(bpu * cells / (t / 1e3) / 1e9, 1) if bpu else None}
        r = {"ms": total_ms, "achieved_gbs": achieved, "frac": achieved / hbm, "hbm_frac": achieved / hbm,
             "kernels": per}
        flops_pc, inst_pc = FP64_PER_CELL_RESIDUAL.get(form, (None, None))
        if fp64_peak and flops_pc:
            # FP64 roofline: the FP64 pipe issues one instruction (dadd, dmul or
            # dfma) per slot at half the measured FMA FLOP rate
            r.update({"bound": "fp64", "fp64_flops_per_cell": flops_pc, "fp64_inst_per_cell": inst_pc,
                      "fp64_tflops": flops_pc * cells / (total_ms / 1e3) / 1e12,
                      "fp64_frac": flops_pc * cells / (total_ms / 1e3) / 1e12 / fp64_peak,
                      "fp64_issue_frac": inst_pc * cells / (total_ms / 1e3) / 1e12 / (fp64_peak / 2.0)})
        out[form] = r
    g.close()
    out["transfers"] = transfer_hbm(torch, gpu, dev, p, blocks, hbm, reps=transfer_reps)
    # the headline fields: the faster form
    best = min(forms, key=lambda f: out[f]["ms"])
    out["form"] = best
    for k in ("ms", "achieved_gbs", "frac", "hbm_frac", "bound", "fp64_tflops", "fp64_frac", "fp64_issue_frac"):
        if k in out[best]:
            out[k] = out[best][k]
    out["note"] = ("FP64 instruction issue bounds this stage: fp64_issue_frac = FP64 instructions per second / the "
                   "FP64 pipe's instruction rate (measured FMA FLOP/s / 2); fp64_frac counts FLOPs, where a dadd or "
                   "dmul is one FLOP in one issue slot")
    return out


def transfer_hbm(torch, gpu, dev, p, blocks, hbm, reps=10):
    """The multigrid transfers on the same 4.19 M-cell grid with a second
    level, each launched through its C-ABI hook (interpolation2h, prolong_U)
    and timed with CUDA events on the library's stream.  Algorithmic bytes:
    the volume-weighted restriction of U (flag 1; per coarse cell read 4 fine
    cells' U and volumes and the coarse volume, write U: 200); the
    restriction of the residual (flag 2; read 4 fine Res, write QF: 160); the
    cycle's forcing (flag 6; also read the coarse Res: 192); the
    prolongation of U (flag 1; per fine cell write U, read a quarter of a
    coarse cell's U: 40); the cycle's correction (flag 3; per fine cell read
    and write U, write deltU, read a quarter of a coarse cell's U and Un:
    112)."""
    g = gpu.Solver([(p.replace(Num_Mesh=2), blocks)], device=dev)
    g.init_flow()
    g.residual(1)
    g.sync()
    st = torch.cuda.ExternalStream(g.stream_handle())
    fine = fine_cells(blocks)
    coarse = sum(((b.nx - 1) // 2) * ((b.ny - 1) // 2) for b in blocks)
    out = {}
    for name, call, nbytes in (("k_restrict U", lambda: g.interpolation2h(1, 2, 1), 200.0 * coarse),
                               ("k_restrict Res", lambda: g.interpolation2h(1, 2, 2), 160.0 * coarse),
                               ("k_restrict QF (cycle)", lambda: g.interpolation2h(1, 2, 6), 192.0 * coarse),
                               ("k_prolong U", lambda: g.prolong(2, 1, 1), 40.0 * fine),
                               ("k_prolong U-Un (cycle)", lambda: g.prolong(2, 1, 3), 112.0 * fine)):
        call()
        g.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            call()
        e1.record(st)
        e1.synchronize()
        us = e0.elapsed_time(e1) / reps * 1e3
        gbs = nbytes / (us * 1e-6) / 1e9
        out[name] = {"us": round(us, 1), "algorithmic_bytes": nbytes, "gbs": round(gbs, 1), "hbm_frac": gbs / hbm}
    g.close()
    out["note"] = f"back-to-back launches; the fine level is {fine / 1e6:.2f} M cells"
    return out


def plain_step_ms(torch, gpu, pc, steps=10, mg_amut=False):
    """Milliseconds per V-cycle of every case as the plain drop-in: one
    context per case, FP64 LU-SGS, the step graph replayed, CUDA events on
    the context's stream after three warm-up V-cycles."""
    out = []
    for case in pc:
        g = gpu.Solver([case[:2]])
        if mg_amut:
            g.mg_eddy_viscosity(1)
        st = torch.cuda.ExternalStream(g.stream_handle())
        g.init_flow()
        g.step(3)
        g.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        g.step(steps)
        e1.record(st)
        e1.synchronize()
        out.append(e0.elapsed_time(e1) / steps)
        g.close()
    return out


def polar_metric(args, torch, gpu):
    """The metric's comparison on the 64-case polar (SA RANS cases from a
    seed: M in [0.3, 0.8], AoA in [-2, 8] deg, Re in [1e6, 1e7], t/c in [0.09,
    0.15], 257x65 to 513x129, 1-4 blocks, 3-level V-cycle, LU-SGS):

    * plain: the GPU drop-in, one case per context, FP64.  Its time to a
      drop D for case c is that case's V-cycles to D times its own ms per
      V-cycle (plain_step_ms).  The V-cycle counts come from the FP64 batch
      (one launch per stage covers every case; cases never read each
      other's data); a lone case runs the eight-lane wavefront, the batch's
      150 blocks the one-lane one, so the two differ in the wavefront's
      summation order only.
    * batched_mixed: all 64 cases in one context, FP32 LU-SGS (FP64
      residual, boundary conditions, transfers, norms), freestream start.
    * learned_batched_mixed: the same from the warm-start network's
      prediction (inference inside the timed region), the network trained
      in this run on fields the solver generated (learned leg, below); a
      case whose residual blows up within its first 200 V-cycles restarts
      from the freestream (the fallback).

    Every context of the comparison (the plain per-case timings included)
    keeps the restricted eddy viscosity on its coarse levels
    (ec2d_mg_eddy_viscosity; off with --no-polar-mg-eddy-viscosity): with the
    reference's laminar coarse levels the LU-SGS V-cycle diverges on some
    turbulent cases (7 of 64 within the cap from the freestream) and on most
    warm starts, on the oracle as on the GPU.

    Every run is capped at args.polar_cap seconds; residuals are checked
    every 25 V-cycles.  The batched arms retire a case when it reaches the
    comparison drop (args.polar_drop) or diverges, and move the others into
    a smaller context once a quarter of the batch has left.  For each drop D
    the comparison uses the cases that reached D in both arms: plain time =
    the sum of their plain times (one context after the other), batched time
    = the wall time until the last of them reached D."""
    import numpy as np
    from ec2d import cases, learn
    pc = cases.polar_cases(64, with_tc=True)
    cells = sum(fine_cells(bl) for _, bl, _ in pc)
    # the FP64 batch gives the plain per-case V-cycle counts and runs every
    # case to the cap (its reached counts show how deep the family gets); the
    # batched arms retire a case at the comparison drop and move the rest
    # into a smaller context as cases finish (or diverge)
    targets = (1e-2, 1e-3, 1e-4, 1e-6, 1e-8)
    drop = args.polar_drop
    arm_targets = tuple(t for t in targets if t >= drop)
    out = {"cases": len(pc), "cells": cells, "cap_s": args.polar_cap, "check_every": 25,
           "targets": [f"{t:.0e}" for t in targets], "comparison_drop": f"{drop:.0e}"}
    net, learned = None, None
    if args.polar_learned:
        net, learned = learned_leg(args, gpu)
        out["learned_training"] = learned
    t0 = time.perf_counter()
    mg = args.polar_mg_amut
    out["mg_eddy_viscosity"] = bool(mg)
    fp64 = learn.converge(gpu, pc, "freestream", 64, targets=targets, max_steps=10 ** 6, check=25,
                          max_seconds=args.polar_cap, mg_amut=mg)
    r0 = fp64["r0"]
    arms = {"batched_fp64": fp64,
            "batched_mixed": learn.converge(gpu, pc, "freestream", 32, r0=r0, targets=arm_targets,
                                            max_steps=10 ** 6, check=25, max_seconds=args.polar_cap, retire=drop,
                                            mg_amut=mg)}
    if net is not None:
        arms["learned_batched_mixed"] = learn.converge(gpu, pc, "warm", 32, r0=r0, net=net, targets=arm_targets,
                                                       max_steps=10 ** 6, check=25, max_seconds=args.polar_cap,
                                                       retire=drop, mg_amut=mg)
        net.close()
    plain_ms = plain_step_ms(torch, gpu, pc, mg_amut=mg)
    out["plain_ms_per_vcycle"] = {"median": float(np.median(plain_ms)), "min": float(np.min(plain_ms)),
                                  "max": float(np.max(plain_ms)), "sum": float(np.sum(plain_ms))}
    for name, r in arms.items():
        out[name] = {"reached": {k: v["reached"] for k, v in r["targets"].items()}, "vcycles": r["steps"],
                     "seconds": r["seconds"], "ms_per_vcycle": r["seconds"] / max(r["steps"], 1) * 1e3,
                     "diverged": r["diverged"], "start_seconds": r["start_seconds"],
                     "setup_seconds": r["setup_seconds"], "download_seconds": r["download_seconds"],
                     "warm_start_fallback_cases": r["fallback"],
                     "restarted_from_freestream": r["restarted_from_freestream"],
                     "context_moves": r["context_moves"]}
    plain_first = fp64["first"]
    comp = {}
    for t in arm_targets:
        key = f"{t:.0e}"
        ok_plain = plain_first[t] >= 0
        row = {"plain_reached": int(ok_plain.sum())}
        for name in [n for n in arms if n != "batched_fp64"]:
            r = arms[name]
            both = ok_plain & (r["first"][t] >= 0)
            if not both.any():
                row[name] = {"common_cases": 0}
                continue
            plain_s = float(np.sum(np.array(plain_ms)[both] * plain_first[t][both]) / 1e3)
            batch_s = float(np.max(r["when"][t][both]))
            e2e_s = batch_s + r["setup_seconds"] + r["download_seconds"]
            row[name] = {"reached": int((r["first"][t] >= 0).sum()), "common_cases": int(both.sum()),
                         "plain_seconds": plain_s, "batched_seconds": batch_s, "speedup": plain_s / batch_s,
                         "e2e_seconds": e2e_s, "e2e_speedup": plain_s / e2e_s}
        comp[key] = row
    out["comparison"] = comp
    # the headline: for the learned and for the freestream batch, the deepest
    # drop that at least a quarter of the cases reached in the plain run and
    # in that batch
    out["headline"] = None
    for head in ("learned_batched_mixed", "batched_mixed"):
        best = None
        for t in arm_targets:
            row = comp[f"{t:.0e}"].get(head, {})
            if row.get("common_cases", 0) >= len(pc) // 4:
                best = {"drop": f"{t:.0e}", "arm": head, **row}
        out[f"headline_{head}"] = best
    out["headline"] = out["headline_learned_batched_mixed"] or out["headline_batched_mixed"]
    out["seconds"] = time.perf_counter() - t0
    out["unit"] = "wall seconds to the drop for the cases both arms reached"
    return out


def learned_leg(args, gpu):
    """The warm-start network of the polar comparison: args.ws_train SA cases
    of the learned family (257x65 C-grid, the polar box, seed 20261203) solved
    in batches in FP32 LU-SGS from the freestream until every case's drop
    reached args.ws_gen_target, or its plateau, or args.ws_gen_steps steps,
    or args.ws_gen_cap seconds per batch; then args.ws_train_steps Adam steps
    on all their cells.  Dataset generation and training are reported here
    and are not part of the time-to-drop comparison."""
    import numpy as np
    from ec2d import learn
    train_cases = learn.warmstart_cases(args.ws_train, seed=20261203)
    net = gpu.WarmStartNet(hidden=6, width=256, seed=1)
    gen = learn.generate(gpu, net, train_cases, steps=args.ws_gen_steps, target=args.ws_gen_target,
                         max_seconds=args.ws_gen_cap)
    tr = learn.train(net, steps=args.ws_train_steps)
    drops = np.array(gen.pop("drops"))
    gen["drops_quartiles"] = [float(x) for x in np.quantile(drops[np.isfinite(drops)], [0.25, 0.5, 0.75])]
    return net, {"network": "6 hidden layers x 256, SiLU, BF16 weights/activations, FP32 accumulate",
                 "generate": gen, "train": tr}


def leg_polar(args):
    """The batched polar, as the default run reports it."""
    import torch
    from ec2d import gpu
    return polar_metric(args, torch, gpu)


def leg_mlp(args):
    """Training-step throughput of the warm-start network (6 hidden layers of
    256, batch 16,384) with the tcgen05 GEMM kernels and with the mma.sync
    ones.  Samples: one 257x65 SA case after 50 steps (the values do not
    change the work).  Algorithmic FLOPs of a step: forward 2 B (7x256 +
    5x256^2 + 256x5), backward twice that less the input-gradient product of
    the first layer."""
    from ec2d import gpu, learn
    case = learn.warmstart_cases(1, seed=5)
    s = gpu.Solver([(case[0][0], case[0][1])])
    s.init_flow()
    s.step(50)
    B, steps = 16384, max(args.steps, 50)
    fwd = 2.0 * B * (7 * 256 + 5 * 256 * 256 + 256 * 5)
    flops = fwd + 2.0 * fwd - 2.0 * B * 7 * 256
    out = {"batch": B, "hidden": "6 x 256", "algorithmic_gflop_per_step": flops / 1e9}
    hbm_peak, _ = peaks()
    try:
        with open(PEAKS) as fh:
            bf16 = float(json.load(fh)["bf16_tflops"])
    except Exception:
        bf16 = 1900.0
    for kind, name in ((1, "tcgen05"), (0, "mma_sync")):
        net = gpu.WarmStartNet(hidden=6, width=256, seed=1)
        net.set_gemm(kind)
        net.add_samples(s)
        net.fit_normalization()
        net.train(20, batch=B)
        t0 = time.perf_counter()
        loss = net.train(steps, batch=B)
        dt = (time.perf_counter() - t0) / steps
        out[name] = {"ms_per_step": dt * 1e3, "tflops": flops / dt / 1e12, "frac_of_bf16_peak": flops / dt / 1e12 / bf16,
                     "loss": loss}
        net.close()
    s.close()
    out["bf16_peak_tflops"] = bf16
    return out


def leg_rans(args):
    """The RANS workload (4-block 513x129 NACA 2412, M 0.73, AoA 2.8,
    Re 6.5e6, Roe, MUSCL3, WENO5 patch on every block, 3-level V-cycle,
    LU-SGS, FP64) with SA and with SST, each with the reference's laminar
    coarse levels and with the coarse eddy viscosity kept: ms per V-cycle
    (20 V-cycles after 20, CUDA graphs, CUDA events on the context's
    stream) and per kernel (10 V-cycles with per-kernel event timing)."""
    import torch
    from ec2d import cases, gpu
    out = {}
    for turb, name in ((2, "sa"), (3, "sst")):
        p, bl, fdm = cases.rans_naca2412(turb=turb)
        for amut in (0, 1):
            g = gpu.Solver([(p, bl)], fdm_blocks=[fdm])
            g.mg_eddy_viscosity(amut)
            g.init_flow()
            g.step(20)
            g.sync()
            st = torch.cuda.ExternalStream(g.stream_handle())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            g.step(20)
            e1.record(st)
            e1.synchronize()
            g.kernel_timing(True)
            g.step(10)
            kt = g.kernel_times()
            g.kernel_timing(False)
            out[f"{name}{'_mg_eddy_viscosity' if amut else ''}"] = {
                "ms_per_vcycle": e0.elapsed_time(e1) / 20,
                "kernels_ms_per_vcycle": {f"{n}@{l}": round(v[2] / 10, 4)
                                          for (n, l), v in sorted(kt.items(), key=lambda kv: -kv[1][2])[:12]},
                "cells": fine_cells(bl), "lusgs_shape": g.lusgs_shape()}
            g.close()
    return out


def leg_fp64(args):
    """The FP64 cost model of the latency-bound kernels: clock64 cycles per
    dependent operation per warp (ec2d_measure_op_cycles) for FP64 fma, the
    FP64 divide, the refined FP64 reciprocal of the face and wavefront paths
    and FP32 fma, with 1-8 warps in one CTA and 1-8 independent chains per
    thread; and the FP64 FMA throughput of the whole GPU."""
    from ec2d import gpu
    ops = {0: "fp64_fma", 1: "fp64_divide", 2: "fp64_refined_reciprocal", 3: "fp32_fma"}
    shapes = [(1, 1), (1, 2), (1, 4), (1, 8), (2, 1), (4, 1), (4, 4), (8, 1)]
    out = {"unit": "clock64 cycles per operation and warp", "shapes": "warps x independent chains per thread"}
    for op, name in ops.items():
        out[name] = {f"{w}x{c}": round(gpu.measure_op_cycles(op, w, c), 2) for w, c in shapes}
    out["cta_barrier_cycles"] = {f"{w} warps": round(gpu.measure_op_cycles(4, w, 1), 1) for w in (1, 3, 8)}
    out["cluster_barrier_cycles"] = {f"{c} CTAs": round(gpu.measure_op_cycles(5, 1, c), 1) for c in (2, 4, 8)}
    rel, ulps = gpu.check_reciprocal(40_000_000)
    out["reciprocal"] = {"inputs": 40_000_000, "range": "[2^-8, 2^9)", "approx_max_rel_err": rel,
                         "refined_max_ulps_from_ieee_quotient": ulps}
    out["fp64_peak_tflops"] = gpu.measure_fp64_peak()
    return out


def leg_learned(args):
    """Learned warm start (512 training + 64 held-out SA cases on a 257x65
    C-grid): data generation, training, and the held-out polar to a 1e-8 drop
    -- warm-started, batched, FP32 LU-SGS against the freestream start and the
    plain drop-in (one case per context, FP64)."""
    from ec2d import gpu, learn
    train_cases = learn.warmstart_cases(args.ws_train, seed=20261203)
    held = learn.warmstart_cases(args.ws_held, seed=20261204)
    net = gpu.WarmStartNet(hidden=6, width=256, seed=1)
    gen = learn.generate(gpu, net, train_cases, steps=args.ws_gen_steps, target=args.ws_gen_target,
                         max_seconds=args.ws_gen_cap)
    tr = learn.train(net, steps=args.ws_train_steps)
    ev = learn.evaluate(gpu, net, held, targets=(1e-4, 1e-6, args.ws_target), max_steps=args.ws_max_steps,
                        plain_sample=args.ws_plain)
    net.close()
    return {"network": "6 hidden layers x 256, SiLU, BF16 weights/activations, FP32 accumulate",
            "generate": gen, "train": tr, "evaluate": ev}


def reduce_max(dist, x: float, device: str) -> float:
    """The slowest rank's time: every rank of a replica run gets the maximum
    of x over all ranks (x itself without a process group)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, steps: int, world: int, ms: float) -> float:
    """Whole-job rate: all ranks' units x steps over the slowest rank's time."""
    return units_per_rank * steps * world / (ms / 1e3)


def run_gb300(args, rank, world):
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
    g.set_lusgs_precision(64)
    g.init_flow()
    stream = torch.cuda.ExternalStream(g.stream_handle())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    for _ in range(max(3, args.warmup)):
        g.step(1)
    g.sync()
    tune = (lambda: g.autotune(3)) if args.autotune else (lambda: (0, 12, 1, None))

    def shape(t):
        # lusgs_ctas 0: bands of at most `rows` rows on a cluster, eight lanes
        # per row up to 16 rows, four above; 1: one CTA per block, `rows` rows
        # per warp; >1: a cluster of that many CTAs with a barrier per plane
        cs, rpw, cc, ms = t
        lanes = g.lusgs_shape()[2]
        kind = "one-lane" if cs != 0 else ("eight-lane bands" if lanes == 8 else "four-lane bands")
        return {"lusgs_kernel": kind, "lusgs_ctas": cs, "rows": rpw, "lanes": lanes if cs == 0 else 1,
                "concurrent_faces": cc, "ms": ms,
                "residual": "one kernel over shared-memory tiles" if g.tile_residual() else "four-kernel chain"}

    tuned = {"fp64": shape(tune())}

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        return reduce_max(dist, x, f"cuda:{dev}")

    # ---- device-timed region: K V-cycles (FP64), L2 flushed before each -----
    barrier()
    with ClockSampler(dev) as clk:
        ms, launches = timed_steps(torch, g, stream, flush, args.steps)
    barrier()
    clocks = clk.summary()
    ms = max_over_ranks(ms)
    value = aggregate_rate(cells, args.steps, world, ms)

    # ---- per-kernel event timing (same K cycles, separate pass) -------------
    kt = kernel_table(g, torch, flush, args.steps)
    sweep_ms = merge_lusgs(kt)
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
                "unit": "GB/s", "frac": (achieved / hbm) if achieved else None,
                "traffic": PROFILED_TRAFFIC.get((kname, klev)),
                "peak_source": f"{peak_kind} hbm_gbs (of {peak_kind})", "avg_launch_us": avg_ms * 1e3,
                "bytes_per_launch": bpu * units,
                "share_of_step": kms / sum(v[2] for v in kt.values()),
                "kernels": {f"{n}@{l}": {"calls": c, "ms_total": round(m, 4)} for (n, l), (c, _, m) in
                            sorted(kt.items(), key=lambda kv: -kv[1][2])[:12]}}
    if kname == "k_lusgs":
        # the wavefront is bound by the latency of its per-plane FP64 chain, not
        # by HBM: 2 (nx + ny - 3) dependent hyperplanes, each one cell update
        mhz = clocks.get("sm_mhz") or 2070.0
        planes = SWEEP_PLANES(blocks, klev)
        s_calls, s_ms = sweep_ms.get(klev, (kcalls, kms))
        cpp = s_ms / s_calls * 1e-3 * mhz * 1e6 / planes
        # the FP64 chain of one plane: 15 operations per cell and lane with
        # eight lanes per row, 18 with four, 31 per cell with one, 64 cycles each
        kind = tuned["fp64"]["lusgs_kernel"]
        floor = {"eight-lane bands": 15, "four-lane bands": 18}.get(kind, 31) * 64
        roofline["bound"] = "latency"
        roofline["hbm_frac"] = roofline["frac"]
        roofline["sweep_avg_launch_us"] = s_ms / s_calls * 1e3
        roofline["cycles_per_plane"] = cpp
        roofline["cycles_per_plane_incl_prep"] = avg_ms * 1e-3 * mhz * 1e6 / planes
        roofline["fp64_chain_floor_cycles_per_plane"] = floor
        roofline["of_chain_floor"] = floor / cpp
        roofline["latency_note"] = ("wavefront sweep: one dependent chain of FP64 operations per hyperplane, FP64 "
                                    "warp instruction latency 64 cycles on this part; cycles_per_plane = the sweep "
                                    "kernel's event time x SM clock / planes; of_chain_floor = the chain's cycles / "
                                    "cycles_per_plane; frac and hbm_frac = algorithmic bytes of prep + sweep "
                                    "(256 B/cell) / their time / measured HBM bandwidth")

    # ---- mixed precision: the same V-cycle with FP32 LU-SGS sweeps ----------
    g.set_lusgs_precision(32)
    for _ in range(3):
        g.step(1)
    g.sync()
    tuned["mixed"] = shape(tune())
    barrier()
    ms32, launches32 = timed_steps(torch, g, stream, flush, args.steps)
    barrier()
    ms32 = max_over_ranks(ms32)
    kt32 = kernel_table(g, torch, flush, args.steps)
    mixed = {"value": cells * args.steps * world / (ms32 / 1e3), "ms_per_step": ms32 / args.steps,
             "lusgs": "fp32", "residual": "fp64",
             "kernels": {f"{n}@{l}": round(m / args.steps, 4) for (n, l), (c, _, m) in
                         sorted(kt32.items(), key=lambda kv: -kv[1][2])[:8]}}
    g.set_lusgs_precision(64)
    tune()

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
    # each step from the host's U to the host's norms (wall clock), after the
    # same 512 MiB L2 flush as the device-timed steps, which stays outside
    t_e2e = 0.0
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for b in range(1, nbl + 1):
            g.upload_U(1, 1, b, host[b - 1][1])
        g.step(1)
        g.norms(1, 1)
        t_e2e += time.perf_counter() - t0
    t_e2e = max_over_ranks(t_e2e)
    e2e = {"value": cells * args.steps * world / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}

    # ---- time to a 1e-8 drop from the freestream start ----------------------
    ttd = None
    hist = None
    if args.drop_cap > 0:
        ttd = {"fp64": time_to_drop(g, cells, cap_s=args.drop_cap)}
        cl, cd, cm = g.forces(1)
        ttd["fp64"]["forces"] = {"cl": cl, "cd": cd, "cm": cm}
        cf_fp64, _ = g.wall_cf(1, 2, 2)
        g.set_lusgs_precision(32)
        tune()
        ttd["mixed"] = time_to_drop(g, cells, cap_s=args.drop_cap)
        cl2, cd2, cm2 = g.forces(1)
        ttd["mixed"]["forces"] = {"cl": cl2, "cd": cd2, "cm": cm2}
        ttd["mixed"]["force_error_vs_fp64"] = max(abs(cl2 - cl), abs(cd2 - cd), abs(cm2 - cm))
        g.set_lusgs_precision(64)
        tune()
        if rank == 0 and world == 1 and args.parity:
            # untimed: the FP64 residual history at every 25th V-cycle, the
            # checks of the run above, for the comparison with the oracle
            g.init_flow()
            g.step(1)
            r0 = g.norms(1, 1)[1][0]
            hist, it = [r0], 1
            while hist[-1] > 1e-8 * r0 and it < ttd["fp64"]["iterations"]:
                g.step(25)
                it += 25
                hist.append(g.norms(1, 1)[1][0])
    cl, cd, cm = g.forces(1)
    g.close()

    big = None
    if args.residual_hbm and rank == 0:
        big = residual_hbm(torch, gpu, dev)
    polar = None
    if args.polar and rank == 0 and world == 1:
        polar = polar_metric(args, torch, gpu)

    if rank == 0:
        cpu = None
        parity = None
        if world == 1 and not args.no_cpu_baseline:
            rate, thr, by, ncores = cpu_port_rates(p, blocks, seconds=args.cpu_seconds)
            cpu = {"value": rate, "unit": UNIT, "cores": thr, "kind": "port-O3", "host_cores": ncores,
                   "by_cores": by,
                   "sample": (f"V-cycles of the same workload on the C++ restatement built -O3 with FMA "
                              f"contraction, {args.cpu_seconds:.0f} s over 1..{ncores} threads; value at the "
                              f"fastest count ({thr})"),
                   "seconds_per_step": by[str(thr)]["seconds_per_step"]}
            if ttd and ttd["fp64"]["reached"]:
                cpu["time_to_drop_estimate_s"] = cpu["seconds_per_step"] * ttd["fp64"]["iterations"]
                cpu["time_to_drop_basis"] = ("CPU seconds per V-cycle x the V-cycles to the drop (the FP64 GPU "
                                             "run and the oracle need the same count, see parity)")
        if hist is not None:
            parity = parity_record(p, blocks, hist, ttd["fp64"]["iterations"],
                                   (ttd["fp64"]["forces"]["cl"], ttd["fp64"]["forces"]["cd"],
                                    ttd["fp64"]["forces"]["cm"]), cf_fp64,
                                   mixed_forces=(ttd["mixed"]["forces"]["cl"], ttd["mixed"]["forces"]["cd"],
                                                 ttd["mixed"]["forces"]["cm"]))
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "cells": cells, "step": "one 3-level V-cycle",
                           "l2": "flushed before every timed step (512 MiB write)", "parallelism": f"replicas{world}",
                           "autotuned": tuned},
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
                "gpu_launches": launches * args.steps, "launches_per_step": launches,
                "mixed_precision": mixed, "time_to_drop": ttd, "parity": parity, "residual_hbm": big,
                "polar": polar, "learned_batched_vs_plain": polar["headline"] if polar else None,
                "forces": {"cl": cl, "cd": cd, "cm": cm}}
        if polar:
            line["config"]["polar"] = (f"64 SA cases of the polar box (257x65..513x129, 1-4 blocks, 3-level "
                                       f"V-cycle), each run capped at {args.polar_cap:g} s; warm-start network "
                                       f"trained in this run on {args.ws_train} generated 257x65 fields")
        print(json.dumps(line), flush=True)
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
    ap.add_argument("--cpu-seconds", type=float, default=16.0,
                    help="seconds of the CPU timing port, spread over 1..all host threads")
    ap.add_argument("--no-parity", dest="parity", action="store_false",
                    help="skip the oracle run to the same drop (converged CL/CD/CM, Cf, residual history)")
    ap.add_argument("--drop-cap", type=float, default=60.0, help="seconds per time-to-drop run (0: skip)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default launch configuration (e.g. under a profiler, whose timing misleads it)")
    ap.add_argument("--no-residual-hbm", dest="residual_hbm", action="store_false",
                    help="skip the residual bandwidth measurement on the 4.19 M-cell grid")
    ap.add_argument("--no-polar-mg-eddy-viscosity", dest="polar_mg_amut", action="store_false",
                    help="polar runs with laminar coarse levels, as the reference (default: the coarse levels keep "
                         "the restricted eddy viscosity, which keeps the turbulent V-cycle from diverging)")
    ap.add_argument("--transfer-reps", type=int, default=10, help="timed launches per transfer form")
    ap.add_argument("--residual-grid", default="2049x1025",
                    help="nodes per block of the residual_hbm leg's 2-block flat plate (NXxNY)")
    ap.add_argument("--leg", default="all", choices=["all", "residual_hbm", "polar", "learned", "mlp", "rans", "fp64"],
                    help="residual_hbm: the 4.19 M-cell residual alone (for profiling); polar: the 64-case "
                         "batched polar; learned: the learned warm start end to end")
    ap.add_argument("--no-polar", dest="polar", action="store_false",
                    help="skip the 64-case polar comparison (learned+batched+mixed vs plain)")
    ap.add_argument("--polar-cap", type=float, default=20.0, help="seconds per polar run")
    ap.add_argument("--polar-drop", type=float, default=1e-3,
                    help="the drop the polar comparison is made at (batched cases retire there)")
    ap.add_argument("--no-polar-learned", dest="polar_learned", action="store_false",
                    help="polar comparison without the warm-start network")
    ap.add_argument("--ws-gen-target", type=float, default=1e-6)
    ap.add_argument("--ws-gen-cap", type=float, default=15.0, help="seconds per generation batch of 64 cases")
    ap.add_argument("--ws-train", type=int, default=64)
    ap.add_argument("--ws-held", type=int, default=64)
    ap.add_argument("--ws-gen-steps", type=int, default=30000)
    ap.add_argument("--ws-train-steps", type=int, default=2000)
    ap.add_argument("--ws-target", type=float, default=1e-8)
    ap.add_argument("--ws-max-steps", type=int, default=30000)
    ap.add_argument("--ws-plain", type=int, default=4, help="held-out cases also run one per context in FP64")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.leg != "all":
        import torch
        from ec2d import gpu
        if args.leg == "residual_hbm":
            out = residual_hbm(torch, gpu, 0, grid=tuple(int(v) for v in args.residual_grid.split("x")),
                               transfer_reps=args.transfer_reps)
        elif args.leg == "polar":
            out = leg_polar(args)
        elif args.leg == "mlp":
            out = leg_mlp(args)
        elif args.leg == "rans":
            out = leg_rans(args)
        elif args.leg == "fp64":
            out = leg_fp64(args)
        else:
            out = leg_learned(args)
        print(json.dumps({args.leg: out}, default=float), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gb300(args, rank, world)


if __name__ == "__main__":
    main()
