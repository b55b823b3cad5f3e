"""Generates tests/golden/converged.json: converged-answer fixtures of the CPU
oracle (the C++ restatement of the reference, test infrastructure) on two of
the benchmark workloads, for the converged-answer parity tests and the bench's
parity record.

* flat_plate: the laminar flat plate (2-block 193x97 H-grid, 3-level V-cycle
  with LU-SGS smoothing, FP64) run from the freestream start until the
  continuity RMS residual Res_rms(1) is at most 1e-8 times its first-iteration
  value, checked every 25 V-cycles as ec2d_run_to_drop checks it.  Recorded:
  the V-cycle count, the residual history at every check, CL/CD/CM and the
  wall skin friction of every wall face.
* naca0012_euler: the inviscid NACA 0012 C-grid (257x65, M 0.8, AoA 1.25,
  Roe + MUSCL van Albada, single-grid LU-SGS, CFL 5), which does not reach a
  steady state with the reference discretisation: CL swings between about
  -0.5 and 0.9 from a few thousand steps on, and near step 13,200 a
  temperature below 1e-5 stops the run (the reference's STOP,
  sub_Residual.f90:143-146).  Recorded: CL, CD, CM and Res_rms(1) every 20
  steps up to 13,000 steps, and where the run stops.

The oracle is built with the parity flags of oracle/Makefile; its results do
not depend on the thread count (no reductions run in parallel).

  python tests/golden/make_converged.py [--threads 8]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "opencfd-ec2d_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

OUT = os.path.join(HERE, "converged.json")


def flat_plate(threads, check=25, target=1e-8, cap=200000):
    import oracle
    from ec2d import cases
    p, blocks = cases.laminar_flat_plate(97, 97, num_mesh=3)
    orc = oracle.Oracle(p, blocks, threads=threads)
    orc.init_flow()
    t0 = time.perf_counter()
    orc.step(1)
    r0 = orc.norms()[1][0]
    it, hist = 1, [r0]
    while hist[-1] > target * r0 and it < cap:
        orc.step(check)
        it += check
        hist.append(orc.norms()[1][0])
    secs = time.perf_counter() - t0
    cl, cd, cm = orc.forces()
    cf, xc = orc.wall_cf(2, 2)
    return {"workload": "laminar flat plate, 2 x 97x97 blocks, 3-level V-cycle, LU-SGS smoothing, FP64",
            "case": "cases.laminar_flat_plate(97, 97, num_mesh=3)", "target": target, "check_every": check,
            "iterations": it, "r0": r0, "history_res_rms1": hist, "reached": bool(hist[-1] <= target * r0),
            "forces": {"cl": cl, "cd": cd, "cm": cm}, "wall": {"block": 2, "sub": 2, "cf": list(cf), "xc": list(xc)},
            "oracle_seconds": secs, "oracle_threads": threads}


def naca0012_euler(threads, steps=13000, every=20, stop_probe=1000):
    import oracle
    from ec2d import cases
    p, blocks = cases.euler_naca0012()
    orc = oracle.Oracle(p, blocks, threads=threads)
    orc.init_flow()
    rec = {"step": [], "cl": [], "cd": [], "cm": [], "res_rms1": []}
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        orc.step(every)
        done += every
        cl, cd, cm = orc.forces()
        rec["step"].append(done)
        rec["cl"].append(cl)
        rec["cd"].append(cd)
        rec["cm"].append(cm)
        rec["res_rms1"].append(orc.norms()[1][0])
    secs = time.perf_counter() - t0
    stop = None
    try:  # where the T < 1e-5 stop comes
        for _ in range(stop_probe):
            orc.step(1)
            done += 1
    except RuntimeError as e:
        stop = {"step": done + 1, "error": str(e)}
    return {"workload": "Euler NACA 0012 C-grid 257x65, M 0.8, AoA 1.25, Roe + MUSCL van Albada, LU-SGS, CFL 5",
            "case": "cases.euler_naca0012()", "steps": steps, "every": every, "record": rec, "stop": stop,
            "oracle_seconds": secs, "oracle_threads": threads}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    import oracle
    oracle.build()
    out = {"generator": "tests/golden/make_converged.py", "oracle_flags": "oracle/Makefile (parity build)",
           "flat_plate": flat_plate(args.threads), "naca0012_euler": naca0012_euler(args.threads)}
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=0)
    fp = out["flat_plate"]
    print(f"flat plate: {fp['iterations']} V-cycles to {fp['target']:g} ({fp['oracle_seconds']:.1f} s), "
          f"CL {fp['forces']['cl']:.12e} CD {fp['forces']['cd']:.12e} CM {fp['forces']['cm']:.12e}")
    print(f"naca0012: {out['naca0012_euler']['oracle_seconds']:.1f} s, stop {out['naca0012_euler']['stop']}")


if __name__ == "__main__":
    main()
