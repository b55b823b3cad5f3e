"""The reference main program (opencfd_ec2d_v1.5.4.f90:142-186) as a Python
host over the C-ABI: read the case directory, hand it to the library, march
until t_end (or a step count), print and record the residuals every
Kstep_show steps and write the flow files every Kstep_save steps and at the
end.  SA and SST runs take the wall distance from the case's dist_wall.dat,
or write it there (and dw.dat) from the distances formed on the device.

The flow files at Kstep_save come from asynchronous snapshots
(ec2d_snapshot): the library copies U to pinned host memory on a stream of
its own while the steps go on, and the files of a snapshot are written once
the next snapshot is taken or the run ends, so the marching does not wait for
the device-to-host copy.

With a tuning cache (--tuning-cache FILE, or the EC2D_TUNING_CACHE
environment variable) the launch choices of the autotuner are taken from the
file when this case's launch signature is stored there, and otherwise timed
once and added to it (ec2d/tuning.py); without one the library's default
choices are used.

  python -m ec2d.driver <case_dir> [--steps N] [--fix-nvar-restart] [--tuning-cache FILE]
"""
from __future__ import annotations

import argparse
import os
import time
import warnings

from . import gpu, inputs, outputs, tuning


def read_fdm(directory: str):
    """Block numbers listed in FDM.in (sub_Finite_Difference.f90:287-308):
    four comment lines, the count, one more line, one block per line."""
    path = os.path.join(directory, "FDM.in")
    if not os.path.exists(path):
        return []
    lines = open(path).read().splitlines()
    n = int(lines[4].split()[0])
    return [int(lines[6 + k].split()[0]) for k in range(n)]


def read_wall_distance(directory: str, p, dims):
    """The distances of the case's dist_wall.dat for an SA or SST run, or
    None: for the other models, without the file, or (with a warning) for a
    file written for another mesh or cut short, whose distances are then
    formed anew and the file rewritten.  The reference would read such a
    file into the mesh's blocks as it stands."""
    if p.Iflag_turbulence_model not in (inputs.TURB_SA, inputs.TURB_SST):
        return None
    path = os.path.join(directory, "dist_wall.dat")
    if not os.path.exists(path):
        return None
    try:
        return inputs.read_dist_wall(path, dims)
    except ValueError as e:
        warnings.warn(f"{e}; the wall distances are formed anew")
        return None


def write_wall_distance(solver, directory: str, dims) -> None:
    """dist_wall.dat and dw.dat from the distances the library formed on the
    device (comput_dw writes both when it had to compute them,
    sub_turbulence_SST.f90:342-362)."""
    dws, cells = [], []
    for k, (nx, ny) in enumerate(dims, start=1):
        dw = solver.field(1, 1, k, gpu.F_DW, shape=(nx + 1, ny + 1))[1:nx, 1:ny]
        x1 = solver.field(1, 1, k, gpu.F_X1, shape=(nx + 3, ny + 3))[2:nx + 1, 2:ny + 1]
        y1 = solver.field(1, 1, k, gpu.F_Y1, shape=(nx + 3, ny + 3))[2:nx + 1, 2:ny + 1]
        dws.append(dw)
        cells.append((x1, y1, dw))
    inputs.write_dist_wall(os.path.join(directory, "dist_wall.dat"), dws, dims)
    inputs.write_dw_tecplot(os.path.join(directory, "dw.dat"), cells)


def run(directory: str, steps: int = None, device: int = 0, fix_nvar: bool = False, quiet: bool = False,
        tuning_cache: str = None) -> dict:
    p, blocks = inputs.read_case(directory)
    fdm = read_fdm(directory)
    # the wall distance of SA and SST runs (comput_dw,
    # opencfd_ec2d_v1.5.4.f90:164): read from dist_wall.dat where the case
    # directory has one, else formed on the device and written there
    dims = [(b.nx, b.ny) for b in blocks]
    turbulent = p.Iflag_turbulence_model in (inputs.TURB_SA, inputs.TURB_SST)
    dw = read_wall_distance(directory, p, dims)
    s = gpu.Solver([(p, blocks)], device=device, fdm_blocks=[fdm], dw=None if dw is None else [dw])
    if turbulent and dw is None:
        write_wall_distance(s, directory, dims)
    if p.Iflag_init == 0:
        s.init_flow()
    else:
        outputs.restart(s, directory, fix_nvar=fix_nvar)
    tuned = None
    if tuning_cache or os.environ.get(tuning.ENV):
        # the autotuner restores U and the step counters it advances
        tuned = tuning.autotune_cached(s, tuning_cache)
    geometry = outputs.read_blocks(s)  # x1, y1 (constant) for the snapshot files
    res_path = os.path.join(directory, "Residual.dat")
    pending, written, done, tt, kstep = None, [], 0, 0.0, 0
    t0 = time.perf_counter()
    while tt < p.t_end and (steps is None or done < steps):
        s.step(1)
        done += 1
        rmax, rrms, kstep, tt = s.norms()
        if kstep % max(1, p.Kstep_show) == 0:  # output_Res(1)
            if not quiet:
                print(f" Kstep, t= {kstep} {tt}  Res_rms(1:{p.nvar()}) = {rrms[:p.nvar()]}")
            with open(res_path, "a") as fh:
                fh.write(inputs.residual_record(kstep, rmax, rrms, p.nvar()))
        if kstep % max(1, p.Kstep_save) == 0:  # output(1), from a snapshot
            if pending is not None:
                written += outputs.write_output(directory, s, p, kstep=pending,
                                                blocks=outputs.snapshot_blocks(s, geometry))
            s.snapshot(1)
            pending = kstep
    if pending is not None:
        written += outputs.write_output(directory, s, p, kstep=pending, blocks=outputs.snapshot_blocks(s, geometry))
    written += outputs.write_output(directory, s, p, kstep=kstep)  # the final output(1)
    forces = s.forces(1)
    s.close()
    return {"steps": done, "kstep": kstep, "tt": tt, "seconds": time.perf_counter() - t0, "files": written,
            "forces": forces, "tuning": tuned}


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("case_dir")
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--fix-nvar-restart", action="store_true",
                    help="read SST2d.dat for 6-variable states on restart (the reference tests NVAR == 5)")
    ap.add_argument("--tuning-cache", default=None,
                    help="JSON file of autotuner results keyed by launch signature (read, and extended on a miss)")
    a = ap.parse_args()
    r = run(a.case_dir, a.steps, a.device, a.fix_nvar_restart, tuning_cache=a.tuning_cache)
    print(f"steps {r['steps']} Kstep {r['kstep']} tt {r['tt']} ({r['seconds']:.2f} s); CL CD CM {r['forces']}")


if __name__ == "__main__":
    main()
