"""The reference's post-processing program read_flow-1.2.f90 as a host tool:
read a case directory's control.in (Ma, line 2), Mesh2d.dat, bc2d_1.in and
flow2d.dat, and write Cp.dat, the wall pressure coefficient of every wall
subface (read_flow-1.2.f90:24-51).

What it keeps from the program, on purpose:
* gamma is the program's own constant 1.4 (read_flow-1.2.f90:10), not the
  case's, in p_inf = 1/(gamma Ma^2);
* the pressure is the p column of flow2d.dat (written F20.10), taken at the
  cell centres (x1, p)(i, j) over the subface's node index range
  ist..iend x jst..jend, so the last entry of a wall's range is the ghost
  cell beyond its end, as in the program;
* one zone per wall subface (neighb = -10), "zone i=" the entry count.

  python -m ec2d.read_flow <case_dir>
"""
from __future__ import annotations

import argparse
import os

from . import inputs, outputs

GAMMA = 1.4  # read_flow-1.2.f90:10
BC_WALL = -10


def cp_zones(directory: str):
    """Per wall subface (in block, subface order) the list of (x1, Cp)."""
    p = inputs.read_control(os.path.join(directory, "control.in"))
    xy = inputs.read_mesh(os.path.join(directory, "Mesh2d.dat"))
    bcs = inputs.read_bc(os.path.join(directory, "bc2d_1.in"))
    if len(bcs) != len(xy):
        raise ValueError("Block number in bc2d.in is not equal to that in Mesh2d.dat")
    zones = outputs._zones(os.path.join(directory, "flow2d.dat"), 7)
    p00 = 1.0 / (GAMMA * p.Ma * p.Ma)
    out = []
    for (x, _), subs, (ni, nj, rows) in zip(xy, bcs, zones):
        nx, ny = x.shape
        if (ni, nj) != (nx + 1, ny + 1):
            raise ValueError(f"flow2d.dat zone {ni}x{nj} does not match block {nx}x{ny}")
        for s in subs:
            if s[6] != BC_WALL:
                continue
            ist, iend, jst, jend = s[2], s[3], s[4], s[5]
            zone = []
            for j in range(jst, jend + 1):
                for i in range(ist, iend + 1):
                    r = rows[j * ni + i]  # records over i = 0..nx fastest, j = 0..ny
                    zone.append((r[0], -(r[6] - p00) * 2.0))
            out.append(zone)
    return out


def write_cp(directory: str) -> str:
    path = os.path.join(directory, "Cp.dat")
    with open(path, "w") as fh:
        fh.write(" variable=x,Cp\n")
        for zone in cp_zones(directory):
            fh.write(f" zone i= {len(zone):11d}\n")
            for x1, cp in zone:
                fh.write(f" {x1:.17g} {cp:.17g}\n")
    return path


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("case_dir", nargs="?", default=".")
    print(write_cp(ap.parse_args().case_dir))


if __name__ == "__main__":
    main()
