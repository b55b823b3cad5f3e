"""Tecplot output of a solved case in the reference's own files (host side).

`output` (opencfd_ec2d_v1.5.4.f90:284-371) writes, per mesh level,
flow2d.dat (variables x, y, d, u, v, T, p, Amut over i = 0..nx, j = 0..ny of
every block, format 8F20.10), on the fine mesh also flow2d-<Kstep>.dat (the
same without Amut, 7F20.10), and SA2d.dat / SST2d.dat with the turbulence
variables.  The arrays come from the device through the C-ABI
(ec2d_download_U, ec2d_get_field); the formatting is plain host work.
"""
from __future__ import annotations

import os
from typing import List, Sequence

import numpy as np


def primitives(U, gamma: float, Ma: float):
    """d, u, v, T, p from conservative U (Cv = 1/(gamma (gamma-1) Ma^2),
    p = d T / (gamma Ma^2), as in `output`)."""
    Cv = 1.0 / (gamma * (gamma - 1.0) * Ma * Ma)
    d = U[0]
    u = U[1] / d
    v = U[2] / d
    T = (U[3] - 0.5 * d * (u * u + v * v)) / (Cv * d)
    p = d * T / (gamma * Ma * Ma)
    return d, u, v, T, p


def _zone_lines(cols, nx: int, ny: int, fmt: str) -> List[str]:
    out = [f"  zone i= {nx + 1:11d} j= {ny + 1:11d}\n"]
    # i fastest over 0..nx, then j over 0..ny (the arrays start at index -1)
    for j in range(1, ny + 2):
        for i in range(1, nx + 2):
            out.append("".join(fmt.format(c[i, j]) for c in cols) + "\n")
    return out


def format_blocks(blocks: Sequence[dict], gamma: float, Ma: float, Re: float, with_amut: bool = True) -> str:
    """Text of flow2d.dat for blocks given as dicts with nx, ny and arrays on
    the index range -1..nx+1, -1..ny+1: U (nvar, nx+3, ny+3), x1, y1, amut
    (nx+3, ny+3)."""
    head = " variables=x,y,d,u,v,T,p,Amut\n" if with_amut else " variables=x,y,d,u,v,T,p\n"
    lines = [head]
    for b in blocks:
        d, u, v, T, p = primitives(b["U"], gamma, Ma)
        cols = [b["x1"], b["y1"], d, u, v, T, p]
        if with_amut:
            cols.append(b["amut"] * Re)
        lines += _zone_lines(cols, b["nx"], b["ny"], "{:20.10f}")
    return "".join(lines)


def format_turbulence(blocks: Sequence[dict]) -> str:
    """SA2d.dat (x, y, vt) or SST2d.dat (x, y, Kt, Wt) text, by the variable count."""
    nv = blocks[0]["U"].shape[0]
    lines = [" variables=x,y,vt\n" if nv == 5 else " variables=x,y,Kt,Wt\n"]
    for b in blocks:
        cols = [b["x1"], b["y1"]] + [b["U"][m] for m in range(4, nv)]
        lines += _zone_lines(cols, b["nx"], b["ny"], "{:20.10f}")
    return "".join(lines)


def read_blocks(solver, case: int = 1, mesh: int = 1) -> List[dict]:
    """U, x1, y1, mu_t of every block of a case from the device."""
    out = []
    b = 1
    while True:
        try:
            nx, ny, nv = solver.dims(case, mesh, b)
        except Exception:
            break
        shp = (nx + 3, ny + 3)
        out.append({"nx": nx, "ny": ny, "U": solver.download_U(case, mesh, b),
                    "x1": solver.field(case, mesh, b, 9, shp), "y1": solver.field(case, mesh, b, 10, shp),
                    "amut": solver.field(case, mesh, b, 8, shp)})
        b += 1
    return out


def write_output(directory: str, solver, params, case: int = 1, mesh: int = 1, kstep: int = 0) -> List[str]:
    """The files `output(nMesh)` writes; returns their paths."""
    blocks = read_blocks(solver, case, mesh)
    paths = []
    name = "flow2d.dat" if mesh == 1 else f"flow2d-{mesh:1d}.dat"
    if mesh == 1:
        path = os.path.join(directory, f"flow2d-{kstep:07d}.dat")
        with open(path, "w") as fh:
            fh.write(format_blocks(blocks, params.gamma, params.Ma, params.Re, with_amut=False))
        paths.append(path)
    path = os.path.join(directory, name)
    with open(path, "w") as fh:
        fh.write(format_blocks(blocks, params.gamma, params.Ma, params.Re, with_amut=True))
    paths.append(path)
    nv = blocks[0]["U"].shape[0]
    if nv in (5, 6):
        path = os.path.join(directory, "SA2d.dat" if nv == 5 else "SST2d.dat")
        with open(path, "w") as fh:
            fh.write(format_turbulence(blocks))
        paths.append(path)
    return paths


def parse_tecplot(text: str):
    """(variable names, [zone arrays (npoints, nvar)]) of a file written above."""
    lines = text.splitlines()
    names = lines[0].split("=", 1)[1].strip().split(",")
    zones, k = [], 1
    while k < len(lines):
        parts = lines[k].split()
        ni, nj = int(parts[2]), int(parts[4])
        rows = [[float(t) for t in lines[k + 1 + r].split()] for r in range(ni * nj)]
        zones.append(np.array(rows))
        k += 1 + ni * nj
    return names, zones
