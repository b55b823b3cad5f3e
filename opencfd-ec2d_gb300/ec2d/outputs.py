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


def snapshot_blocks(solver, geometry: Sequence[dict]) -> List[dict]:
    """The blocks of the solver's last asynchronous snapshot (ec2d_snapshot)
    in the form of read_blocks; `geometry`: read_blocks' x1/y1 of the same
    case (constant, read once)."""
    out = []
    for b, g in enumerate(geometry, start=1):
        out.append({"nx": g["nx"], "ny": g["ny"], "U": solver.snapshot_U(b), "x1": g["x1"], "y1": g["y1"],
                    "amut": solver.snapshot_amut(b)})
    return out


def write_output(directory: str, solver, params, case: int = 1, mesh: int = 1, kstep: int = 0,
                 blocks: Sequence[dict] = None) -> List[str]:
    """The files `output(nMesh)` writes; returns their paths.  blocks: the
    data to write (read_blocks / snapshot_blocks), by default read from the
    device now."""
    if blocks is None:
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


class RestartError(RuntimeError):
    pass


def _zones(path: str, ncols: int):
    """The zones of a Tecplot file written by `output`: per zone (ni, nj) and
    the first `ncols` numbers of every record (list-directed reads take the
    leading values of a record)."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    zones, k = [], 1
    while k < len(lines):
        parts = lines[k].replace("=", " ").split()
        if not parts:
            k += 1
            continue
        ni, nj = int(parts[parts.index("i") + 1]), int(parts[parts.index("j") + 1])
        rows = np.array([[float(t) for t in lines[k + 1 + r].split()[:ncols]] for r in range(ni * nj)])
        zones.append((ni, nj, rows))
        k += 1 + ni * nj
    return zones


def read_flow(directory: str, params, dims: Sequence[tuple], fix_nvar: bool = False) -> List[np.ndarray]:
    """init_flow_read (sub_init.f90:499-560): the state of every block from
    flow2d.dat (d, u, v, T on i = 0..nx, j = 0..ny; U(4) = d Cv T +
    0.5 d (u^2 + v^2)) and the turbulence variables from SA2d.dat / SST2d.dat.

    dims: per block (nx, ny, nvar).  Returns U(NVAR,-1:nx+1,-1:ny+1) per
    block with the ring -1 / nx+1 left at zero; the caller uploads these over
    the freestream state and applies the boundary conditions and the halo, as
    init_flow_read ends.

    The reference reads the turbulence files under one condition, NVAR == 5,
    for both (sub_init.f90:523, 541): an SA restart then also reads
    SST2d.dat into U(5:6) of a 5-variable array, and an SST restart never
    reloads k and omega.  fix_nvar=False keeps that behaviour as far as it is
    defined: an SA restart raises RestartError where the reference would go on
    to read SST2d.dat, and an SST restart leaves U(5:6) as the caller's
    freestream.  fix_nvar=True reads SST2d.dat when NVAR == 6, as intended."""
    gamma, Ma = params.gamma, params.Ma
    Cv = 1.0 / (gamma * (gamma - 1.0) * Ma * Ma)
    zones = _zones(os.path.join(directory, "flow2d.dat"), 6)
    if len(zones) < len(dims):
        raise RestartError("flow2d.dat holds fewer blocks than the mesh")
    out = []
    for (nx, ny, nv), (ni, nj, rows) in zip(dims, zones):
        if (ni, nj) != (nx + 1, ny + 1):
            raise RestartError(f"flow2d.dat zone {ni}x{nj} does not match block {nx}x{ny}")
        U = np.zeros((nv, nx + 3, ny + 3), order="F")
        # records run i fastest over 0..nx, then j over 0..ny
        d, u, v, T = (rows[:, c].reshape(nj, ni).T for c in (2, 3, 4, 5))
        U[0, 1:nx + 2, 1:ny + 2] = d
        U[1, 1:nx + 2, 1:ny + 2] = d * u
        U[2, 1:nx + 2, 1:ny + 2] = d * v
        U[3, 1:nx + 2, 1:ny + 2] = d * Cv * T + 0.5 * d * (u * u + v * v)
        out.append(U)
    nv = dims[0][2]
    if nv == 5:
        for (nx, ny, _), (ni, nj, rows), U in zip(dims, _zones(os.path.join(directory, "SA2d.dat"), 3), out):
            U[4, 1:nx + 2, 1:ny + 2] = rows[:, 2].reshape(nj, ni).T
        if not fix_nvar:
            raise RestartError("sub_init.f90:541 reads SST2d.dat into U(5:6) of a 5-variable (SA) state as well; "
                               "restart with fix_nvar=True")
    if nv == 6 and fix_nvar:
        for (nx, ny, _), (ni, nj, rows), U in zip(dims, _zones(os.path.join(directory, "SST2d.dat"), 4), out):
            U[4, 1:nx + 2, 1:ny + 2] = rows[:, 2].reshape(nj, ni).T
            U[5, 1:nx + 2, 1:ny + 2] = rows[:, 3].reshape(nj, ni).T
    return out


def restart(solver, directory: str, case: int = 1, fix_nvar: bool = False) -> None:
    """Iflag_init = 1 for one case of a context: the freestream everywhere
    (ec2d_init_flow), then every block's 0..nx x 0..ny from the files of
    `directory` (read_flow), then the boundary conditions and the block halo
    on the fine mesh (init_flow_read ends with Boundary_condition_onemesh(1)
    and update_buffer_onemesh(1)).  The step counter and time restart at
    zero, as in the reference; with dual time stepping U(n) and U(n-1) are
    the restart state (ec2d_dual_time_start), for every case of the
    context."""
    params = solver.params[case - 1]
    dims = [solver.dims(case, 1, b) for b in range(1, solver.nblocks[case - 1] + 1)]
    Us = read_flow(directory, params, dims, fix_nvar=fix_nvar)
    solver.init_flow()
    for b, U in enumerate(Us, start=1):
        cur = solver.download_U(case, 1, b)
        nx, ny, nv = dims[b - 1]
        keep = U.shape[0] if (nv != 6 or fix_nvar) else 4
        cur[:keep, 1:nx + 2, 1:ny + 2] = U[:keep, 1:nx + 2, 1:ny + 2]
        solver.upload_U(case, 1, b, cur)
    solver.bc(1)
    solver.halo(1)
    # dual time stepping: the physical-time history starts from the restart
    # state (ec2d_dual_time_start; a no-op for the other time methods)
    solver.dual_time_start()
