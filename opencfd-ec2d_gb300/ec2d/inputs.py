"""Readers and writers for the OpenCFD-EC2D input and output files.

The formats are the reference's, unchanged, so a case directory prepared for
the Fortran code runs here and vice versa:

* ``control.in``  -- positional free-format parameters, read at
  opencfd_ec2d_v1.5.4.f90:201-211 (lines 2,4,6,8,10; line 12 ``xaxis yaxis
  deltAoA`` is not read by the reference and is used here for the moment
  reference point).
* ``bc2d_1.in``   -- block connectivity, read at sub_init.f90:228-248.
* ``Mesh2d.dat``  -- node coordinates, read at sub_init.f90:121-127,176.
* ``Residual.dat`` records, written at opencfd_ec2d_v1.5.4.f90:275-277.
* ``flow2d.dat`` Tecplot snapshot, written at opencfd_ec2d_v1.5.4.f90:323-339.
* ``dist_wall.dat`` cell wall distances, read or written by comput_dw
  (sub_turbulence_SST.f90:295-348), and its Tecplot view ``dw.dat``
  (:350-362).
"""
from __future__ import annotations

import dataclasses
import re
from typing import List, Sequence

import numpy as np

# enumerations, opencfd_ec2d_v1.5.4.f90:42-47
SCHEME = {"UD1": 0, "NND2": 1, "UD3": 2, "WENO3": 3, "MUSCL2": 4, "MUSCL3": 5, "OMUSCL2": 6}
FLUX = {"SW": 1, "HLL": 2, "HLLC": 3, "ROE": 4, "VANLEER": 5, "AUSM": 6}
RECON = {"ORIGINAL": 0, "CONSERVATIVE": 1, "CHARACTERISTIC": 2}
BC_WALL, BC_FARFIELD, BC_SYMMETRY, BC_INLET, BC_OUTLET = -10, -20, -30, -40, -50
TIME_EULER1, TIME_RK3, TIME_LUSGS, TIME_DUAL = 1, 3, 0, -1
TURB_NONE, TURB_BL, TURB_SA, TURB_SST = 0, 1, 2, 3


@dataclasses.dataclass
class Params:
    """The scalars of control.in (Global_Var, opencfd_ec2d_v1.5.4.f90:103-110).

    AoA is in degrees and Twall in kelvin, as written in control.in.
    """
    Ma: float = 0.8
    Re: float = 1.0e6
    gamma: float = 1.4
    AoA: float = 0.0
    Pr: float = 0.72
    t_end: float = 1.0
    Kstep_save: int = 1000000
    If_viscous: int = 0
    Iflag_turbulence_model: int = 0
    Iflag_init: int = 0
    Iflag_local_dt: int = 1
    dt_global: float = 1.0e-6
    CFL: float = 5.0
    dtmax: float = 1.0
    dtmin: float = 1.0e-8
    Time_Method: int = 0
    P_outlet: float = -1.0
    T_inf: float = 288.15
    Twall: float = -1.0
    vt_inf: float = 3.0
    Kt_inf: float = 1.0e-8
    Wt_inf: float = 1.0e-6
    Iflag_Scheme: int = 5
    Iflag_flux: int = 4
    IFlag_Reconstruction: int = 0
    Kstep_show: int = 10
    Num_Mesh: int = 1
    Num_Threads: int = 1
    Nstep_Inner_Limit: int = 20
    Res_Inner_Limit: float = 1.0e-6
    Pre_Step_Mesh: Sequence[int] = (0, 0, 0)
    xaxis: float = 0.25
    yaxis: float = 0.0
    mg_lusgs: int = 1

    def nvar(self) -> int:
        if self.Iflag_turbulence_model == TURB_SST:
            return 6
        if self.Iflag_turbulence_model == TURB_SA:
            return 5
        return 4

    def replace(self, **kw) -> "Params":
        return dataclasses.replace(self, **kw)


@dataclasses.dataclass
class Block:
    """One structured block: node coordinates x[i,j], y[i,j] (0-based arrays of
    shape (nx, ny), node (1,1) of the reference at [0,0]) and its subfaces, each
    ``[f_no, face, ist, iend, jst, jend, neighb, subface, orient]``."""
    x: np.ndarray
    y: np.ndarray
    bc: List[List[int]]

    @property
    def nx(self) -> int:
        return self.x.shape[0]

    @property
    def ny(self) -> int:
        return self.x.shape[1]

    @property
    def ncell(self) -> int:
        return (self.nx - 1) * (self.ny - 1)


def _fnum(tok: str) -> float:
    # Fortran list-directed reals accept d/D exponents
    return float(tok.replace("d", "e").replace("D", "E"))


def _data_lines(text: str) -> List[str]:
    return [ln for ln in text.replace("\r", "").split("\n")]


def read_control(path: str) -> Params:
    """Parse control.in exactly as read_parameter does (opencfd_ec2d_v1.5.4.f90:201-211)."""
    lines = _data_lines(open(path, encoding="latin-1").read())
    def toks(k):
        return lines[k].split()
    t = toks(1)
    p = Params()
    p.Ma, p.Re, p.gamma, p.AoA, p.Pr, p.t_end = map(_fnum, t[:6])
    p.Kstep_save, p.If_viscous, p.Iflag_turbulence_model, p.Iflag_init = (int(_fnum(v)) for v in t[6:10])
    t = toks(3)
    p.Iflag_local_dt = int(_fnum(t[0]))
    p.dt_global, p.CFL, p.dtmax, p.dtmin = map(_fnum, t[1:5])
    p.Time_Method = int(_fnum(t[5]))
    p.P_outlet, p.T_inf, p.Twall, p.vt_inf, p.Kt_inf, p.Wt_inf = map(_fnum, t[6:12])
    t = toks(5)
    p.Iflag_Scheme, p.Iflag_flux, p.IFlag_Reconstruction, p.Kstep_show = (int(_fnum(v)) for v in t[:4])
    t = toks(7)
    p.Num_Mesh, p.Num_Threads, p.Nstep_Inner_Limit = (int(_fnum(v)) for v in t[:3])
    p.Res_Inner_Limit = _fnum(t[3])
    t = toks(9)
    pre = [int(_fnum(v)) for v in t[: p.Num_Mesh]]
    p.Pre_Step_Mesh = tuple(pre + [0] * (3 - len(pre)))
    if len(lines) > 11 and len(lines[11].split()) >= 2:
        try:
            t = toks(11)
            p.xaxis, p.yaxis = _fnum(t[0]), _fnum(t[1])
        except ValueError:
            pass
    return p


def write_control(path: str, p: Params) -> None:
    def f(v):
        return repr(float(v)).replace("e", "d") if "e" in repr(float(v)) else repr(float(v)) + "d0"
    with open(path, "w") as fh:
        fh.write("  Ma Re gamma AoA Pr t_end Kstep_save If_viscous Iflag_turbulence_model Iflag_init\n")
        fh.write(f" {f(p.Ma)} {f(p.Re)} {f(p.gamma)} {f(p.AoA)} {f(p.Pr)} {f(p.t_end)} {p.Kstep_save} "
                 f"{p.If_viscous} {p.Iflag_turbulence_model} {p.Iflag_init}\n")
        fh.write("  Iflag_local_dt dt_global CFL dtmax dtmin Time_Method P_outlet T_inf Twall vt_inf Kt_inf Wt_inf\n")
        fh.write(f" {p.Iflag_local_dt} {f(p.dt_global)} {f(p.CFL)} {f(p.dtmax)} {f(p.dtmin)} {p.Time_Method} "
                 f"{f(p.P_outlet)} {f(p.T_inf)} {f(p.Twall)} {f(p.vt_inf)} {f(p.Kt_inf)} {f(p.Wt_inf)}\n")
        fh.write("  Iflag_scheme Iflag_flux IFlag_Reconstruction Kstep_show\n")
        fh.write(f" {p.Iflag_Scheme} {p.Iflag_flux} {p.IFlag_Reconstruction} {p.Kstep_show}\n")
        fh.write("  Num_Mesh Num_THREADS Nstep_Inner_Limit Res_Inner_Limit\n")
        fh.write(f" {p.Num_Mesh} {p.Num_Threads} {p.Nstep_Inner_Limit} {f(p.Res_Inner_Limit)}\n")
        fh.write("  Pre_Step_Mesh(1:Num_Mesh)\n")
        fh.write(" " + " ".join(str(int(v)) for v in list(p.Pre_Step_Mesh)[: p.Num_Mesh]) + "\n")
        fh.write("  xaxis yaxis deltAoA\n")
        fh.write(f" {f(p.xaxis)} {f(p.yaxis)} 0.d0\n")


def read_bc(path: str) -> List[List[List[int]]]:
    """Parse bc2d_1.in (sub_init.f90:228-248): per block, a list of 9-int subfaces."""
    lines = [ln for ln in _data_lines(open(path, encoding="latin-1").read())]
    k = 2
    nb = int(lines[k].split()[0]); k += 1
    out = []
    for _ in range(nb):
        k += 2  # " Block n", " Subface"
        ns = int(lines[k].split()[0]); k += 1
        k += 1  # header
        subs = []
        for _ in range(ns):
            subs.append([int(v) for v in lines[k].split()[:9]]); k += 1
        out.append(subs)
    return out


def write_bc(path: str, blocks: Sequence[Block], title: str = "ec2d case") -> None:
    with open(path, "w") as fh:
        fh.write(f" 2D BC file for multi-block mesh:  {title}\n # Blocks\n")
        fh.write(f" {len(blocks):10d}\n")
        for m, b in enumerate(blocks):
            fh.write(f" Block {m + 1:12d}\n Subface\n  {len(b.bc)}\n")
            fh.write(" f_no, face, istart,iend, jstart, jend,  neighb, subface orient\n")
            for s in b.bc:
                fh.write(" " + " ".join(f"{v:5d}" for v in s) + "\n")


def read_mesh(path: str) -> List[tuple]:
    """Parse Mesh2d.dat (sub_init.f90:121-127,176): list of (x, y) arrays (nx, ny)."""
    vals = open(path, encoding="latin-1").read().replace("\r", " ").split()
    pos = 0
    nb = int(vals[pos]); pos += 1
    dims = []
    for _ in range(nb):
        dims.append((int(vals[pos]), int(vals[pos + 1]))); pos += 2
    out = []
    for nx, ny in dims:
        n = nx * ny
        x = np.array([_fnum(v) for v in vals[pos:pos + n]]).reshape(ny, nx).T.copy(); pos += n
        y = np.array([_fnum(v) for v in vals[pos:pos + n]]).reshape(ny, nx).T.copy(); pos += n
        out.append((x, y))
    return out


def write_mesh(path: str, blocks: Sequence[Block]) -> None:
    with open(path, "w") as fh:
        fh.write(f"{len(blocks):12d}\n")
        fh.write(" ".join(f"{b.nx:12d}{b.ny:12d}" for b in blocks) + "\n")
        for b in blocks:
            for arr in (b.x, b.y):
                flat = np.asarray(arr).T.reshape(-1)
                for k in range(0, flat.size, 3):
                    fh.write("".join(f"{v:24.16e}" for v in flat[k:k + 3]) + "\n")


def read_case(directory: str):
    """Read control.in, bc2d_1.in and Mesh2d.dat of a case directory."""
    import os
    p = read_control(os.path.join(directory, "control.in"))
    bcs = read_bc(os.path.join(directory, "bc2d_1.in"))
    xy = read_mesh(os.path.join(directory, "Mesh2d.dat"))
    if len(bcs) != len(xy):
        raise ValueError("Block number in bc2d.in is not equal to that in Mesh2d.dat")
    blocks = [Block(x, y, bc) for (x, y), bc in zip(xy, bcs)]
    return p, blocks


def write_case(directory: str, p: Params, blocks: Sequence[Block], title: str = "ec2d case") -> None:
    import os
    os.makedirs(directory, exist_ok=True)
    write_control(os.path.join(directory, "control.in"), p)
    write_bc(os.path.join(directory, "bc2d_1.in"), blocks, title)
    write_mesh(os.path.join(directory, "Mesh2d.dat"), blocks)


def _list_directed(text: str) -> List[str]:
    """The values of Fortran list-directed records: separated by blanks,
    commas or line ends, ``r*c`` standing for r copies of c."""
    out: List[str] = []
    for tok in re.split(r"[\s,]+", text.strip()):
        if not tok:
            continue
        if "*" in tok:
            r, c = tok.split("*", 1)
            out.extend([c] * int(r))
        else:
            out.append(tok)
    return out


def read_dist_wall(path: str, dims: Sequence) -> List[np.ndarray]:
    """dist_wall.dat as comput_dw reads it (sub_turbulence_SST.f90:295-306):
    the block count, the (nx, ny) node counts of every block, then each
    block's cell distances dw(1:nx-1,1:ny-1), i fastest.  `dims` holds the
    (nx, ny) of the mesh's blocks; one Fortran-ordered (nx-1, ny-1) array per
    block is returned.  A file written for another mesh (other block count
    or sizes) raises ValueError; the reference would read its numbers into
    the mesh's blocks all the same."""
    v = _list_directed(open(path).read())
    nb = int(v[0])
    sizes = [(int(v[1 + 2 * k]), int(v[2 + 2 * k])) for k in range(nb)]
    want = [(int(nx), int(ny)) for nx, ny in dims]
    if sizes != want:
        raise ValueError(f"{path} was written for blocks {sizes}, the mesh has {want}")
    pos, out = 1 + 2 * nb, []
    for nx, ny in sizes:
        n = (nx - 1) * (ny - 1)
        vals = [float(t.replace("D", "E").replace("d", "e")) for t in v[pos:pos + n]]
        if len(vals) != n:
            raise ValueError(f"{path} ends inside a block")
        out.append(np.array(vals).reshape((nx - 1, ny - 1), order="F"))
        pos += n
    return out


def write_dist_wall(path: str, dws: Sequence, dims: Sequence) -> None:
    """dist_wall.dat as comput_dw writes it (sub_turbulence_SST.f90:342-348),
    every value with 17 significant digits, as list-directed output writes a
    double: it reads back to the same double."""
    with open(path, "w") as fh:
        fh.write(f" {len(dws)}\n")
        fh.write(" " + " ".join(f"{int(nx)} {int(ny)}" for nx, ny in dims) + "\n")
        for d in dws:
            flat = np.asarray(d, dtype=np.float64).reshape(-1, order="F")
            for k in range(0, flat.size, 4):
                fh.write(" " + " ".join(f"{float(x):.17g}" for x in flat[k:k + 4]) + "\n")


def write_dw_tecplot(path: str, cells: Sequence) -> None:
    """dw.dat (sub_turbulence_SST.f90:350-362): per block a zone of its cell
    centres and wall distances, i fastest; `cells` holds one (x1, y1, dw)
    triple of (nx-1, ny-1) arrays per block."""
    with open(path, "w") as fh:
        fh.write(" variables=x,y,dw\n")
        for x1, y1, dw in cells:
            ni, nj = np.shape(dw)
            fh.write(f" zone i= {ni} j= {nj}\n")
            for j in range(nj):
                for i in range(ni):
                    fh.write(f" {float(x1[i, j]):.17g} {float(y1[i, j]):.17g} {float(dw[i, j]):.17g}\n")


def residual_record(kstep: int, res_max6, res_rms, nvar: int) -> str:
    """One Residual.dat line, format (I8,13E24.10) (opencfd_ec2d_v1.5.4.f90:276)."""
    vals = list(res_max6[:6]) + list(res_rms[:nvar])
    return f"{kstep:8d}" + "".join(_e24(v) for v in vals) + "\n"


def _e24(v: float) -> str:
    # Fortran E24.10: 0.dddddddddddE+xx
    if v == 0.0 or not np.isfinite(v):
        return f"{'0.0000000000E+00' if v == 0.0 else str(v):>24s}"
    m, e = f"{abs(v):.9e}".split("e")
    ex = int(e) + 1
    mant = f"0.{m.replace('.', '')}"
    s = ("-" if v < 0 else "") + f"{mant}E{ex:+03d}"
    return f"{s:>24s}"
