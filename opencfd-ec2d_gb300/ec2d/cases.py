"""The benchmark workloads as (Params, blocks) pairs, built from seeded
synthetic grids (no external data).

Choices the workload descriptions leave open are fixed here:
* reconstruction: primitive variables (IFlag_Reconstruction = 0) for all
  workloads; "MUSCL" means the van Albada limiter (Iflag_Scheme = 5);
* "WENO5" is the reference's finite-difference WENO5 / Steger-Warming patch
  on every block (FDM.in lists all blocks) with Roe + MUSCL on the four
  finite-volume border layers, the only WENO5 the reference has;
* "LU-SGS smoothing" inside multigrid lifts the reference's refusal of that
  combination (mg_lusgs = 1; every level is smoothed by one LU-SGS sweep).
"""
from __future__ import annotations

import math

import numpy as np

from . import grids
from .inputs import (FLUX, SCHEME, TIME_LUSGS, TURB_NONE, TURB_SA, TURB_SST, Params)


def euler_naca0012(nx=257, ny=65):
    """Inviscid Euler, single block 257x65 C-grid, NACA 0012 (closed TE),
    M 0.8, AoA 1.25 deg, Roe + MUSCL van Albada, LU-SGS, CFL 5."""
    p = Params(Ma=0.8, AoA=1.25, Re=1.0e6, If_viscous=0, Iflag_turbulence_model=TURB_NONE,
               Iflag_local_dt=1, CFL=5.0, dtmax=1.0e3, dtmin=1.0e-12, Time_Method=TIME_LUSGS,
               Iflag_Scheme=SCHEME["MUSCL3"], Iflag_flux=FLUX["ROE"], IFlag_Reconstruction=0,
               Num_Mesh=1, xaxis=0.25, yaxis=0.0)
    n_wake = (nx - 1) // 8 + 1
    blocks = grids.naca_cgrid(nx, ny, m=0.0, p=0.0, t=0.12, radius=20.0, n_wake=n_wake, first=2.0e-3)
    return p, blocks


def laminar_flat_plate(nxb=97, ny=97, num_mesh=3):
    """Laminar flat plate, 2-block 193x97 H-grid, dy1 = 1e-4, ratio 1.1,
    M 0.3, Re 1e4, adiabatic wall, AUSM+ + MUSCL, 3-level V-cycle with
    LU-SGS smoothing; free-stream back pressure at the exit face."""
    p = Params(Ma=0.3, AoA=0.0, Re=1.0e4, Pr=0.72, If_viscous=1, Iflag_turbulence_model=TURB_NONE,
               Iflag_local_dt=1, CFL=10.0, dtmax=1.0e3, dtmin=1.0e-12, Time_Method=TIME_LUSGS,
               P_outlet=1.0 / (1.4 * 0.3 ** 2),
               Iflag_Scheme=SCHEME["MUSCL3"], Iflag_flux=FLUX["AUSM"], IFlag_Reconstruction=0,
               Num_Mesh=num_mesh, Twall=-1.0, T_inf=288.15, mg_lusgs=1, xaxis=0.0, yaxis=0.0)
    blocks = grids.flat_plate(nxb, ny, first=1.0e-4, ratio=1.1, x_lead=0.5, plate=1.0)
    return p, blocks


def rans_naca2412(nx=513, ny=129, nblocks=4, turb=TURB_SA, num_mesh=3, weno5=True):
    """RANS on a 4-block 513x129 C-grid around NACA 2412 (2% camber at 40%,
    12%), y+ ~ 1 at Re 6.5e6, M 0.73, AoA 2.8 deg, Roe, WENO5 patch,
    3-level multigrid, LU-SGS.  SA by default, SST as the second run."""
    p = Params(Ma=0.73, AoA=2.8, Re=6.5e6, Pr=0.72, If_viscous=1, Iflag_turbulence_model=turb,
               Iflag_local_dt=1, CFL=5.0, dtmax=1.0e3, dtmin=1.0e-12, Time_Method=TIME_LUSGS,
               Iflag_Scheme=SCHEME["MUSCL3"], Iflag_flux=FLUX["ROE"], IFlag_Reconstruction=0,
               Num_Mesh=num_mesh, Twall=-1.0, T_inf=288.15, vt_inf=3.0, Kt_inf=1.0e-6, Wt_inf=1.0e-2,
               mg_lusgs=1, xaxis=0.25, yaxis=0.0)
    n_wake = (nx - 1) // 8 + 1
    blocks = grids.naca_cgrid(nx, ny, m=0.02, p=0.4, t=0.12, radius=20.0, n_wake=n_wake, first=4.0e-6,
                              nblocks=nblocks)
    fdm = list(range(1, nblocks + 1)) if weno5 else []
    return p, blocks, fdm


def polar_cases(n=64, seed=20261203, min_size=(257, 65), max_size=(513, 129), with_tc=False):
    """Batched polar: n SA RANS cases drawn from a seed.  M ~ U[0.3,0.8],
    AoA ~ U[-2,8] deg, log10 Re ~ U[6,7], t/c ~ U[0.09,0.15], 1..4 blocks,
    grids between 257x65 and 513x129 (node counts that keep three multigrid
    levels).  with_tc: (params, blocks, t/c) triples."""
    rng = np.random.default_rng(seed)
    sizes = [(257, 65), (385, 97), (513, 129)]
    sizes = [s for s in sizes if min_size[0] <= s[0] <= max_size[0]]
    out = []
    for k in range(n):
        M = rng.uniform(0.3, 0.8)
        aoa = rng.uniform(-2.0, 8.0)
        re = 10.0 ** rng.uniform(6.0, 7.0)
        tc = rng.uniform(0.09, 0.15)
        nb = int(rng.integers(1, 5))
        nx, ny = sizes[int(rng.integers(0, len(sizes)))]
        while (nx - 1) % nb:
            nb -= 1
        p = Params(Ma=M, AoA=aoa, Re=re, Pr=0.72, If_viscous=1, Iflag_turbulence_model=TURB_SA,
                   Iflag_local_dt=1, CFL=5.0, dtmax=1.0e3, dtmin=1.0e-12, Time_Method=TIME_LUSGS,
                   Iflag_Scheme=SCHEME["MUSCL3"], Iflag_flux=FLUX["ROE"], IFlag_Reconstruction=0,
                   Num_Mesh=3, Twall=-1.0, vt_inf=3.0, mg_lusgs=1, xaxis=0.25)
        n_wake = (nx - 1) // 8 + 1
        first = 1.0e-6 * 6.5e6 / re * 4.0
        blocks = grids.naca_cgrid(nx, ny, m=0.0, p=0.0, t=tc, radius=20.0, n_wake=n_wake, first=first,
                                  nblocks=nb)
        out.append((p, blocks, tc) if with_tc else (p, blocks))
    return out


def small_cgrid_case(nx=65, ny=17, **kw):
    """A small C-grid case for parity tests (seconds on the CPU oracle)."""
    n_wake = (nx - 1) // 8 + 1
    nblocks = kw.pop("nblocks", 1)
    first = kw.pop("first", 1.0e-3)
    t = kw.pop("t", 0.12)
    m = kw.pop("m", 0.0)
    pp = kw.pop("p", 0.0)
    blocks = grids.naca_cgrid(nx, ny, m=m, p=pp, t=t, radius=10.0, n_wake=n_wake, first=first, nblocks=nblocks)
    params = Params(**kw)
    return params, blocks
