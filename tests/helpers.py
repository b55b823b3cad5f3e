"""Shared helpers: build a case on the CPU oracle and on the GPU library,
copy states between them, and compare fields with the tolerances of the
parity contract."""
from __future__ import annotations

import numpy as np

from ec2d import cases, grids
from ec2d.inputs import Params

# One residual evaluation: per-cell error relative to the larger of |Res| and
# a face-flux scale of that cell must stay below RES_TOL (FP64, 1e-12).
RES_TOL = 1.0e-12
# Fields produced by pointwise formulas (primitives, spectral radii, dt,
# ghost cells): relative error per entry.
FIELD_TOL = 1.0e-12


def make_oracle(p, blocks, fdm=(), dw=None, threads=4):
    import oracle
    return oracle.Oracle(p, blocks, fdm_blocks=fdm, dw=dw, threads=threads)


def make_gpu(p, blocks, fdm=(), dw=None):
    from ec2d import gpu
    return gpu.Solver([(p, blocks)], fdm_blocks=[list(fdm)], dw=None if dw is None else [dw])


def copy_state(orc, g, mesh=1, nblocks=None, case=1):
    """Upload the oracle's U of every block of `mesh` to the GPU case."""
    nb = nblocks or orc.nblocks
    for b in range(1, nb + 1):
        g.upload_U(case, mesh, b, orc.get_U(mesh, b))


def perturb_state(orc, mesh=1, amp=0.02, seed=0):
    """Smooth seeded perturbation of the oracle's U (all cells incl. ghosts)."""
    rng = np.random.default_rng(seed)
    for b in range(1, orc.nblocks + 1):
        U = orc.get_U(mesh, b)
        nv, ni, nj = U.shape
        ii, jj = np.meshgrid(np.arange(ni), np.arange(nj), indexing="ij")
        for m in range(nv):
            ph = rng.uniform(0, 2 * np.pi, 3)
            f = (np.sin(0.37 * ii + ph[0]) * np.cos(0.23 * jj + ph[1]) + 0.5 * np.sin(0.11 * (ii + jj) + ph[2]))
            if m in (1, 2):
                U[m] = U[m] + amp * f * max(1e-3, np.abs(U[m]).max())
            else:
                U[m] = U[m] * (1.0 + amp * f)
        orc.set_U(mesh, b, U)


def flux_scale(orc, mesh, block, gamma):
    """Per-cell, per-variable scale of the face-flux terms entering Res:
    inviscid flux magnitude of the cell state times its perimeter; for the
    turbulence variables (nu_tilde, or rho k and rho omega) their convected
    amount |U_m| (|u| + c) times the perimeter."""
    Uall = orc.get_U(mesh, block)
    U = Uall[:4]
    nx, ny = orc.dims(mesh, block)
    si = orc.field(mesh, block, 12, (nx, ny))
    sj = orc.field(mesh, block, 13, (nx, ny))
    per = si[1:nx, 0:ny - 1] + si[0:nx - 1, 0:ny - 1] + sj[0:nx - 1, 1:ny] + sj[0:nx - 1, 0:ny - 1]
    Uc = U[:, 2:nx + 1, 2:ny + 1]  # cells 1..nx-1, 1..ny-1
    d = Uc[0]
    u, v = Uc[1] / d, Uc[2] / d
    p = (gamma - 1.0) * (Uc[3] - 0.5 * d * (u * u + v * v))
    c = np.sqrt(np.abs(gamma * p / d))
    q = np.sqrt(u * u + v * v) + c
    rows = [d * q, d * np.abs(u) * q + p, d * np.abs(v) * q + p, (Uc[3] + p) * q]
    for m in range(4, Uall.shape[0]):
        rows.append(np.abs(Uall[m, 2:nx + 1, 2:ny + 1]) * q)
    return np.stack(rows) * per[None]


def rel_err(a, b, scale=None):
    a = np.asarray(a); b = np.asarray(b)
    den = np.maximum(np.abs(a), np.abs(b))
    if scale is not None:
        den = np.maximum(den, scale)
    den = np.where(den == 0, 1.0, den)
    return np.max(np.abs(a - b) / den)


def compare_residual(orc, g, mesh=1, tol=RES_TOL, gamma=1.4, nvar=None):
    worst = 0.0
    for b in range(1, orc.nblocks + 1):
        nx, ny = orc.dims(mesh, b)
        nv = nvar or orc.nvar(mesh)
        ro = orc.field(mesh, b, 0, (nv, nx - 1, ny - 1))
        rg = g.field(1, mesh, b, 0, (nv, nx - 1, ny - 1))
        sc = flux_scale(orc, mesh, b, gamma)
        for m in range(nv):
            # turbulence rows: their own face-flux scale, or the block's
            # largest |Res_m| where that is larger
            s = sc[m] if m < 4 else np.maximum(sc[m], np.abs(ro[m]).max())
            e = rel_err(ro[m], rg[m], s)
            worst = max(worst, e)
    assert worst <= tol, f"residual mismatch {worst:.3e} > {tol:.1e}"
    return worst


def compare_fields(orc, g, fields, mesh=1, tol=FIELD_TOL, absfloor=0.0):
    worst = {}
    for b in range(1, orc.nblocks + 1):
        for f in fields:
            a = orc.field(mesh, b, f)
            c = g.field(1, mesh, b, f)
            assert a.shape == c.shape, (f, a.shape, c.shape)
            sc = absfloor * max(1e-300, np.abs(a).max())
            e = rel_err(a, c, sc if absfloor else None)
            worst[f] = max(worst.get(f, 0.0), e)
    bad = {k: v for k, v in worst.items() if v > tol}
    assert not bad, f"field mismatch {bad}"
    return worst


def compare_U(orc, g, mesh=1, tol=1e-12, interior_only=False):
    worst = 0.0
    for b in range(1, orc.nblocks + 1):
        a = orc.get_U(mesh, b)
        c = g.download_U(1, mesh, b)
        if interior_only:
            nx, ny = orc.dims(mesh, b)
            a = a[:, 2:nx + 1, 2:ny + 1]; c = c[:, 2:nx + 1, 2:ny + 1]
        for m in range(a.shape[0]):
            sc = np.abs(a[m]).max()
            e = np.max(np.abs(a[m] - c[m])) / (sc if sc > 0 else 1.0)
            worst = max(worst, e)
    assert worst <= tol, f"U mismatch {worst:.3e} > {tol:.1e}"
    return worst


def small_case(**kw):
    nx = kw.pop("nx", 65)
    ny = kw.pop("ny", 17)
    return cases.small_cgrid_case(nx, ny, **kw)
