"""Synthetic multi-block structured grids in the reference's Mesh2d.dat /
bc2d_1.in layout (seeded, deterministic; no external data).

* ``naca_cgrid``  -- C-grid around a NACA four-digit airfoil (closed trailing
  edge thickness polynomial), far field at ``R`` chords, split into 1-4 blocks
  along i.  The wake cut is a subface pair on the j- faces, reversed
  orientation, as in the reference's RAE2822 case (bc2d_1.in).
* ``flat_plate``  -- 2-block H-grid for the laminar flat plate: a symmetry
  block ahead of the plate and a no-slip block over it, geometric wall
  stretching.

Every subface start/end index is 1 modulo 4 so that check_mesh_multigrid
(sub_init.f90:39-107) admits three multigrid levels.  Node arrays are (nx, ny)
with x[i-1, j-1] = x(i, j) of the reference.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np

from .inputs import BC_FARFIELD, BC_OUTLET, BC_SYMMETRY, BC_WALL, Block


def naca4(m: float, p: float, t: float, xc: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Camber line and half thickness of a NACA four-digit section at stations
    ``xc`` (0..1); closed trailing edge (last thickness coefficient -0.1036)."""
    yt = 5.0 * t * (0.2969 * np.sqrt(xc) - 0.1260 * xc - 0.3516 * xc ** 2 + 0.2843 * xc ** 3 - 0.1036 * xc ** 4)
    if m <= 0.0 or p <= 0.0:
        return np.zeros_like(xc), yt
    yc = np.where(xc < p, m / p ** 2 * (2 * p * xc - xc ** 2),
                  m / (1 - p) ** 2 * ((1 - 2 * p) + 2 * p * xc - xc ** 2))
    return yc, yt


def _airfoil_surface(m, p, t, n_half):
    """Airfoil nodes from the trailing edge along the lower surface to the
    leading edge and back along the upper surface (2*n_half-1 nodes)."""
    beta = np.linspace(0.0, math.pi, n_half)
    xc = 0.5 * (1.0 - np.cos(beta))  # cosine clustering at LE and TE
    yc, yt = naca4(m, p, t, xc)
    if m > 0:
        dyc = np.where(xc < p, 2 * m / p ** 2 * (p - xc), 2 * m / (1 - p) ** 2 * (p - xc))
        th = np.arctan(dyc)
    else:
        th = np.zeros_like(xc)
    xu, yu = xc - yt * np.sin(th), yc + yt * np.cos(th)
    xl, yl = xc + yt * np.sin(th), yc - yt * np.cos(th)
    # lower: TE -> LE ; upper: LE -> TE
    x = np.concatenate([xl[::-1], xu[1:]])
    y = np.concatenate([yl[::-1], yu[1:]])
    y[0] = y[-1] = 0.5 * (y[0] + y[-1])
    x[0] = x[-1] = 0.5 * (x[0] + x[-1])
    return x, y


def _tanh_dist(n: int, first: float) -> np.ndarray:
    """n points on [0,1] clustered at 0 with first spacing ~first (tanh stretching)."""
    eta = np.linspace(0.0, 1.0, n)
    if first >= 1.0 / (n - 1):
        return eta
    lo, hi = 1e-6, 50.0
    for _ in range(200):
        b = 0.5 * (lo + hi)
        s1 = 1.0 + math.tanh(b * (eta[1] - 1.0)) / math.tanh(b)
        if s1 > first:
            lo = b
        else:
            hi = b
    b = 0.5 * (lo + hi)
    return 1.0 + np.tanh(b * (eta - 1.0)) / math.tanh(b)


def naca_cgrid(nx: int = 257, ny: int = 65, m: float = 0.0, p: float = 0.0, t: float = 0.12,
               radius: float = 20.0, n_wake: int = 33, first: float = 2.0e-3,
               nblocks: int = 1) -> List[Block]:
    """C-grid of nx*ny nodes (1..4 blocks split along i).

    i runs lower-wake outflow -> trailing edge -> lower surface -> leading edge
    -> upper surface -> trailing edge -> upper-wake outflow; j runs from the
    surface/cut to the far field (a right-handed grid, so the reference's face
    normals point to increasing i and j)."""
    n_af = nx - 2 * (n_wake - 1)
    if n_af % 2 == 0 or n_af < 9:
        raise ValueError("nx - 2*(n_wake-1) must be odd and >= 9")
    xa, ya = _airfoil_surface(m, p, t, (n_af + 1) // 2)
    x_te = xa[0]
    x_out = x_te + radius
    # wake: from outflow to the trailing edge, clustered at the TE
    ds_te = math.hypot(xa[1] - xa[0], ya[1] - ya[0])
    sw = _tanh_dist(n_wake, ds_te / radius)
    xw = x_te + radius * sw[::-1]
    yw = np.full(n_wake, ya[0])
    xin = np.concatenate([xw, xa[1:-1], xw[::-1]])
    yin = np.concatenate([yw, ya[1:-1], yw[::-1]])
    assert xin.size == nx
    # outer C boundary: bottom line, semicircle centred at the TE, top line
    xo = np.empty(nx); yo = np.empty(nx)
    xo[:n_wake] = xw; yo[:n_wake] = -radius
    xo[nx - n_wake:] = xw[::-1]; yo[nx - n_wake:] = radius
    na = n_af
    th = -0.5 * math.pi - math.pi * np.linspace(0.0, 1.0, na)
    xo[n_wake - 1:n_wake - 1 + na] = x_te + radius * np.cos(th)
    yo[n_wake - 1:n_wake - 1 + na] = radius * np.sin(th)
    # inner normals (into the fluid) and outer normals (outward)
    tx = np.gradient(xin); ty = np.gradient(yin)
    nin = np.stack([-ty, tx], 1)  # tangent rotated by +90 degrees: into the fluid
    nin /= np.linalg.norm(nin, axis=1, keepdims=True)
    nin[:n_wake - 1] = [0.0, -1.0]
    nin[nx - n_wake + 1:] = [0.0, 1.0]
    # j-lines: straight segments inner->outer bent near the wall so that they
    # leave the surface along its normal; the bend fades out within 20% chord of
    # the trailing edge so the fan there cannot cross the vertical wake lines.
    d = np.stack([xo - xin, yo - yin], 1)
    L = np.linalg.norm(d, axis=1)
    dh = d / L[:, None]
    dist_te = np.minimum(np.hypot(xin - x_te, yin - ya[0]), 1.0)
    w = np.clip(dist_te / 0.2, 0.0, 1.0)
    w[:n_wake] = 0.0
    w[nx - n_wake:] = 0.0
    nw = (1.0 - w)[:, None] * dh + w[:, None] * nin
    nw /= np.linalg.norm(nw, axis=1, keepdims=True)
    s = _tanh_dist(ny, first / radius)
    g = s * (1.0 - s) ** 16
    X = np.outer(xin, 1 - s) + np.outer(xo, s) + np.outer(L * (nw[:, 0] - dh[:, 0]), g)
    Y = np.outer(yin, 1 - s) + np.outer(yo, s) + np.outer(L * (nw[:, 1] - dh[:, 1]), g)
    X[:, 0] = xin; Y[:, 0] = yin
    # wake cut nodes coincide
    X[:n_wake, 0] = X[nx - n_wake:, 0][::-1]
    Y[:n_wake, 0] = Y[nx - n_wake:, 0][::-1]
    return split_cgrid(X, Y, n_wake, nblocks)


def split_cgrid(X: np.ndarray, Y: np.ndarray, n_wake: int, nblocks: int) -> List[Block]:
    """Split a single-block C-grid into ``nblocks`` blocks along i and build the
    bc2d_1.in subfaces (wake cut on j-, wall on j-, far field elsewhere)."""
    nx, ny = X.shape
    if (nx - 1) % nblocks:
        raise ValueError("(nx-1) must divide into nblocks")
    w = (nx - 1) // nblocks
    cuts = [b * w + 1 for b in range(nblocks + 1)]  # global 1-based node index of block starts
    te_lo, te_hi = n_wake, nx - n_wake + 1
    blocks = []
    for b in range(nblocks):
        g0, g1 = cuts[b], cuts[b + 1]
        blocks.append(Block(X[g0 - 1:g1].copy(), Y[g0 - 1:g1].copy(), []))
    # j- face pieces in global indices: [lo, hi] with kind
    pieces = [(1, te_lo, "cutlo"), (te_lo, te_hi, "wall"), (te_hi, nx, "cuthi")]
    sub_of = {}
    for b in range(nblocks):
        g0, g1 = cuts[b], cuts[b + 1]
        nxb = g1 - g0 + 1
        subs = []
        if b == 0:
            subs.append([1, 1, 1, 1, 1, ny, BC_FARFIELD, 0, 0])
        else:
            subs.append([1, 1, 1, 1, 1, ny, b, None, 2])  # neighbour fixed below
        for lo, hi, kind in pieces:
            a, c = max(lo, g0), min(hi, g1)
            if c <= a:
                continue
            entry = [0, 2, a - g0 + 1, c - g0 + 1, 1, 1, 0, 0, 0]
            if kind == "wall":
                entry[6] = BC_WALL
            else:
                entry[6] = kind  # resolved below
                entry[7] = (a, c)
            subs.append(entry)
        if b == nblocks - 1:
            subs.append([0, 3, nxb, nxb, 1, ny, BC_FARFIELD, 0, 0])
        else:
            subs.append([0, 3, nxb, nxb, 1, ny, b + 2, None, 2])
        subs.append([0, 4, 1, nxb, ny, ny, BC_FARFIELD, 0, 0])
        for k, e in enumerate(subs):
            e[0] = k + 1
        blocks[b].bc = subs
        for k, e in enumerate(subs):
            if isinstance(e[6], str):
                sub_of[(e[6], e[7])] = (b, k)
    # resolve block-to-block neighbours
    for b in range(nblocks):
        for e in blocks[b].bc:
            if e[1] == 1 and e[7] is None:
                nb = b - 1
                e[6] = nb + 1
                e[7] = next(k + 1 for k, s in enumerate(blocks[nb].bc) if s[1] == 3)
            elif e[1] == 3 and e[7] is None:
                nb = b + 1
                e[6] = nb + 1
                e[7] = next(k + 1 for k, s in enumerate(blocks[nb].bc) if s[1] == 1)
    # resolve the wake cut: lower piece [a,c] in global i maps to the mirrored
    # upper piece [nx+1-c, nx+1-a]; pieces may be split by block edges.
    lo_items = [(key, v) for key, v in sub_of.items() if key[0] == "cutlo"]
    hi_items = [(key, v) for key, v in sub_of.items() if key[0] == "cuthi"]
    for key, (b, k) in lo_items:
        a, c = key[1]
        mirror = (nx + 1 - c, nx + 1 - a)
        match = [(kk, vv) for kk, vv in hi_items if kk[1] == mirror]
        if not match:
            raise ValueError("wake cut pieces do not mirror; choose nblocks so block edges are symmetric")
        (_, (b2, k2)) = match[0]
        blocks[b].bc[k][6] = b2 + 1; blocks[b].bc[k][7] = k2 + 1; blocks[b].bc[k][8] = 1
        blocks[b2].bc[k2][6] = b + 1; blocks[b2].bc[k2][7] = k + 1; blocks[b2].bc[k2][8] = 1
    return blocks


def flat_plate(nx_block: int = 97, ny: int = 97, first: float = 1.0e-4, ratio: float = 1.1,
               x_lead: float = 0.5, plate: float = 1.0, outlet: int = BC_OUTLET) -> List[Block]:
    """2-block H-grid: block 1 over [-x_lead, 0] (symmetry floor), block 2 over
    [0, plate] (no-slip wall); geometric wall-normal stretching.  The exit face
    is a back-pressure outlet (BC_OUTLET, with P_outlet > 0 in control.in): a
    far-field face there extrapolates every variable on subsonic outflow
    (sub_boundary.f90:529-531), which leaves the exit pressure floating."""
    yj = np.concatenate([[0.0], np.cumsum(first * ratio ** np.arange(ny - 1))])
    # streamwise: cluster at the leading edge x=0 from both sides
    s = _tanh_dist(nx_block, 2.0e-3)
    x1 = -x_lead * s[::-1]
    x2 = plate * _tanh_dist(nx_block, 2.0e-3 / plate * 1.0)
    b1 = Block(np.repeat(x1[:, None], ny, 1), np.repeat(yj[None, :], nx_block, 0), [])
    b2 = Block(np.repeat(x2[:, None], ny, 1), np.repeat(yj[None, :], nx_block, 0), [])
    n = nx_block
    b1.bc = [[1, 1, 1, 1, 1, ny, BC_FARFIELD, 0, 0],
             [2, 2, 1, n, 1, 1, BC_SYMMETRY, 0, 0],
             [3, 3, n, n, 1, ny, 2, 1, 2],
             [4, 4, 1, n, ny, ny, BC_FARFIELD, 0, 0]]
    b2.bc = [[1, 1, 1, 1, 1, ny, 1, 3, 2],
             [2, 2, 1, n, 1, 1, BC_WALL, 0, 0],
             [3, 3, n, n, 1, ny, outlet, 0, 0],
             [4, 4, 1, n, ny, ny, BC_FARFIELD, 0, 0]]
    return [b1, b2]


def cell_volumes(b: Block) -> np.ndarray:
    """Signed cell areas (positive for a right-handed block)."""
    x, y = b.x, b.y
    return 0.5 * ((x[1:, 1:] - x[:-1, :-1]) * (y[:-1, 1:] - y[1:, :-1]) -
                  (x[:-1, 1:] - x[1:, :-1]) * (y[1:, 1:] - y[:-1, :-1]))
