"""Mixed precision: the LU-SGS sweeps in FP32 (ec2d_set_lusgs_precision(32))
against the all-FP64 oracle.

The FP32 sweep preconditions only: the residual is FP64 on both sides, so a
converged state must agree with the FP64 run to the level of the residual
drop.  Per sweep, dU must agree with the FP64 oracle's to float accuracy
accumulated along the wavefront: max|dU32 - dU64| <= 2e-5 max|dU64| per
variable and block (float epsilon 6e-8 times a few hundred dependent planes)."""
import numpy as np
import pytest

from helpers import copy_state, make_gpu, make_oracle, perturb_state, small_case

pytestmark = pytest.mark.gpu


def _sweep_pair(p, bl, nv):
    orc = make_oracle(p, bl)
    orc.init_flow()
    orc.step(3)
    perturb_state(orc, seed=5)
    g = make_gpu(p, bl)
    g.init_flow()
    copy_state(orc, g)
    g.set_lusgs_precision(32)
    orc.residual()
    nb = len(bl)
    for b in range(1, nb + 1):
        for f in (0, 1, 2, 3, 4, 5):
            g.set_field(1, 1, b, f, orc.field(1, b, f))
        orc.lusgs(1, b, 0.0)
    g.lusgs(1, 0.0)
    worst = 0.0
    for b in range(1, nb + 1):
        nx, ny = orc.dims(1, b)
        a = orc.field(1, b, 6, (nv, nx, ny))[:, :nx - 1, :ny - 1]
        c = g.field(1, 1, b, 6, (nv, nx, ny))[:, :nx - 1, :ny - 1]
        for m in range(nv):
            scale = np.abs(a[m]).max()
            assert scale > 0
            worst = max(worst, np.abs(a[m] - c[m]).max() / scale)
    return worst


@pytest.mark.parametrize("case", ["euler", "viscous", "sa", "sst"])
def test_lusgs32_sweep_matches_fp64(gpu_lib, case):
    kw = dict(Ma=0.7, AoA=2.0, nblocks=2, Iflag_flux=4)
    nv = 4
    if case != "euler":
        kw.update(If_viscous=1, Re=1e4 if case == "viscous" else 1e6, first=2e-4)
    if case == "sa":
        kw.update(Iflag_turbulence_model=2); nv = 5
    if case == "sst":
        kw.update(Iflag_turbulence_model=3, Kt_inf=1e-6, Wt_inf=1e-2); nv = 6
    p, bl = small_case(**kw)
    worst = _sweep_pair(p, bl, nv)
    assert worst <= 2e-5, worst


def test_lusgs32_steps_track_fp64(gpu_lib):
    """A few hundred steps from freestream: the FP32-preconditioned run follows
    the FP64 run closely (the residual history has the same shape)."""
    p, bl = small_case(Ma=0.5, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, CFL=5.0)
    runs = []
    for bits in (64, 32):
        g = make_gpu(p, bl)
        g.set_lusgs_precision(bits)
        g.init_flow()
        hist = []
        for k in range(10):
            g.step(30)
            hist.append(g.norms()[1][0])
        runs.append((g, np.sqrt(np.array(hist))))
    (g64, h64), (g32, h32) = runs
    np.testing.assert_allclose(h32, h64, rtol=1e-3)
    f64, f32 = np.array(g64.forces()), np.array(g32.forces())
    assert np.abs(f32 - f64).max() <= 1e-4, (f32, f64)


def test_fp32_coarse_levels_track_fp64(gpu_lib):
    """Flat plate, 3-level V-cycle: FP32 LU-SGS on every level plus FP32 face
    fluxes on the coarse levels against the all-FP64 run: over 1,500 cycles
    the residual drop stays within a factor of two and the forces within
    1e-6.  (Deeper down the FP32 rounding carried by the FAS forcing stalls
    the drop near 1e-7 of the first residual, so the mixed mode of the bench
    keeps the coarse fluxes in FP64.)"""
    from ec2d import cases
    p, bl = cases.laminar_flat_plate(49, 49, num_mesh=3)
    out = []
    for mixed in (False, True):
        g = make_gpu(p, bl)
        if mixed:
            g.set_lusgs_precision(32)
            g.set_coarse_precision(32)
        g.init_flow()
        g.step(1)
        r0 = g.norms()[1][0]
        g.step(1499)
        out.append((g.norms()[1][0] / r0, np.array(g.forces())))
    (d64, f64), (d32, f32) = out
    assert d32 <= 2.0 * d64 and d64 <= 2.0 * d32, (d64, d32)
    assert np.abs(f32 - f64).max() <= 1e-6, (f64, f32)
