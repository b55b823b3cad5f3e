"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden outputs, so the oracle is checked
against properties derived from the code and from mathematics: consistency
of every face flux, limiter identities, freestream preservation on closed
multi-block grids, exact conservation of the multigrid restriction, mirror
symmetry, and convergence of the reference's own RAE2822 case when present."""
import math
import os

import numpy as np
import pytest

from helpers import make_oracle, small_case

GAMMA = 1.4


def euler_flux(q, gamma=GAMMA):
    d, u, v, p = q
    E = p / (gamma - 1.0) + 0.5 * d * (u * u + v * v)
    return np.array([d * u, d * u * u + p, d * u * v, u * (E + p)])


@pytest.mark.parametrize("iflux", [1, 2, 3, 4, 5, 6])
def test_flux_consistency(oracle_lib, iflux):
    """F(q, q) equals the exact Euler flux for every flux function
    (sub_flux_split.f90), subsonic and supersonic, both directions."""
    rng = np.random.default_rng(iflux)
    for _ in range(200):
        d = rng.uniform(0.2, 3.0)
        p = rng.uniform(0.2, 3.0)
        c = math.sqrt(GAMMA * p / d)
        u = rng.uniform(-2.5, 2.5) * c
        v = rng.uniform(-1.0, 1.0)
        q = np.array([d, u, v, p])
        F = oracle_lib.flux(iflux, q, q)
        np.testing.assert_allclose(F, euler_flux(q), rtol=1e-12, atol=1e-12 * (abs(u) + c) * (d + p))


@pytest.mark.parametrize("iflux", [1, 2, 3, 4, 5, 6])
def test_flux_upwinding(oracle_lib, iflux):
    """Supersonic flow to the right takes the left flux only (all six fluxes
    are upwind for |M| > 1 except Roe, whose entropy fix keeps it upwind too)."""
    qL = np.array([1.0, 2.5, 0.3, 0.7])
    qR = np.array([0.8, 2.4, -0.1, 0.6])
    F = oracle_lib.flux(iflux, qL, qR)
    if iflux in (1, 2, 3, 5, 6):
        np.testing.assert_allclose(F, euler_flux(qL), rtol=1e-12)


@pytest.mark.parametrize("flag", [0, 1, 2, 3, 4, 5, 6])
def test_limiters_exact_on_constants_and_lines(oracle_lib, flag):
    """Every scheme reproduces a constant; UD3/MUSCL3 are exact on lines."""
    for c in (0.0, 1.5, -2.25):
        assert oracle_lib.scheme(0, c, c, c, c, flag) == pytest.approx(c, abs=1e-15)
        assert oracle_lib.scheme(1, c, c, c, c, flag) == pytest.approx(c, abs=1e-15)
    if flag in (2, 5):
        u = [1.0, 2.0, 3.0, 4.0]
        assert oracle_lib.scheme(0, *u, flag) == pytest.approx(2.5, rel=1e-6)
        assert oracle_lib.scheme(1, *u, flag) == pytest.approx(2.5, rel=1e-6)


def test_minmod_limiters_tvd(oracle_lib):
    """NND2 and MUSCL2 (minmod) return the first-order value at extrema."""
    for flag in (1, 4):
        assert oracle_lib.scheme(0, 0.0, 1.0, 0.0, 1.0, flag) == pytest.approx(1.0)
        assert oracle_lib.scheme(1, 0.0, 1.0, 0.0, 1.0, flag) == pytest.approx(0.0)


@pytest.mark.parametrize("recon", [0, 1, 2])
@pytest.mark.parametrize("iflux", [1, 4, 5, 6])
def test_freestream_preservation(oracle_lib, recon, iflux):
    """A uniform state on a closed multi-block C-grid (wall replaced by far
    field) gives a zero inviscid residual to round-off: the face normals
    times lengths of every cell sum to zero (sub_init.f90:188-204)."""
    p, bl = small_case(nx=65, ny=17, nblocks=2, Ma=0.7, AoA=3.0, IFlag_Reconstruction=recon, Iflag_flux=iflux,
                       Iflag_Scheme=5, Time_Method=1)
    for b in bl:  # wall -> far field, so every ghost cell holds the freestream
        for s in b.bc:
            if s[6] == -10:
                s[6] = -20
    orc = make_oracle(p, bl)
    orc.init_flow()
    orc.residual()
    # scale: mass flux * typical face length
    for b in (1, 2):
        nx, ny = orc.dims(1, b)
        r = orc.field(1, b, 0, (4, nx - 1, ny - 1))
        si = orc.field(1, b, 12, (nx, ny))
        # far-field ghost states are freestream as well, so every face sees
        # the same state and the residual vanishes
        assert np.max(np.abs(r)) < 1e-12 * 10.0 * si.max() * 10.0


def test_restriction_conserves_residual(oracle_lib):
    """interpolation2h(flag 2) sums the four children: the coarse forcing
    before -R_2h conserves the fine residual (sub_NS_multigrid.f90:381-395)."""
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Num_Mesh=3, Time_Method=1, Iflag_flux=4, Iflag_Scheme=5,
                       CFL=1.0)
    orc = make_oracle(p, bl)
    orc.init_flow()
    orc.step(3)
    orc.residual(1)
    orc.interpolation2h(1, 2, 2)
    nx, ny = orc.dims(1, 1)
    rf = orc.field(1, 1, 0, (4, nx - 1, ny - 1))
    cx, cy = orc.dims(2, 1)
    qf = orc.field(2, 1, 19, (4, cx - 1, cy - 1))
    np.testing.assert_allclose(qf.sum(axis=(1, 2)), rf.sum(axis=(1, 2)), rtol=1e-10, atol=1e-13)


def test_volume_weighted_restriction_of_constant(oracle_lib):
    """Restricting a uniform U with volume weights returns the same U."""
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Num_Mesh=2, Time_Method=1)
    orc = make_oracle(p, bl)
    orc.init_flow()
    U = orc.get_U(1, 1)
    U[:] = np.array([1.0, 0.9, 0.1, 2.5])[:, None, None]
    orc.set_U(1, 1, U)
    orc.interpolation2h(1, 2, 1)
    Uc = orc.get_U(2, 1)
    cx, cy = orc.dims(2, 1)
    nx, ny = orc.dims(1, 1)
    vf = orc.field(1, 1, 11, (nx, ny))[:nx - 1, :ny - 1]
    vc = orc.field(2, 1, 11, (cx, cy))[:cx - 1, :cy - 1]
    # the coarse value is U * (sum of the four child areas) / (coarse area);
    # on a curved grid the coarse quadrilateral is not the union of its children
    ratio = (vf[0::2, 0::2] + vf[0::2, 1::2] + vf[1::2, 0::2] + vf[1::2, 1::2]) / vc
    np.testing.assert_allclose(Uc[:, 2:cx + 1, 2:cy + 1], U[:, 2:3, 2:3] * ratio[None], rtol=1e-13)
    assert np.abs(ratio - 1.0).max() < 0.5


def test_symmetric_airfoil_zero_lift(oracle_lib):
    """NACA 0012 at AoA = 0 with a pointwise (RK3) update: lift and moment
    stay zero to round-off by the mirror symmetry of grid, scheme and force
    integration.  (LU-SGS sweeps in i+j order are not mirror-symmetric, so
    there the symmetry is only reached at convergence.)"""
    p, bl = small_case(nx=65, ny=17, Ma=0.5, AoA=0.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=3, CFL=1.0)
    orc = make_oracle(p, bl)
    orc.init_flow()
    orc.step(120)
    cl, cd, cm = orc.forces()
    assert abs(cl) < 1e-12 and abs(cm) < 1e-12


def test_lusgs_converges_euler_small(oracle_lib):
    """The single-grid LU-SGS loop drives the residual down on a small
    C-grid (a regression check of the time-marching restatement)."""
    p, bl = small_case(nx=65, ny=17, Ma=0.5, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0, CFL=5.0)
    orc = make_oracle(p, bl)
    orc.init_flow()
    orc.step(1)
    r0 = orc.norms()[1][0]
    orc.step(300)
    r1 = orc.norms()[1][0]
    assert r1 < 1e-2 * r0


def test_reference_rae2822_case_runs(oracle_lib):
    """The reference's own RAE2822 grid and connectivity (3 blocks, wake cut
    j-/j- reversed) parse and run: Euler LU-SGS drives the residual down."""
    from conftest import reference_file
    from ec2d import inputs
    reference_file("Mesh2d.dat")
    p, blocks = inputs.read_case(os.path.dirname(reference_file("control.in")))
    assert [b.nx for b in blocks] == [33, 305, 33] and all(b.ny == 65 for b in blocks)
    p = p.replace(If_viscous=0, Iflag_turbulence_model=0, Iflag_flux=4, IFlag_Reconstruction=0, CFL=3.0)
    orc = make_oracle(p, blocks, threads=8)
    orc.init_flow()
    orc.step(1)
    r0 = orc.norms()[1][0]
    orc.step(100)
    assert orc.norms()[1][0] < r0


def test_flat_plate_converged_cf_is_blasius():
    """The oracle's converged laminar flat plate (the committed fixture:
    2 x 97x97, Re 1e4 per unit length, M 0.3, 1e-8 drop) against the Blasius
    solution: wall skin friction within 3 % of 0.664 / sqrt(Re_x) over
    x = 0.2..0.9 (measured 0.6-2.1 %), drag within 5 % of 1.328 / sqrt(Re)
    (measured 3.3 %, the leading edge included)."""
    import json
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "converged.json")) as fh:
        fx = json.load(fh)["flat_plate"]
    cf, xc = np.array(fx["wall"]["cf"]), np.array(fx["wall"]["xc"])
    m = (xc > 0.2) & (xc < 0.9)
    blasius = 0.664 / np.sqrt(1.0e4 * xc[m])
    assert np.max(np.abs(cf[m] / blasius - 1.0)) <= 0.03
    assert abs(fx["forces"]["cd"] / (1.328 / np.sqrt(1.0e4)) - 1.0) <= 0.05
    assert fx["reached"] and fx["iterations"] == 6751


def test_mg_eddy_viscosity_keeps_turbulent_cycle_stable():
    """A transonic SA case of the polar family (case 62: 257x65 C-grid,
    M 0.716, AoA 6.35, Re 4.2e6) under the 3-level LU-SGS V-cycle from the
    freestream: with laminar coarse levels (the reference's
    Comput_Residual_one_mesh zeroes Amu_t, sub_Residual.f90:158-191) the
    cycle stops on T < 1e-5 in the wake next to the cut after about 750
    V-cycles (measured: 751); with the coarse levels keeping the eddy
    viscosity restricted from the finer level it runs on."""
    import oracle
    from ec2d import cases
    p, bl, _ = cases.polar_cases(64, with_tc=True)[62]
    orc = oracle.Oracle(p, bl, threads=8, fast=True)
    orc.init_flow()
    with pytest.raises(RuntimeError, match="code 2"):
        orc.step(1000)
    orc = oracle.Oracle(p, bl, threads=8, fast=True)
    orc.set_mg_amut(True)
    orc.init_flow()
    orc.step(1)
    r0 = orc.norms()[1][0]
    orc.step(999)
    assert np.isfinite(orc.norms()[1][0]) and orc.norms()[1][0] < r0


def test_dual_time_start_is_the_whole_history(oracle_lib):
    """orc_dual_time_start makes U(n) = U(n-1) = U and the next physical step
    the one-step form: an oracle handed a developed state and started there
    steps exactly as the oracle that developed it and was started there; one
    left with the freestream history of its own start steps differently."""
    p, bl = small_case(Ma=0.5, AoA=3.0, Re=5e3, If_viscous=1, Iflag_flux=4, Iflag_Scheme=5, Time_Method=-1,
                       CFL=5.0, dt_global=0.05, Nstep_Inner_Limit=4, Res_Inner_Limit=1e-12)
    a = make_oracle(p, bl)
    a.init_flow()
    a.step(2)
    state = a.get_U(1, 1)
    b, c = make_oracle(p, bl), make_oracle(p, bl)
    for o in (b, c):
        o.init_flow()
        o.set_U(1, 1, state)
    a.dual_time_start()
    b.dual_time_start()
    for o in (a, b, c):
        o.step(1)
    np.testing.assert_array_equal(a.get_U(1, 1), b.get_U(1, 1))
    assert not np.array_equal(a.get_U(1, 1), c.get_U(1, 1))
