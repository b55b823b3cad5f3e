"""GPU parity: the CUDA path (through the C-ABI) against the CPU oracle on
the same seeded inputs.

Tolerances (FP64): one residual evaluation matches per cell within 1e-12
relative to the larger of |Res| and the cell's face-flux scale; pointwise
fields (primitives, spectral radii, dt, ghost cells, dU) within 1e-12
relative; multi-step states within the bounds stated per test."""
import numpy as np
import pytest

from helpers import (compare_U, compare_fields, compare_residual, copy_state, make_gpu, make_oracle,
                     perturb_state, small_case)

pytestmark = pytest.mark.gpu

GEOM = [9, 10, 11, 12, 13, 14, 15, 16, 17, 22, 23]  # x1 y1 vol si sj ni1 ni2 nj1 nj2 x y


def _pair(p, blocks, fdm=(), steps=0, perturb=True, seed=1):
    orc = make_oracle(p, blocks, fdm=fdm)
    orc.init_flow()
    if steps:
        orc.step(steps)
    if perturb:
        perturb_state(orc, seed=seed)
    g = make_gpu(p, blocks, fdm=fdm)
    g.init_flow()
    copy_state(orc, g)
    return orc, g


def test_geometry_all_levels(gpu_lib):
    p, bl = small_case(nx=65, ny=17, nblocks=2, Num_Mesh=3, Time_Method=1)
    orc = make_oracle(p, bl)
    g = make_gpu(p, bl)
    assert g.num_mesh == orc.num_mesh == 3
    for mesh in (1, 2, 3):
        compare_fields(orc, g, GEOM, mesh=mesh, tol=1e-13)


@pytest.mark.parametrize("case", ["cgrid4", "flat_plate", "rans513"])
def test_device_setup_geometry_bit_identical(gpu_lib, case):
    """The set-up kernels (node skipping, areas, faces, ghost nodes across
    block interfaces and physical faces, corners, cell centres) reproduce the
    oracle's geometry bit for bit on every multigrid level."""
    from ec2d import cases
    if case == "cgrid4":
        p, bl = small_case(nx=129, ny=33, nblocks=4, Num_Mesh=3, Time_Method=1)
    elif case == "flat_plate":
        p, bl = cases.laminar_flat_plate(97, 97, num_mesh=3)
    else:
        p, bl, _ = cases.rans_naca2412()
    orc = make_oracle(p, bl)
    g = make_gpu(p, bl)
    assert g.num_mesh == orc.num_mesh == 3
    for mesh in (1, 2, 3):
        for b in range(1, len(bl) + 1):
            for f in GEOM:
                np.testing.assert_array_equal(g.field(1, mesh, b, f), orc.field(mesh, b, f),
                                              err_msg=f"mesh {mesh} block {b} field {f}")
    g.close()


@pytest.mark.parametrize("kind", ["euler_roe_char", "viscous_ausm_cons", "mg3_flat_plate", "sa_coarse_levels"])
def test_tile_residual_equals_chain(gpu_lib, monkeypatch, kind):
    """The one-kernel residual over shared-memory tiles (EC2D_TILE_RESIDUAL=1,
    used where no turbulence model or FDM patch is on the level) against the
    four-kernel chain (0, the default) on the same state: Res, spectral radii,
    dt, mu and the norms of one evaluation, then U after a few steps.  Both
    run the same face arithmetic; the agreement asked is 1e-13 of each
    field's scale."""
    from ec2d import cases
    if kind == "euler_roe_char":
        p, bl = small_case(nx=97, ny=33, Ma=0.7, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, IFlag_Reconstruction=2,
                           nblocks=2)
    elif kind == "viscous_ausm_cons":
        p, bl = small_case(nx=97, ny=33, Ma=0.5, AoA=3.0, Re=5e3, If_viscous=1, Iflag_flux=6, Iflag_Scheme=4,
                           IFlag_Reconstruction=1, nblocks=2)
    elif kind == "mg3_flat_plate":
        p, bl = cases.laminar_flat_plate(97, 97, num_mesh=3)
    else:  # SA: the fine level keeps the chain, the coarse levels take the tile kernel
        p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2,
                           Iflag_flux=4, Iflag_Scheme=5, first=2e-4, Num_Mesh=3, mg_lusgs=1, nblocks=2)
    orc = make_oracle(p, bl)
    orc.init_flow()
    orc.step(3)
    perturb_state(orc, seed=4)
    runs = []
    for tile in ("1", "0"):
        monkeypatch.setenv("EC2D_TILE_RESIDUAL", tile)
        g = make_gpu(p, bl)
        g.init_flow()
        copy_state(orc, g)
        g.residual()
        f = {fid: [g.field(1, 1, b, fid) for b in range(1, len(bl) + 1)] for fid in (0, 1, 2, 3, 4, 5, 7)}
        nrm = g.norms()[:2]
        g.step(4)
        U = [g.download_U(1, 1, b) for b in range(1, len(bl) + 1)]
        runs.append((f, nrm, U))
        g.close()
    (fa, na, Ua), (fb, nb, Ub) = runs
    for fid in fa:
        for a, b in zip(fa[fid], fb[fid]):
            sc = np.abs(b).max()
            assert np.max(np.abs(a - b)) <= 1e-13 * (sc if sc > 0 else 1.0), (kind, fid)
    np.testing.assert_allclose(na[1], nb[1], rtol=1e-13)
    np.testing.assert_allclose(na[0], nb[0], rtol=1e-12)
    for a, b in zip(Ua, Ub):
        for m in range(a.shape[0]):
            assert np.max(np.abs(a[m] - b[m])) <= 1e-12 * np.abs(b[m]).max(), (kind, m)
    # and the tile path against the oracle, one evaluation at 1e-12 per cell
    monkeypatch.setenv("EC2D_TILE_RESIDUAL", "1")
    g = make_gpu(p, bl)
    g.init_flow()
    copy_state(orc, g)
    orc.residual()
    g.residual()
    compare_residual(orc, g)
    compare_fields(orc, g, [1, 2, 3, 4, 5] + ([7] if p.If_viscous else []))
    g.close()


@pytest.mark.parametrize("flux", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("recon", [0, 1, 2])
def test_residual_inviscid(gpu_lib, flux, recon):
    p, bl = small_case(Ma=0.7, AoA=2.0, Iflag_flux=flux, IFlag_Reconstruction=recon, Iflag_Scheme=5)
    orc, g = _pair(p, bl, steps=5)
    orc.residual(); g.residual()
    compare_residual(orc, g)
    compare_fields(orc, g, [1, 2, 3, 4, 5])


@pytest.mark.parametrize("scheme", [0, 1, 2, 3, 4, 5, 6])
def test_residual_schemes(gpu_lib, scheme):
    p, bl = small_case(Ma=0.6, AoA=1.0, Iflag_flux=4, IFlag_Reconstruction=0, Iflag_Scheme=scheme)
    orc, g = _pair(p, bl, steps=3)
    orc.residual(); g.residual()
    compare_residual(orc, g)


@pytest.mark.parametrize("recon", [0, 2])
def test_residual_viscous(gpu_lib, recon):
    p, bl = small_case(Ma=0.5, AoA=3.0, Re=5.0e3, If_viscous=1, Iflag_flux=6, IFlag_Reconstruction=recon,
                       Iflag_Scheme=5, nblocks=2)
    orc, g = _pair(p, bl, steps=5)
    orc.residual(); g.residual()
    compare_residual(orc, g)
    compare_fields(orc, g, [1, 2, 3, 4, 5, 7])


def test_residual_sa(gpu_lib):
    p, bl = small_case(Ma=0.6, AoA=2.0, Re=1.0e6, If_viscous=1, Iflag_turbulence_model=2, Iflag_flux=4,
                       Iflag_Scheme=5, first=2e-4)
    orc, g = _pair(p, bl, steps=5)
    compare_fields(orc, g, [18], tol=1e-13)  # wall distance
    orc.residual(); g.residual()
    compare_residual(orc, g)
    compare_fields(orc, g, [1, 2, 3, 4, 5, 7, 8])


def test_residual_sst(gpu_lib):
    p, bl = small_case(Ma=0.6, AoA=2.0, Re=1.0e6, If_viscous=1, Iflag_turbulence_model=3, Iflag_flux=4,
                       Iflag_Scheme=5, first=2e-4, Kt_inf=1e-6, Wt_inf=1e-2)
    orc, g = _pair(p, bl, steps=5)
    orc.residual(); g.residual()
    compare_residual(orc, g)
    compare_fields(orc, g, [1, 2, 3, 7])
    # mu_t from k, omega, the blending F2 and the vorticity limiter: the
    # primitives' last-ulp differences (reciprocal-multiply against the
    # oracle's divides) grow to ~1e-11 there, and to ~1e-12 in Lv = f(mu_t)
    compare_fields(orc, g, [4, 5, 8], tol=1e-10)


@pytest.mark.parametrize("visc", [0, 1])
def test_residual_fdm_weno5(gpu_lib, visc):
    p, bl = small_case(nx=97, ny=33, Ma=0.6, AoA=1.5, Re=1.0e4, If_viscous=visc, Iflag_flux=4, Iflag_Scheme=5,
                       nblocks=2)
    orc, g = _pair(p, bl, fdm=(1, 2), steps=3)
    orc.residual(); g.residual()
    compare_residual(orc, g)


def test_boundary_and_halo(gpu_lib):
    p, bl = small_case(Ma=0.7, AoA=4.0, nblocks=2, If_viscous=0)
    orc, g = _pair(p, bl, steps=2)
    orc.bc(); g.bc()
    compare_U(orc, g, tol=1e-15)
    orc.halo(); g.halo()
    compare_U(orc, g, tol=1e-15)


def test_boundary_wall_isothermal_symmetry_sa(gpu_lib):
    from ec2d import grids
    from ec2d.inputs import Params
    bl = grids.flat_plate(33, 17, first=1e-3, ratio=1.2)
    p = Params(Ma=0.3, Re=1e4, If_viscous=1, Iflag_turbulence_model=2, Twall=300.0, Iflag_flux=6, Iflag_Scheme=5)
    orc, g = _pair(p, bl, steps=2)
    orc.bc(); g.bc(); orc.halo(); g.halo()
    compare_U(orc, g, tol=1e-14)


# NV = 4 (default shape): 16, 40 and 70 rows per block run eight lanes per
# row in bands of 8, 10 and 12 rows on clusters of 2, 4 and 6 CTAs (the last
# band short).  NV = 5 (SA) and 6 (SST) take the same eight-lane bands, the
# turbulence rows carried by every lane.
@pytest.mark.parametrize("ny", [17, 41, 71])
@pytest.mark.parametrize("turb", [0, 2, 3])
def test_lusgs_sweep(gpu_lib, ny, turb):
    kw = dict(Ma=0.7, AoA=2.0, nblocks=2, If_viscous=1, Re=1e4, Iflag_flux=4, ny=ny)
    nv = 4
    if turb == 2:
        kw.update(Iflag_turbulence_model=2, Re=1e6, first=2e-4); nv = 5
    if turb == 3:
        kw.update(Iflag_turbulence_model=3, Re=1e6, first=2e-4, Kt_inf=1e-6, Wt_inf=1e-2); nv = 6
    p, bl = small_case(**kw)
    orc, g = _pair(p, bl, steps=3)
    orc.residual()
    # identical inputs on both sides: Res, dt and spectral radii from the oracle
    for b in (1, 2):
        for f in (0, 1, 2, 3, 4, 5):
            g.set_field(1, 1, b, f, orc.field(1, b, f))
    for b in (1, 2):
        orc.lusgs(1, b, 0.0)
    g.lusgs(1, 0.0)
    # dU = (Res + dui + duj)/alfa with dui built from F(U+dU) - F(U) and the
    # dissipation (0.5 Lc + Lv) dU of the upstream neighbours: the round-off
    # of those sums scales with the magnitudes added, F(U) s / alfa and
    # (0.5 Lc + Lv) U_nb / alfa, i.e. with |U| of the cell and of its
    # neighbours (and with p in the momentum and energy rows, where F carries
    # p n and (E + p) un), not with |dU|, and it accumulates along the sweep's
    # dependency chain, one rounding of those magnitudes per hyperplane at
    # most.  Per cell: |ddU_m| <= 1e-12 |dU_m| + eps (nx + ny) S_m with eps =
    # 2^-52, nx + ny the planes of a sweep and S_m = max |U_m| over the cell
    # and its four neighbours (+ p for m = 1..3).  The SST omega row sums
    # source and flux terms thousands of times its increment next to walls:
    # its relative term is 2e-12 (the row reached 0.9-1.1e-12 with either
    # accumulation order of the wavefront).
    worst = 0.0
    for b in (1, 2):
        nx, ny = orc.dims(1, b)
        chain = np.finfo(np.float64).eps * (nx + ny)
        a = orc.field(1, b, 6, (nv, nx, ny))[:, :nx - 1, :ny - 1]
        c = g.field(1, 1, b, 6, (nv, nx, ny))[:, :nx - 1, :ny - 1]
        Ug = np.abs(orc.get_U(1, b)[:nv])  # ghost-padded: interior at 2..nx, 2..ny
        Um = np.maximum.reduce([Ug[:, 2:nx + 1, 2:ny + 1], Ug[:, 1:nx, 2:ny + 1], Ug[:, 3:nx + 2, 2:ny + 1],
                                Ug[:, 2:nx + 1, 1:ny], Ug[:, 2:nx + 1, 3:ny + 2]])
        Uc = orc.get_U(1, b)[:4, 2:nx + 1, 2:ny + 1]
        pr = 0.4 * (Uc[3] - 0.5 * (Uc[1] ** 2 + Uc[2] ** 2) / Uc[0])
        S = Um.copy()
        S[1:4] += pr
        rel = np.full((nv, 1, 1), 1e-12)
        rel[4:] = 2e-12
        bound = rel * np.maximum(np.abs(a), np.abs(c)) + chain * S
        worst = max(worst, np.max(np.abs(a - c) / bound))
    assert worst <= 1.0, worst


@pytest.mark.parametrize("turb,ny,shape", [(0, 41, "auto"), (0, 71, "auto"), (0, 41, "four"), (0, 71, "four"),
                                           (0, 41, "one"), (0, 41, "barrier"), (2, 41, "auto"),
                                           (0, 97, "warp4"), (0, 97, "eight8"), (0, 97, "six8"), (0, 97, "six4")])
def test_lusgs_steps_wide_blocks(gpu_lib, monkeypatch, turb, ny, shape):
    """LU-SGS time steps on 40- to 96-row blocks (U updated inside the
    sweep) against the oracle, with each wavefront shape: auto (eight lanes
    per row in bands of at most 12 rows on a cluster for NV = 4, one lane per
    row otherwise), four lanes per row in bands of at most 24 rows, one CTA
    per block with one lane per row, a two-CTA cluster with a barrier per
    plane, and the narrow bands on clusters of 12 and 16 CTAs (8 rows with
    four lanes: one warp per CTA; 8 rows with eight lanes; 6 rows with eight
    or four lanes), where the device places such clusters."""
    monkeypatch.setenv("EC2D_LUSGS_CLUSTER", {"auto": "0", "four": "0", "one": "1", "barrier": "2"}.get(shape, "0"))
    monkeypatch.setenv("EC2D_LUSGS_ROWS", {"four": "24", "one": "32", "barrier": "32", "warp4": "8", "eight8": "8",
                                           "six8": "6", "six4": "6"}.get(shape, "12"))
    monkeypatch.setenv("EC2D_LUSGS_LANES", {"warp4": "4", "six4": "4", "eight8": "8", "six8": "8"}.get(shape, "0"))
    kw = dict(ny=ny, Ma=0.6, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0, CFL=5.0)
    if turb == 2:
        kw.update(If_viscous=1, Iflag_turbulence_model=2, Re=1e6, first=2e-4)
    p, bl = small_case(**kw)
    orc = make_oracle(p, bl)
    orc.init_flow()
    g = make_gpu(p, bl)
    g.init_flow()
    orc.step(15); g.step(15)
    compare_U(orc, g, tol=1e-10)


@pytest.mark.parametrize("tm", [0, 1, 3])
def test_steps_single_grid(gpu_lib, tm):
    p, bl = small_case(Ma=0.75, AoA=1.25, Iflag_flux=4, Iflag_Scheme=5, Time_Method=tm, CFL={0: 5.0, 1: 0.8, 3: 1.5}[tm])
    orc = make_oracle(p, bl)
    orc.init_flow()
    g = make_gpu(p, bl)
    g.init_flow()
    compare_U(orc, g, tol=1e-15)
    orc.step(20); g.step(20)
    compare_U(orc, g, tol=1e-10)
    a_o, r_o, k_o, t_o = orc.norms()
    a_g, r_g, k_g, t_g = g.norms()
    assert k_o == k_g == 20
    np.testing.assert_allclose(r_g, r_o, rtol=1e-8, atol=1e-300)


@pytest.mark.parametrize("tm", [1, 3, 0])
def test_multigrid_cycles(gpu_lib, tm):
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Iflag_flux=6, Iflag_Scheme=5, Time_Method=tm, Num_Mesh=3,
                       CFL={0: 4.0, 1: 0.8, 3: 1.5}[tm], Pre_Step_Mesh=(0, 5, 5), mg_lusgs=1, nblocks=2)
    orc = make_oracle(p, bl)
    orc.init_flow()
    g = make_gpu(p, bl)
    g.init_flow()
    assert g.num_mesh == 3
    compare_U(orc, g, tol=1e-11)
    orc.step(5); g.step(5)
    compare_U(orc, g, tol=1e-9)


def test_multigrid_eddy_viscosity_extension(gpu_lib):
    """The coarse-level eddy viscosity extension (ec2d_mg_eddy_viscosity; the
    oracle's set_mg_amut) on an SA case under the 3-level LU-SGS V-cycle:
    the fine U after 4 V-cycles within the multigrid bound, the coarse
    levels' eddy viscosity (restricted after the finer residual, then frozen)
    within 1e-9 of its scale and not zero, and the default still laminar."""
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2,
                       Iflag_flux=4, Iflag_Scheme=5, first=2e-4, Num_Mesh=3, mg_lusgs=1, nblocks=2,
                       Time_Method=0, CFL=2.0)
    orc = make_oracle(p, bl)
    orc.set_mg_amut(True)
    orc.init_flow()
    g = make_gpu(p, bl)
    assert g.mg_eddy_viscosity() == 0
    assert g.mg_eddy_viscosity(1) == 1
    g.init_flow()
    orc.step(4); g.step(4)
    compare_U(orc, g, tol=1e-9)
    for mesh in (2, 3):
        compare_fields(orc, g, [8], mesh=mesh, tol=1e-9)
        assert max(np.abs(g.field(1, mesh, b, 8)).max() for b in (1, 2)) > 0.0
    g.close()
    g = make_gpu(p, bl)
    g.init_flow()
    g.step(2)
    assert max(np.abs(g.field(1, 2, b, 8)).max() for b in (1, 2)) == 0.0
    g.close()


@pytest.mark.parametrize("nblocks", [1, 2])
def test_transfer_operators(gpu_lib, nblocks):
    """Each multigrid transfer against the oracle's reference routines on
    seeded random states (the operators are linear, so any state exercises
    every weight), levels 1 <-> 2 and 2 <-> 3: interpolation2h flags 1 and 2;
    the cycle's QF = sum Res_h - Res_2h (flag 6) against flag 2 then
    comput_force_function; prolong_U flags 1 and 2 over fine cells 0..nx,
    0..ny (the ghost ring included); the cycle's fused prolongation (flag 3)
    against comput_delt_U, prolong_U flag 2 and comput_new_U.  Within 1e-14
    of the field's largest value (FMA contraction on the GPU only)."""
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Num_Mesh=3, Time_Method=1, nblocks=nblocks)
    orc = make_oracle(p, bl)
    orc.init_flow()
    g = make_gpu(p, bl)
    g.init_flow()
    rng = np.random.default_rng(11 + nblocks)
    nb = len(bl)
    F_RES, F_QF, F_DELTU, F_UN = 0, 19, 20, 21

    def seed_U(mesh):
        for b in range(1, nb + 1):
            U = orc.get_U(mesh, b) * rng.uniform(0.8, 1.2, (orc.nvar(mesh), 1, 1)) + \
                rng.uniform(-0.05, 0.05, orc.get_U(mesh, b).shape)
            orc.set_U(mesh, b, U)
            g.upload_U(1, mesh, b, U)

    def seed_field(mesh, fid):
        for b in range(1, nb + 1):
            r = rng.standard_normal(orc.field(mesh, b, fid).size)
            assert g.field(1, mesh, b, fid).size == r.size
            orc.set_field(mesh, b, fid, r)
            g.set_field(1, mesh, b, fid, r)

    def same_field(mesh, fid):
        for b in range(1, nb + 1):
            a, c = orc.field(mesh, b, fid), g.field(1, mesh, b, fid)
            assert a.shape == c.shape
            np.testing.assert_allclose(c, a, rtol=0, atol=1e-14 * np.abs(a).max())

    for f, c in ((1, 2), (2, 3)):
        seed_U(f); seed_U(c)
        orc.interpolation2h(f, c, 1); g.interpolation2h(f, c, 1)
        compare_U(orc, g, mesh=c, tol=1e-14)
        seed_field(f, F_RES); seed_field(c, F_RES); seed_field(c, F_QF)
        orc.interpolation2h(f, c, 2); g.interpolation2h(f, c, 2)
        same_field(c, F_QF)
        orc.interpolation2h(f, c, 2); orc.force_function(c)
        g.interpolation2h(f, c, 6)
        same_field(c, F_QF)
        seed_U(f); seed_U(c)
        orc.prolong(c, f, 1); g.prolong(c, f, 1)
        compare_U(orc, g, mesh=f, tol=1e-14)
        seed_field(c, F_DELTU); seed_field(f, F_DELTU)
        orc.prolong(c, f, 2); g.prolong(c, f, 2)
        same_field(f, F_DELTU)
        seed_U(f); seed_U(c); seed_field(c, F_UN); seed_field(f, F_DELTU)
        orc.delt_u(c); orc.prolong(c, f, 2); orc.new_u(f)
        g.prolong(c, f, 3)
        same_field(f, F_DELTU)
        compare_U(orc, g, mesh=f, tol=1e-14)


def test_multigrid_viscous_lusgs_flat_plate(gpu_lib):
    from ec2d import cases
    p, bl = cases.laminar_flat_plate(33, 33, num_mesh=3)
    orc = make_oracle(p, bl)
    orc.init_flow()
    g = make_gpu(p, bl)
    g.init_flow()
    orc.step(4); g.step(4)
    compare_U(orc, g, tol=1e-9)


def test_norms_and_forces(gpu_lib):
    p, bl = small_case(Ma=0.5, AoA=3.0, Re=2e3, If_viscous=1, Iflag_flux=4, Iflag_Scheme=5)
    orc, g = _pair(p, bl, steps=10, perturb=False)
    orc.residual(); g.residual()
    a_o, r_o, _, _ = orc.norms()
    a_g, r_g, _, _ = g.norms()
    np.testing.assert_allclose(a_g, a_o, rtol=1e-12)
    np.testing.assert_allclose(r_g, r_o, rtol=1e-12)
    fo = np.array(orc.forces())
    fg = np.array(g.forces())
    np.testing.assert_allclose(fg, fo, rtol=1e-11, atol=1e-13)
    cfo, xo = orc.wall_cf(1, 3)
    cfg, xg = g.wall_cf(1, 1, 3)
    np.testing.assert_allclose(cfg, cfo, rtol=1e-10, atol=1e-13)


def test_batch_equals_single(gpu_lib):
    from ec2d import gpu
    p1, bl1 = small_case(Ma=0.6, AoA=1.0, Iflag_flux=4, Iflag_Scheme=5)
    p2, bl2 = small_case(nx=97, ny=17, Ma=0.7, AoA=3.0, Iflag_flux=4, Iflag_Scheme=5, nblocks=2)
    batch = gpu.Solver([(p1, bl1), (p2, bl2)])
    batch.init_flow(); batch.step(8)
    for ci, (p, bl) in enumerate([(p1, bl1), (p2, bl2)], start=1):
        one = gpu.Solver([(p, bl)])
        one.init_flow(); one.step(8)
        for b in range(1, len(bl) + 1):
            np.testing.assert_array_equal(batch.download_U(ci, 1, b), one.download_U(1, 1, b))
        np.testing.assert_array_equal(batch.norms(ci)[1], one.norms(1)[1])


def test_batch_equals_single_turbulent_multigrid(gpu_lib):
    """Two SA cases under the 3-level LU-SGS V-cycle with the coarse eddy
    viscosity kept (the polar's configuration), batched in one context and
    each alone: U and norms bit-identical, so the batch's V-cycle counts are
    the single runs'."""
    from ec2d import gpu
    kw = dict(Re=1e6, If_viscous=1, Iflag_turbulence_model=2, Iflag_flux=4, Iflag_Scheme=5, first=2e-4,
              Num_Mesh=3, mg_lusgs=1, Time_Method=0, CFL=2.0)
    cs = [small_case(Ma=0.6, AoA=1.0, **kw), small_case(nx=97, ny=17, Ma=0.7, AoA=3.0, nblocks=2, **kw)]
    batch = gpu.Solver(cs)
    batch.mg_eddy_viscosity(1)
    batch.init_flow(); batch.step(6)
    for ci, (p, bl) in enumerate(cs, start=1):
        one = gpu.Solver([(p, bl)])
        one.mg_eddy_viscosity(1)
        one.init_flow(); one.step(6)
        for b in range(1, len(bl) + 1):
            np.testing.assert_array_equal(batch.download_U(ci, 1, b), one.download_U(1, 1, b))
        np.testing.assert_array_equal(batch.norms(ci)[1], one.norms(1)[1])
        one.close()
    batch.close()


def test_symmetric_airfoil_zero_lift(gpu_lib):
    """NACA 0012 at AoA 0 with the pointwise RK3 update (an i+j LU-SGS sweep
    is not mirror-symmetric): the mirror symmetry of grid, scheme and force
    integration keeps CL and CM zero to round-off on the GPU, as on the
    oracle (test_oracle_kat)."""
    p, bl = small_case(nx=65, ny=17, Ma=0.5, AoA=0.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=3, CFL=1.0)
    g = make_gpu(p, bl)
    g.init_flow()
    g.step(120)
    cl, cd, cm = g.forces(1)
    assert abs(cl) < 1e-11 and abs(cm) < 1e-11
    g.close()
