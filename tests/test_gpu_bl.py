"""Baldwin-Lomax eddy viscosity (turbulence_model_BL, sub_turbulence_BL.f90)
on the GPU against the oracle.

Walls on all four block faces: a channel with walls on faces 2 and 4, the
same channel with the index directions swapped (walls on faces 1 and 3), the
C-grid airfoil (partial wall on face 2, two blocks) and the flat plate (wall
and symmetry floor in different blocks).  Two wall subfaces in one block
exercise the minimum taken where a second wall's lines cross cells set by the
first.  Amu_t must match to 1e-10 relative (the model's branches are discrete,
so a mismatch shows up as an O(1) jump, not as round-off; the primitives come
from a Newton-refined reciprocal of the density, an ulp or two from the
oracle's divide, and the F_max search and the Klebanoff factor carry that to
about 1e-11), and the residual to the standard 1e-12 face-flux-scaled bound."""
import numpy as np
import pytest

from helpers import compare_fields, compare_residual, compare_U, copy_state, make_gpu, make_oracle, perturb_state, \
    small_case

pytestmark = pytest.mark.gpu

AMU, AMUT = 7, 8


def _channel(nx=49, ny=33, swap=False, h=0.2, first=2e-3):
    from ec2d.grids import cell_volumes
    from ec2d.inputs import BC_FARFIELD, BC_WALL, Block
    xs = np.linspace(0.0, 1.0, nx)
    s = np.linspace(-1.0, 1.0, ny)
    ys = 0.5 * h * (1.0 + np.tanh(2.5 * s) / np.tanh(2.5))  # clustered at both walls
    if not swap:
        x = np.repeat(xs[:, None], ny, 1)
        y = np.repeat(ys[None, :], nx, 0)
        bc = [[1, 1, 1, 1, 1, ny, BC_FARFIELD, 0, 0], [2, 2, 1, nx, 1, 1, BC_WALL, 0, 0],
              [3, 3, nx, nx, 1, ny, BC_FARFIELD, 0, 0], [4, 4, 1, nx, ny, ny, BC_WALL, 0, 0]]
        blk = Block(x, y, bc)
    else:
        # i runs across the channel (towards -y), j downstream: right-handed
        x = np.repeat(xs[None, :], ny, 0)
        y = -np.repeat(ys[:, None], nx, 1)
        bc = [[1, 1, 1, 1, 1, nx, BC_WALL, 0, 0], [2, 2, 1, ny, 1, 1, BC_FARFIELD, 0, 0],
              [3, 3, ny, ny, 1, nx, BC_WALL, 0, 0], [4, 4, 1, ny, nx, nx, BC_FARFIELD, 0, 0]]
        blk = Block(x, y, bc)
    assert (cell_volumes(blk) > 0).all()
    return blk


def _params(**kw):
    from ec2d.inputs import Params
    base = dict(Ma=0.3, AoA=0.0, Re=2.0e6, If_viscous=1, Iflag_turbulence_model=1, Iflag_flux=4, Iflag_Scheme=5,
                Time_Method=0, CFL=2.0)
    base.update(kw)
    return Params(**base)


def _check(p, blocks, steps=4, seed=3):
    orc = make_oracle(p, blocks)
    orc.init_flow()
    orc.step(steps)
    perturb_state(orc, seed=seed, amp=0.01)
    g = make_gpu(p, blocks)
    g.init_flow()
    copy_state(orc, g)
    orc.residual(); g.residual()
    compare_fields(orc, g, [AMU], tol=1e-13)
    compare_fields(orc, g, [AMUT], tol=1e-10)
    compare_residual(orc, g)
    return orc, g


@pytest.mark.parametrize("swap", [False, True])
def test_bl_channel_walls_every_face(gpu_lib, swap):
    orc, g = _check(_params(), [_channel(swap=swap)])
    at = g.field(1, 1, 1, AMUT)
    assert np.abs(at).max() > 0.0


def test_bl_airfoil_two_blocks(gpu_lib):
    p, bl = small_case(Ma=0.6, AoA=2.0, Re=3.0e6, If_viscous=1, Iflag_turbulence_model=1, Iflag_flux=4,
                       Iflag_Scheme=5, first=2e-4, nblocks=2)
    _check(p, bl)


def test_bl_flat_plate_steps(gpu_lib):
    from ec2d import cases
    p, bl = cases.laminar_flat_plate(33, 33, num_mesh=1)
    p.Re = 1.0e6
    p.Iflag_turbulence_model = 1
    orc = make_oracle(p, bl)
    orc.init_flow()
    g = make_gpu(p, bl)
    g.init_flow()
    orc.step(6); g.step(6)
    compare_U(orc, g, tol=1e-10)
