"""Error behaviour of the C-ABI, with every failure made on the host.

* Inputs the library refuses with EC2D_ERR_ARG before any device work: a
  subface off its block face, a neighbour that does not exist, interface
  strips of different lengths, cases of one batch with different methods.
* The reference's refusals (opencfd_ec2d_v1.5.4.f90:216-221): LU-SGS inside
  multigrid without mg_lusgs, a turbulence model without viscosity ->
  EC2D_ERR_UNSUPPORTED.
* The T < 1e-5 stop (sub_Residual.f90:143-146) as a status word per case: a
  state with a negative internal energy uploaded into one case of a batch
  stops that case with EC2D_ERR_STATE and its block and cell, the other case
  steps on unchanged; replacing the state and clearing the status resumes it.
"""
import ctypes

import numpy as np
import pytest

from helpers import make_gpu, small_case

pytestmark = pytest.mark.gpu

EC2D_ERR_ARG, EC2D_ERR_STATE, EC2D_ERR_UNSUPPORTED = 1, 3, 5


def _solver_error(cases):
    from ec2d import gpu
    with pytest.raises(gpu.EC2DError) as e:
        gpu.Solver(cases)
    return e.value.code


def test_rejects_bad_subfaces_and_neighbours(gpu_lib):
    p, bl = small_case(nx=65, ny=17, nblocks=2)
    # a subface that leaves its face: i-range on face 1 (i = 1 only)
    bad = [[list(s) for s in b.bc] for b in bl]
    bad[0][0][3] = 5 if bad[0][0][1] == 1 else bad[0][0][3]
    b0 = type(bl[0])(bl[0].x, bl[0].y, bad[0])
    if bad[0][0][1] == 1:
        assert _solver_error([(p, [b0, bl[1]])]) == EC2D_ERR_ARG
    # a neighbour block that does not exist
    nb = [[list(s) for s in b.bc] for b in bl]
    k = next(k for k, s in enumerate(nb[0]) if s[6] > 0)
    nb[0][k][6] = 7
    assert _solver_error([(p, [type(bl[0])(bl[0].x, bl[0].y, nb[0]), bl[1]])]) == EC2D_ERR_ARG
    # a neighbour subface whose strip has another length
    ln = [[list(s) for s in b.bc] for b in bl]
    ln[0][k][7] = next(q + 1 for q, s in enumerate(ln[1]) if s[6] < 0)
    assert _solver_error([(p, [type(bl[0])(bl[0].x, bl[0].y, ln[0]), bl[1]])]) == EC2D_ERR_ARG


def test_rejects_mixed_methods_and_reference_refusals(gpu_lib):
    p1, bl1 = small_case(Iflag_flux=4)
    p2, bl2 = small_case(Iflag_flux=6)
    assert _solver_error([(p1, bl1), (p2, bl2)]) == EC2D_ERR_ARG
    p3, bl3 = small_case(Time_Method=0, Num_Mesh=3, mg_lusgs=0)
    assert _solver_error([(p3, bl3)]) == EC2D_ERR_UNSUPPORTED
    p4, bl4 = small_case(If_viscous=0, Iflag_turbulence_model=2)
    assert _solver_error([(p4, bl4)]) == EC2D_ERR_UNSUPPORTED


def test_bad_arguments_return_err_arg(gpu_lib):
    g = make_gpu(*small_case())
    L, h = g.L, g.h
    U = np.zeros(10)
    dp = U.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert L.ec2d_download_U(h, 2, 1, 1, dp) == EC2D_ERR_ARG    # no case 2
    assert L.ec2d_download_U(h, 1, 1, 3, dp) == EC2D_ERR_ARG    # no block 3
    assert L.ec2d_get_field(h, 1, 1, 1, 99, dp) == EC2D_ERR_ARG  # no field 99
    assert L.ec2d_set_lusgs_precision(h, 16) == EC2D_ERR_ARG
    assert L.ec2d_clear_status(h, 5) == EC2D_ERR_ARG
    g.close()


def test_t_stop_per_case_in_a_batch(gpu_lib):
    from ec2d import gpu
    p, bl = small_case(Ma=0.6, AoA=1.0, Iflag_flux=4, Iflag_Scheme=5)
    g = gpu.Solver([(p, bl), (p, bl)])
    ref = gpu.Solver([(p, bl)])
    for s in (g, ref):
        s.init_flow()
        s.step(3)
    U = g.download_U(2, 1, 1)
    good = U.copy()
    U[3, 10, 6] = 0.05 * U[3, 10, 6]  # energy below the kinetic part: T < 0 in cell (9, 5)
    g.upload_U(2, 1, 1, U)
    g.step(1)
    ref.step(1)
    with pytest.raises(gpu.EC2DError) as e:
        g.norms(2)
    assert e.value.code == EC2D_ERR_STATE
    code, blk, i, j = g.status(2)
    assert code == EC2D_ERR_STATE and blk == 1 and (i, j) == (9, 5)
    # case 1 is untouched by case 2's stop: bit-identical to the lone case
    np.testing.assert_array_equal(g.download_U(1, 1, 1), ref.download_U(1, 1, 1))
    assert g.status(1)[0] == 0
    # the host replaces the failed state and clears the stop: case 2 resumes
    g.upload_U(2, 1, 1, good)
    g.clear_status(2)
    g.step(2)
    assert g.status(2)[0] == 0 and np.all(np.isfinite(g.norms(2)[1][:4]))
    g.close()
    ref.close()
