"""Dual time stepping (Dual_time_LU_SGS, sub_NS_singlegrid.f90:231-310): the
physical-time source term of the residual (sub_Residual.f90:29-34,55-65) and
the inner LU-SGS loop with its residual exit test, GPU against the oracle."""
import numpy as np
import pytest

from helpers import compare_U, make_gpu, make_oracle, small_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("visc", [0, 1])
def test_dual_time_steps(gpu_lib, visc):
    p, bl = small_case(Ma=0.5, AoA=3.0, Re=5e3, If_viscous=visc, Iflag_flux=4, Iflag_Scheme=5, Time_Method=-1,
                       CFL=5.0, dt_global=0.05, Nstep_Inner_Limit=6, Res_Inner_Limit=1e-12)
    orc = make_oracle(p, bl)
    orc.init_flow()
    g = make_gpu(p, bl)
    g.init_flow()
    orc.step(3)
    g.step(3)
    compare_U(orc, g, tol=1e-10)
    a_o, r_o, k_o, t_o = orc.norms()
    a_g, r_g, k_g, t_g = g.norms()
    assert k_o == k_g == 3
    assert t_g == pytest.approx(t_o, rel=1e-15)
    np.testing.assert_allclose(r_g, r_o, rtol=1e-8, atol=1e-300)


def test_dual_time_start_from_a_developed_state(gpu_lib):
    """ec2d_dual_time_start against the oracle's: both take the oracle's state
    after three physical steps as U(n) = U(n-1), then take two more steps."""
    p, bl = small_case(Ma=0.5, AoA=3.0, Re=5e3, If_viscous=1, Iflag_flux=4, Iflag_Scheme=5, Time_Method=-1,
                       CFL=5.0, dt_global=0.05, Nstep_Inner_Limit=6, Res_Inner_Limit=1e-12)
    orc = make_oracle(p, bl)
    orc.init_flow()
    orc.step(3)
    g = make_gpu(p, bl)
    g.init_flow()
    for b in range(1, len(bl) + 1):
        g.upload_U(1, 1, b, orc.get_U(1, b))
    orc.dual_time_start()
    g.dual_time_start()
    orc.step(2)
    g.step(2)
    compare_U(orc, g, tol=1e-10)
