"""The wavefront shape changes rounding, not convergence.

A batch of many turbulent cases runs the one-lane LU-SGS wavefront (its
blocks leave no SMs for bands), a lone case the eight-lane bands; both keep
the reference's Gauss-Seidel order and differ only in the summation order
of a cell's neighbour terms.  The polar comparison takes a lone case's
V-cycle counts from the batch, so the two shapes must need the same
V-cycles to a drop: checked here on an SA case under the 3-level LU-SGS
cycle (coarse eddy viscosity kept, as in the polar) and on the laminar
flat plate."""
import pytest

from helpers import make_gpu, small_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["sa_mg3", "flat_plate_mg3"])
def test_one_lane_and_eight_lane_reach_the_drop_together(gpu_lib, monkeypatch, kind):
    from ec2d import cases
    if kind == "sa_mg3":
        # 40 rows per block: more than the four-lane one-CTA kernel takes,
        # so EC2D_LUSGS_CLUSTER=1 runs one lane per row
        p, bl = small_case(nx=65, ny=41, Ma=0.6, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2,
                           Iflag_flux=4, Iflag_Scheme=5, first=2e-4, Num_Mesh=3, mg_lusgs=1, nblocks=2,
                           Time_Method=0, CFL=2.0)
        drop = 1e-2
    else:
        p, bl = cases.laminar_flat_plate(97, 97, num_mesh=3)
        drop = 1e-4
    steps = {}
    for cs in ("1", "0"):  # one CTA per block with one lane per row; the eight-lane bands
        monkeypatch.setenv("EC2D_LUSGS_CLUSTER", cs)
        g = make_gpu(p, bl)
        g.mg_eddy_viscosity(1)
        g.init_flow()
        n, worst, _ = g.run_to_drop(drop=drop, max_steps=20000, check_every=5)
        assert worst <= drop
        steps[cs] = n
        g.close()
    assert abs(steps["1"] - steps["0"]) <= max(5, 0.01 * steps["0"]), steps
