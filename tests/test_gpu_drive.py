"""ec2d_run_to_drop (iterate to a residual drop, with timers): the steps it
takes are ordinary ec2d_step calls, so a second solver stepped by hand the
same number of times must hold the identical state and norms."""
import os

import numpy as np
import pytest

from helpers import make_gpu, small_case

pytestmark = pytest.mark.gpu


def test_run_to_drop_matches_manual_stepping(gpu_lib):
    p, bl = small_case(Ma=0.5, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, CFL=5.0)
    a = make_gpu(p, bl)
    a.init_flow()
    n, ratio, secs = a.run_to_drop(drop=0.2, max_steps=400, check_every=10)
    assert 1 < n <= 400 and secs > 0.0
    assert ratio <= 0.2 or n == 400
    b = make_gpu(p, bl)
    b.init_flow()
    b.step(1)
    r0 = b.norms()[1][0]
    b.step(n - 1)
    np.testing.assert_array_equal(a.norms()[1], b.norms()[1])
    assert b.norms()[1][0] / r0 == ratio
    np.testing.assert_array_equal(a.download_U(1, 1, 1), b.download_U(1, 1, 1))


def test_run_to_drop_limits(gpu_lib):
    p, bl = small_case(Ma=0.5, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, CFL=5.0)
    g = make_gpu(p, bl)
    g.init_flow()
    n, ratio, _ = g.run_to_drop(drop=1e-30, max_steps=37, check_every=10)
    assert n == 37 and ratio > 1e-30
    # a given reference residual: one check, no step needed when already below
    n2, ratio2, _ = g.run_to_drop(drop=1.0, r0=[1e30], max_steps=5, check_every=5)
    assert n2 == 5 or ratio2 <= 1.0


def test_output_files_from_the_device(gpu_lib, tmp_path):
    from ec2d import outputs
    p, bl = small_case(Ma=0.5, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2, Iflag_flux=4,
                       Iflag_Scheme=5, CFL=5.0, first=2e-4, nblocks=2)
    g = make_gpu(p, bl)
    g.init_flow()
    g.step(20)
    paths = outputs.write_output(str(tmp_path), g, p, kstep=20)
    assert [os.path.basename(x) for x in paths] == ["flow2d-0000020.dat", "flow2d.dat", "SA2d.dat"]
    names, zones = outputs.parse_tecplot(open(paths[1]).read())
    assert len(zones) == 2 and names[-1] == "Amut"
    U = g.download_U(1, 1, 2)
    nx, ny, _ = g.dims(1, 1, 2)
    np.testing.assert_allclose(zones[1][:, 2].reshape(ny + 1, nx + 1), U[0, 1:nx + 2, 1:ny + 2].T, atol=1e-10)


@pytest.mark.parametrize("method", ["lusgs_mg3", "dual"])
def test_init_flow_restarts_a_used_context(gpu_lib, method):
    """ec2d_init_flow on a context that has stepped starts as a new context
    does (the reference starts right after the mesh set-up): the coarse
    pre-steps, which add the coarse forcing, run with it zero; the dual-time
    first-step flags are unset; the counters are back at zero.  The steps
    after it are bit-identical to a new context's."""
    if method == "lusgs_mg3":
        p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0, Num_Mesh=3,
                           CFL=4.0, Pre_Step_Mesh=(0, 5, 5), mg_lusgs=1, nblocks=2)
    else:
        p, bl = small_case(Ma=0.5, AoA=3.0, Re=5e3, If_viscous=1, Iflag_flux=4, Iflag_Scheme=5, Time_Method=-1,
                           CFL=5.0, dt_global=0.05, Nstep_Inner_Limit=6, Res_Inner_Limit=1e-12)
    a = make_gpu(p, bl)
    a.init_flow()
    a.step(7)
    a.init_flow()
    a.step(4)
    b = make_gpu(p, bl)
    b.init_flow()
    b.step(4)
    for blk in range(1, len(bl) + 1):
        np.testing.assert_array_equal(a.download_U(1, 1, blk), b.download_U(1, 1, blk))
    na, nb = a.norms(), b.norms()
    np.testing.assert_array_equal(na[0], nb[0])
    np.testing.assert_array_equal(na[1], nb[1])
    assert na[2] == nb[2] == 4 and na[3] == nb[3]
    a.close()
    b.close()


def test_driver_wall_distance_file(gpu_lib, tmp_path):
    """An SA run of the main-loop driver without dist_wall.dat writes it (and
    dw.dat) from the distances formed on the device, bit for bit; a run whose
    case directory holds that file reads it and marches exactly as the first
    run did; a file with other distances changes the run (it is read)."""
    import shutil

    from ec2d import driver, gpu, inputs
    p, bl = small_case(Ma=0.5, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2, Iflag_flux=4,
                       Iflag_Scheme=5, CFL=5.0, first=2e-4, nblocks=2, Kstep_show=5, Kstep_save=1000, t_end=1.0e9)
    dims = [(b.nx, b.ny) for b in bl]
    dirs = [tmp_path / n for n in ("computed", "read", "scaled")]
    inputs.write_case(str(dirs[0]), p, bl)
    r0 = driver.run(str(dirs[0]), steps=10, quiet=True)
    assert os.path.exists(dirs[0] / "dist_wall.dat") and os.path.exists(dirs[0] / "dw.dat")
    dws = inputs.read_dist_wall(str(dirs[0] / "dist_wall.dat"), dims)
    g = make_gpu(p, bl)
    for k, (nx, ny) in enumerate(dims, start=1):
        np.testing.assert_array_equal(dws[k - 1], g.field(1, 1, k, gpu.F_DW, shape=(nx + 1, ny + 1))[1:nx, 1:ny])
    g.close()
    inputs.write_case(str(dirs[1]), p, bl)
    shutil.copy(dirs[0] / "dist_wall.dat", dirs[1] / "dist_wall.dat")
    r1 = driver.run(str(dirs[1]), steps=10, quiet=True)
    assert open(dirs[1] / "Residual.dat").read() == open(dirs[0] / "Residual.dat").read()
    assert r1["forces"] == r0["forces"] and not os.path.exists(dirs[1] / "dw.dat")
    inputs.write_case(str(dirs[2]), p, bl)
    inputs.write_dist_wall(str(dirs[2] / "dist_wall.dat"), [2.0 * d for d in dws], dims)
    driver.run(str(dirs[2]), steps=10, quiet=True)
    assert open(dirs[2] / "Residual.dat").read() != open(dirs[0] / "Residual.dat").read()
