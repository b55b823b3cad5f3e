"""Restart and snapshots.

* ec2d_snapshot: an asynchronous copy of a case's U (and eddy viscosity)
  taken between steps equals what a synchronous download at that step gives,
  bit for bit, while later steps run on.
* A binary checkpoint (download U, upload into a new context) continues
  bit-identically to the uninterrupted run.
* The Tecplot restart (init_flow_read, sub_init.f90:499-560) from the files
  `output` writes: the state comes back within the F20.10 format's rounding
  and the run continues from it; the reference's NVAR test at
  sub_init.f90:541 is kept unless fix_nvar is set.
* The Python main loop (ec2d.driver, opencfd_ec2d_v1.5.4.f90:142-186) writes
  its Kstep_save files from snapshots: they equal the files written from a
  synchronous read at the same step.
"""
import os

import numpy as np
import pytest

from helpers import make_gpu, small_case

pytestmark = pytest.mark.gpu


def _sa_case(**kw):
    return small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2, Iflag_flux=4,
                      Iflag_Scheme=5, first=2e-4, nblocks=2, **kw)


def test_snapshot_equals_synchronous_download(gpu_lib):
    p, bl = _sa_case()
    g = make_gpu(p, bl)
    g.init_flow()
    g.step(7)
    ref = [g.download_U(1, 1, b) for b in (1, 2)]
    amut = [g.field(1, 1, b, 8, (bl[b - 1].nx + 3, bl[b - 1].ny + 3)) for b in (1, 2)]
    g.snapshot(1)
    g.step(5)  # queued behind the snapshot's device copy
    case, kstep, _ = g.snapshot_wait()
    assert (case, kstep) == (1, 7)
    for b in (1, 2):
        np.testing.assert_array_equal(g.snapshot_U(b), ref[b - 1])
        np.testing.assert_array_equal(g.snapshot_amut(b), amut[b - 1])
    assert not np.array_equal(g.download_U(1, 1, 1), ref[0])
    # a second snapshot replaces the first
    now = [g.download_U(1, 1, b) for b in (1, 2)]
    g.snapshot(1)
    assert g.snapshot_wait()[1] == 12
    np.testing.assert_array_equal(g.snapshot_U(2), now[1])
    g.close()


def test_binary_checkpoint_continues_bit_identically(gpu_lib):
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Iflag_flux=6, Iflag_Scheme=5, Num_Mesh=3, mg_lusgs=1,
                       CFL=4.0, nblocks=2)
    a = make_gpu(p, bl)
    a.init_flow()
    a.step(6)
    saved = [a.download_U(1, 1, b) for b in (1, 2)]
    a.step(9)
    b_ = make_gpu(p, bl)
    b_.init_flow()
    for k, U in enumerate(saved, start=1):
        b_.upload_U(1, 1, k, U)
    b_.step(9)
    for k in (1, 2):
        np.testing.assert_array_equal(b_.download_U(1, 1, k), a.download_U(1, 1, k))
    a.close()
    b_.close()


def test_tecplot_restart_round_trip(gpu_lib, tmp_path):
    from ec2d import outputs
    p, bl = _sa_case()
    a = make_gpu(p, bl)
    a.init_flow()
    a.step(20)
    outputs.write_output(str(tmp_path), a, p, kstep=20)
    assert os.path.exists(tmp_path / "SA2d.dat")
    b_ = make_gpu(p, bl)
    # the reference's SA restart goes on to read SST2d.dat into U(5:6)
    with pytest.raises(outputs.RestartError):
        outputs.restart(b_, str(tmp_path))
    outputs.restart(b_, str(tmp_path), fix_nvar=True)
    for k in (1, 2):
        Ua, Ub = a.download_U(1, 1, k), b_.download_U(1, 1, k)
        nx, ny = bl[k - 1].nx, bl[k - 1].ny
        sl = (slice(None), slice(1, nx + 2), slice(1, ny + 2))
        # F20.10: absolute rounding 5e-11 on d, u, v, T, nu_tilde
        assert np.max(np.abs(Ua[sl] - Ub[sl])) <= 1e-9 * np.abs(Ua[sl]).max()
    a.step(10)
    b_.step(10)
    for k in (1, 2):
        Ua, Ub = a.download_U(1, 1, k), b_.download_U(1, 1, k)
        assert np.max(np.abs(Ua - Ub)) <= 1e-8 * np.abs(Ua).max()
    a.close()
    b_.close()


def test_tecplot_restart_sst_keeps_reference_behaviour(gpu_lib, tmp_path):
    from ec2d import outputs
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=3, Iflag_flux=4,
                       Iflag_Scheme=5, first=2e-4, Kt_inf=1e-6, Wt_inf=1e-2)
    a = make_gpu(p, bl)
    a.init_flow()
    fs = a.download_U(1, 1, 1)
    # two steps: on this coarse wall spacing the SST iteration grows omega
    # without bound within ten steps (the oracle does the same)
    a.step(2)
    outputs.write_output(str(tmp_path), a, p, kstep=2)
    Ua = a.download_U(1, 1, 1)
    nx, ny = bl[0].nx, bl[0].ny
    sl = (slice(4, 6), slice(2, nx + 1), slice(2, ny + 1))
    b_ = make_gpu(p, bl)
    outputs.restart(b_, str(tmp_path))  # sub_init.f90:541 never reads SST2d.dat: k, omega stay freestream
    np.testing.assert_array_equal(b_.download_U(1, 1, 1)[sl], fs[sl])
    outputs.restart(b_, str(tmp_path), fix_nvar=True)
    assert np.max(np.abs(b_.download_U(1, 1, 1)[sl] - Ua[sl])) <= 1e-9 * np.abs(Ua[sl]).max()
    a.close()
    b_.close()


def test_driver_writes_kstep_save_files_from_snapshots(gpu_lib, tmp_path):
    from ec2d import driver, gpu, inputs, outputs
    p, bl = _sa_case(Kstep_show=5, Kstep_save=10, t_end=1.0e9)
    d1, d2 = tmp_path / "run", tmp_path / "ref"
    inputs.write_case(str(d1), p, bl)
    r = driver.run(str(d1), steps=25, quiet=True)
    assert r["steps"] == 25 and r["kstep"] == 25
    recs = open(d1 / "Residual.dat").read().splitlines()
    assert [int(x[:8]) for x in recs] == [5, 10, 15, 20, 25]
    # the same steps, outputs written from synchronous reads
    os.makedirs(d2)
    g = gpu.Solver([(p, bl)])
    g.init_flow()
    for k in (10, 20):
        g.step(10)
        outputs.write_output(str(d2), g, p, kstep=k)
    g.close()
    for name in ("flow2d-0000010.dat", "flow2d-0000020.dat"):
        assert open(d1 / name).read() == open(d2 / name).read()


def test_dual_time_restart_starts_the_history_from_the_files(gpu_lib, tmp_path):
    """A dual-time restart: U(n) after outputs.restart is the restart state
    (ec2d_dual_time_start), not the freestream that init_flow set, and the
    next physical step starts from it in the one-step form, as the stepping
    of a context handed the same state does."""
    from ec2d import gpu, outputs
    p, bl = small_case(Ma=0.5, AoA=3.0, Re=5e3, If_viscous=1, Iflag_flux=4, Iflag_Scheme=5, Time_Method=-1,
                       CFL=5.0, dt_global=0.05, Nstep_Inner_Limit=6, Res_Inner_Limit=1e-12)
    a = make_gpu(p, bl)
    a.init_flow()
    a.step(3)
    outputs.write_output(str(tmp_path), a, p, kstep=3)
    b_ = make_gpu(p, bl)
    outputs.restart(b_, str(tmp_path))
    c = make_gpu(p, bl)
    c.init_flow()
    for k in range(1, len(bl) + 1):
        nx, ny, nv = b_.dims(1, 1, k)
        U = b_.download_U(1, 1, k)
        un = b_.field(1, 1, k, gpu.F_UN, shape=(nv, nx + 1, ny + 1))
        np.testing.assert_array_equal(un[:, 1:nx, 1:ny], U[:, 2:nx + 1, 2:ny + 1])
        c.upload_U(1, 1, k, U)
    c.dual_time_start()
    b_.step(2)
    c.step(2)
    for k in range(1, len(bl) + 1):
        np.testing.assert_array_equal(b_.download_U(1, 1, k), c.download_U(1, 1, k))
    for g in (a, b_, c):
        g.close()
