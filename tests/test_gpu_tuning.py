"""Launch choices through the C-ABI (ec2d_launch_config, ec2d_set_launch_config,
ec2d_launch_signature) and the autotuner cache over them (ec2d/tuning.py):
a context keyed by the same signature takes the stored choices without
timing and then steps exactly as the context that was tuned; the setter is
the same as the choices fixed by the EC2D_* variables at create, and a change
after steps drops the captured step graph."""
import ctypes

import numpy as np
import pytest

from helpers import make_gpu, small_case

pytestmark = pytest.mark.gpu


def _case(ny=17):
    return small_case(nx=65, ny=ny, Ma=0.6, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0, Num_Mesh=3,
                      CFL=4.0, Pre_Step_Mesh=(0, 5, 5), mg_lusgs=1, nblocks=2)


def _same_U(a, b, nblocks=2):
    for blk in range(1, nblocks + 1):
        np.testing.assert_array_equal(a.download_U(1, 1, blk), b.download_U(1, 1, blk))


def test_cached_choices_reproduce_the_tuned_run(gpu_lib, tmp_path):
    from ec2d import tuning
    path = str(tmp_path / "tuning.json")
    p, bl = _case()
    a = make_gpu(p, bl)
    sig = a.launch_signature()
    assert sig.startswith("ec2d-launch-1 ") and " sm=103 " in sig and " L3:nv4," in sig and " cases=1" in sig
    ra = tuning.autotune_cached(a, path, trial_steps=2)
    assert ra["source"] == "autotune" and ra["ms_per_step"] > 0.0
    b = make_gpu(p, bl)
    assert b.launch_signature() == sig
    rb = tuning.autotune_cached(b, path, trial_steps=2)
    assert rb["source"] == "cache"
    assert rb["config"] == ra["config"] == a.launch_config() == b.launch_config()
    for g in (a, b):
        g.init_flow()
        g.step(6)
    _same_U(a, b)
    c = make_gpu(*_case(ny=33))
    assert c.launch_signature() != sig
    b.set_lusgs_precision(32)
    assert b.launch_signature() == sig.replace(" lusgs=64 ", " lusgs=32 ") != sig
    for g in (a, b, c):
        g.close()


def test_setter_matches_create_time_choices(gpu_lib, monkeypatch):
    cfg = {"lusgs_cs": 1, "rows": 16, "lanes": 0, "concurrent": 0, "tile_residual": 1}
    p, bl = _case()
    x = make_gpu(p, bl)
    x.set_launch_config(cfg)
    assert x.launch_config() == cfg and x.lusgs_shape()[:2] == (1, 16) and x.tile_residual() == 1
    for k, v in (("EC2D_LUSGS_CLUSTER", "1"), ("EC2D_LUSGS_ROWS", "16"), ("EC2D_CONCURRENT", "0"),
                 ("EC2D_TILE_RESIDUAL", "1")):
        monkeypatch.setenv(k, v)
    y = make_gpu(p, bl)
    assert y.launch_config() == cfg
    for g in (x, y):
        g.init_flow()
        g.step(5)
    _same_U(x, y)
    x.close()
    y.close()


def test_change_after_steps_recaptures(gpu_lib):
    """Two contexts step twice with the default choices, then switch to the
    one-lane wavefront: one replays its new step graph, the other launches
    kernel by kernel; graph replay equals direct launches bit for bit, so
    they stay equal only if the switch dropped the old graph."""
    cfg = {"lusgs_cs": 1, "rows": 32, "lanes": 0, "concurrent": 1, "tile_residual": 0}
    p, bl = _case()
    x, y = make_gpu(p, bl), make_gpu(p, bl)
    for g in (x, y):
        g.init_flow()
        g.step(2)
        g.set_launch_config(cfg)
    y.set_graphs(False)
    x.step(3)
    y.step(3)
    _same_U(x, y)
    x.close()
    y.close()


def test_refusals(gpu_lib):
    p, bl = _case()
    g = make_gpu(p, bl)
    cfg = g.launch_config()
    L = g.L
    for bad in ((9, 12, 0, 1, 0), (-1, 12, 0, 1, 0), (0, 3, 0, 1, 0), (0, 33, 0, 1, 0), (0, 12, 6, 1, 0),
                (0, 12, 0, 2, 0), (0, 12, 0, 1, -1)):
        assert L.ec2d_set_launch_config(g.h, *bad) == 1, bad
    assert g.launch_config() == cfg
    n = ctypes.c_int()
    assert L.ec2d_launch_signature(g.h, None, 0, ctypes.byref(n)) == 0 and n.value > 60
    short = ctypes.create_string_buffer(8)
    assert L.ec2d_launch_signature(g.h, short, 8, ctypes.byref(n)) == 1
    assert L.ec2d_launch_signature(None, None, 0, ctypes.byref(n)) == 1
    g.close()


def test_driver_takes_the_cache(gpu_lib, tmp_path):
    """The main-loop driver with --tuning-cache: the first run times the
    candidates and stores them, the second run of the same case takes them
    from the file; both write the same residual records and end on the same
    coefficients."""
    import json

    from ec2d import driver, inputs
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0, Num_Mesh=3,
                       CFL=4.0, Pre_Step_Mesh=(0, 5, 5), mg_lusgs=1, nblocks=2, Kstep_show=5, Kstep_save=1000,
                       t_end=1.0e9)
    cache = str(tmp_path / "tuning.json")
    runs = []
    for name in ("first", "second"):
        d = tmp_path / name
        inputs.write_case(str(d), p, bl)
        runs.append((d, driver.run(str(d), steps=20, quiet=True, tuning_cache=cache)))
    (d1, r1), (d2, r2) = runs
    assert r1["tuning"]["source"] == "autotune" and r2["tuning"]["source"] == "cache"
    assert r1["tuning"]["config"] == r2["tuning"]["config"]
    assert len(json.load(open(cache))["entries"]) == 1
    assert r1["kstep"] == r2["kstep"] == 20 and r1["forces"] == r2["forces"]
    assert open(d1 / "Residual.dat").read() == open(d2 / "Residual.dat").read()


def test_autotune_restores_dual_time_levels(gpu_lib):
    """With dual time stepping the autotuner's trial steps advance the two
    physical time levels and the first-step flags; it restores them with U,
    so the steps after it equal those of a context given the same launch
    choices without trials, bit for bit."""
    p, bl = small_case(Ma=0.5, AoA=3.0, Re=5e3, If_viscous=1, Iflag_flux=4, Iflag_Scheme=5, Time_Method=-1,
                       CFL=5.0, dt_global=0.05, Nstep_Inner_Limit=6, Res_Inner_Limit=1e-12)
    a, b = make_gpu(p, bl), make_gpu(p, bl)
    for g in (a, b):
        g.init_flow()
        g.step(2)
    a.autotune(trial_steps=2)
    b.set_launch_config(a.launch_config())
    a.step(3)
    b.step(3)
    _same_U(a, b, nblocks=len(bl))
    na, nb = a.norms(), b.norms()
    np.testing.assert_array_equal(na[1], nb[1])
    assert na[2] == nb[2] == 5 and na[3] == nb[3]
    a.close()
    b.close()


def test_autotune_restores_status_words(gpu_lib):
    """Trial steps on a state that trips the T < 1e-5 test (a context not yet
    started: U is zero) set the case's status word; the autotuner restores
    it with U, so the stop is not reported for the restored state."""
    p, bl = _case()
    g = make_gpu(p, bl)
    assert g.status(1)[0] == 0
    g.autotune(trial_steps=1)
    assert g.status(1)[0] == 0
    g.init_flow()
    g.step(2)
    assert g.status(1)[0] == 0
    g.close()
