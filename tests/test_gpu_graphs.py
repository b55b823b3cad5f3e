"""CUDA-graph replay of ec2d_step against one-by-one kernel launches: the
same kernels in the same order, so the states must be bit-identical, and the
launch and step counters must advance the same way."""
import numpy as np
import pytest

from helpers import make_gpu, small_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tm,num_mesh", [(0, 1), (3, 1), (0, 3), (1, 2)])
def test_graph_replay_equals_direct(gpu_lib, tm, num_mesh):
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=tm,
                       Num_Mesh=num_mesh, CFL={0: 4.0, 1: 0.8, 3: 1.5}[tm], Pre_Step_Mesh=(0, 5, 5), mg_lusgs=1,
                       nblocks=2)
    runs = []
    for graphs in (False, True):
        g = make_gpu(p, bl)
        g.set_graphs(graphs)
        g.init_flow()
        n0 = g.launch_count()
        g.step(3)
        g.step(4)
        runs.append((g, g.launch_count() - n0))
    (a, na), (b, nb) = runs
    assert na == nb > 7
    for blk in range(1, len(bl) + 1):
        np.testing.assert_array_equal(b.download_U(1, 1, blk), a.download_U(1, 1, blk))
    ra, rb = a.norms(1), b.norms(1)
    np.testing.assert_array_equal(rb[0], ra[0])
    np.testing.assert_array_equal(rb[1], ra[1])
    assert rb[2] == ra[2] == 7
    assert rb[3] == ra[3]


def test_autotune_keeps_state_and_results(gpu_lib):
    """The autotuner restores U and the counters, and its choice changes only
    the launch configuration: the steps after it match an untuned solver to
    round-off (the banded wavefronts form the energy flux as H w - p cc and
    sum the neighbours in another order than the one-lane one, so the shapes
    differ in the last bits of U, whose entries are O(1))."""
    p, bl = small_case(nx=65, ny=17, Ma=0.6, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0,
                       Num_Mesh=3, CFL=4.0, Pre_Step_Mesh=(0, 5, 5), mg_lusgs=1, nblocks=2)
    a = make_gpu(p, bl)
    a.init_flow()
    a.step(2)
    u0 = [a.download_U(1, 1, b) for b in (1, 2)]
    k0 = a.norms(1)[2]
    cs, rpw, cc, ms = a.autotune(trial_steps=3)
    # the autotuner's candidates: bands of 6, 8, 12, 16, 24 or 32 rows (cs 0),
    # rows per warp of the one-CTA kernel (cs 1), clusters with a barrier
    assert cs in (0, 1, 2, 4, 8) and rpw in (6, 8, 12, 16, 24, 32) and cc in (0, 1) and ms > 0.0
    for b in (1, 2):
        np.testing.assert_array_equal(a.download_U(1, 1, b), u0[b - 1])
    assert a.norms(1)[2] == k0
    ref = make_gpu(p, bl)
    ref.init_flow()
    ref.step(2)
    a.step(4)
    ref.step(4)
    for b in (1, 2):
        np.testing.assert_allclose(a.download_U(1, 1, b), ref.download_U(1, 1, b), rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("num_mesh", [2, 3])
def test_concurrent_branches_bit_identical(gpu_lib, monkeypatch, num_mesh):
    """The concurrent graph branches (i- and j-face kernels; at each multigrid
    transfer the fine residual beside the restriction, coarse boundary
    conditions and coarse entry residual) write disjoint arrays, so U and the
    norms after a few V-cycles equal those of the one-stream order bit for
    bit."""
    p, bl = small_case(nx=65, ny=33, Ma=0.6, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0,
                       Num_Mesh=num_mesh, CFL=4.0, Pre_Step_Mesh=(0, 5, 5), mg_lusgs=1, nblocks=2)
    runs = []
    for conc in ("1", "0"):
        monkeypatch.setenv("EC2D_CONCURRENT", conc)
        g = make_gpu(p, bl)
        g.init_flow()
        g.step(4)
        runs.append(g)
    a, b = runs
    for blk in range(1, len(bl) + 1):
        np.testing.assert_array_equal(a.download_U(1, 1, blk), b.download_U(1, 1, blk))
    for mesh in range(1, num_mesh + 1):
        na, nb = a.norms(1, mesh), b.norms(1, mesh)
        np.testing.assert_array_equal(na[0], nb[0])
        np.testing.assert_array_equal(na[1], nb[1])
