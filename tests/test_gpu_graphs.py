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
