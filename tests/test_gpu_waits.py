"""Failure detection of the banded LU-SGS wavefront without a GPU fault.

The bands of a tall block hand their edge rows to the next band through
bounded waits.  With the band edges silenced (the EC2D_TEST_SILENT_BAND_EDGE
test hook read by ec2d_create) nothing arrives, every downstream wait runs
out after its poll limit, the case's status records the timeout, and the
next status read reports EC2D_ERR_TIMEOUT while the context keeps working."""
import numpy as np
import pytest

from helpers import make_gpu, small_case

pytestmark = pytest.mark.gpu

EC2D_ERR_TIMEOUT = 4


# Euler (4 variables) and SA (5: the SA row rides on the same bands and its
# inbox entries are 80 bytes)
CASES = {"euler": dict(), "sa": dict(If_viscous=1, Iflag_turbulence_model=2, Re=1e6, first=2e-4)}


@pytest.mark.parametrize("kind", ["euler", "sa"])
def test_band_edge_wait_runs_out(gpu_lib, monkeypatch, kind):
    from ec2d import gpu
    monkeypatch.setenv("EC2D_TEST_SILENT_BAND_EDGE", "1")
    monkeypatch.setenv("EC2D_LUSGS_CLUSTER", "0")  # banded wavefront, 40 rows: four bands of 10
    p, bl = small_case(ny=41, Ma=0.6, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0, CFL=5.0,
                       **CASES[kind])
    nv = 4 if kind == "euler" else 5
    g = make_gpu(p, bl)
    g.init_flow()
    g.step(1)
    with pytest.raises(gpu.EC2DError) as e:
        g.norms()
    assert e.value.code == EC2D_ERR_TIMEOUT
    code, blk, i, j = g.status()
    assert code == EC2D_ERR_TIMEOUT and blk >= 1 and i >= 1 and j >= 1
    # the context still answers: the state can be read back
    g.sync()
    assert g.download_U(1, 1, 1).shape[0] == nv
    g.close()
    # and the process's GPU context stays usable: with the hook cleared, a new
    # context in the same process steps with a clean status and finite U, and
    # its sweeps agree with a context that never saw the hook
    monkeypatch.delenv("EC2D_TEST_SILENT_BAND_EDGE")
    outs = []
    for _ in range(2):
        h = make_gpu(p, bl)
        h.init_flow()
        h.step(3)
        h.norms()
        assert h.status()[0] == 0
        outs.append(h.download_U(1, 1, 1))
        h.close()
    assert np.all(np.isfinite(outs[0]))
    np.testing.assert_array_equal(outs[0], outs[1])


def test_band_edges_deliver_without_the_hook(gpu_lib, monkeypatch):
    monkeypatch.delenv("EC2D_TEST_SILENT_BAND_EDGE", raising=False)
    monkeypatch.setenv("EC2D_LUSGS_CLUSTER", "0")
    p, bl = small_case(ny=41, Ma=0.6, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0, CFL=5.0)
    g = make_gpu(p, bl)
    g.init_flow()
    g.step(3)
    g.norms()  # raises on any recorded status
    assert g.status()[0] == 0
    assert np.all(np.isfinite(g.download_U(1, 1, 1)))
