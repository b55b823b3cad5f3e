"""The measured cost model behind the latency-bound kernels (no reference
counterpart): the FP64 FMA throughput of the device and the cycles of
dependent FP64 and FP32 operations per warp.  Checked as orderings and
ranges that the kernels' design relies on, not as exact figures: a
dependent FP64 operation costs tens of cycles, an order of magnitude more
than an FP32 one; a divide costs several FMAs and the refined reciprocal
fewer than a divide; more independent chains per thread do not make a
warp's FP64 instructions cheaper."""
import pytest

pytestmark = pytest.mark.gpu


def test_fp64_cost_model(gpu_lib):
    from ec2d import gpu
    fma = gpu.measure_op_cycles(0, 1, 1)
    assert 16.0 <= fma <= 256.0
    assert gpu.measure_op_cycles(3, 1, 1) * 4.0 < fma           # FP32 fma
    div, rcp = gpu.measure_op_cycles(1, 1, 1), gpu.measure_op_cycles(2, 1, 1)
    assert div > 3.0 * fma and rcp < div
    assert gpu.measure_op_cycles(0, 1, 8) >= 0.8 * fma          # no overlap of one warp's FP64 work
    with pytest.raises(gpu.EC2DError):
        gpu.measure_op_cycles(0, 33, 1)
    assert gpu.measure_fp64_peak() > 0.1
    # a cluster barrier costs more than a CTA barrier
    assert gpu.measure_op_cycles(5, 1, 4) > gpu.measure_op_cycles(4, 4, 1)


def test_refined_reciprocal_within_an_ulp(gpu_lib):
    """rcp<double> of the face and wavefront paths (the hardware
    approximation refined by one third-order step) against the IEEE quotient
    on 4 M inputs: the approximation within 2^-19 relative, the refined
    value within one ulp."""
    from ec2d import gpu
    rel, ulps = gpu.check_reciprocal(4_000_000)
    assert 0.0 < rel < 2.0 ** -19
    assert ulps <= 1.0
