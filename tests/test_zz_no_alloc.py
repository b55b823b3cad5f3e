"""The allocation-free residual-norm entry point (ec2d_residual_norms_noalloc).

It exists for hosts that cannot call cudaMalloc -- e.g. a Fortran/OpenACC
host whose device memory belongs to another allocator, or a host that must
not allocate after start-up -- and already hold the residual on the device.
Its tile partials live in a fixed file-scope device array, so this test
checks it against the context-based entry point (ec2d_residual) on two calls
in a row, plus the size limit.  Collected last on purpose (test_zz_*)."""
import ctypes

import numpy as np
import pytest

from helpers import make_gpu, small_case

pytestmark = pytest.mark.gpu


def _noalloc(lib, dev_res, nvar, ncell, dev_out):
    f = lib.ec2d_residual_norms_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f(ctypes.c_void_p(dev_res), nvar, ncell, ctypes.c_void_p(dev_out), None)


def test_noalloc_norms_match_context_entry_point(gpu_lib):
    import torch
    lib = gpu_lib.lib()
    p, bl = small_case(Ma=0.6, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2, Iflag_flux=4,
                       Iflag_Scheme=5, first=2e-4)
    g = make_gpu(p, bl)
    g.init_flow()
    nx, ny, nv = g.dims(1, 1, 1)
    ncell = (nx - 1) * (ny - 1)
    out = torch.zeros(12, dtype=torch.float64, device="cuda")
    for call in range(2):  # two calls in a row, on two different residual states
        g.step(3 + 5 * call)
        g.residual(1)
        rmax, rrms, _, _ = g.norms(1, 1)
        res = g.field(1, 1, 1, 0)  # Res(NVAR,1:nx-1,1:ny-1), Fortran order
        dres = torch.from_numpy(res).to("cuda")
        torch.cuda.synchronize()
        rc = _noalloc(lib, dres.data_ptr(), nv, ncell, out.data_ptr())
        assert rc == 0
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        np.testing.assert_allclose(o[:6], rmax, rtol=1e-12, atol=0)
        np.testing.assert_allclose(np.sqrt(o[6:6 + nv] / ncell), rrms[:nv], rtol=1e-12, atol=0)
        assert np.all(o[6 + nv:] == 0.0)
    g.close()


def test_noalloc_max_carries_nan(gpu_lib):
    """A host that watches max|Res| for divergence must see a NaN cell: the
    max of a residual holding one NaN is NaN for that variable, finite for
    the others, as in the context path."""
    import torch
    lib = gpu_lib.lib()
    nv, ncell = 4, 3000
    rng = np.random.default_rng(3)
    res = rng.standard_normal((ncell, nv))
    res[1234, 2] = np.nan
    dres = torch.from_numpy(res.reshape(-1)).to("cuda")
    out = torch.zeros(12, dtype=torch.float64, device="cuda")
    assert _noalloc(lib, dres.data_ptr(), nv, ncell, out.data_ptr()) == 0
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    assert np.isnan(o[2]) and np.isnan(o[6 + 2])
    for m in (0, 1, 3):
        assert o[m] == np.max(np.abs(res[:, m]))
        np.testing.assert_allclose(o[6 + m], np.sum(res[:, m] ** 2), rtol=1e-13)


def test_noalloc_rejects_oversize(gpu_lib):
    import torch
    lib = gpu_lib.lib()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = torch.zeros(12, dtype=torch.float64, device="cuda")
    # rejected before any launch: the size check comes first
    assert _noalloc(lib, buf.data_ptr(), 4, 2097152 + 1, out.data_ptr()) == 1
    assert _noalloc(lib, buf.data_ptr(), 7, 4, out.data_ptr()) == 1
    assert _noalloc(lib, buf.data_ptr(), 4, 4, out.data_ptr()) == 0
    torch.cuda.synchronize()
