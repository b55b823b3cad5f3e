"""Host-side checks without a GPU: input-file formats, grid generators, the
multigrid depth rule, and that libec2d_gpu.so loads and exports every entry
point declared in include/ec2d_gpu.h."""
import ctypes
import os
import re

import numpy as np
import pytest

from ec2d import cases, grids, inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_symbols_exported():
    import ec2d_build
    lib = ec2d_build.build()
    hdr = open(os.path.join(ROOT, "include", "ec2d_gpu.h")).read()
    names = sorted(set(re.findall(r"\b(ec2d_[a-z0-9_]+)\s*\(", hdr)))
    assert len(names) >= 25
    L = ctypes.CDLL(lib)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    L.ec2d_version.restype = ctypes.c_int
    assert L.ec2d_version() >= 10000


def test_params_struct_matches_header():
    """The ctypes mirror lists the header's fields in the header's order."""
    from ec2d import gpu
    hdr = open(os.path.join(ROOT, "include", "ec2d_gpu.h")).read()
    body = hdr[hdr.index("typedef struct ec2d_params"):hdr.index("} ec2d_params;")]
    fields = re.findall(r"([A-Za-z_][A-Za-z0-9_]*)(?:\[\d+\])?\s*[,;]", body.split("{", 1)[1])
    assert [f for f, _ in gpu.Params._fields_] == fields


def test_control_roundtrip(tmp_path):
    p = inputs.Params(Ma=0.73, Re=6.5e6, AoA=2.8, If_viscous=1, Iflag_turbulence_model=2, Num_Mesh=3,
                      Pre_Step_Mesh=(0, 100, 200), CFL=7.5, xaxis=0.3)
    f = tmp_path / "control.in"
    inputs.write_control(str(f), p)
    q = inputs.read_control(str(f))
    for k in ("Ma", "Re", "AoA", "If_viscous", "Iflag_turbulence_model", "Num_Mesh", "CFL", "xaxis"):
        assert getattr(q, k) == getattr(p, k)
    assert tuple(q.Pre_Step_Mesh) == (0, 100, 200)


def test_reads_reference_inputs():
    from conftest import reference_file
    reference_file("Mesh2d.dat")
    p, blocks = inputs.read_case(os.path.dirname(reference_file("control.in")))
    assert p.Ma == 0.729 and p.Iflag_turbulence_model == 3 and p.Iflag_Scheme == 5
    assert len(blocks) == 3 and blocks[1].bc[1] == [2, 2, 1, 305, 1, 1, -10, 0, 0]


def test_mesh_bc_roundtrip(tmp_path):
    p, bl = cases.euler_naca0012(129, 33)
    inputs.write_case(str(tmp_path), p, bl)
    q, bl2 = inputs.read_case(str(tmp_path))
    assert len(bl2) == len(bl)
    for a, b in zip(bl, bl2):
        np.testing.assert_allclose(a.x, b.x, rtol=1e-15)
        assert a.bc == b.bc


@pytest.mark.parametrize("nb", [1, 2, 4])
def test_cgrid_valid(nb):
    bl = grids.naca_cgrid(257, 65, m=0.02, p=0.4, nblocks=nb)
    for b in bl:
        assert grids.cell_volumes(b).min() > 0.0
        for s in b.bc:
            assert all((v - 1) % 4 == 0 for v in s[2:6])


def test_flat_plate_grid():
    bl = grids.flat_plate(97, 97, first=1e-4, ratio=1.1)
    assert len(bl) == 2 and bl[0].nx == 97
    assert abs(bl[1].y[0, 1] - 1e-4) < 1e-15
    assert abs((bl[1].y[0, 2] - bl[1].y[0, 1]) / (bl[1].y[0, 1]) - 1.1) < 1e-12
    for b in bl:
        assert grids.cell_volumes(b).min() > 0


def test_polar_cases_seeded():
    a = cases.polar_cases(6)
    b = cases.polar_cases(6)
    assert [x[0].Ma for x in a] == [x[0].Ma for x in b]
    for p, bl in a:
        assert 0.3 <= p.Ma <= 0.8 and -2 <= p.AoA <= 8 and 1e6 <= p.Re <= 1e7
        assert 1 <= len(bl) <= 4


def test_residual_record_format():
    s = inputs.residual_record(10, [1.0, 2.5e-3, 0, 0, 0, 0], [3.25e-7, 1, 1, 1], 4)
    assert s.startswith("      10") and len(s) == 8 + 10 * 24 + 1
    assert "0.3250000000E-06" in s
