"""Tecplot writers of `output` (opencfd_ec2d_v1.5.4.f90:284-371): layout,
variables and values, checked by parsing the text back."""
import numpy as np

from ec2d import outputs


def _block(nx, ny, nv, seed):
    rng = np.random.default_rng(seed)
    U = np.zeros((nv, nx + 3, ny + 3))
    d = 1.0 + 0.1 * rng.random((nx + 3, ny + 3))
    u, v = 0.5 + 0.1 * rng.random(d.shape), 0.1 * rng.random(d.shape)
    p = 1.0 / (1.4 * 0.5 ** 2) * (1.0 + 0.05 * rng.random(d.shape))
    U[0], U[1], U[2] = d, d * u, d * v
    U[3] = p / 0.4 + 0.5 * d * (u * u + v * v)
    for m in range(4, nv):
        U[m] = rng.random(d.shape)
    x1 = np.add.outer(np.arange(-1, nx + 2), np.zeros(ny + 3)) * 0.1
    y1 = np.add.outer(np.zeros(nx + 3), np.arange(-1, ny + 2)) * 0.2
    return {"nx": nx, "ny": ny, "U": U, "x1": x1, "y1": y1, "amut": 1e-6 * rng.random(d.shape)}, (d, u, v, p)


def test_flow2d_layout_and_values():
    b1, (d, u, v, p) = _block(5, 4, 4, 0)
    b2, _ = _block(3, 6, 4, 1)
    txt = outputs.format_blocks([b1, b2], gamma=1.4, Ma=0.5, Re=1e6)
    names, zones = outputs.parse_tecplot(txt)
    assert names == ["x", "y", "d", "u", "v", "T", "p", "Amut"]
    assert [z.shape for z in zones] == [(6 * 5, 8), (4 * 7, 8)]
    z = zones[0]
    # row r = j*(nx+1) + i for i, j = 0..nx, 0..ny: array index (i+1, j+1)
    for (i, j) in [(0, 0), (5, 0), (2, 3), (5, 4)]:
        r = j * 6 + i
        np.testing.assert_allclose(z[r, 0], b1["x1"][i + 1, j + 1], atol=1e-10)
        np.testing.assert_allclose(z[r, 2], d[i + 1, j + 1], atol=1e-10)
        np.testing.assert_allclose(z[r, 3], u[i + 1, j + 1], atol=1e-10)
        np.testing.assert_allclose(z[r, 6], p[i + 1, j + 1], atol=1e-9)
        np.testing.assert_allclose(z[r, 7], b1["amut"][i + 1, j + 1] * 1e6, atol=1e-10)


def test_turbulence_files():
    b, _ = _block(4, 3, 5, 2)
    names, zones = outputs.parse_tecplot(outputs.format_turbulence([b]))
    assert names == ["x", "y", "vt"] and zones[0].shape == (5 * 4, 3)
    np.testing.assert_allclose(zones[0][7, 2], b["U"][4][7 % 5 + 1, 7 // 5 + 1], atol=1e-10)
    b6, _ = _block(4, 3, 6, 3)
    names, zones = outputs.parse_tecplot(outputs.format_turbulence([b6]))
    assert names == ["x", "y", "Kt", "Wt"] and zones[0].shape == (20, 4)


def test_dist_wall_round_trip_and_fortran_records(tmp_path):
    """dist_wall.dat (comput_dw, sub_turbulence_SST.f90:295-348): what is
    written reads back to the same doubles, a file in the Fortran compiler's
    list-directed style (repeat counts, D exponents, records wrapped across
    lines) reads as the numbers it holds, and a file for another mesh is
    refused."""
    import numpy as np

    from ec2d import inputs
    rng = np.random.default_rng(5)
    dims = [(5, 4), (3, 3)]
    dws = [rng.random((nx - 1, ny - 1)) * 10.0 ** rng.integers(-6, 2, (nx - 1, ny - 1)) for nx, ny in dims]
    path = str(tmp_path / "dist_wall.dat")
    inputs.write_dist_wall(path, dws, dims)
    back = inputs.read_dist_wall(path, dims)
    for a, b in zip(dws, back):
        assert b.shape == a.shape and np.array_equal(a, b)
    text = ("           2\n           5           4           3\n           3\n"
            "   1.0000000000000000       0.50000000000000000     3*0.25000000000000000\n"
            "   1.5D-002   2.5E-003  6*7.0000000000000000    \n"
            "   0.125000000000000000       4.0000000000000000E-004   1.0 2.0\n")
    with open(path, "w") as fh:
        fh.write(text)
    got = inputs.read_dist_wall(path, dims)
    assert got[0].reshape(-1, order="F").tolist() == [1.0, 0.5, 0.25, 0.25, 0.25, 1.5e-2, 2.5e-3] + [7.0] * 5
    assert got[1].reshape(-1, order="F").tolist() == [7.0, 0.125, 4.0e-4, 1.0]
    import pytest
    with pytest.raises(ValueError):
        inputs.read_dist_wall(path, [(5, 4), (3, 4)])
    x1 = [np.arange(12.0).reshape(4, 3), np.zeros((2, 2))]
    inputs.write_dw_tecplot(str(tmp_path / "dw.dat"), [(x, x, d) for x, d in zip(x1, got)])
    lines = open(tmp_path / "dw.dat").read().splitlines()
    assert lines[0].split() == ["variables=x,y,dw"] and lines[1].split() == ["zone", "i=", "4", "j=", "3"]
    assert len(lines) == 2 + 12 + 1 + 4


def test_read_flow_cp_file(tmp_path):
    """read_flow-1.2.f90 as ec2d.read_flow: Cp.dat holds one zone per wall
    subface (neighb = -10) over its node index range, Cp = -2 (p - p_inf)
    with p the p column of flow2d.dat and p_inf = 1/(1.4 Ma^2) -- the
    program's own gamma, not the case's."""
    import numpy as np

    from ec2d import cases, inputs, outputs, read_flow
    p, bl = cases.small_cgrid_case(33, 9, Ma=0.5, gamma=1.3, nblocks=2)
    inputs.write_case(str(tmp_path), p, bl)
    rng = np.random.default_rng(11)
    blocks = []
    for b in bl:
        shape = (b.nx + 3, b.ny + 3)
        d = 1.0 + 0.1 * rng.random(shape)
        U = np.stack([d, 0.2 * d, 0.05 * d, 2.0 + rng.random(shape)])
        blocks.append({"nx": b.nx, "ny": b.ny, "U": U, "x1": rng.random(shape), "y1": rng.random(shape),
                       "amut": np.zeros(shape)})
    with open(tmp_path / "flow2d.dat", "w") as fh:
        fh.write(outputs.format_blocks(blocks, p.gamma, p.Ma, p.Re, with_amut=True))
    read_flow.write_cp(str(tmp_path))
    lines = open(tmp_path / "Cp.dat").read().splitlines()
    assert lines[0].split() == ["variable=x,Cp"]
    walls = [(k, s) for k, b in enumerate(bl) for s in b.bc if s[6] == -10]
    assert walls
    flow = outputs._zones(str(tmp_path / "flow2d.dat"), 7)
    p00 = 1.0 / (1.4 * p.Ma * p.Ma)
    pos = 1
    for k, s in walls:
        ni, _, rows = flow[k]
        n = (s[5] - s[4] + 1) * (s[3] - s[2] + 1)
        assert lines[pos].split() == ["zone", "i=", str(n)]
        got = np.array([[float(t) for t in ln.split()] for ln in lines[pos + 1:pos + 1 + n]])
        want = np.array([(rows[j * ni + i][0], -(rows[j * ni + i][6] - p00) * 2.0)
                         for j in range(s[4], s[5] + 1) for i in range(s[2], s[3] + 1)])
        np.testing.assert_array_equal(got, want)
        pos += 1 + n
    assert pos == len(lines)


def test_driver_wall_distance_choice(tmp_path):
    """Which distances the main-loop driver hands to the library: the file's
    for SA and SST runs, none (formed on the device) for the other models,
    without the file, or -- with a warning -- for a file of another mesh."""
    import numpy as np
    import pytest

    from ec2d import driver, inputs
    dims = [(5, 4), (3, 3)]
    dws = [np.full((nx - 1, ny - 1), 0.5) for nx, ny in dims]
    sa, lam = inputs.Params(Iflag_turbulence_model=2), inputs.Params(Iflag_turbulence_model=0)
    assert driver.read_wall_distance(str(tmp_path), sa, dims) is None
    inputs.write_dist_wall(str(tmp_path / "dist_wall.dat"), dws, dims)
    got = driver.read_wall_distance(str(tmp_path), sa, dims)
    assert all(np.array_equal(a, b) for a, b in zip(got, dws))
    assert driver.read_wall_distance(str(tmp_path), lam, dims) is None
    with pytest.warns(UserWarning):
        assert driver.read_wall_distance(str(tmp_path), sa, [(5, 4), (3, 5)]) is None
