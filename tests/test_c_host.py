"""The C-ABI from hosts other than ctypes.

* include/ec2d_gpu_mod.f90, the Fortran (iso_c_binding) module a Fortran
  host uses: every function it binds is declared in include/ec2d_gpu.h and
  exported by libec2d_gpu.so (no Fortran compiler exists here, so the module
  is checked against the header and the library as text).
* opencfd-ec2d_gb300/host/ec2d_host.c, the C replica of the reference
  driver: it reads control.in / bc2d_1.in / Mesh2d.dat in the reference's
  formats and runs the spliced main loop (opencfd_ec2d_v1.5.4.f90:172-186),
  writing Residual.dat.  On a GPU its records and forces equal those of the
  same case driven through ctypes, bit for bit (same library, same kernels).
"""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def _host():
    import ec2d_build
    ec2d_build.build()
    return ec2d_build.HOST


def test_fortran_module_matches_header_and_library():
    import ec2d_build
    lib = ec2d_build.build()
    f90 = open(os.path.join(INC, "ec2d_gpu_mod.f90")).read()
    hdr = open(os.path.join(INC, "ec2d_gpu.h")).read()
    names = re.findall(r"(?:function|subroutine)\s+(ec2d_\w+)\s*\([^)]*\)\s*bind\(C\)", f90, re.I)
    assert len(names) >= 40
    declared = set(re.findall(r"\b(ec2d_\w+)\s*\(", hdr))
    exported = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (ec2d_\w+)", exported))
    for n in names:
        assert n in declared, f"{n} is bound in ec2d_gpu_mod.f90 but not declared in ec2d_gpu.h"
        assert n in exported, f"{n} is bound in ec2d_gpu_mod.f90 but not exported by the library"
    # the parameter type mirrors struct ec2d_params member by member
    fields_c = re.search(r"typedef struct ec2d_params \{(.*?)\} ec2d_params;", hdr, re.S).group(1)
    fields_f = re.search(r"type, bind\(C\) :: ec2d_params(.*?)end type", f90, re.S).group(1)
    norm = lambda s: re.findall(r"[A-Za-z_][A-Za-z_0-9]*(?=\s*[,;\n(\[])", s)
    cf = [w for w in norm(fields_c) if w not in ("double", "int")]
    ff = [w for w in re.findall(r"::\s*(.*)", fields_f)]
    ff = [v.split("(")[0].strip() for line in ff for v in line.split(",")]
    assert [v.lower() for v in cf] == [v.lower() for v in ff]


def test_c_host_reads_the_reference_inputs(tmp_path):
    """Without a GPU the host parses the case and stops at ec2d_create with
    EC2D_ERR_CUDA; with one it runs.  Either way it exits cleanly."""
    from ec2d import cases, inputs
    p, bl = cases.small_cgrid_case(65, 17, Ma=0.7, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0, CFL=5.0,
                                   Kstep_show=1)
    inputs.write_case(str(tmp_path), p, bl)
    r = subprocess.run([_host(), str(tmp_path), "--steps", "2"], capture_output=True, text=True, timeout=120)
    if r.returncode == 2:
        assert "ec2d_create" in r.stderr
    else:
        assert r.returncode == 0, r.stderr
    # a missing input file is reported before any device call
    os.remove(tmp_path / "bc2d_1.in")
    r = subprocess.run([_host(), str(tmp_path), "--steps", "2"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "bc2d_1.in" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["single", "mg3"])
def test_c_host_main_loop_equals_ctypes(gpu_lib, tmp_path, kind):
    from ec2d import cases, gpu, inputs
    if kind == "single":
        p, bl = cases.small_cgrid_case(97, 33, Ma=0.7, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0,
                                       CFL=5.0, Kstep_show=5, nblocks=2)
        fdm = []
    else:
        p, bl = cases.laminar_flat_plate(33, 33, num_mesh=3)
        p = p.replace(Kstep_show=5)
        fdm = []
    inputs.write_case(str(tmp_path), p, bl)
    steps = 20
    r = subprocess.run([_host(), str(tmp_path), "--steps", str(steps)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    recs = open(tmp_path / "Residual.dat").read().splitlines()
    assert len(recs) == steps // 5
    g = gpu.Solver([(p, bl)], fdm_blocks=[fdm])
    g.init_flow()
    expect = []
    for k in range(steps // 5):
        g.step(5)
        rmax, rrms, kstep, _ = g.norms()
        expect.append(inputs.residual_record(kstep, rmax, rrms, p.nvar()).rstrip("\n"))
    assert recs == expect
    out = dict(line.split(None, 1) for line in r.stdout.splitlines() if line.startswith(("forces", "res_rms")))
    np.testing.assert_array_equal(np.array(out["forces"].split(), dtype=float), np.array(g.forces(1)))
    np.testing.assert_array_equal(np.array(out["res_rms"].split(), dtype=float), g.norms()[1][:p.nvar()])
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["euler", "sa"])
def test_c_host_restart_equals_python_restart(gpu_lib, tmp_path, kind):
    """Iflag_init = 1: the C host's init_flow_read (flow2d.dat, and SA2d.dat
    with --fix-nvar-restart) leaves the state outputs.restart leaves, so both
    hosts write the same Residual.dat records after the restart; an SA
    restart without the flag stops with the reference's NVAR problem named."""
    from ec2d import cases, gpu, inputs, outputs
    if kind == "euler":
        p, bl = cases.small_cgrid_case(65, 17, Ma=0.7, AoA=2.0, Iflag_flux=4, Iflag_Scheme=5, Time_Method=0,
                                       CFL=5.0, Kstep_show=5, nblocks=2)
    else:
        p, bl = cases.small_cgrid_case(65, 17, Ma=0.6, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2,
                                       Iflag_flux=4, Iflag_Scheme=5, CFL=5.0, first=2e-4, nblocks=2, Kstep_show=5)
    g = gpu.Solver([(p, bl)])
    g.init_flow()
    g.step(10)
    inputs.write_case(str(tmp_path), p.replace(Iflag_init=1), bl)
    outputs.write_output(str(tmp_path), g, p, kstep=10)
    g.close()
    # the Python host restarts from its own copy: the C host's final output(1)
    # replaces flow2d.dat in the case directory
    import shutil
    py_dir = tmp_path.parent / (tmp_path.name + "_py")
    shutil.copytree(tmp_path, py_dir)
    fix = kind == "sa"
    if fix:
        r = subprocess.run([_host(), str(tmp_path), "--steps", "10"], capture_output=True, text=True, timeout=120)
        assert r.returncode == 1 and "sub_init.f90:541" in r.stderr
    args = [_host(), str(tmp_path), "--steps", "10"] + (["--fix-nvar-restart"] if fix else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    recs = open(tmp_path / "Residual.dat").read().splitlines()
    h = gpu.Solver([(p, bl)])
    outputs.restart(h, str(py_dir), fix_nvar=fix)
    expect = []
    for _ in range(2):
        h.step(5)
        rmax, rrms, kstep, _ = h.norms()
        expect.append(inputs.residual_record(kstep, rmax, rrms, p.nvar()).rstrip("\n"))
    assert recs == expect
    h.close()


@pytest.mark.gpu
def test_c_host_wall_distance_file(gpu_lib, tmp_path):
    """SA: without dist_wall.dat the C host writes it from the device's
    distances (bit for bit); given one (here with doubled distances) it reads
    it, and marches as the Python driver does with the same file."""
    import shutil

    from ec2d import cases, driver, gpu, inputs
    p, bl = cases.small_cgrid_case(65, 17, Ma=0.6, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2,
                                   Iflag_flux=4, Iflag_Scheme=5, CFL=5.0, first=2e-4, nblocks=2, Kstep_show=5,
                                   t_end=1.0e9)
    dims = [(b.nx, b.ny) for b in bl]
    a, b_, c = tmp_path / "a", tmp_path / "b", tmp_path / "c"
    inputs.write_case(str(a), p, bl)
    r = subprocess.run([_host(), str(a), "--steps", "2"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    dws = inputs.read_dist_wall(str(a / "dist_wall.dat"), dims)
    g = gpu.Solver([(p, bl)])
    for k, (nx, ny) in enumerate(dims, start=1):
        np.testing.assert_array_equal(dws[k - 1], g.field(1, 1, k, gpu.F_DW, shape=(nx + 1, ny + 1))[1:nx, 1:ny])
    g.close()
    assert open(a / "dw.dat").readline().split() == ["variables=x,y,dw"]
    for d in (b_, c):
        inputs.write_case(str(d), p, bl)
        inputs.write_dist_wall(str(d / "dist_wall.dat"), [2.0 * x for x in dws], dims)
    r = subprocess.run([_host(), str(b_), "--steps", "10"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    driver.run(str(c), steps=10, quiet=True)
    assert open(b_ / "Residual.dat").read() == open(c / "Residual.dat").read()
    assert not os.path.exists(b_ / "dw.dat")
    shutil.rmtree(a)


@pytest.mark.gpu
def test_c_host_flow_files_equal_the_python_driver(gpu_lib, tmp_path):
    """output(1) of the C host every Kstep_save steps and at the end
    (flow2d-<Kstep>.dat, flow2d.dat, SA2d.dat) is the Python driver's text,
    byte for byte, for the same SA run."""
    from ec2d import cases, driver, inputs
    p, bl = cases.small_cgrid_case(65, 17, Ma=0.6, AoA=2.0, Re=1e6, If_viscous=1, Iflag_turbulence_model=2,
                                   Iflag_flux=4, Iflag_Scheme=5, CFL=5.0, first=2e-4, nblocks=2, Kstep_show=5,
                                   Kstep_save=10, t_end=1.0e9)
    a, b_ = tmp_path / "c", tmp_path / "py"
    for d in (a, b_):
        inputs.write_case(str(d), p, bl)
    r = subprocess.run([_host(), str(a), "--steps", "20"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    driver.run(str(b_), steps=20, quiet=True)
    for name in ("flow2d-0000010.dat", "flow2d-0000020.dat", "flow2d.dat", "SA2d.dat", "Residual.dat",
                 "dist_wall.dat", "dw.dat"):
        assert open(a / name).read() == open(b_ / name).read(), name
