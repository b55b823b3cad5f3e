"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
module.  It restates the reference Fortran on the CPU; parity is UNPINNED by
the reference (no golden vectors, no Fortran compiler), see ec2d_oracle.h.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libec2d_oracle.so")
# the same source built -O3 with FMA contraction: the benchmark's CPU timing
# baseline, never a parity reference
LIB_FAST = os.path.join(HERE, "_build", "libec2d_oracle_fast.so")

F_RES, F_DT, F_LCI, F_LCJ, F_LVI, F_LVJ, F_DU, F_AMU, F_AMUT, F_X1, F_Y1, F_VOL = range(12)
F_SI, F_SJ, F_NI1, F_NI2, F_NJ1, F_NJ2, F_DW, F_QF, F_DELTU, F_UN, F_X, F_Y = range(12, 24)


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("Ma", ctypes.c_double), ("Re", ctypes.c_double), ("gamma", ctypes.c_double),
        ("AoA", ctypes.c_double), ("Pr", ctypes.c_double), ("t_end", ctypes.c_double),
        ("Kstep_save", ctypes.c_int), ("If_viscous", ctypes.c_int),
        ("Iflag_turbulence_model", ctypes.c_int), ("Iflag_init", ctypes.c_int),
        ("Iflag_local_dt", ctypes.c_int),
        ("dt_global", ctypes.c_double), ("CFL", ctypes.c_double), ("dtmax", ctypes.c_double),
        ("dtmin", ctypes.c_double),
        ("Time_Method", ctypes.c_int),
        ("P_outlet", ctypes.c_double), ("T_inf", ctypes.c_double), ("Twall", ctypes.c_double),
        ("vt_inf", ctypes.c_double), ("Kt_inf", ctypes.c_double), ("Wt_inf", ctypes.c_double),
        ("Iflag_Scheme", ctypes.c_int), ("Iflag_flux", ctypes.c_int),
        ("IFlag_Reconstruction", ctypes.c_int), ("Kstep_show", ctypes.c_int),
        ("Num_Mesh", ctypes.c_int), ("Num_Threads", ctypes.c_int), ("Nstep_Inner_Limit", ctypes.c_int),
        ("Res_Inner_Limit", ctypes.c_double),
        ("Pre_Step_Mesh", ctypes.c_int * 3),
        ("xaxis", ctypes.c_double), ("yaxis", ctypes.c_double),
        ("mg_lusgs", ctypes.c_int),
    ]


def to_struct(p, cls=OrcParams):
    s = cls()
    for name, _ in cls._fields_:
        v = getattr(p, name)
        if name == "Pre_Step_Mesh":
            arr = (ctypes.c_int * 3)(*[int(t) for t in (list(v) + [0, 0, 0])[:3]])
            setattr(s, name, arr)
        else:
            setattr(s, name, v)
    return s


_libs = {}


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib(fast=False):
    """The parity build (default) or, with fast=True, the timing build."""
    path = LIB_FAST if fast else LIB
    if path not in _libs:
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        L.orc_new.restype = vp
        L.orc_new.argtypes = [ctypes.POINTER(OrcParams)]
        L.orc_free.argtypes = [vp]
        L.orc_add_block.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int, ip]
        for name in ("orc_setup", "orc_init_flow", "orc_dual_time_start", "orc_num_mesh"):
            getattr(L, name).argtypes = [vp]
        L.orc_set_fdm_block.argtypes = [vp, ctypes.c_int]
        L.orc_set_dw.argtypes = [vp, ctypes.c_int, dp]
        L.orc_nvar.argtypes = [vp, ctypes.c_int]
        L.orc_block_dims.argtypes = [vp, ctypes.c_int, ctypes.c_int, ip, ip]
        L.orc_get_U.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp]
        L.orc_set_U.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp]
        L.orc_get_field.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        L.orc_field_size.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        for name in ("orc_residual", "orc_bc", "orc_halo", "orc_time_advance", "orc_force_function",
                     "orc_set_un", "orc_delt_u", "orc_new_u"):
            getattr(L, name).argtypes = [vp, ctypes.c_int]
        L.orc_step.argtypes = [vp, ctypes.c_int]
        L.orc_lusgs.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.orc_norms.argtypes = [vp, ctypes.c_int, dp, dp, ip, dp]
        L.orc_interpolation2h.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_prolong.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_forces.argtypes = [vp, dp, dp, dp]
        L.orc_wall_cf.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int]
        L.orc_last_error.argtypes = [vp, ip, ip, ip]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_set_mg_amut.argtypes = [vp, ctypes.c_int]
        L.orc_flux.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double]
        L.orc_scheme.argtypes = [ctypes.c_int] + [ctypes.c_double] * 4 + [ctypes.c_int]
        L.orc_scheme.restype = ctypes.c_double
        L.orc_set_field.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        _libs[path] = L
    return _libs[path]


def flux(iflux, QL, QR, gamma=1.4):
    QL = np.ascontiguousarray(QL, dtype=np.float64); QR = np.ascontiguousarray(QR, dtype=np.float64)
    F = np.zeros(4)
    lib().orc_flux(int(iflux), _dp(QL), _dp(QR), _dp(F), gamma)
    return F


def scheme(side, u1, u2, u3, u4, flag):
    return lib().orc_scheme(side, u1, u2, u3, u4, flag)


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One case on the CPU oracle, driven like the reference main program."""

    def __init__(self, params, blocks, fdm_blocks=(), dw=None, threads=None, fast=False):
        L = lib(fast)
        if threads is not None:
            L.orc_set_threads(int(threads))
        self.L = L
        self.p = params
        sp = to_struct(params)
        self.h = L.orc_new(ctypes.byref(sp))
        for b in blocks:
            x = np.asfortranarray(b.x, dtype=np.float64)
            y = np.asfortranarray(b.y, dtype=np.float64)
            bc = np.ascontiguousarray(np.array(b.bc, dtype=np.int32).reshape(-1))
            r = L.orc_add_block(self.h, b.nx, b.ny, _dp(x), _dp(y), len(b.bc),
                                bc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
            if r:
                raise RuntimeError("orc_add_block failed")
        for k in fdm_blocks:
            L.orc_set_fdm_block(self.h, int(k))
        if dw is not None:
            for k, d in enumerate(dw):
                d = np.asfortranarray(d, dtype=np.float64)
                L.orc_set_dw(self.h, k + 1, _dp(d))
        r = L.orc_setup(self.h)
        if r:
            raise RuntimeError(f"orc_setup failed ({r})")
        self.nblocks = len(blocks)

    def __del__(self):
        try:
            self.L.orc_free(self.h)
        except Exception:
            pass

    @property
    def num_mesh(self):
        return self.L.orc_num_mesh(self.h)

    def nvar(self, mesh=1):
        return self.L.orc_nvar(self.h, mesh)

    def dims(self, mesh, block):
        nx, ny = ctypes.c_int(), ctypes.c_int()
        self.L.orc_block_dims(self.h, mesh, block, ctypes.byref(nx), ctypes.byref(ny))
        return nx.value, ny.value

    def _check(self, r, what):
        if r:
            b, i, j = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            code = self.L.orc_last_error(self.h, ctypes.byref(b), ctypes.byref(i), ctypes.byref(j))
            raise RuntimeError(f"{what} failed: code {code} at block {b.value} cell ({i.value},{j.value})")

    def init_flow(self):
        self._check(self.L.orc_init_flow(self.h), "init_flow")

    def dual_time_start(self):
        """Dual time stepping restarts its physical-time history from the current U."""
        self._check(self.L.orc_dual_time_start(self.h), "dual_time_start")

    def get_U(self, mesh, block):
        nx, ny = self.dims(mesh, block)
        nv = self.nvar(mesh)
        U = np.zeros((nv, nx + 3, ny + 3), order="F")
        self.L.orc_get_U(self.h, mesh, block, _dp(U))
        return U

    def set_U(self, mesh, block, U):
        U = np.asfortranarray(U, dtype=np.float64)
        self.L.orc_set_U(self.h, mesh, block, _dp(U))

    def field(self, mesh, block, fid, shape=None):
        n = self.L.orc_field_size(self.h, mesh, block, fid)
        out = np.zeros(n)
        self.L.orc_get_field(self.h, mesh, block, fid, _dp(out))
        if shape is not None:
            out = out.reshape(shape, order="F")
        return out

    def set_field(self, mesh, block, fid, arr):
        a = np.asfortranarray(arr, dtype=np.float64).reshape(-1, order="F").copy()
        n = self.L.orc_field_size(self.h, mesh, block, fid)
        assert a.size == n, (a.size, n)
        self.L.orc_set_field(self.h, mesh, block, fid, _dp(a))

    def residual(self, mesh=1):
        self._check(self.L.orc_residual(self.h, mesh), "residual")

    def bc(self, mesh=1):
        self.L.orc_bc(self.h, mesh)

    def halo(self, mesh=1):
        self.L.orc_halo(self.h, mesh)

    def lusgs(self, mesh, block, alfa1=0.0):
        self.L.orc_lusgs(self.h, mesh, block, alfa1)

    def time_advance(self, mesh=1):
        self._check(self.L.orc_time_advance(self.h, mesh), "time_advance")

    def step(self, n=1):
        self._check(self.L.orc_step(self.h, n), "step")

    def norms(self, mesh=1):
        a = np.zeros(6); b = np.zeros(6)
        k = ctypes.c_int(); t = ctypes.c_double()
        self.L.orc_norms(self.h, mesh, _dp(a), _dp(b), ctypes.byref(k), ctypes.byref(t))
        return a, b, k.value, t.value

    def interpolation2h(self, m1, m2, flag):
        self.L.orc_interpolation2h(self.h, m1, m2, flag)

    def prolong(self, m1, m2, flag):
        self.L.orc_prolong(self.h, m1, m2, flag)

    def set_mg_amut(self, enable=True):
        """Extension: coarse levels keep the eddy viscosity restricted from
        the next finer level (the reference zeroes it there)."""
        self.L.orc_set_mg_amut(self.h, int(enable))

    def force_function(self, mesh):
        """QF -= Res (comput_force_function, sub_NS_multigrid.f90:156-173)."""
        self.L.orc_force_function(self.h, mesh)

    def set_un(self, mesh):
        """Un = U (Set_Un, sub_NS_multigrid.f90:219-237)."""
        self.L.orc_set_un(self.h, mesh)

    def delt_u(self, mesh):
        """deltU = U - Un (comput_delt_U, sub_NS_multigrid.f90:199-216)."""
        self.L.orc_delt_u(self.h, mesh)

    def new_u(self, mesh):
        """U += deltU on the interior (comput_new_U, sub_NS_multigrid.f90:240-260)."""
        self.L.orc_new_u(self.h, mesh)

    def forces(self):
        cl, cd, cm = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self.L.orc_forces(self.h, ctypes.byref(cl), ctypes.byref(cd), ctypes.byref(cm))
        return cl.value, cd.value, cm.value

    def wall_cf(self, block, sub, maxn=4096):
        cf = np.zeros(maxn); xc = np.zeros(maxn)
        n = self.L.orc_wall_cf(self.h, block, sub, _dp(cf), _dp(xc), maxn)
        return cf[:n], xc[:n]
