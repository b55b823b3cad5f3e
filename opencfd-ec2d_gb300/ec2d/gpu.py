"""ctypes binding of libec2d_gpu.so (the C-ABI declared in include/ec2d_gpu.h).

This is the same binding a Python host of the Fortran code's logic would use;
it adds nothing to the computation.  There is no CPU fallback: if the library
cannot be loaded, or no CUDA device is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB = os.path.join(PKG, "lib", "libec2d_gpu.so")

F_RES, F_DT, F_LCI, F_LCJ, F_LVI, F_LVJ, F_DU, F_AMU, F_AMUT, F_X1, F_Y1, F_VOL = range(12)
F_SI, F_SJ, F_NI1, F_NI2, F_NJ1, F_NJ2, F_DW, F_QF, F_DELTU, F_UN, F_X, F_Y = range(12, 24)

ERRORS = {1: "invalid argument or call order", 2: "CUDA error", 3: "non-physical state (T < 1e-5)",
          4: "device wait timed out", 5: "option combination not supported", 6: "out of device memory"}


class EC2DError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f"{what}: {ERRORS.get(code, code)} (code {code})")
        self.code = code


class Params(ctypes.Structure):
    """ec2d_params of include/ec2d_gpu.h (field order matters)."""
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

    @classmethod
    def from_params(cls, p):
        s = cls()
        for name, _ in cls._fields_:
            v = getattr(p, name)
            if name == "Pre_Step_Mesh":
                s.Pre_Step_Mesh = (ctypes.c_int * 3)(*[int(t) for t in (list(v) + [0, 0, 0])[:3]])
            else:
                setattr(s, name, v)
        return s


_lib = None


def lib():
    """Load libec2d_gpu.so (built by build.py); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise OSError(f"{LIB} not built; run ec2d_build.py")
    L = ctypes.CDLL(LIB)
    vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    fp = ctypes.POINTER(ctypes.c_float)
    cpp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "ec2d_version": ([], ctypes.c_int),
        "ec2d_error_string": ([ctypes.c_int], ctypes.c_char_p),
        "ec2d_create": ([ctypes.c_int, cpp], ctypes.c_int),
        "ec2d_destroy": ([vp], None),
        "ec2d_add_case": ([vp, ctypes.POINTER(Params), ip], ctypes.c_int),
        "ec2d_add_block": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int, ip], ctypes.c_int),
        "ec2d_set_fdm_block": ([vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "ec2d_set_wall_distance": ([vp, ctypes.c_int, ctypes.c_int, dp], ctypes.c_int),
        "ec2d_setup": ([vp], ctypes.c_int),
        "ec2d_num_mesh": ([vp, ip], ctypes.c_int),
        "ec2d_block_dims": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, ip, ip], ctypes.c_int),
        "ec2d_init_flow": ([vp], ctypes.c_int),
        "ec2d_dual_time_start": ([vp], ctypes.c_int),
        "ec2d_upload_U": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp], ctypes.c_int),
        "ec2d_download_U": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp], ctypes.c_int),
        "ec2d_step": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_residual": ([vp, ctypes.c_int, ctypes.c_int, dp, dp, ip, dp], ctypes.c_int),
        "ec2d_status": ([vp, ctypes.c_int, ip, ip, ip, ip], ctypes.c_int),
        "ec2d_forces": ([vp, ctypes.c_int, dp, dp, dp], ctypes.c_int),
        "ec2d_wall_cf": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int, ip], ctypes.c_int),
        "ec2d_get_field": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp], ctypes.c_int),
        "ec2d_field_size": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip], ctypes.c_int),
        "ec2d_set_field": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp], ctypes.c_int),
        "ec2d_comput_residual": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_boundary_condition": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_update_buffer": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_du_lusgs": ([vp, ctypes.c_int, ctypes.c_double], ctypes.c_int),
        "ec2d_time_advance": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_interpolation2h": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "ec2d_prolong": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "ec2d_force_function": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_sync": ([vp], ctypes.c_int),
        "ec2d_stream": ([vp, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
        "ec2d_launch_count": ([vp, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "ec2d_kernel_timing": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_kernel_times": ([vp, ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
        "ec2d_set_graphs": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_set_lusgs_precision": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_set_coarse_precision": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_run_to_drop": ([vp, ctypes.c_double, dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ip, dp, dp],
                             ctypes.c_int),
        "ec2d_set_case_shape": ([vp, ctypes.c_int, ctypes.c_double], ctypes.c_int),
        "ec2d_autotune": ([vp, ctypes.c_int, ip, ip, ip, dp], ctypes.c_int),
        "ec2d_mlp_create": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, cpp], ctypes.c_int),
        "ec2d_mlp_destroy": ([vp], None),
        "ec2d_mlp_add_samples": ([vp, vp], ctypes.c_int),
        "ec2d_mlp_num_samples": ([vp, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "ec2d_mlp_clear_samples": ([vp], ctypes.c_int),
        "ec2d_mlp_fit_normalization": ([vp], ctypes.c_int),
        "ec2d_mlp_train": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp], ctypes.c_int),
        "ec2d_mlp_warm_start": ([vp, vp, ip], ctypes.c_int),
        "ec2d_mlp_num_layers": ([vp, ip], ctypes.c_int),
        "ec2d_mlp_layer_shape": ([vp, ctypes.c_int, ip, ip], ctypes.c_int),
        "ec2d_mlp_get_weights": ([vp, ctypes.c_int, fp, fp], ctypes.c_int),
        "ec2d_mlp_set_weights": ([vp, ctypes.c_int, fp, fp], ctypes.c_int),
        "ec2d_mlp_get_grads": ([vp, ctypes.c_int, fp, fp], ctypes.c_int),
        "ec2d_mlp_get_normalization": ([vp, fp], ctypes.c_int),
        "ec2d_mlp_set_normalization": ([vp, fp], ctypes.c_int),
        "ec2d_mlp_loss_grad": ([vp, fp, fp, ctypes.c_int, dp], ctypes.c_int),
        "ec2d_mlp_predict": ([vp, fp, ctypes.c_longlong, fp], ctypes.c_int),
        "ec2d_mlp_set_gemm": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_measure_fp64_peak": ([dp], ctypes.c_int),
        "ec2d_measure_op_cycles": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, dp], ctypes.c_int),
        "ec2d_check_reciprocal": ([ctypes.c_longlong, dp, dp], ctypes.c_int),
        "ec2d_snapshot": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_tile_residual": ([vp, ctypes.c_int, ip], ctypes.c_int),
        "ec2d_launch_config": ([vp, ip, ip, ip, ip, ip], ctypes.c_int),
        "ec2d_set_launch_config": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int],
                                   ctypes.c_int),
        "ec2d_launch_signature": ([vp, ctypes.c_char_p, ctypes.c_int, ip], ctypes.c_int),
        "ec2d_mg_eddy_viscosity": ([vp, ctypes.c_int, ip], ctypes.c_int),
        "ec2d_clear_status": ([vp, ctypes.c_int], ctypes.c_int),
        "ec2d_lusgs_shape": ([vp, ip, ip, ip], ctypes.c_int),
        "ec2d_snapshot_wait": ([vp, ip, ip, dp], ctypes.c_int),
        "ec2d_snapshot_U": ([vp, ctypes.c_int, dp], ctypes.c_int),
        "ec2d_snapshot_amut": ([vp, ctypes.c_int, dp], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def measure_fp64_peak():
    """Measured FP64 FMA throughput of the current device, TFLOP/s."""
    t = ctypes.c_double()
    _ck(lib().ec2d_measure_fp64_peak(ctypes.byref(t)), "ec2d_measure_fp64_peak")
    return t.value


def check_reciprocal(n=40_000_000):
    """(largest relative error of the hardware reciprocal approximation,
    largest distance of the refined reciprocal from the IEEE quotient in
    ulps) over n inputs in [2^-8, 2^9)."""
    a, u = ctypes.c_double(), ctypes.c_double()
    _ck(lib().ec2d_check_reciprocal(int(n), ctypes.byref(a), ctypes.byref(u)), "ec2d_check_reciprocal")
    return a.value, u.value


def measure_op_cycles(op, warps=1, chains=1):
    """clock64 cycles per dependent operation per warp (op 0 FP64 fma, 1 FP64
    divide, 2 refined FP64 reciprocal, 3 FP32 fma), or per barrier (4 CTA
    barrier with `warps` warps, 5 cluster barrier among `chains` CTAs)."""
    c = ctypes.c_double()
    _ck(lib().ec2d_measure_op_cycles(int(op), int(warps), int(chains), ctypes.byref(c)), "ec2d_measure_op_cycles")
    return c.value


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _ck(r, what):
    if r:
        raise EC2DError(r, what)


class Solver:
    """A context of one or more cases sharing the method flags (a batch)."""

    def __init__(self, cases, device=0, fdm_blocks=None, dw=None):
        """cases: list of (Params, [Block, ...]); fdm_blocks: per case list of
        1-based block ids; dw: per case list of per-block wall distances."""
        self.L = lib()
        h = ctypes.c_void_p()
        _ck(self.L.ec2d_create(device, ctypes.byref(h)), "ec2d_create")
        self.h = h
        self.ncase = len(cases)
        self.params = [c[0] for c in cases]
        self.nblocks = [len(c[1]) for c in cases]
        for ci, (p, blocks) in enumerate(cases):
            sp = Params.from_params(p)
            cid = ctypes.c_int()
            _ck(self.L.ec2d_add_case(self.h, ctypes.byref(sp), ctypes.byref(cid)), "ec2d_add_case")
            for b in blocks:
                x = np.asfortranarray(b.x, dtype=np.float64)
                y = np.asfortranarray(b.y, dtype=np.float64)
                bc = np.ascontiguousarray(np.array(b.bc, dtype=np.int32).reshape(-1))
                _ck(self.L.ec2d_add_block(self.h, cid.value, b.nx, b.ny, _dp(x), _dp(y), len(b.bc),
                                          bc.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), "ec2d_add_block")
            if fdm_blocks is not None:
                for k in fdm_blocks[ci]:
                    _ck(self.L.ec2d_set_fdm_block(self.h, cid.value, int(k)), "ec2d_set_fdm_block")
            if dw is not None and dw[ci] is not None:
                for k, d in enumerate(dw[ci]):
                    d = np.asfortranarray(d, dtype=np.float64)
                    _ck(self.L.ec2d_set_wall_distance(self.h, cid.value, k + 1, _dp(d)), "ec2d_set_wall_distance")
        _ck(self.L.ec2d_setup(self.h), "ec2d_setup")

    def close(self):
        if getattr(self, "h", None):
            self.L.ec2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_mesh(self):
        n = ctypes.c_int()
        _ck(self.L.ec2d_num_mesh(self.h, ctypes.byref(n)), "ec2d_num_mesh")
        return n.value

    def dims(self, case, mesh, block):
        nx, ny, nv = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _ck(self.L.ec2d_block_dims(self.h, case, mesh, block, ctypes.byref(nx), ctypes.byref(ny), ctypes.byref(nv)),
            "ec2d_block_dims")
        return nx.value, ny.value, nv.value

    def init_flow(self):
        _ck(self.L.ec2d_init_flow(self.h), "ec2d_init_flow")

    def dual_time_start(self):
        """Dual time stepping: U(n) = U(n-1) = the current U, first step one-step form."""
        _ck(self.L.ec2d_dual_time_start(self.h), "ec2d_dual_time_start")

    def upload_U(self, case, mesh, block, U):
        U = np.asfortranarray(U, dtype=np.float64)
        _ck(self.L.ec2d_upload_U(self.h, case, mesh, block, _dp(U)), "ec2d_upload_U")

    def download_U(self, case, mesh, block, out=None):
        nx, ny, nv = self.dims(case, mesh, block)
        U = out if out is not None else np.zeros((nv, nx + 3, ny + 3), order="F")
        _ck(self.L.ec2d_download_U(self.h, case, mesh, block, _dp(U)), "ec2d_download_U")
        return U

    def step(self, n=1):
        _ck(self.L.ec2d_step(self.h, n), "ec2d_step")

    def snapshot(self, case=1):
        """Enqueue an asynchronous copy of the case's fine-mesh U (returns at once)."""
        _ck(self.L.ec2d_snapshot(self.h, case), "ec2d_snapshot")

    def snapshot_wait(self):
        """Wait for the last snapshot; returns (case, Kstep, tt) at which it was taken."""
        c, k, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _ck(self.L.ec2d_snapshot_wait(self.h, ctypes.byref(c), ctypes.byref(k), ctypes.byref(t)),
            "ec2d_snapshot_wait")
        return c.value, k.value, t.value

    def snapshot_U(self, block, case=None):
        """One block of the last snapshot, U(NVAR,-1:nx+1,-1:ny+1)."""
        if case is None:
            case = self.snapshot_wait()[0]
        nx, ny, nv = self.dims(case, 1, block)
        U = np.zeros((nv, nx + 3, ny + 3), order="F")
        _ck(self.L.ec2d_snapshot_U(self.h, block, _dp(U)), "ec2d_snapshot_U")
        return U

    def snapshot_amut(self, block, case=None):
        """Amu_t(-1:nx+1,-1:ny+1) of one block at the last snapshot."""
        if case is None:
            case = self.snapshot_wait()[0]
        nx, ny, _ = self.dims(case, 1, block)
        a = np.zeros((nx + 3, ny + 3), order="F")
        _ck(self.L.ec2d_snapshot_amut(self.h, block, _dp(a)), "ec2d_snapshot_amut")
        return a

    def norms(self, case=1, mesh=1):
        a = np.zeros(6); b = np.zeros(6)
        k = ctypes.c_int(); t = ctypes.c_double()
        _ck(self.L.ec2d_residual(self.h, case, mesh, _dp(a), _dp(b), ctypes.byref(k), ctypes.byref(t)),
            "ec2d_residual")
        return a, b, k.value, t.value

    def status(self, case=1):
        c, b, i, j = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _ck(self.L.ec2d_status(self.h, case, ctypes.byref(c), ctypes.byref(b), ctypes.byref(i), ctypes.byref(j)),
            "ec2d_status")
        return c.value, b.value, i.value, j.value

    def forces(self, case=1):
        cl, cd, cm = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _ck(self.L.ec2d_forces(self.h, case, ctypes.byref(cl), ctypes.byref(cd), ctypes.byref(cm)), "ec2d_forces")
        return cl.value, cd.value, cm.value

    def wall_cf(self, case, block, sub, maxn=8192):
        cf = np.zeros(maxn); xc = np.zeros(maxn); n = ctypes.c_int()
        _ck(self.L.ec2d_wall_cf(self.h, case, block, sub, _dp(cf), _dp(xc), maxn, ctypes.byref(n)), "ec2d_wall_cf")
        return cf[:n.value], xc[:n.value]

    def field(self, case, mesh, block, fid, shape=None):
        n = ctypes.c_int()
        _ck(self.L.ec2d_field_size(self.h, case, mesh, block, fid, ctypes.byref(n)), "ec2d_field_size")
        out = np.zeros(n.value)
        _ck(self.L.ec2d_get_field(self.h, case, mesh, block, fid, _dp(out)), "ec2d_get_field")
        if shape is not None:
            out = out.reshape(shape, order="F")
        return out

    def set_field(self, case, mesh, block, fid, arr):
        a = np.asfortranarray(arr, dtype=np.float64).reshape(-1, order="F").copy()
        _ck(self.L.ec2d_set_field(self.h, case, mesh, block, fid, _dp(a)), "ec2d_set_field")

    def residual(self, mesh=1):
        _ck(self.L.ec2d_comput_residual(self.h, mesh), "ec2d_comput_residual")

    def bc(self, mesh=1):
        _ck(self.L.ec2d_boundary_condition(self.h, mesh), "ec2d_boundary_condition")

    def halo(self, mesh=1):
        _ck(self.L.ec2d_update_buffer(self.h, mesh), "ec2d_update_buffer")

    def lusgs(self, mesh=1, alfa1=0.0):
        _ck(self.L.ec2d_du_lusgs(self.h, mesh, alfa1), "ec2d_du_lusgs")

    def time_advance(self, mesh=1):
        _ck(self.L.ec2d_time_advance(self.h, mesh), "ec2d_time_advance")

    def interpolation2h(self, m1, m2, flag):
        _ck(self.L.ec2d_interpolation2h(self.h, m1, m2, flag), "ec2d_interpolation2h")

    def prolong(self, m1, m2, flag):
        _ck(self.L.ec2d_prolong(self.h, m1, m2, flag), "ec2d_prolong")

    def force_function(self, mesh):
        _ck(self.L.ec2d_force_function(self.h, mesh), "ec2d_force_function")

    def sync(self):
        _ck(self.L.ec2d_sync(self.h), "ec2d_sync")

    def stream_handle(self):
        """The context's cudaStream_t as an integer (for CUDA events)."""
        s = ctypes.c_void_p()
        _ck(self.L.ec2d_stream(self.h, ctypes.byref(s)), "ec2d_stream")
        return s.value or 0

    def launch_count(self):
        n = ctypes.c_longlong()
        _ck(self.L.ec2d_launch_count(self.h, ctypes.byref(n)), "ec2d_launch_count")
        return n.value

    def set_graphs(self, enable=True):
        """Replay each step as one CUDA graph (default) or launch kernels one by one."""
        _ck(self.L.ec2d_set_graphs(self.h, 1 if enable else 0), "ec2d_set_graphs")

    def run_to_drop(self, drop=1e-8, r0=None, max_steps=1000000, max_seconds=0.0, check_every=25):
        """Iterate until every case's Res_rms(1) <= drop * r0 (r0: the first
        step's residual unless given).  Returns (steps, worst ratio, seconds)."""
        n = ctypes.c_int(); w = ctypes.c_double(); t = ctypes.c_double()
        r0a = None if r0 is None else np.ascontiguousarray(r0, dtype=np.float64)
        r0p = None if r0a is None else _dp(r0a)
        _ck(self.L.ec2d_run_to_drop(self.h, drop, r0p, int(max_steps), float(max_seconds), int(check_every),
                                    ctypes.byref(n), ctypes.byref(w), ctypes.byref(t)), "ec2d_run_to_drop")
        return n.value, w.value, t.value

    def autotune(self, trial_steps=5):
        """Pick the fastest launch configuration; returns (cluster CTAs, rows
        per warp, concurrent flux kernels, ms per step)."""
        cs, rpw, cc, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _ck(self.L.ec2d_autotune(self.h, int(trial_steps), ctypes.byref(cs), ctypes.byref(rpw), ctypes.byref(cc),
                                 ctypes.byref(ms)), "ec2d_autotune")
        return cs.value, rpw.value, cc.value, ms.value

    def set_case_shape(self, case, shape):
        """Per-case shape feature of the warm-start network (the airfoil t/c)."""
        _ck(self.L.ec2d_set_case_shape(self.h, case, float(shape)), "ec2d_set_case_shape")

    def lusgs_shape(self):
        """(lusgs_cs, rows, lanes) of the FP64 wavefront in use."""
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _ck(self.L.ec2d_lusgs_shape(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "ec2d_lusgs_shape")
        return a.value, b.value, c.value

    def clear_status(self, case=0):
        """Clear a case's status word (0: every case)."""
        _ck(self.L.ec2d_clear_status(self.h, case), "ec2d_clear_status")

    def tile_residual(self, enable=-1):
        """The one-kernel residual on (1) / off (0); -1 reads; returns the setting."""
        c = ctypes.c_int()
        _ck(self.L.ec2d_tile_residual(self.h, int(enable), ctypes.byref(c)), "ec2d_tile_residual")
        return c.value

    LAUNCH_KEYS = ("lusgs_cs", "rows", "lanes", "concurrent", "tile_residual")

    def launch_config(self):
        """The launch choices in use (what ec2d_autotune picks), as a dict."""
        v = [ctypes.c_int() for _ in self.LAUNCH_KEYS]
        _ck(self.L.ec2d_launch_config(self.h, *[ctypes.byref(x) for x in v]), "ec2d_launch_config")
        return {k: x.value for k, x in zip(self.LAUNCH_KEYS, v)}

    def set_launch_config(self, cfg):
        """Apply launch choices (a dict as launch_config returns) without timing them."""
        _ck(self.L.ec2d_set_launch_config(self.h, *[int(cfg[k]) for k in self.LAUNCH_KEYS]),
            "ec2d_set_launch_config")

    def launch_signature(self):
        """What the launch choices depend on (device, library build, method
        flags, block shapes per level), one line; the autotuner cache's key."""
        n = ctypes.c_int()
        _ck(self.L.ec2d_launch_signature(self.h, None, 0, ctypes.byref(n)), "ec2d_launch_signature")
        buf = ctypes.create_string_buffer(n.value)
        _ck(self.L.ec2d_launch_signature(self.h, buf, n.value, ctypes.byref(n)), "ec2d_launch_signature")
        return buf.value.decode()

    def mg_eddy_viscosity(self, enable=-1):
        """Coarse multigrid levels keep the restricted eddy viscosity (1) or
        are laminar as in the reference (0); -1 reads; returns the setting."""
        c = ctypes.c_int()
        _ck(self.L.ec2d_mg_eddy_viscosity(self.h, int(enable), ctypes.byref(c)), "ec2d_mg_eddy_viscosity")
        return c.value

    def set_coarse_precision(self, bits):
        """64 (default) or 32: arithmetic of the coarse multigrid levels' face fluxes."""
        _ck(self.L.ec2d_set_coarse_precision(self.h, int(bits)), "ec2d_set_coarse_precision")

    def set_lusgs_precision(self, bits):
        """64 (default) or 32: arithmetic of the LU-SGS sweeps on every level."""
        _ck(self.L.ec2d_set_lusgs_precision(self.h, int(bits)), "ec2d_set_lusgs_precision")

    def kernel_timing(self, enable=True):
        _ck(self.L.ec2d_kernel_timing(self.h, 1 if enable else 0), "ec2d_kernel_timing")

    def kernel_times(self):
        """{(name, level): (calls, kernels, total_ms)} since timing was enabled."""
        buf = ctypes.create_string_buffer(1 << 16)
        _ck(self.L.ec2d_kernel_times(self.h, buf, len(buf)), "ec2d_kernel_times")
        out = {}
        for line in buf.value.decode().splitlines():
            name, lvl, calls, nk, ms = line.split()
            out[(name, int(lvl))] = (int(calls), int(nk), float(ms))
        return out


class WarmStartNet:
    """The learned warm start (ec2d_mlp_*): a coordinate-conditioned MLP over
    (x, y, log10 dw, M, AoA, log10 Re, shape) -> (rho, rho u, rho v, E,
    log1p(nu_tilde Re)), trained on solved fields by the library's kernels."""

    NIN, NOUT = 7, 5

    def __init__(self, hidden=6, width=256, seed=1, device=0):
        self.L = lib()
        h = ctypes.c_void_p()
        _ck(self.L.ec2d_mlp_create(device, hidden, width, seed, ctypes.byref(h)), "ec2d_mlp_create")
        self.h = h
        n = ctypes.c_int()
        _ck(self.L.ec2d_mlp_num_layers(self.h, ctypes.byref(n)), "ec2d_mlp_num_layers")
        self.nlin = n.value

    def close(self):
        if self.h:
            self.L.ec2d_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_gemm(self, kind):
        """1: tcgen05 GEMM kernels, 0: mma.sync GEMM kernels."""
        _ck(self.L.ec2d_mlp_set_gemm(self.h, int(kind)), "ec2d_mlp_set_gemm")

    def add_samples(self, solver):
        _ck(self.L.ec2d_mlp_add_samples(self.h, solver.h), "ec2d_mlp_add_samples")

    def num_samples(self):
        n = ctypes.c_longlong()
        _ck(self.L.ec2d_mlp_num_samples(self.h, ctypes.byref(n)), "ec2d_mlp_num_samples")
        return n.value

    def clear_samples(self):
        _ck(self.L.ec2d_mlp_clear_samples(self.h), "ec2d_mlp_clear_samples")

    def fit_normalization(self):
        _ck(self.L.ec2d_mlp_fit_normalization(self.h), "ec2d_mlp_fit_normalization")

    def train(self, steps, batch=16384, lr=1e-3):
        l = ctypes.c_double()
        _ck(self.L.ec2d_mlp_train(self.h, int(steps), int(batch), float(lr), ctypes.byref(l)), "ec2d_mlp_train")
        return l.value

    def warm_start(self, solver):
        """Write the predicted field into every case of `solver`; returns the
        number of cases that kept the freestream."""
        n = ctypes.c_int()
        _ck(self.L.ec2d_mlp_warm_start(self.h, solver.h, ctypes.byref(n)), "ec2d_mlp_warm_start")
        return n.value

    def layer_shape(self, layer):
        r, c = ctypes.c_int(), ctypes.c_int()
        _ck(self.L.ec2d_mlp_layer_shape(self.h, layer, ctypes.byref(r), ctypes.byref(c)), "ec2d_mlp_layer_shape")
        return r.value, c.value

    def get_weights(self, layer):
        r, c = self.layer_shape(layer)
        w = np.zeros((r, c), np.float32); b = np.zeros(r, np.float32)
        _ck(self.L.ec2d_mlp_get_weights(self.h, layer, _fp(w), _fp(b)), "ec2d_mlp_get_weights")
        return w, b

    def set_weights(self, layer, w, b):
        w = np.ascontiguousarray(w, np.float32); b = np.ascontiguousarray(b, np.float32)
        _ck(self.L.ec2d_mlp_set_weights(self.h, layer, _fp(w), _fp(b)), "ec2d_mlp_set_weights")

    def get_grads(self, layer):
        r, c = self.layer_shape(layer)
        w = np.zeros((r, c), np.float32); b = np.zeros(r, np.float32)
        _ck(self.L.ec2d_mlp_get_grads(self.h, layer, _fp(w), _fp(b)), "ec2d_mlp_get_grads")
        return w, b

    def get_normalization(self):
        a = np.zeros(2 * self.NIN + 2 * self.NOUT, np.float32)
        _ck(self.L.ec2d_mlp_get_normalization(self.h, _fp(a)), "ec2d_mlp_get_normalization")
        return a

    def set_normalization(self, a):
        a = np.ascontiguousarray(a, np.float32)
        _ck(self.L.ec2d_mlp_set_normalization(self.h, _fp(a)), "ec2d_mlp_set_normalization")

    def loss_grad(self, x, y):
        x = np.ascontiguousarray(x, np.float32); y = np.ascontiguousarray(y, np.float32)
        l = ctypes.c_double()
        _ck(self.L.ec2d_mlp_loss_grad(self.h, _fp(x), _fp(y), x.shape[0], ctypes.byref(l)), "ec2d_mlp_loss_grad")
        return l.value

    def predict(self, feat):
        feat = np.ascontiguousarray(feat, np.float32)
        out = np.zeros((feat.shape[0], self.NOUT), np.float32)
        _ck(self.L.ec2d_mlp_predict(self.h, _fp(feat), feat.shape[0], _fp(out)), "ec2d_mlp_predict")
        return out
