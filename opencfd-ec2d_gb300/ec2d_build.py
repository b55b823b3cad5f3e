"""Build libec2d_gpu.so (sm_103a) in-tree: one nvcc process per translation
unit, in parallel, then a shared-library link.  Usage: python ec2d_build.py [-v]"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib", "libec2d_gpu.so")
SOURCES = ["ec2d_api.cu", "k_residual.cu", "k_turb.cu", "k_bl.cu", "k_bc.cu", "k_lusgs.cu", "k_sweep.cu",
           "k_sweep32.cu", "k_misc.cu", "k_noalloc.cu", "k_mlp.cu", "k_peak.cu", "k_setup.cu",
           "k_gemm_tc.cu"]
# per-file flags: the Baldwin-Lomax switch is discrete, and the mesh set-up
# must give the reference's geometry bit for bit, so their products and sums
# are rounded one by one like the reference's
FILE_FLAGS = {"k_bl.cu": ["-fmad=false"], "k_setup.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _write_build_id(paths, extra) -> str:
    """A translation unit holding a digest of the library's sources, headers
    and flags (ec2d_launch_signature reports it, so launch choices cached by
    a host are not reused after the kernels change); rewritten only when the
    digest changes, so an unchanged tree rebuilds nothing."""
    h = hashlib.sha256()
    for p in sorted(paths, key=os.path.basename):
        h.update(os.path.basename(p).encode() + b"\0")
        with open(p, "rb") as fh:
            h.update(fh.read())
    h.update(repr((ARCH, FLAGS, sorted(FILE_FLAGS.items()), list(extra))).encode())
    src = os.path.join(OUT, "build_id.cpp")
    text = f'extern "C" const char ec2d_internal_build_id[] = "{h.hexdigest()[:16]}";\n'
    old = open(src).read() if os.path.exists(src) else None
    if old != text:
        with open(src, "w") as fh:
            fh.write(text)
    return src


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    headers = [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "ec2d_gpu.h"))
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(SRC, s))]
    objs, jobs = [], []
    bid = _write_build_id([os.path.join(SRC, s) for s in srcs] + headers, extra)
    bid_obj = os.path.join(OUT, "build_id.o")
    objs.append(bid_obj)
    if _stale(bid_obj, [bid]):
        jobs.append([nvcc(), "-Xcompiler", "-fPIC", "-c", bid, "-o", bid_obj])
    for s in srcs:
        src = os.path.join(SRC, s)
        obj = os.path.join(OUT, s.replace(".cu", ".o"))
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc(), *ARCH, *FLAGS, *FILE_FLAGS.get(s, []), *extra, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    build_host(verbose)
    return LIB


HOST_SRC = os.path.join(HERE, "host", "ec2d_host.c")
HOST = os.path.join(HERE, "lib", "ec2d_host")


def build_host(verbose: bool = False) -> str:
    """The C replica of the reference driver (host/ec2d_host.c), linked
    against the library beside it (rpath $ORIGIN)."""
    inc = os.path.join(HERE, "..", "include")
    if os.path.exists(HOST) and not _stale(HOST, [HOST_SRC, LIB, os.path.join(inc, "ec2d_gpu.h")]):
        return HOST
    # no contraction of products into FMAs (aarch64 has them in its base
    # ISA): the host's output arithmetic rounds like the Python host's
    cmd = [os.environ.get("CC", "gcc"), "-O2", "-std=c11", "-ffp-contract=off", "-Wall", "-I", inc, HOST_SRC, "-o", HOST,
           "-L", os.path.dirname(LIB), "-lec2d_gpu", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return HOST


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
