"""Build libqgt_gb300.so in-tree: C11 host code (gcc) + CUDA kernels (nvcc, sm_103a).

    python -m quantum_geometric_tensor_gb300.build        # or __graft_entry__.build()

Translation units compile in parallel into quantum_geometric_tensor_gb300/lib/obj;
the shared library lands in quantum_geometric_tensor_gb300/lib/libqgt_gb300.so.
CUDA runtime is linked statically (one self-contained .so); the driver API
entry point for tensor maps is fetched at run time; NVRTC (the toolkit's
runtime compiler, for the per-plan pass kernels) is linked dynamically.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libqgt_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDES = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    c = sorted(glob.glob(os.path.join(CSRC, "host", "*.c")))
    cu = sorted(glob.glob(os.path.join(CSRC, "cuda", "*.cu")))
    return c, cu


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, r.returncode, r.stdout + r.stderr


def _embed_ops_header() -> str:
    """The gate routines of qgt_pass2_ops.cuh as a C array for the pass-kernel compiler (qgt_jit_rt.cu)."""
    gen = os.path.join(OBJDIR, "gen")
    os.makedirs(gen, exist_ok=True)
    data = open(os.path.join(CSRC, "cuda", "qgt_pass2_ops.cuh"), "rb").read()
    body = ",".join(str(b) for b in data)
    text = ("/* generated from qgt_pass2_ops.cuh by build.py */\n"
            f"static const char qgt_pass2_ops_src[] = {{{body},0}};\n")
    out = os.path.join(gen, "qgt_pass2_ops_src.h")
    if not os.path.exists(out) or open(out).read() != text:
        with open(out, "w") as f:
            f.write(text)
    return gen


def build(verbose: bool = False, extra_nvcc=None) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    gen = _embed_ops_header()
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "lib64")
    csrcs, cusrcs = sources()
    jobs = []
    objs = []
    for s in csrcs:
        o = os.path.join(OBJDIR, os.path.basename(s) + ".o")
        objs.append(o)
        jobs.append(["gcc", "-std=gnu11", "-O2", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter",
                     "-fvisibility=default", *INCLUDES, "-I/usr/local/cuda/include", "-c", s, "-o", o])
    for s in cusrcs:
        o = os.path.join(OBJDIR, os.path.basename(s) + ".o")
        objs.append(o)
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-v" if verbose else "-O3", *INCLUDES, "-I" + gen, *(extra_nvcc or []), "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        results = list(ex.map(_compile, jobs))
    failed = [(c, out) for c, rc, out in results if rc != 0]
    if verbose:
        for c, rc, out in results:
            if out.strip():
                print(os.path.basename(c[-3]), out, file=sys.stderr)
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + out for c, out in failed)
        raise RuntimeError("libqgt_gb300 build failed:\n" + msg)
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-cudart", "static", "-o", tmp, *objs,
            "-L" + cuda_lib, "-lnvrtc", "-Xlinker", "-rpath=" + cuda_lib, "-lm", "-ldl", "-lpthread", "-lrt"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("libqgt_gb300 link failed:\n" + " ".join(link) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
