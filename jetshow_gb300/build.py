"""Build recipe of the in-tree CUDA library ``_build/libjetshow_gb300.so``.

nvcc compiles the kernels for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``); g++ compiles the host translation units.
Every unit is compiled in parallel, then nvcc links one shared library.
Host code is built with ``-ffp-contract=off``: the image-plane constants it
computes feed the bit-exact FP64 geometry kernels.  The mixed-precision
kernels are built with ``--fmad=false`` (no implicit fma contraction), so that
the same lane-machine code rounds the same way in each kernel it is
instantiated in.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
REPO = os.path.dirname(HERE)
LIB = os.path.join(OUT, "libjetshow_gb300.so")

CU_SOURCES = ["jsh_kernels.cu", "jsh_fp64.cu", "jsh_persistent.cu", "jsh_persistent_ft.cu", "jsh_noalloc.cu", "jsh_stripe.cu",
              "jsh_visibility.cu"]
CPP_SOURCES = ["jsh_host.cpp", "jsh_capi.cpp", "jsh_server.cpp", "jsh_autotune.cpp", "jsh_grid.cpp", "jsh_hull.cpp", "jsh_cells.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Units whose kernels must round identically in every instantiation: the
# mixed-precision lane machine runs in several kernels (static, single
# persistent, split tau and IQUV kernels) whose images are bitwise equal
# only if the compiler fuses no multiply-add on its own (the explicit fmaf
# calls stay fused).
NO_CONTRACT = {"jsh_persistent.cu", "jsh_persistent_ft.cu"}
# Sources that include another source file.
INCLUDED = {"jsh_persistent_ft.cu": ["jsh_persistent.cu"]}


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + CSRC, "-I" + os.path.join(REPO, "include")]
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(REPO, "include", "jetshow_capi.h"))
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
               "-Xptxas", "-v", "-Xcompiler", "-fPIC,-ffp-contract=off", *inc, "-c", s, "-o", o]
        if src in NO_CONTRACT:
            cmd.insert(1, "--fmad=false")
        jobs.append((o, [s, *headers, *(os.path.join(CSRC, f) for f in INCLUDED.get(src, []))], cmd))
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
               *inc, "-I" + os.path.join(cuda, "include"), "-c", s, "-o", o]
        jobs.append((o, [s, *headers], cmd))
    logs = {}
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        futs = {}
        for o, deps, cmd in jobs:
            if not force and _newer(o, deps):
                continue
            futs[ex.submit(_run, cmd)] = o
        for f in cf.as_completed(futs):
            logs[futs[f]] = f.result()
    objs = [o for o, _, _ in jobs]
    if force or not _newer(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", LIB,
              "-lcudart_static", "-ldl", "-lrt", "-lpthread"])
    for o, txt in logs.items():  # one resource report per recompiled object
        with open(o + ".ptxas.log", "w") as fh:
            fh.write(txt)
    if verbose:
        for o, txt in logs.items():
            print(f"== {os.path.basename(o)}\n{txt}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
