"""In-tree build of libseiswg.so (CUDA kernels for sm_103a + C++ host + C ABI)
and the `seiswg` command-line tool.

    python -m seiswg_gb300.build          # or __graft_entry__.build()

Objects go to seiswg_gb300/_lib/obj, the library and the tool to
seiswg_gb300/_lib.  Translation units compile in parallel; a unit is rebuilt
when it or any header is newer than its object.  No cmake, no -march flags:
the same sources build on x86-64 and on aarch64.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libseiswg.so")
CLI = os.path.join(OUT, "seiswg")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills"]
# -fmad=false: the forward stencil keeps the reference's separate multiply and
# add (fd2d.wgsl); those kernels are bandwidth-bound, so this costs nothing.
# The reverse step (no counterpart in the reference), the two-step forward
# kernel and the spin kernel are issue-bound, so they contract multiply-add
# pairs.
FMAD = {"fd_adjoint.cu": "true", "fd_step2.cu": "true", "fd_step2pc.cu": "true", "fd_adjointpc.cu": "true", "fd_spin.cu": "true", "fd_queue.cu": "true"}
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fno-strict-aliasing", "-Wall", "-Wextra", f"-I{CUDA_HOME}/include",
             f"-I{os.path.join(ROOT, 'include')}"]

CU_SOURCES = ["fd_step.cu", "fd_step2.cu", "fd_step2pc.cu", "fd_spin.cu", "fd_cluster.cu", "fd_aux.cu", "fd_adjoint.cu", "fd_adjointpc.cu", "fd_batch.cu", "fd_queue.cu", "noalloc.cu"]
CXX_SOURCES = ["engine.cpp", "host.cpp", "batch.cpp", "capi.cpp"]
CLI_SOURCES = ["cli.cpp"]


def _headers():
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _stale(src, obj, hdr_mtime):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or hdr_mtime > t


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, force=False):
    """Compile every translation unit that changed, then link. Returns LIB."""
    os.makedirs(OBJ, exist_ok=True)
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    hdr = _headers()
    jobs = []
    for s in CU_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(OBJ, s + ".o")
        if force or _stale(src, obj, hdr):
            jobs.append([NVCC] + NVCC_FLAGS + [f"-fmad={FMAD.get(s, 'false')}", "-c", src, "-o", obj])
    for s in CXX_SOURCES + CLI_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(OBJ, s + ".o")
        if force or _stale(src, obj, hdr):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
        if verbose:
            for j, log in zip(jobs, logs):
                print(" ".join(j))
                if log.strip():
                    print(log)
    lib_objs = [os.path.join(OBJ, s + ".o") for s in CU_SOURCES + CXX_SOURCES]
    newest = max(os.path.getmtime(o) for o in lib_objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        _run(["g++", "-shared", "-o", tmp] + lib_objs +
             [f"-L{CUDA_HOME}/lib64", "-lcudart_static", "-ldl", "-lpthread", "-lrt"])
        os.replace(tmp, LIB)
    cli_obj = os.path.join(OBJ, "cli.cpp.o")
    if force or not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(cli_obj),
                                                                         os.path.getmtime(LIB)):
        _run(["g++", "-o", CLI, cli_obj, f"-L{OUT}", "-lseiswg", "-Wl,-rpath,$ORIGIN"])
    return LIB


def clean():
    shutil.rmtree(OUT, ignore_errors=True)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
