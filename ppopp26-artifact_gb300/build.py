"""In-tree build of the CUDA library (libppfr.so) and the C++ host layer.

    python ppopp26-artifact_gb300/build.py

Compiles every ``csrc/*.cu`` for sm_103a in parallel (one ``-gencode``,
``-lineinfo``) and links ``libppfr.so`` next to this file; then builds the
SyncedMemory-compatible host layer ``libppcompat.so`` and its driver
``pp_compat_driver`` from ``host/``.  Objects go to ``_build/`` (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libppfr.so")
COMPAT_LIB = os.path.join(HERE, "libppcompat.so")
COMPAT_DRIVER = os.path.join(HERE, "pp_compat_driver")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Montgomery multiply formulation (csrc/fr.cuh), the transform's twiddle
# multiply (PP_NTT_MUL) and the pass kernels' blocks per SM (PP_NTT_MINB);
# overridable for experiments
MUL_VARIANT = os.environ.get("PP_MUL_VARIANT", "9")
NTT_MUL = os.environ.get("PP_NTT_MUL", "")
NTT_MINB = os.environ.get("PP_NTT_MINB", "")
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-DPP_MUL_VARIANT=" + MUL_VARIANT,
              "-I" + os.path.join(ROOT, "include")]
if NTT_MUL:
    NVCC_FLAGS.append("-DPP_NTT_MUL=" + NTT_MUL)
if NTT_MINB:
    NVCC_FLAGS.append("-DPP_NTT_MINB=" + NTT_MINB)


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(ROOT, "include", "pp_ops.h")]
    objs = []
    jobs = []
    for src in sources:
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *NVCC_FLAGS, *ARCH, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs])
    _build_host(nvcc, force)
    return LIB


def _build_host(nvcc: str, force: bool) -> None:
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    if not srcs:
        return
    hdrs = sorted(glob.glob(os.path.join(HOST, "*.h*"))) + [os.path.join(ROOT, "include", "pp_ops.h")]
    lib_srcs = [s for s in srcs if not os.path.basename(s).startswith("driver")]
    drv_srcs = [s for s in srcs if os.path.basename(s).startswith("driver")]
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    cxx = shutil.which("g++") or "g++"
    flags = ["-std=c++17", "-O2", "-fPIC", "-I" + os.path.join(ROOT, "include"), "-I" + HOST,
             "-I" + cuda_inc]
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "lib64")
    if force or _stale(COMPAT_LIB, lib_srcs + hdrs + [LIB]):
        _run([cxx, *flags, "-shared", "-o", COMPAT_LIB, *lib_srcs, "-L" + HERE, "-lppfr",
              "-L" + cuda_lib, "-lcudart", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + cuda_lib, "-pthread"])
    if drv_srcs and (force or _stale(COMPAT_DRIVER, drv_srcs + hdrs + [COMPAT_LIB])):
        _run([cxx, *flags, "-o", COMPAT_DRIVER, *drv_srcs, "-L" + HERE, "-lppcompat", "-lppfr",
              "-L" + cuda_lib, "-lcudart", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + cuda_lib, "-pthread"])


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
