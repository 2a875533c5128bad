"""Build libcolore_cuda.so (sm_103a kernels + C ABI + C host side) and the
colore_gpu driver in-tree, compiling translation units in parallel.

Outputs:
    colore_gb300/lib/libcolore_cuda.so
    colore_gb300/lib/colore_gpu
Objects go to colore_gb300/_build/ and are reused while newer than every
source and header.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(CSRC, "host")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libcolore_cuda.so")
DRIVER = os.path.join(LIBDIR, "colore_gpu")

FIELD_SIZES = [64, 96, 128, 192, 256, 384, 512, 1024, 2048]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    return "nvcc"


NVFLAGS = ["-std=c++17", "-O3", ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-diag-suppress", "177",
           "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
CFLAGS = ["-O2", "-fPIC", "-std=gnu11", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _headers():
    hs = []
    for d in (CSRC, HOST, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                hs.append(os.path.join(d, f))
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _jobs():
    units = []  # (out, cmd, deps)
    hdr = _headers()
    for n in FIELD_SIZES:
        src = os.path.join(CSRC, "field_impl.cu")
        out = os.path.join(BUILD, "field_%d.o" % n)
        units.append((out, [nvcc()] + NVFLAGS + ["-DCG_N=%d" % n, "-c", src, "-o", out], [src] + hdr))
    for name in ("dens", "srcs", "imap", "kappa", "capi", "fp64"):
        src = os.path.join(CSRC, name + ".cu")
        out = os.path.join(BUILD, name + ".o")
        units.append((out, [nvcc()] + NVFLAGS + ["-c", src, "-o", out], [src] + hdr))
    for name in ("host_cosmo", "host_params", "host_io", "host_pred"):
        src = os.path.join(HOST, name + ".c")
        out = os.path.join(BUILD, name + ".o")
        units.append((out, ["gcc"] + CFLAGS + ["-c", src, "-o", out], [src] + hdr))
    return units


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    units = _jobs()
    todo = [u for u in units if _stale(u[0], u[2])]
    jobs = jobs or min(32, max(2, os.cpu_count() or 2))
    if todo:
        with ThreadPoolExecutor(jobs) as ex:
            list(ex.map(lambda u: _run(u[1], verbose), todo))
    objs = [u[0] for u in units]
    if _stale(LIB, objs):
        cudalib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "lib64")
        _run([nvcc(), "-shared", ARCH, "-o", LIB] + objs +
             ["-cudart=static", "-L" + cudalib, "-lcufft", "-Xlinker", "-rpath=" + cudalib, "-lm"], verbose)
    drv = os.path.join(HOST, "colore_gpu.c")
    if os.path.exists(drv) and _stale(DRIVER, [drv, LIB] + _headers()):
        _run(["gcc"] + CFLAGS + ["-o", DRIVER, drv, "-L" + LIBDIR, "-lcolore_cuda",
                                 "-Wl,-rpath,$ORIGIN", "-lm"], verbose)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
