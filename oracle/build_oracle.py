"""ORACLE build recipe (test infrastructure only): compiles the CPU
restatement in oracle/ into oracle/_lib/liboracle.so with OpenMP.

The library also carries its own build of the host C side (the param-file
reader and the FP64 cosmology and tracer tables, colore_gb300/csrc/host/),
so that the CPU reference arm of bench.py reads its configuration without
loading the GPU library.  -Bsymbolic binds those copies to each other when
both libraries live in one process.

Only tests/, the smoke check and bench.py's CPU-baseline leg load it.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUTDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUTDIR, "liboracle.so")
SRCS = ["or_fft.c", "or_ref64.c", "or_dev32.c", "or_checks.c", "or_sht.c"]
HOST = os.path.join(ROOT, "colore_gb300", "csrc", "host")
HOST_SRCS = ["host_cosmo.c", "host_params.c", "host_io.c", "host_pred.c"]


def build(verbose=False):
    os.makedirs(OUTDIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SRCS] + [os.path.join(HOST, s) for s in HOST_SRCS]
    csrc = os.path.join(ROOT, "colore_gb300", "csrc")
    deps = srcs + [os.path.join(HERE, "oracle.h"),
                   os.path.join(ROOT, "include", "colore_cuda.h"),
                   os.path.join(ROOT, "include", "colore_host.h")]
    deps += [os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith(".h")]
    deps += [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-fopenmp", "-ffp-contract=off",
           "-Wall", "-Wno-unused-function", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "colore_gb300", "csrc"), "-Wl,-Bsymbolic", "-o", LIB] + srcs + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
