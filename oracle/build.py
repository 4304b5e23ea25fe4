"""Build recipe for the oracle (test infrastructure only).

Compiles the plain-C restatement of the reference path (oracle/*.c) into
oracle/_build/liboracle.so with gcc. The product library never links it.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["orc_basis.c", "orc_mesh.c", "orc_gmsh.c", "orc_ipdg.c", "orc_solver.c"]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build_oracle(force=False, verbose=False):
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    hdrs = [os.path.join(HERE, h) for h in ("orc_internal.h", "oracle.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(f) <= t for f in srcs + hdrs + [__file__]):
            return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    # -ffp-contract=off: the same rounding on x86-64 and aarch64 (no fused multiply-adds)
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-D_GNU_SOURCE",
           "-Wall", "-Wno-unused-function", "-o", tmp] + srcs + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True, verbose=True))
