"""Build recipe for the oracle (test infrastructure only).

Compiles the plain-C restatement of the reference path (oracle/*.c) into
oracle/_build/liboracle.so with gcc, and the reference's own Ax and gather kernels
(translated from its OKL) into oracle/_ref/libref.so. The product library never links
either.
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


# The reference's own kernels (oracle/_ref/): OKL text translated to C by okl_translate.py
# from the reference tree when it is on this machine, then compiled with the reference's
# release flags (make.top: -fopenmp -O3 -ftree-vectorize; its -march=native/-mavx2 are left
# out so the same recipe builds on x86-64 and aarch64; contraction of multiply-adds stays
# gcc's default, as in the reference's build). Everything lands in oracle/_ref/, which is
# not committed; where the reference tree is absent (the GPU host) the generated C file
# that travelled with the working tree is compiled.
REF_TREE = os.environ.get("LIBPARANUMAL_DIR", "/root/reference")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "libref.so")


def build_ref(force=False, verbose=False):
    """oracle/_ref/libref.so, or None when neither the reference tree nor a generated
    oracle/_ref/ref_kernels.c is present."""
    from . import okl_translate as tr
    gen = tr.GENERATED
    if os.path.isdir(REF_TREE) and (force or not os.path.exists(gen) or
                                   os.path.getmtime(gen) < os.path.getmtime(tr.__file__)):
        tr.generate(REF_TREE)
    if not os.path.exists(gen):
        return None
    harness = os.path.join(HERE, "ref_harness.c")
    if not force and os.path.exists(REF_LIB):
        t = os.path.getmtime(REF_LIB)
        if all(os.path.getmtime(f) <= t for f in (gen, harness, __file__)):
            return REF_LIB
    tmp = REF_LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-ftree-vectorize", "-std=gnu11", "-fPIC", "-shared", "-w", "-o", tmp,
           harness, gen, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force=True, verbose=True))
    print(build_ref(force=True, verbose=True))
