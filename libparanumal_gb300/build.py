"""Build the GB300 (sm_103a) shared library in-tree.

Compiles the CUDA kernels (csrc/*.cu) with nvcc for sm_103a only and the host
objects (csrc/host/*.cpp) with g++ and OpenMP, in parallel, and links them into
libparanumal_gb300/_build/liblpg.so. No cmake, no torch extension machinery.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblpg.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    host = os.path.join(CSRC, "host")
    cpp = sorted(os.path.join(host, f) for f in os.listdir(host) if f.endswith(".cpp"))
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh"))]
    hdrs += [os.path.join(host, f) for f in os.listdir(host) if f.endswith(".hpp")]
    hdrs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return cu, cpp, hdrs


def _fingerprint(files, flags):
    h = hashlib.sha256()
    for f in sorted(files):
        h.update(f.encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def build_library(force=False, verbose=False, jobs=None):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    cu, cpp, hdrs = _sources()
    nvflags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                      "-Xcompiler", "-fPIC,-fopenmp", "-I" + INCLUDE]
    # -ffp-contract=off: host arithmetic rounds the same on x86-64 and aarch64 (where g++
    # would otherwise fuse multiply-adds)
    ccflags = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-I" + INCLUDE,
               "-I" + os.path.join(cuda, "include")]
    fp = _fingerprint(cu + cpp + hdrs + [__file__], nvflags + ccflags)
    stamp = os.path.join(OUT, "fingerprint")
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == fp:
        return LIB
    os.makedirs(OUT, exist_ok=True)
    jobs = jobs or max(1, min(8, os.cpu_count() or 1))
    cmds = []
    objs = []
    for src in cu:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        cmds.append([nvcc] + nvflags + ["-c", src, "-o", obj])
        objs.append(obj)
    for src in cpp:
        obj = os.path.join(OUT, "host_" + os.path.basename(src) + ".o")
        cmds.append(["g++"] + ccflags + ["-c", src, "-o", obj])
        objs.append(obj)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
        return p.stderr

    with cf.ThreadPoolExecutor(jobs) as ex:
        for err in ex.map(run, cmds):
            if verbose and err.strip():
                print(err)
    tmp = LIB + ".tmp%d" % os.getpid()
    run([nvcc] + ARCH + ["-shared", "-cudart=static", "-o", tmp] + objs +
        ["-Xcompiler", "-fopenmp", "-lgomp", "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(fp)
    return LIB


if __name__ == "__main__":
    import sys
    print(build_library(force="--force" in sys.argv, verbose=True))
