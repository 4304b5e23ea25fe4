"""ctypes wrapper of the reference's own operator kernels (test infrastructure only).

oracle/_ref/libref.so holds ellipticPartialAxHex3D and the ogs gather kernel as the
reference wrote them (translated from OKL by oracle/okl_translate.py, driven by
oracle/ref_harness.c the way elliptic_t::Operator drives them on one rank). Only tests/
and bench.py's CPU baseline and reference arm use it, as a checker and as the
reference's CPU implementation; the product path never does.
"""
import ctypes

import numpy as np

from . import build as _build

_lib = None


def available():
    """True when the reference's kernels could be built (the reference tree, or the C file
    generated from it, is present)."""
    return lib() is not None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_ref()
        if path is None:
            return None
        L = ctypes.CDLL(path)
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.ref_op_create.restype = vp
        L.ref_op_create.argtypes = [ip, ip, vp, ip, vp, vp, vp, dp]
        L.ref_op_destroy.argtypes = [vp]
        L.ref_op_apply.argtypes = [vp, vp, vp]
        L.ref_op_partial_ax.argtypes = [vp, vp, vp]
        L.ref_op_time.restype = dp
        L.ref_op_time.argtypes = [vp, vp, vp, ip, ip]
        L.ref_threads.restype = ip
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefOperator:
    """The reference's elliptic_t::Operator (partialAx + Gather(Add, Trans)) on host arrays:
    GlobalToLocal (int32, E*Np, -1 masked), wJ (E*Np), ggeo (E*6*Np, the reference layout),
    D ((N+1)^2, row-major) and a scalar lambda."""

    def __init__(self, N, E, g2l, Ngather, wJ, ggeo, D, lam):
        L = lib()
        if L is None:
            raise RuntimeError("reference kernels not built (no reference tree or generated oracle/_ref)")
        Np = (N + 1) ** 3
        self.g2l = np.ascontiguousarray(g2l, dtype=np.int32)
        self.wJ = np.ascontiguousarray(wJ, dtype=np.float64)
        self.ggeo = np.ascontiguousarray(ggeo, dtype=np.float64)
        self.D = np.ascontiguousarray(D, dtype=np.float64)
        assert self.g2l.size == E * Np and self.wJ.size == E * Np and self.ggeo.size == 6 * E * Np
        if E * Np >= 2 ** 31:
            raise ValueError("the reference's dlong (int) indexing holds at most 2^31 - 1 local nodes")
        self.N, self.E, self.Np, self.Ngather = N, E, Np, Ngather
        self.h = L.ref_op_create(N, E, _p(self.g2l), Ngather, _p(self.wJ), _p(self.ggeo), _p(self.D), float(lam))
        if not self.h:
            raise ValueError("ref_op_create failed")

    @classmethod
    def from_oracle(cls, o, lam):
        """Built on the arrays of an oracle.Oracle object (same mesh, numbering and factors)."""
        N = o.info("nq") - 1
        return cls(N, o.info("nelements"), o.array("GlobalToLocal"), o.Ngather, o.array("wJ"),
                   o.array("ggeo"), o.array("D"), lam)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_op_destroy(self.h)
            self.h = None

    def apply(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros(self.Ngather)
        lib().ref_op_apply(self.h, _p(q), _p(out))
        return out

    def partial_ax(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros(self.E * self.Np)
        lib().ref_op_partial_ax(self.h, _p(q), _p(out))
        return out

    def time(self, q, reps, nthreads=0):
        """Wall seconds of `reps` operator applications (after one warm-up)."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros(self.Ngather)
        return lib().ref_op_time(self.h, _p(q), _p(out), reps, nthreads)


def threads():
    return lib().ref_threads()
