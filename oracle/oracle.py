"""ctypes wrapper of the oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import
this module, and only as the checker; the product path never does.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

INFO = dict(nelements=0, np=1, ngather=2, nlocal=3, nq=4, allneumann=5,
            mg_plevels=6, mg_amglevels=7, coarse_n=8)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        vp, cp, ip, dp = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_double
        L.orc_create.restype = vp
        L.orc_create.argtypes = [cp, ctypes.POINTER(ctypes.c_int)]
        L.orc_destroy.argtypes = [vp]
        L.orc_info.restype = ctypes.c_longlong
        L.orc_info.argtypes = [vp, ip]
        L.orc_get_array.argtypes = [vp, cp, vp]
        for f in ("orc_operator_apply", "orc_partial_ax_apply", "orc_precon_apply", "orc_matrix_apply",
                  "orc_scatter_apply"):
            getattr(L, f).argtypes = [vp, vp, vp]
        L.orc_gather.argtypes = [vp, vp, vp, ip]
        L.orc_build_rhs.argtypes = [vp, vp]
        L.orc_pcg.argtypes = [vp, vp, vp, dp, ip, ctypes.POINTER(ctypes.c_double)]
        L.orc_run.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_int),
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.orc_time_operator.restype = dp
        L.orc_time_operator.argtypes = [vp, ip, ip]
        L.orc_u01.restype = dp
        L.orc_u01.argtypes = [ctypes.c_uint64] * 3
        L.orc_jacobiGLL.argtypes = [ip, vp, vp]
        L.orc_dmatrix1D.argtypes = [ip, vp, vp]
        L.orc_hessenberg_eigenvalues.argtypes = [ip, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def settings_text(d):
    """Render a {KEY: value} dict in the reference's .rc format."""
    return "".join("[%s]\n%s\n\n" % (k, v) for k, v in d.items())


class Oracle:
    """CPU restatement of elliptic_t for one settings file."""

    def __init__(self, settings):
        if isinstance(settings, dict):
            settings = settings_text(settings)
        st = ctypes.c_int(0)
        self.h = lib().orc_create(settings.encode(), ctypes.byref(st))
        if not self.h:
            raise ValueError("oracle: bad settings (status %d)" % st.value)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def info(self, what):
        return int(lib().orc_info(self.h, INFO[what]))

    @property
    def Ngather(self):
        return self.info("ngather")

    @property
    def Nlocal(self):
        return self.info("nlocal")

    def array(self, name):
        E, Np, Nq = self.info("nelements"), self.info("np"), self.info("nq")
        Nl = E * Np
        spec = {"ggeo": (E * 6 * Np, np.float64), "wJ": (Nl, np.float64),
                "D": (Nq * Nq, np.float64), "gllz": (Nq, np.float64), "gllw": (Nq, np.float64),
                "x": (Nl, np.float64), "y": (Nl, np.float64), "z": (Nl, np.float64),
                "EX": (E * 8, np.float64), "EY": (E * 8, np.float64), "EZ": (E * 8, np.float64),
                "GlobalToLocal": (Nl, np.int32), "globalIds": (Nl, np.int64),
                "mapB": (Nl, np.int32), "weightG": (self.Ngather, np.float64),
                "lambdaE": (E, np.float64), "invDiag": (self.Ngather, np.float64)}[name]
        out = np.zeros(spec[0], dtype=spec[1])
        rc = lib().orc_get_array(self.h, name.encode(), _p(out))
        if rc != 0:
            raise KeyError(name)
        return out

    def operator(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros(self.Ngather)
        lib().orc_operator_apply(self.h, _p(q), _p(out))
        return out

    def partial_ax(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros(self.Nlocal)
        lib().orc_partial_ax_apply(self.h, _p(q), _p(out))
        return out

    def matrix_apply(self, x):
        """A x with the assembled matrix (explicitly built, as the AMG setup does)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(self.Ngather)
        lib().orc_matrix_apply(self.h, _p(x), _p(out))
        return out

    def precon(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        out = np.zeros(self.Ngather)
        lib().orc_precon_apply(self.h, _p(r), _p(out))
        return out

    def gather(self, qL, trans=True):
        qL = np.ascontiguousarray(qL, dtype=np.float64)
        out = np.zeros(self.Ngather)
        lib().orc_gather(self.h, _p(qL), _p(out), 1 if trans else 0)
        return out

    def scatter(self, qG):
        qG = np.ascontiguousarray(qG, dtype=np.float64)
        out = np.zeros(self.Nlocal)
        lib().orc_scatter_apply(self.h, _p(qG), _p(out))
        return out

    def rhs(self):
        out = np.zeros(self.Ngather)
        lib().orc_build_rhs(self.h, _p(out))
        return out

    def pcg(self, r, tol=1e-8, maxit=5000, x0=None):
        r = np.array(r, dtype=np.float64)
        x = np.zeros(self.Ngather) if x0 is None else np.array(x0, dtype=np.float64)
        res = ctypes.c_double(0)
        it = lib().orc_pcg(self.h, _p(x), _p(r), tol, maxit, ctypes.byref(res))
        return x, it, res.value

    def run(self):
        xL = np.zeros(self.Nlocal)
        it, nrm, err = ctypes.c_int(0), ctypes.c_double(0), ctypes.c_double(0)
        lib().orc_run(self.h, _p(xL), ctypes.byref(it), ctypes.byref(nrm), ctypes.byref(err))
        return dict(xL=xL, iterations=it.value, norm=nrm.value, error=err.value)

    def time_operator(self, reps, nthreads=0):
        return lib().orc_time_operator(self.h, reps, nthreads)


def u01(seed, stream, key):
    return lib().orc_u01(seed, stream, key)


def threads():
    return lib().orc_threads()
