"""libparanumal_gb300: GB300-native C0 hexahedral elliptic path.

Python view of the C ABI in include/lpg.h. The compute path is the CUDA library
libparanumal_gb300/_build/liblpg.so (built by libparanumal_gb300.build); importing
an entry point without it raises -- there is no CPU fallback.

Device buffers are passed as integers (device addresses), e.g. torch tensors'
``data_ptr()``; streams as integers (``torch.cuda.current_stream().cuda_stream``) or 0.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liblpg.so")

LPG_OK = 0
STATUS = {0: "OK", -1: "INVALID", -2: "CUDA", -3: "UNSUPPORTED", -4: "NOT_CONVERGED",
          -5: "ALLOC", -6: "SETTINGS", -7: "BREAKDOWN", -8: "TIMEOUT"}
INFO = dict(nelements=0, np=1, nglobal=2, nlocal=3, n=4, allneumann=5, mg_plevels=6,
            mg_amglevels=7, coarse_n=8, device_bytes=9, vcycles=10, fallbacks=11, host_chunks=12,
            ig_history=13, operator_applications=14, learned_timeouts=15, morton_order=16)

_lib = None


class LPGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "?"), status, msg))
        self.status = status


def lib():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libparanumal_gb300: %s is missing; build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    vp, i32, i64, f64, f32 = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double,
                              ctypes.c_float)
    L.lpg_last_error.restype = ctypes.c_char_p
    L.lpg_version.restype = ctypes.c_char_p
    ax64 = [i32, i64, vp, vp, vp, i64, vp, i64, vp, f64, vp, vp, vp, i64, vp]
    ax32 = [i32, i64, vp, vp, vp, i64, vp, i64, vp, f32, vp, vp, vp, i64, vp]
    sig = {
        "lpg_device_malloc": [ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint64],
        "lpg_device_free": [vp],
        "lpg_memcpy_h2d": [vp, vp, ctypes.c_uint64, vp],
        "lpg_memcpy_d2h": [vp, vp, ctypes.c_uint64, vp],
        "lpg_memcpy_d2d": [vp, vp, ctypes.c_uint64, vp],
        "lpg_set_device": [i32],
        "lpg_elliptic_zero_mean": [vp, vp, vp],
        "lpg_elliptic_mass": [vp, vp, vp, vp],
        "lpg_stream_sync": [vp],
        "lpg_ax_hex_f64": ax64,
        "lpg_ax_hex_f32": ax32,
        "lpg_ax_hex_bf16g": ax32,
        "lpg_partial_ax_hex_f64": [i32, i64, vp, vp, vp, i64, vp, i64, vp, f64, vp, vp, vp, vp],
        "lpg_ogs_gather_add_f64": [i64, vp, vp, vp, i64, vp],
        "lpg_ogs_gather_owner_f64": [i64, vp, vp, vp, vp],
        "lpg_ogs_scatter_f64": [i64, vp, vp, vp, vp],
        "lpg_axpy_f64": [i64, f64, vp, f64, vp, vp],
        "lpg_amxpy_f64": [i64, f64, vp, vp, f64, vp, vp],
        "lpg_dot_f64": [i64, vp, vp, vp, vp],
        "lpg_norm2sq_f64": [i64, vp, vp, vp],
        "lpg_dot_f64_noalloc": [i64, vp, vp, vp, vp],
        "lpg_pcg_update_f64": [i64, f64, vp, vp, vp, vp, vp, vp],
        "lpg_norm2_f64": [i64, vp, vp, vp],
        "lpg_box_partition": [i32, i32, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp],
        "lpg_halo_pack_f64": [i64, vp, vp, vp, vp],
        "lpg_halo_unpack_add_f64": [i64, vp, vp, vp, vp],
        "lpg_jacobi_f64": [i64, vp, vp, vp, vp],
        "lpg_pmg_restrict_f64": [i32, i32, i64, vp, vp, vp, vp, vp, vp, i64, vp],
        "lpg_pmg_restrict_f32": [i32, i32, i64, vp, vp, vp, vp, vp, vp, i64, vp],
        "lpg_pmg_prolong_add_f64": [i32, i32, i64, vp, vp, vp, vp, vp, vp, vp],
        "lpg_pmg_prolong_add_f32": [i32, i32, i64, vp, vp, vp, vp, vp, vp, vp],
        "lpg_cheb_start_f64": [i64, vp, vp, vp, vp, vp, vp, f64, i32, vp],
        "lpg_cheb_start_f32": [i64, vp, vp, vp, vp, vp, vp, f32, i32, vp],
        "lpg_cheb_update_f64": [i64, vp, vp, vp, vp, vp, f64, f64, vp],
        "lpg_cheb_update_f32": [i64, vp, vp, vp, vp, vp, f32, f32, vp],
        "lpg_csr_spmv_f64": [i64, vp, vp, vp, f64, vp, f64, vp, vp],
        "lpg_csr_cheb_start_f64": [i64, f64, vp, vp, vp, vp, vp, vp],
        "lpg_csr_cheb_residual_f64": [i64, vp, vp, vp, f64, f64, vp, vp, vp, vp, vp],
        "lpg_csr_cheb_update_f64": [i64, f64, f64, i32, vp, vp, vp, vp],
        "lpg_gemv_f64": [i64, vp, vp, vp, vp],
        "lpg_elliptic_create": [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)],
        "lpg_elliptic_destroy": [vp],
        "lpg_elliptic_get": [vp, ctypes.c_char_p, vp, ctypes.c_uint64],
        "lpg_elliptic_device_ptr": [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)],
        "lpg_elliptic_random_vector": [vp, ctypes.c_uint64, vp, vp],
        "lpg_elliptic_operator": [vp, vp, vp, vp],
        "lpg_elliptic_operator_f32": [vp, vp, vp, i32, vp],
        "lpg_elliptic_operator_host": [vp, vp, vp],
        "lpg_elliptic_operator_df64": [vp, vp, vp, vp],
        "lpg_elliptic_initial_guess": [vp, vp, vp, vp],
        "lpg_extrap_coeffs": [i32, i32, i32, vp],
        "lpg_elliptic_operator_host_f32": [vp, vp, vp, i32],
        "lpg_elliptic_precon": [vp, vp, vp, vp],
        "lpg_elliptic_solve": [vp, vp, vp, f64, i32, ctypes.POINTER(ctypes.c_int)],
        "lpg_elliptic_rhs": [vp, vp, vp],
        "lpg_elliptic_run": [vp, vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
    }
    sig.update({
        "lpg_mlp_forward_f32": [vp, i64, vp, vp, vp, vp],
        "lpg_mlp_backward_f32": [vp, i64, vp, vp, vp, vp, vp, vp],
        "lpg_mlp_adam_f32": [i64, vp, vp, vp, vp, f32, i32, vp],
        "lpg_mlp_forward_bf16": [vp, i64, vp, vp, vp],
        "lpg_smoother_train": [ctypes.c_char_p, i32, i32, i32, i32, f32, ctypes.c_uint64, vp, vp],
        "lpg_elliptic_set_learned_smoother": [vp, vp, f64],
        "lpg_debug_mlp_hold": [ctypes.c_uint64],
        "lpg_elliptic_plot_fields": [vp, vp, ctypes.c_char_p],
        "lpg_hex_mesh_info": [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                              ctypes.POINTER(ctypes.c_int64)],
        "lpg_hex_mesh_numbering": [ctypes.c_char_p, i32, vp, ctypes.POINTER(ctypes.c_int64)],
    })
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.lpg_elliptic_info.argtypes = [vp, i32]
    L.lpg_elliptic_info.restype = i64
    L.lpg_mlp_param_count.argtypes = []
    L.lpg_mlp_param_count.restype = i64
    L.lpg_mlp_workspace_floats.argtypes = [i64]
    L.lpg_mlp_workspace_floats.restype = i64
    _lib = L
    return L


def declared_symbols():
    """Entry points declared in include/lpg.h (parsed from the header)."""
    import re
    hdr = os.path.join(os.path.dirname(_HERE), "include", "lpg.h")
    txt = open(hdr).read()
    return sorted(set(re.findall(r"\b(lpg_[a-z0-9_]+)\s*\(", txt)))


def check(status):
    if status != LPG_OK:
        raise LPGError(status, lib().lpg_last_error().decode())
    return status


def settings_text(d):
    """Render {KEY: value} in the reference's .rc format ([KEY] newline value)."""
    if isinstance(d, str):
        return d
    return "".join("[%s]\n%s\n\n" % (k, v) for k, v in d.items())


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _host_ptr(x, dtype, n, writable=False):
    """Address of a contiguous host array of n entries of dtype (numpy or CPU tensor)."""
    if isinstance(x, np.ndarray):
        if x.dtype != np.dtype(dtype) or not x.flags["C_CONTIGUOUS"] or x.size != n:
            raise ValueError("host array must be contiguous %s of %d entries" % (dtype, n))
        if writable and not x.flags["WRITEABLE"]:
            raise ValueError("output array is read-only")
        return x.ctypes.data
    import torch
    if (not isinstance(x, torch.Tensor) or x.is_cuda or str(x.dtype) != "torch." + dtype
            or not x.is_contiguous() or x.numel() != n):
        raise ValueError("host tensor must be a contiguous CPU %s tensor of %d entries" % (dtype, n))
    return x.data_ptr()


class Elliptic:
    """elliptic_t for a box mesh (solvers/elliptic/elliptic.hpp:56-170).

    Settings use the reference's .rc keys (lpg_elliptic_create). Operator / precon /
    Solve act on device vectors of length Nglobal.
    """

    def __init__(self, settings):
        h = ctypes.c_void_p()
        check(lib().lpg_elliptic_create(settings_text(settings).encode(), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().lpg_elliptic_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self, what):
        return int(lib().lpg_elliptic_info(self.h, INFO[what]))

    @property
    def Nglobal(self):
        return self.info("nglobal")

    @property
    def Nlocal(self):
        return self.info("nlocal")

    def get(self, name):
        E, Np, Ng, Nl = self.info("nelements"), self.info("np"), self.Nglobal, self.Nlocal
        Nq = self.info("n") + 1
        spec = {"GlobalToLocal": (Nl, np.int32), "ownerLocal": (Ng, np.int32),
                "weightG": (Ng, np.float64), "D": (Nq * Nq, np.float64),
                "lambdaE": (E, np.float64), "ggeo": (E * 6 * Np, np.float64),
                "wJ": (E * Np, np.float64), "geo": (E * 7 * Np, np.float64),
                "invDiag": (Ng, np.float64)}[name]
        out = np.zeros(spec[0], dtype=spec[1])
        check(lib().lpg_elliptic_get(self.h, name.encode(), out.ctypes.data_as(ctypes.c_void_p),
                                     out.nbytes))
        return out

    def device_ptr(self, name):
        p = ctypes.c_void_p()
        check(lib().lpg_elliptic_device_ptr(self.h, name.encode(), ctypes.byref(p)))
        return p.value

    def random_vector(self, q, seed, stream=0):
        check(lib().lpg_elliptic_random_vector(self.h, seed, _ptr(q), stream or None))

    def Operator(self, q, Aq, stream=0):
        check(lib().lpg_elliptic_operator(self.h, _ptr(q), _ptr(Aq), stream or None))

    def OperatorF32(self, q, Aq, bf16geo=False, stream=0):
        """Reduced-precision operator (FP32 vectors; FP32 or BF16 geometric factors)."""
        check(lib().lpg_elliptic_operator_f32(self.h, _ptr(q), _ptr(Aq), 1 if bf16geo else 0,
                                              stream or None))

    def initial_guess(self, x, rhs, stream=0):
        """x = the configured initial-guess strategy's guess for rhs (device vectors)."""
        check(lib().lpg_elliptic_initial_guess(self.h, _ptr(x), _ptr(rhs), stream or None))

    def OperatorDF64(self, q, Aq, stream=0):
        """FP64-accurate operator in double-FP32 words (device vectors, FP64 in and out)."""
        check(lib().lpg_elliptic_operator_df64(self.h, _ptr(q), _ptr(Aq), stream or None))

    def OperatorHost(self, q, Aq, precision="FP64"):
        """Aq = A q on host arrays (numpy arrays or CPU tensors of Nglobal entries: float64
        for FP64, float32 for FP32 and BF16GEO). Upload, operator and download are pipelined
        over element chunks; page-locked (pinned) tensors are needed for the overlap."""
        dt = "float64" if precision == "FP64" else "float32"
        pq, pa = _host_ptr(q, dt, self.Nglobal), _host_ptr(Aq, dt, self.Nglobal, writable=True)
        if precision == "FP64":
            check(lib().lpg_elliptic_operator_host(self.h, pq, pa))
        elif precision in ("FP32", "BF16GEO"):
            check(lib().lpg_elliptic_operator_host_f32(self.h, pq, pa, 1 if precision == "BF16GEO" else 0))
        else:
            raise ValueError("precision must be FP64, FP32 or BF16GEO")

    def precon(self, r, z, stream=0):
        check(lib().lpg_elliptic_precon(self.h, _ptr(r), _ptr(z), stream or None))

    def mass(self, u, Mu, stream=0):
        """Mu = M u, the assembled diagonal mass product (device vectors of Nglobal)."""
        check(lib().lpg_elliptic_mass(self.h, _ptr(u), _ptr(Mu), stream or None))

    def rhs(self, r):
        check(lib().lpg_elliptic_rhs(self.h, _ptr(r), None))

    def Solve(self, x, r, tol=1e-8, maxit=5000):
        it = ctypes.c_int(0)
        st = lib().lpg_elliptic_solve(self.h, _ptr(x), _ptr(r), tol, maxit, ctypes.byref(it))
        if st not in (LPG_OK, -4):
            check(st)
        return it.value

    def set_learned_smoother(self, weights, threshold=0.5):
        """Use the element-local network (FP32 weights, lpg_mlp_param_count() values) as the
        fine-level smoother, with per-V-cycle fallback above `threshold`; None restores the
        plain smoother."""
        if weights is None:
            check(lib().lpg_elliptic_set_learned_smoother(self.h, None, threshold))
            return
        w = np.ascontiguousarray(weights, dtype=np.float32)
        check(lib().lpg_elliptic_set_learned_smoother(self.h, w.ctypes.data_as(ctypes.c_void_p), threshold))

    def Run(self, want_solution=False):
        xL = np.zeros(self.Nlocal) if want_solution else None
        it, nrm, err, sec = ctypes.c_int(0), ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
        st = lib().lpg_elliptic_run(self.h, xL.ctypes.data_as(ctypes.c_void_p) if xL is not None else None,
                                    ctypes.byref(it), ctypes.byref(nrm), ctypes.byref(err),
                                    ctypes.byref(sec))
        if st not in (LPG_OK, -4):
            check(st)
        return dict(iterations=it.value, norm=nrm.value, error=err.value, solve_seconds=sec.value,
                    xL=xL, converged=(st == LPG_OK))

    def PlotFields(self, qL, file_name):
        """VTU file of the local field qL (Nlocal doubles, device tensor or pointer)."""
        check(lib().lpg_elliptic_plot_fields(self.h, _ptr(qL), str(file_name).encode()))


def hex_mesh_info(path):
    """(elements, nodes, tagged boundary faces) of a Gmsh hexahedral mesh (host only)."""
    E, Nn, Nb = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
    check(lib().lpg_hex_mesh_info(str(path).encode(), ctypes.byref(E), ctypes.byref(Nn), ctypes.byref(Nb)))
    return E.value, Nn.value, Nb.value


def hex_mesh_numbering(path, N):
    """(GlobalToLocal int32[E*(N+1)^3], Nglobal) of the degree-N nodes of a Gmsh mesh (host only)."""
    E = hex_mesh_info(path)[0]
    g2l = np.zeros(E * (N + 1) ** 3, dtype=np.int32)
    ng = ctypes.c_int64(0)
    check(lib().lpg_hex_mesh_numbering(str(path).encode(), N, g2l.ctypes.data_as(ctypes.c_void_p), ctypes.byref(ng)))
    return g2l, ng.value


def box_partition(nx, ny, nz, N, bcflag, nranks, rank):
    """z-slab partition of a box for `rank` of `nranks` (host only): dict with e0, e1,
    nowned, nlocal and the arrays global_to_local, below, above, lattice."""
    info = np.zeros(6, dtype=np.int64)
    L = lib()
    check(L.lpg_box_partition(nx, ny, nz, N, bcflag, nranks, rank, info.ctypes.data_as(ctypes.c_void_p),
                              None, None, None, None))
    e0, e1, nowned, nlocal, nb, na = (int(v) for v in info)
    g2l = np.zeros((e1 - e0) * (N + 1) ** 3, dtype=np.int32)
    below, above = np.zeros(nb, dtype=np.int32), np.zeros(na, dtype=np.int32)
    lattice = np.zeros(nlocal, dtype=np.int64)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    check(L.lpg_box_partition(nx, ny, nz, N, bcflag, nranks, rank, vp(info), vp(g2l), vp(below), vp(above),
                              vp(lattice)))
    return dict(e0=e0, e1=e1, nowned=nowned, nlocal=nlocal, global_to_local=g2l, below=below, above=above,
                lattice=lattice)


def extrap_coeffs(degree, history, cpqr=False):
    """Extrapolation weights of the EXTRAP initial guess (host computation)."""
    c = np.zeros(history)
    check(lib().lpg_extrap_coeffs(degree, history, 1 if cpqr else 0, c.ctypes.data_as(ctypes.c_void_p)))
    return c


def train_smoother(settings, nsolves=4, samples_per_solve=5000, epochs=30, batch=250, lr=1e-3, seed=7):
    """Train the learned smoother on (residual, exact error) pairs of the plain solver of
    `settings`; returns (weights float32[492800], per-epoch loss float32[epochs])."""
    n = int(lib().lpg_mlp_param_count())
    w = np.zeros(n, dtype=np.float32)
    hist = np.zeros(epochs, dtype=np.float32)
    check(lib().lpg_smoother_train(settings_text(settings).encode(), nsolves, samples_per_solve, epochs,
                                   batch, lr, seed, w.ctypes.data_as(ctypes.c_void_p),
                                   hist.ctypes.data_as(ctypes.c_void_p)))
    return w, hist


def ax_hex(prec, N, Nelements, g2l, ggeo, geo_stride, wJ, wJ_stride, D, lam, q, Aq, Nglobal,
           lambdaE=None, element_list=None, stream=0):
    """Assembled Ax through lpg_ax_hex_{f64,f32,bf16g}; device pointers or tensors."""
    fn = {"f64": lib().lpg_ax_hex_f64, "f32": lib().lpg_ax_hex_f32,
          "bf16g": lib().lpg_ax_hex_bf16g}[prec]
    check(fn(N, Nelements, _ptr(element_list), _ptr(g2l), _ptr(ggeo), geo_stride, _ptr(wJ),
             wJ_stride, _ptr(D), lam, _ptr(lambdaE), _ptr(q), _ptr(Aq), Nglobal, stream or None))
