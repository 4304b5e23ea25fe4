"""The level-kernel entry points of the C ABI against numpy restatements of the
reference's kernels, through ctypes on device tensors:

* lpg_pmg_restrict / lpg_pmg_prolong_add: ellipticPreconCoarsenHex3D.okl:209-294 and
  ellipticPreconProlongateHex3D.okl:216-301 -- per element, (P^T x P^T x P^T)(w .* r_local)
  assembled, and P x P x P of the coarse local values -- on two meshes of one box whose
  numberings, weights and owners come from the library's own setup arrays;
* lpg_cheb_start / lpg_cheb_update: MGLevel::smoothChebyshev's vector steps
  (ellipticPreconMultiGridLevel.cpp:154-206);
* lpg_csr_spmv / lpg_csr_cheb_*: parCSR::SpMV and the SmoothChebyshev.okl kernels on a
  random sparse matrix; lpg_gemv: dGEMV.okl;
* lpg_norm2 (linAlg_t::norm2) and lpg_jacobi (JacobiPrecon::Operator).
FP64 to 1e-13 relative (max-norm), FP32 to 1e-5."""
import ctypes

import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from gpu_helpers import box, rel_err
from oracle.oracle import lib as olib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


def gll(N):
    r, w = np.zeros(N + 1), np.zeros(N + 1)
    olib().orc_jacobiGLL(N, r.ctypes.data_as(ctypes.c_void_p), w.ctypes.data_as(ctypes.c_void_p))
    return r


def interp(Nf, Nc):
    rf, rc = gll(Nf), gll(Nc)
    P = np.ones((Nf + 1, Nc + 1))
    for j in range(Nc + 1):
        for m in range(Nc + 1):
            if m != j:
                P[:, j] *= (rf - rc[m]) / (rc[j] - rc[m])
    return P


def dev(a, dtype=None):
    return torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=dtype)


def tensor3(P, u, E, nin):
    """apply P in each direction to u[e][k][j][i] (i fastest)"""
    u = u.reshape(E, nin, nin, nin)
    return np.einsum("ai,bj,ck,ekji->ecba", P, P, P, u).reshape(E, -1)


@pytest.mark.parametrize("Nf,Nc", [(7, 3), (3, 1), (5, 2), (4, 4)])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_pmg_restrict_and_prolong(Nf, Nc, prec):
    base = box(**{"BOX NX": 3, "BOX NY": 2, "BOX NZ": 2, "LAMBDA": 1.0})
    ef = lpg.Elliptic(dict(base, **{"POLYNOMIAL DEGREE": Nf}))
    ec = lpg.Elliptic(dict(base, **{"POLYNOMIAL DEGREE": Nc}))
    E = ef.info("nelements")
    g2lf, g2lc = ef.get("GlobalToLocal"), ec.get("GlobalToLocal")
    wf, owner = ef.get("weightG"), ef.get("ownerLocal")
    P = interp(Nf, Nc)
    rng = np.random.default_rng(Nf * 10 + Nc)
    rF = rng.uniform(-1, 1, ef.Nglobal)
    xC = rng.uniform(-1, 1, ec.Nglobal)
    xF0 = rng.uniform(-1, 1, ef.Nglobal)
    # numpy restatement
    uF = np.where(g2lf >= 0, (wf * rF)[np.maximum(g2lf, 0)], 0.0)
    uC = tensor3(P.T, uF, E, Nf + 1).ravel()
    refC = np.zeros(ec.Nglobal)
    np.add.at(refC, g2lc[g2lc >= 0], uC[g2lc >= 0])
    vC = np.where(g2lc >= 0, xC[np.maximum(g2lc, 0)], 0.0)
    vF = tensor3(P, vC, E, Nc + 1).ravel()
    refF = xF0.copy()
    refF += vF[owner]
    dt, tol = (torch.float64, 1e-13) if prec == "f64" else (torch.float32, 1e-5)
    L = lpg.lib()
    restrict = getattr(L, "lpg_pmg_restrict_" + prec)
    prolong = getattr(L, "lpg_pmg_prolong_add_" + prec)
    d_g2lf, d_g2lc, d_owner = dev(g2lf), dev(g2lc), dev(owner)
    d_w, d_r, d_P = dev(wf, dt), dev(rF, dt), dev(P, dt)
    d_rC = torch.full((ec.Nglobal,), np.nan, device="cuda", dtype=dt)
    lpg.check(restrict(Nf, Nc, E, d_g2lf.data_ptr(), d_w.data_ptr(), d_r.data_ptr(), d_P.data_ptr(),
                       d_g2lc.data_ptr(), d_rC.data_ptr(), ec.Nglobal, None))
    d_xC, d_xF = dev(xC, dt), dev(xF0, dt)
    lpg.check(prolong(Nf, Nc, E, d_g2lc.data_ptr(), d_xC.data_ptr(), d_P.data_ptr(), d_g2lf.data_ptr(),
                      d_owner.data_ptr(), d_xF.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_err(d_rC.double().cpu().numpy(), refC) < tol
    assert rel_err(d_xF.double().cpu().numpy(), refF) < tol
    # a coarse degree above the fine one is refused
    assert restrict(Nc, Nf + 1, E, 0, 0, 0, 0, 0, 0, 1, None) == -1


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_chebyshev_passes(prec):
    n = 100_003
    rng = np.random.default_rng(4)
    inv, r, Ax, d0, x0, Ad = (rng.uniform(0.5, 2, n), rng.standard_normal(n), rng.standard_normal(n),
                              rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(n))
    dt, tol = (torch.float64, 1e-13) if prec == "f64" else (torch.float32, 1e-5)
    L = lpg.lib()
    start = getattr(L, "lpg_cheb_start_" + prec)
    update = getattr(L, "lpg_cheb_update_" + prec)
    # device copies stay referenced until the kernels have run
    d_inv, d_r, d_Ax, d_Ad = dev(inv, dt), dev(r, dt), dev(Ax, dt), dev(Ad, dt)
    for xIsZero in (1, 0):
        res, d, x = (torch.empty(n, device="cuda", dtype=dt), torch.empty(n, device="cuda", dtype=dt),
                     dev(x0, dt))
        lpg.check(start(n, d_inv.data_ptr(), d_r.data_ptr(), d_Ax.data_ptr(), res.data_ptr(),
                        d.data_ptr(), x.data_ptr(), 0.7, xIsZero, None))
        rr = inv * (r if xIsZero else r - Ax)
        dd = 0.7 * rr
        xx = dd if xIsZero else x0 + dd
        torch.cuda.synchronize()
        assert rel_err(res.double().cpu().numpy(), rr) < tol
        assert rel_err(d.double().cpu().numpy(), dd) < tol
        assert rel_err(x.double().cpu().numpy(), xx) < tol
        lpg.check(update(n, d_inv.data_ptr(), d_Ad.data_ptr(), res.data_ptr(), d.data_ptr(),
                         x.data_ptr(), 0.3, 1.9, None))
        rr = rr - inv * Ad
        dd = 0.3 * dd + 1.9 * rr
        xx = xx + dd
        torch.cuda.synchronize()
        assert rel_err(res.double().cpu().numpy(), rr) < tol
        assert rel_err(d.double().cpu().numpy(), dd) < tol
        assert rel_err(x.double().cpu().numpy(), xx) < tol


def random_csr(n, nnz_row, rng):
    rs = np.arange(0, n * nnz_row + 1, nnz_row, dtype=np.int64)
    rs[1:] -= rng.integers(0, 2, n).cumsum()   # ragged rows
    rs[-1] = max(rs[-1], rs[-2])
    cols = rng.integers(0, n, rs[-1]).astype(np.int32)
    vals = rng.standard_normal(rs[-1])
    A = np.zeros((n, n))
    for i in range(n):
        np.add.at(A[i], cols[rs[i]:rs[i + 1]], vals[rs[i]:rs[i + 1]])
    return rs, cols, vals, A


def test_csr_kernels_and_gemv():
    rng = np.random.default_rng(9)
    n = 777
    rs, cols, vals, A = random_csr(n, 9, rng)
    x, y0, b = rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(n)
    dinv = rng.uniform(0.5, 2, n)
    L = lpg.lib()
    d_rs, d_cols, d_vals, d_x, d_dinv, d_b = dev(rs), dev(cols), dev(vals), dev(x), dev(dinv), dev(b)
    y = dev(y0)
    lpg.check(L.lpg_csr_spmv_f64(n, d_rs.data_ptr(), d_cols.data_ptr(), d_vals.data_ptr(), 0.5, d_x.data_ptr(),
                                 -2.0, y.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_err(y.cpu().numpy(), 0.5 * A @ x - 2.0 * y0) < 1e-13
    # Chebyshev pieces
    r, d, xx = torch.empty(n, device="cuda", dtype=torch.float64), torch.empty(n, device="cuda",
                                                                                 dtype=torch.float64), dev(x)
    lpg.check(L.lpg_csr_cheb_start_f64(n, 0.8, d_dinv.data_ptr(), d_b.data_ptr(), r.data_ptr(), d.data_ptr(),
                                       xx.data_ptr(), None))
    rr = dinv * b
    torch.cuda.synchronize()
    assert rel_err(r.cpu().numpy(), rr) < 1e-14 and rel_err(xx.cpu().numpy(), 0.8 * rr) < 1e-14
    r0 = r.cpu().numpy()
    xcur = xx.cpu().numpy()
    lpg.check(L.lpg_csr_cheb_residual_f64(n, d_rs.data_ptr(), d_cols.data_ptr(), d_vals.data_ptr(), 1.0, 1.0,
                                          d_dinv.data_ptr(), d_b.data_ptr(), xx.data_ptr(), r.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_err(r.cpu().numpy(), r0 + dinv * (b - A @ xcur)) < 1e-13
    r1 = r.cpu().numpy()
    d0 = d.cpu().numpy()
    lpg.check(L.lpg_csr_cheb_update_f64(n, 0.25, 1.5, 0, r.data_ptr(), d.data_ptr(), xx.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_err(d.cpu().numpy(), 0.25 * d0 + 1.5 * r1) < 1e-14
    assert rel_err(xx.cpu().numpy(), xcur + 0.25 * d0 + 1.5 * r1) < 1e-14
    # dense coarse inverse
    m = 300
    M = rng.standard_normal((m, m))
    v = rng.standard_normal(m)
    out = torch.empty(m, device="cuda", dtype=torch.float64)
    d_M, d_v = dev(M), dev(v)
    lpg.check(L.lpg_gemv_f64(m, d_M.data_ptr(), d_v.data_ptr(), out.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_err(out.cpu().numpy(), M @ v) < 1e-13


def test_norm2_and_jacobi():
    rng = np.random.default_rng(2)
    n = 3_000_017
    x, inv = rng.standard_normal(n), rng.uniform(0.1, 3, n)
    L = lpg.lib()
    dx = dev(x)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    lpg.check(L.lpg_norm2_f64(n, dx.data_ptr(), out.data_ptr(), None))
    z = torch.empty_like(dx)
    d_inv = dev(inv)
    lpg.check(L.lpg_jacobi_f64(n, d_inv.data_ptr(), dx.data_ptr(), z.data_ptr(), None))
    torch.cuda.synchronize()
    assert abs(float(out) - np.linalg.norm(x)) < 1e-12 * np.linalg.norm(x)
    assert rel_err(z.cpu().numpy(), inv * x) < 1e-15
    assert L.lpg_norm2_f64(-1, dx.data_ptr(), out.data_ptr(), None) == -1
