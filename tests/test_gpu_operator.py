"""Parity of the CUDA operator path with the oracle (CPU restatement of the
reference): box numbering, geometric factors, matrix-free Ax with fused assembly,
the reference-layout partial Ax contract, FP32/BF16 variants, gather-scatter and
reductions. FP64 results must agree to 1e-12 relative (max-norm); integer maps
must be identical."""
import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from gpu_helpers import box, lattice_q, rel_err
from oracle import refimpl
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

CASES = [
    box(),                                                   # jittered, N=7, lambda=1
    box(**{"POLYNOMIAL DEGREE": 5, "MESH JITTER": 0.0, "LAMBDA": 0.0, "BOX NX": 4, "BOX NY": 4, "BOX NZ": 4}),
    box(**{"POLYNOMIAL DEGREE": 1, "BOX NX": 5, "BOX NY": 3, "BOX NZ": 2}),
    box(**{"POLYNOMIAL DEGREE": 3, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0, "BOX NX": 3,
           "BOX NY": 4, "BOX NZ": 2}),                      # periodic
    box(**{"POLYNOMIAL DEGREE": 4, "LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2}),
    box(**{"POLYNOMIAL DEGREE": 8, "BOX NX": 2, "BOX NY": 2, "BOX NZ": 2}),
    box(**{"POLYNOMIAL DEGREE": 2, "BOX NX": 1, "BOX NY": 1, "BOX NZ": 1}),   # one element
    box(**{"LAMBDA": 0.3}),                                  # N=7, lambda neither 0 nor 1
    box(**{"POLYNOMIAL DEGREE": 3, "LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2}),   # N=3 even-odd, field
]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


def ids(c):
    return "N%s_%sx%sx%s_bc%s_j%s_%s" % (c["POLYNOMIAL DEGREE"], c["BOX NX"], c["BOX NY"], c["BOX NZ"],
                                         c["BOX BOUNDARY FLAG"], c["MESH JITTER"], c.get("LAMBDA FIELD", "const"))


@pytest.mark.parametrize("cfg", CASES, ids=ids)
def test_numbering_and_geometry_match_oracle(cfg):
    e = lpg.Elliptic(cfg)
    o = Oracle(cfg)
    assert e.Nglobal == o.Ngather
    assert np.array_equal(e.get("GlobalToLocal"), o.array("GlobalToLocal"))
    assert rel_err(e.get("ggeo"), o.array("ggeo")) < 1e-13
    assert rel_err(e.get("wJ"), o.array("wJ")) < 1e-13
    assert rel_err(e.get("D"), o.array("D")) < 1e-13
    assert np.allclose(e.get("weightG"), o.array("weightG"), rtol=0, atol=0)
    # owners are the first appearance of each dof in local order
    g2l = o.array("GlobalToLocal")
    first = np.full(e.Nglobal, -1)
    idx = np.nonzero(g2l >= 0)[0]
    rev = idx[::-1]
    first[g2l[rev]] = rev
    assert np.array_equal(e.get("ownerLocal"), first)
    if cfg.get("LAMBDA FIELD") == "LOGNORMAL":
        assert np.array_equal(e.get("lambdaE"), o.array("lambdaE"))


@pytest.mark.parametrize("cfg", CASES, ids=ids)
def test_operator_matches_oracle(cfg):
    e = lpg.Elliptic(cfg)
    o = Oracle(cfg)
    rng = np.random.default_rng(7)
    for _ in range(2):
        qh = rng.uniform(-1, 1, e.Nglobal)
        q = torch.tensor(qh, device="cuda")
        Aq = torch.full_like(q, np.nan)
        e.Operator(q, Aq)
        torch.cuda.synchronize()
        assert rel_err(Aq.cpu().numpy(), o.operator(qh)) < 1e-12


REF_CASES = [box(**{"POLYNOMIAL DEGREE": N}) for N in range(1, 9)] + [
    box(**{"POLYNOMIAL DEGREE": 3, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0}),   # periodic
    box(**{"POLYNOMIAL DEGREE": 7, "LAMBDA": 0.0, "BOX NX": 4, "BOX NY": 4, "BOX NZ": 4}),
    box(**{"POLYNOMIAL DEGREE": 7, "LAMBDA": 2.5}),
]


@pytest.mark.skipif(not refimpl.available(), reason="reference kernels not built here")
@pytest.mark.parametrize("cfg", REF_CASES, ids=ids)
def test_operator_matches_reference_kernels(cfg):
    """The CUDA operators (FP64 and double-FP32 words) and the reference-contract partial Ax
    against the reference's own ellipticPartialAxHex3D + ogs gather (translated from its OKL,
    compiled for the host), both fed this library's own setup arrays."""
    e = lpg.Elliptic(cfg)
    N, E, Np = cfg["POLYNOMIAL DEGREE"], e.info("nelements"), e.info("np")
    ggeo, wJ, D, g2lh = e.get("ggeo"), e.get("wJ"), e.get("D"), e.get("GlobalToLocal")
    r = refimpl.RefOperator(N, E, g2lh, e.Nglobal, wJ, ggeo, D, cfg["LAMBDA"])
    rng = np.random.default_rng(11)
    qh = rng.uniform(-1, 1, e.Nglobal)
    q = torch.tensor(qh, device="cuda")
    ref = r.apply(qh)
    Aq = torch.full_like(q, np.nan)
    e.Operator(q, Aq)
    torch.cuda.synchronize()
    assert rel_err(Aq.cpu().numpy(), ref) < 1e-12
    e.OperatorDF64(q, Aq)
    torch.cuda.synchronize()
    assert rel_err(Aq.cpu().numpy(), ref) < 1e-12
    AqL = torch.full((E * Np,), np.nan, dtype=torch.float64, device="cuda")
    dg = [torch.tensor(x, device="cuda") for x in (ggeo, wJ, D, g2lh)]
    lpg.check(lpg.lib().lpg_partial_ax_hex_f64(N, E, None, dg[3].data_ptr(), dg[0].data_ptr(), 6 * Np,
                                               dg[1].data_ptr(), Np, dg[2].data_ptr(), cfg["LAMBDA"], None,
                                               q.data_ptr(), AqL.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_err(AqL.cpu().numpy(), r.partial_ax(qh)) < 1e-12


def test_lattice_keyed_input_and_linearity():
    cfg = box(**{"BOX NX": 2, "BOX NY": 3, "BOX NZ": 2})
    e = lpg.Elliptic(cfg)
    o = Oracle(cfg)
    qh = lattice_q(o.array("GlobalToLocal"), 7, 2, 3, 2)
    q = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.random_vector(q, 1)
    torch.cuda.synchronize()
    assert np.array_equal(q.cpu().numpy(), qh)
    Aq = torch.zeros_like(q)
    e.Operator(q, Aq)
    ref = o.operator(qh)
    assert rel_err(Aq.cpu().numpy(), ref) < 1e-12
    # linearity: A(2q) = 2 A q exactly up to rounding; A(q1+q2) = Aq1 + Aq2
    Aq2 = torch.zeros_like(q)
    e.Operator(2 * q, Aq2)
    assert rel_err(Aq2.cpu().numpy(), 2 * Aq.cpu().numpy()) < 1e-14


def test_partial_ax_reference_contract():
    """lpg_partial_ax_hex_f64 with the reference's separate ggeo/wJ arrays and an
    element list reproduces the oracle's unassembled AqL on the listed elements."""
    cfg = box(**{"POLYNOMIAL DEGREE": 6})
    e = lpg.Elliptic(cfg)
    o = Oracle(cfg)
    N, E, Np = 6, e.info("nelements"), e.info("np")
    ggeo = torch.tensor(o.array("ggeo"), device="cuda")
    wJ = torch.tensor(o.array("wJ"), device="cuda")
    D = torch.tensor(o.array("D"), device="cuda")
    g2l = torch.tensor(o.array("GlobalToLocal"), device="cuda")
    rng = np.random.default_rng(3)
    qh = rng.uniform(-1, 1, e.Nglobal)
    q = torch.tensor(qh, device="cuda")
    lst = torch.tensor([E - 1, 0, 5, 2], dtype=torch.int32, device="cuda")
    AqL = torch.full((E * Np,), 7.0, dtype=torch.float64, device="cuda")
    L = lpg.lib()
    lpg.check(L.lpg_partial_ax_hex_f64(N, 4, lst.data_ptr(), g2l.data_ptr(), ggeo.data_ptr(), 6 * Np,
                                       wJ.data_ptr(), Np, D.data_ptr(), 1.0, None, q.data_ptr(),
                                       AqL.data_ptr(), None))
    torch.cuda.synchronize()
    ref = o.partial_ax(qh).reshape(E, Np)
    got = AqL.cpu().numpy().reshape(E, Np)
    for el in (E - 1, 0, 5, 2):
        assert rel_err(got[el], ref[el]) < 1e-12
    untouched = [x for x in range(E) if x not in (E - 1, 0, 5, 2)]
    assert np.all(got[untouched] == 7.0)
    # assembled kernel entry with the same reference layout
    Aq = torch.zeros_like(q)
    lpg.ax_hex("f64", N, E, g2l, ggeo, 6 * Np, wJ, Np, D, 1.0, q, Aq, e.Nglobal)
    torch.cuda.synchronize()
    assert rel_err(Aq.cpu().numpy(), o.operator(qh)) < 1e-12
    # empty element list is a no-op that still zeroes the output
    Aq.fill_(3.0)
    lpg.ax_hex("f64", N, 0, g2l, ggeo, 6 * Np, wJ, Np, D, 1.0, q, Aq, e.Nglobal)
    torch.cuda.synchronize()
    assert float(Aq.abs().max()) == 0.0


@pytest.mark.parametrize("prec,tol", [("f32", 2e-6), ("bf16g", 2e-2)])
def test_reduced_precision_operator(prec, tol):
    cfg = box(**{"POLYNOMIAL DEGREE": 7, "LAMBDA": 1.0})
    e = lpg.Elliptic(cfg)
    o = Oracle(cfg)
    N, E, Np = 7, e.info("nelements"), e.info("np")
    geo64 = e.get("geo")
    g2l = torch.tensor(e.get("GlobalToLocal"), device="cuda")
    D = torch.tensor(e.get("D"), dtype=torch.float32, device="cuda")
    if prec == "f32":
        geo = torch.tensor(geo64, dtype=torch.float32, device="cuda")
    else:
        geo = torch.tensor(geo64, dtype=torch.float64, device="cuda").to(torch.bfloat16)
    rng = np.random.default_rng(5)
    qh = rng.uniform(-1, 1, e.Nglobal)
    q = torch.tensor(qh, dtype=torch.float32, device="cuda")
    Aq = torch.zeros_like(q)
    lpg.ax_hex(prec, N, E, g2l, geo, 7 * Np, geo.data_ptr() + 6 * Np * geo.element_size(), 7 * Np, D,
               1.0, q, Aq, e.Nglobal)
    torch.cuda.synchronize()
    err = rel_err(Aq.double().cpu().numpy(), o.operator(qh))
    assert err < tol, err


@pytest.mark.parametrize("lam", [1.0, 0.0])
@pytest.mark.parametrize("bf16", [False, True])
def test_reduced_precision_operator_many_groups(bf16, lam):
    """16384 elements: every persistent CTA of the staged FP32 / BF16-geometry kernel
    walks many element groups through its shared-memory ring (the small cases give a
    CTA one group). Checked against the oracle on three consecutive applications;
    lambda = 0 runs the instantiation that neither copies nor uses wJ."""
    cfg = box(**{"BOX NX": 32, "BOX NY": 32, "BOX NZ": 16, "LAMBDA": lam})
    e = lpg.Elliptic(cfg)
    o = Oracle(cfg)
    rng = np.random.default_rng(21)
    tol = 2e-2 if bf16 else 2e-6
    for _ in range(3):
        qh = rng.uniform(-1, 1, e.Nglobal)
        q = torch.tensor(qh, dtype=torch.float32, device="cuda")
        Aq = torch.full_like(q, np.nan)
        e.OperatorF32(q, Aq, bf16)
        torch.cuda.synchronize()
        err = rel_err(Aq.double().cpu().numpy(), o.operator(qh))
        assert err < tol, err


DW_CASES = [
    box(),                                                                     # jittered, N=7
    box(**{"POLYNOMIAL DEGREE": 3, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0, "BOX NX": 3,
           "BOX NY": 4, "BOX NZ": 2}),                                        # periodic, N=3
    box(**{"LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2, "BOX NX": 32, "BOX NY": 32, "BOX NZ": 16}),
    box(**{"LAMBDA": 0.0, "BOX NX": 9, "BOX NY": 7, "BOX NZ": 5}),            # N=7 without the mass term
    box(**{"LAMBDA": 2.5}),                                                    # N=7, general constant lambda
    # degrees without an even-odd kernel (thread-per-node double-word kernel)
    box(**{"POLYNOMIAL DEGREE": 1, "BOX NX": 6, "BOX NY": 5, "BOX NZ": 4}),
    box(**{"POLYNOMIAL DEGREE": 2, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0, "BOX NX": 3, "BOX NY": 4,
           "BOX NZ": 2}),
    box(**{"POLYNOMIAL DEGREE": 4, "LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2}),
    box(**{"POLYNOMIAL DEGREE": 5, "BOX BOUNDARY FLAG": 2}),
    box(**{"POLYNOMIAL DEGREE": 6, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0}),
    box(**{"POLYNOMIAL DEGREE": 8}),
]


@pytest.mark.parametrize("cfg", DW_CASES, ids=ids)
def test_double_word_operator_matches_oracle(cfg):
    """The double-FP32 operator agrees with the FP64 oracle to the FP64 bar (1e-12
    relative, max-norm), also for inputs scaled by 1e-12 and 1e+12."""
    e = lpg.Elliptic(cfg)
    o = Oracle(cfg)
    rng = np.random.default_rng(11)
    for scale in (1.0, 1e-12, 1e12):
        qh = scale * rng.uniform(-1, 1, e.Nglobal)
        q = torch.tensor(qh, device="cuda")
        Aq = torch.full_like(q, np.nan)
        e.OperatorDF64(q, Aq)
        torch.cuda.synchronize()
        err = rel_err(Aq.cpu().numpy(), o.operator(qh))
        print("double-word operator, scale %g: max rel err %.3g" % (scale, err))
        assert err < 1e-12, (scale, err)


HOST_CASES = [
    box(**{"BOX NX": 32, "BOX NY": 32, "BOX NZ": 16}),                 # 16384 elements: 4 chunks
    box(**{"POLYNOMIAL DEGREE": 3, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0, "BOX NX": 24,
           "BOX NY": 16, "BOX NZ": 24}),                              # periodic: the last chunk wraps
    box(),                                                            # a single chunk
]


@pytest.mark.parametrize("cfg", HOST_CASES, ids=ids)
def test_host_buffer_operator_matches_oracle(cfg):
    """The host-buffer operator (upload, per-chunk operator and download pipelined over
    element chunks) gives the oracle's Aq from pinned tensors and from pageable numpy
    arrays, in FP64 and in the reduced precisions, on consecutive calls."""
    e = lpg.Elliptic(cfg)
    o = Oracle(cfg)
    E = e.info("nelements")
    rng = np.random.default_rng(3)
    for pinned in (True, False, True):
        qh = rng.uniform(-1, 1, e.Nglobal)
        ref = o.operator(qh)
        if pinned:
            q = torch.tensor(qh).pin_memory()
            Aq = torch.full_like(q, np.nan).pin_memory()
        else:
            q, Aq = qh.copy(), np.full_like(qh, np.nan)
        e.OperatorHost(q, Aq)
        out = Aq.numpy() if pinned else Aq
        assert rel_err(out, ref) < 1e-12
        for prec, tol in (("FP32", 2e-6), ("BF16GEO", 2e-2)):
            q32 = np.ascontiguousarray(qh, dtype=np.float32)
            A32 = np.full_like(q32, np.nan)
            e.OperatorHost(q32, A32, prec)
            assert rel_err(A32.astype(np.float64), ref) < tol, prec
    assert e.info("host_chunks") == max(1, min(32, E // 4096))
    with pytest.raises(ValueError):
        e.OperatorHost(np.zeros(e.Nglobal + 1), np.zeros(e.Nglobal + 1))


def test_gather_scatter_and_reductions():
    cfg = box(**{"POLYNOMIAL DEGREE": 4})
    e = lpg.Elliptic(cfg)
    o = Oracle(cfg)
    L = lpg.lib()
    g2l = torch.tensor(o.array("GlobalToLocal"), device="cuda")
    owner = torch.tensor(e.get("ownerLocal"), device="cuda")
    Nl, Ng = e.Nlocal, e.Nglobal
    rng = np.random.default_rng(11)
    vL = rng.standard_normal(Nl)
    v = torch.tensor(vL, device="cuda")
    gv = torch.full((Ng,), np.nan, dtype=torch.float64, device="cuda")
    lpg.check(L.lpg_ogs_gather_add_f64(Nl, g2l.data_ptr(), v.data_ptr(), gv.data_ptr(), Ng, None))
    torch.cuda.synchronize()
    assert rel_err(gv.cpu().numpy(), o.gather(vL, trans=True)) < 1e-14
    lpg.check(L.lpg_ogs_gather_owner_f64(Ng, owner.data_ptr(), v.data_ptr(), gv.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.array_equal(gv.cpu().numpy(), o.gather(vL, trans=False))
    back = torch.zeros_like(v)
    lpg.check(L.lpg_ogs_scatter_f64(Nl, g2l.data_ptr(), gv.data_ptr(), back.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.array_equal(back.cpu().numpy(), o.scatter(gv.cpu().numpy()))
    # reductions: deterministic and equal to a compensated host sum to rounding
    for n in (0, 1, 1000, 3_000_001):
        x = torch.tensor(rng.standard_normal(n), device="cuda")
        y = torch.tensor(rng.standard_normal(n), device="cuda")
        out = torch.zeros(2, dtype=torch.float64, device="cuda")
        lpg.check(L.lpg_dot_f64(n, x.data_ptr(), y.data_ptr(), out.data_ptr(), None))
        lpg.check(L.lpg_dot_f64(n, x.data_ptr(), y.data_ptr(), out.data_ptr() + 8, None))
        torch.cuda.synchronize()
        ref = float(np.dot(x.cpu().numpy(), y.cpu().numpy()))
        got = out.cpu().numpy()
        assert got[0] == got[1]
        assert abs(got[0] - ref) <= 1e-12 * max(1.0, np.sqrt(n))
    # fused PCG update
    n = 100_003
    p, Ap, xx, r = (torch.tensor(rng.standard_normal(n), device="cuda") for _ in range(4))
    x0, r0 = xx.clone(), r.clone()
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    lpg.check(L.lpg_pcg_update_f64(n, 0.37, p.data_ptr(), Ap.data_ptr(), xx.data_ptr(), r.data_ptr(),
                                   res.data_ptr(), None))
    torch.cuda.synchronize()
    assert torch.allclose(xx, x0 + 0.37 * p, rtol=0, atol=1e-15)
    assert torch.allclose(r, r0 - 0.37 * Ap, rtol=0, atol=1e-15)
    assert abs(float(res) - float((r * r).sum())) < 1e-9


def test_invalid_degree_and_empty_mesh_are_errors():
    with pytest.raises(lpg.LPGError) as ei:
        lpg.Elliptic(box(**{"POLYNOMIAL DEGREE": 9}))
    assert ei.value.status == -3
    with pytest.raises(lpg.LPGError):
        lpg.Elliptic(box(**{"POLYNOMIAL DEGREE": 1, "BOX NX": 1, "BOX NY": 1, "BOX NZ": 1}))
