"""IPDG discretisation (DISCRETIZATION = IPDG) on the CUDA path against the oracle's
restatement of the reference's IPDG kernels, and against the reference's golden norms.

Bars: operator, diagonal and right-hand side within 1e-12 relative of the oracle (FP64,
different summation order); Jacobi-PCG solves with the oracle's iteration count and
solution (1e-7); golden norms within the reference's 1e-5."""
import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from conftest import golden_case_settings
from gmsh_mesh import write_box
from gpu_helpers import rel_err
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

BASE = {"BOX NX": 4, "BOX NY": 3, "BOX NZ": 3, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
        "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 5, "LAMBDA": 0.7, "DISCRETIZATION": "IPDG",
        "LINEAR SOLVER": "PCG", "PRECONDITIONER": "JACOBI", "MESH JITTER": 0.1}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


def _cases(tmp_path):
    f = write_box(str(tmp_path / "m.msh"), 4, 3, 3, rotate_seed=3, shuffle_seed=1, jitter=0.15, jitter_seed=2,
                  tags=(1, 2, 1, 2, 2, 1))
    return {
        "dirichlet_N5": dict(BASE),
        "dirichlet_N1": dict(BASE, **{"POLYNOMIAL DEGREE": 1}),
        "dirichlet_N8": dict(BASE, **{"POLYNOMIAL DEGREE": 8, "BOX NX": 2, "BOX NY": 2, "BOX NZ": 2}),
        "periodic_N7": dict(BASE, **{"POLYNOMIAL DEGREE": 7, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0}),
        "lognormal_N3": dict(BASE, **{"POLYNOMIAL DEGREE": 3, "LAMBDA FIELD": "LOGNORMAL"}),
        "file_mixed_N4": dict(BASE, **{"POLYNOMIAL DEGREE": 4, "MESH FILE": f, "MESH JITTER": 0.0}),
    }


CASE_NAMES = ["dirichlet_N5", "dirichlet_N1", "dirichlet_N8", "periodic_N7", "lognormal_N3", "file_mixed_N4"]


@pytest.mark.parametrize("name", CASE_NAMES)
def test_ipdg_operator_diagonal_rhs_match_oracle(tmp_path, name):
    s = _cases(tmp_path)[name]
    e = lpg.Elliptic(s)
    o = Oracle(s)
    assert e.Nglobal == o.Ngather == e.Nlocal
    rng = np.random.default_rng(7)
    q = rng.standard_normal(e.Nglobal)
    Aq = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.Operator(torch.tensor(q, device="cuda"), Aq)
    torch.cuda.synchronize()
    assert rel_err(Aq.cpu().numpy(), o.operator(q)) < 1e-12
    # symmetric: q' A q == q A q'
    q2 = rng.standard_normal(e.Nglobal)
    Aq2 = torch.zeros_like(Aq)
    e.Operator(torch.tensor(q2, device="cuda"), Aq2)
    torch.cuda.synchronize()
    a, b = float(q2 @ Aq.cpu().numpy()), float(q @ Aq2.cpu().numpy())
    assert abs(a - b) < 1e-10 * max(abs(a), 1.0)
    # Jacobi application (inverse diagonal)
    z = torch.zeros_like(Aq)
    e.precon(torch.tensor(q, device="cuda"), z)
    torch.cuda.synchronize()
    assert rel_err(z.cpu().numpy(), o.precon(q)) < 1e-12
    r = torch.zeros_like(Aq)
    e.rhs(r)
    torch.cuda.synchronize()
    assert rel_err(r.cpu().numpy(), o.rhs()) < 1e-12


@pytest.mark.parametrize("name", ["dirichlet_N5", "periodic_N7", "file_mixed_N4"])
def test_ipdg_jacobi_solve_matches_oracle(tmp_path, name):
    s = _cases(tmp_path)[name]
    r = lpg.Elliptic(s).Run(want_solution=True)
    ro = Oracle(s).run()
    assert r["converged"]
    assert abs(r["iterations"] - ro["iterations"]) <= 1, (r["iterations"], ro["iterations"])
    assert rel_err(r["xL"], ro["xL"]) < 1e-7
    assert abs(r["norm"] - ro["norm"]) < 1e-9 * ro["norm"]


@pytest.mark.parametrize("name", ["testEllipticHex_Ipdg", "testEllipticHex_Ipdg_Jacobi"])
def test_ipdg_reference_golden_norms(reference_norms, name):
    case = reference_norms["cases"][name]
    s = golden_case_settings(case)
    r = lpg.Elliptic(s).Run()
    ro = Oracle(s).run()
    assert r["converged"]
    assert abs(r["norm"] - case["norm"]) < reference_norms["tolerance"]
    assert abs(r["norm"] - ro["norm"]) < 1e-9
    assert abs(r["iterations"] - ro["iterations"]) <= (1 if "Jacobi" in name else 2)


MG_CASES = {
    "pmg_5_2_1": {"PRECONDITIONER": "MULTIGRID", "MULTIGRID DEGREES": "5,2,1", "LINEAR SOLVER": "FPCG"},
    "pmg_halfdofs_N4_lognormal": {"PRECONDITIONER": "MULTIGRID", "POLYNOMIAL DEGREE": 4, "LAMBDA FIELD": "LOGNORMAL"},
    "paralmond_N2": {"PRECONDITIONER": "PARALMOND", "POLYNOMIAL DEGREE": 2, "PARALMOND AGGREGATION": "UNSMOOTHED",
                     "BOX NX": 6, "BOX NY": 5, "BOX NZ": 4},
    "pmg_all_neumann_periodic": {"PRECONDITIONER": "MULTIGRID", "BOX BOUNDARY FLAG": -1, "LAMBDA": 0.0,
                                 "MESH JITTER": 0.0, "POLYNOMIAL DEGREE": 3},
}


@pytest.mark.parametrize("name", sorted(MG_CASES))
def test_ipdg_multigrid_matches_oracle(name):
    """p-multigrid on IPDG levels (element-local transfers, Chebyshev on the IPDG diagonal)
    with AMG on the degree-1 IPDG matrix; the library builds that matrix by probing its
    operator, the oracle by the reference's explicit formula."""
    s = dict(BASE, **MG_CASES[name])
    r = lpg.Elliptic(s).Run(want_solution=True)
    ro = Oracle(s).run()
    assert r["converged"]
    assert abs(r["iterations"] - ro["iterations"]) <= 1, (r["iterations"], ro["iterations"])
    assert rel_err(r["xL"], ro["xL"]) < 1e-7
    jac = Oracle(dict(s, **{"PRECONDITIONER": "JACOBI"})).run()
    assert r["iterations"] < jac["iterations"]


@pytest.mark.parametrize("name", ["testEllipticHex_Ipdg_Multigrid", "testEllipticHex_Ipdg_AllNeumann",
                                  "testEllipticHex_Ipdg_ParAlmond", "testEllipticHex_Ipdg_OAS"])
def test_ipdg_multigrid_reference_golden_norms(reference_norms, name):
    case = reference_norms["cases"][name]
    s = golden_case_settings(case)
    r = lpg.Elliptic(s).Run()
    assert r["converged"]
    assert abs(r["norm"] - case["norm"]) < reference_norms["tolerance"], (r["norm"], case["norm"])


@pytest.mark.parametrize("name", ["dirichlet_N5", "dirichlet_N1", "periodic_N7", "lognormal_N3", "file_mixed_N4"])
def test_ipdg_fp32_operator_matches_oracle(tmp_path, name):
    """FP32 operator of the preconditioner levels (FP32 copies of vgeo/sgeo, float4
    gradients) against the FP64 oracle applied to the same FP32-rounded input: 1e-5
    relative to the largest entry (FP32 rounding of ~3 Nq-term sums)."""
    s = _cases(tmp_path)[name]
    e = lpg.Elliptic(s)
    o = Oracle(s)
    q = np.random.default_rng(11).standard_normal(e.Nglobal).astype(np.float32)
    Aq = torch.zeros(e.Nglobal, dtype=torch.float32, device="cuda")
    e.OperatorF32(torch.tensor(q, device="cuda"), Aq)
    torch.cuda.synchronize()
    err = rel_err(Aq.cpu().numpy().astype(np.float64), o.operator(q.astype(np.float64)))
    assert err < 1e-5, err
    with pytest.raises(RuntimeError):
        e.OperatorF32(torch.tensor(q, device="cuda"), Aq, bf16geo=True)


@pytest.mark.parametrize("name", CASE_NAMES)
def test_ipdg_df64_operator_matches_oracle(tmp_path, name):
    """OPERATOR PRECISION DF64: the operator in double-FP32 words is held to the FP64 bar
    (1e-12 relative to the largest entry), through the object's Operator and the C entry."""
    s = dict(_cases(tmp_path)[name], **{"OPERATOR PRECISION": "DF64"})
    e = lpg.Elliptic(s)
    o = Oracle(_cases(tmp_path)[name])
    q = np.random.default_rng(13).standard_normal(e.Nglobal)
    qd = torch.tensor(q, device="cuda")
    Aq = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.Operator(qd, Aq)
    Aq2 = torch.zeros_like(Aq)
    e.OperatorDF64(qd, Aq2)
    torch.cuda.synchronize()
    ref = o.operator(q)
    assert rel_err(Aq.cpu().numpy(), ref) < 1e-12
    assert torch.equal(Aq, Aq2)
    # scale-independent: 1e-6 q and 1e6 q
    for scale in (1e-6, 1e6):
        e.Operator(qd * scale, Aq)
        torch.cuda.synchronize()
        assert rel_err(Aq.cpu().numpy(), ref * scale) < 1e-12


def test_ipdg_df64_fp32_multigrid_solve_matches_oracle():
    """FP32 p-levels inside FPCG whose operator runs in double-FP32 words: the oracle's
    discrete solution (1e-7) in at most two iterations more than the all-FP64 solve."""
    s = dict(BASE, **MG_CASES["pmg_5_2_1"])
    s["POLYNOMIAL DEGREE"] = 5
    ro = Oracle(s).run()
    r64 = lpg.Elliptic(s).Run()
    r = lpg.Elliptic(dict(s, **{"PRECONDITIONER PRECISION": "FP32", "OPERATOR PRECISION": "DF64"})).Run(
        want_solution=True)
    assert r["converged"]
    assert r["iterations"] <= r64["iterations"] + 2
    assert rel_err(r["xL"], ro["xL"]) < 1e-7
    assert abs(r["norm"] - ro["norm"]) < 1e-9 * ro["norm"]


@pytest.mark.parametrize("name", ["pmg_5_2_1", "pmg_halfdofs_N4_lognormal", "pmg_all_neumann_periodic"])
def test_ipdg_fp32_multigrid_reaches_the_fp64_solution(name):
    """PRECONDITIONER PRECISION FP32 on IPDG levels inside the FP64 FPCG: same discrete
    solution as the oracle (1e-7) in at most two iterations more than the FP64 V-cycle."""
    s = dict(BASE, **MG_CASES[name])
    s["LINEAR SOLVER"] = "FPCG"
    r64 = lpg.Elliptic(s).Run()
    r32 = lpg.Elliptic(dict(s, **{"PRECONDITIONER PRECISION": "FP32"})).Run(want_solution=True)
    ro = Oracle(s).run()
    assert r32["converged"]
    assert r32["iterations"] <= r64["iterations"] + 2, (r32["iterations"], r64["iterations"])
    assert rel_err(r32["xL"], ro["xL"]) < 1e-7


def test_ipdg_fp32_oas_reference_golden_norm(reference_norms):
    case = reference_norms["cases"]["testEllipticHex_Ipdg_OAS"]
    s = dict(golden_case_settings(case), **{"PRECONDITIONER PRECISION": "FP32"})
    r = lpg.Elliptic(s).Run()
    assert r["converged"]
    assert abs(r["norm"] - case["norm"]) < reference_norms["tolerance"], (r["norm"], case["norm"])


def test_ipdg_unsupported_combinations_fail_loudly():
    for over in ({"PRECONDITIONER": "SEMFEM"}, {"PRECONDITIONER": "MULTIGRID", "PRECONDITIONER PRECISION": "BF16GEO"},
                 {"OPERATOR PRECISION": "FP32"}):
        with pytest.raises(RuntimeError):
            lpg.Elliptic(dict(BASE, **over))
