"""End-to-end parity of the CUDA solver path (FPCG/PCG with Jacobi, p-multigrid
and AMG preconditioners) with the oracle and with the reference's golden norms.

Bars: the reference's own tolerance on `Solution norm` (1e-5 absolute,
test/test.py:63), identical iteration counts to the oracle for FP64 paths, and
for reduced-precision preconditioners a discretisation error within 1 % of the
FP64 oracle's."""
import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from conftest import golden_case_settings
from gpu_helpers import box, rel_err
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

GOLDEN = ("testEllipticHex_C0", "testEllipticHex_C0_Jacobi", "testEllipticHex_C0_ParAlmond",
          "testEllipticHex_C0_Multigrid", "testEllipticHex_C0_AllNeumann", "testEllipticHex_C0_Semfem",
          "testEllipticHex_C0_OAS")


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


@pytest.mark.parametrize("name", GOLDEN)
def test_reference_golden_norms(reference_norms, name):
    case = reference_norms["cases"][name]
    s = golden_case_settings(case)
    r = lpg.Elliptic(s).Run()
    ro = Oracle(s).run()
    assert r["converged"]
    assert abs(r["norm"] - case["norm"]) < reference_norms["tolerance"], (r["norm"], case["norm"])
    assert abs(r["norm"] - ro["norm"]) < 1e-9
    amg = "ParAlmond" in name or "Semfem" in name or "OAS" in name
    assert abs(r["iterations"] - ro["iterations"]) <= (1 if amg else 0), \
        (r["iterations"], ro["iterations"])


def config1(**over):
    d = {"BOX NX": 8, "BOX NY": 8, "BOX NZ": 8, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
         "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 5, "LAMBDA": 0.0, "LINEAR SOLVER": "FPCG",
         "PRECONDITIONER": "JACOBI"}
    d.update(over)
    return d


def test_config1_fpcg_jacobi_iterations_and_error():
    s = config1()
    r = lpg.Elliptic(s).Run(want_solution=True)
    ro = Oracle(s).run()
    assert r["iterations"] == ro["iterations"]
    assert abs(r["error"] - ro["error"]) <= 1e-6 * ro["error"]
    assert rel_err(r["xL"], ro["xL"]) < 1e-7
    assert r["error"] < 1e-3


def test_pcg_and_fpcg_agree_on_solution():
    s = config1(**{"BOX NX": 4, "BOX NY": 4, "BOX NZ": 4})
    a = lpg.Elliptic(dict(s, **{"LINEAR SOLVER": "PCG"})).Run(want_solution=True)
    b = lpg.Elliptic(s).Run(want_solution=True)
    assert rel_err(a["xL"], b["xL"]) < 1e-7


MG = dict(config1(), **{"BOX NX": 6, "BOX NY": 5, "BOX NZ": 4, "POLYNOMIAL DEGREE": 7,
                        "MESH JITTER": 0.1, "PRECONDITIONER": "MULTIGRID", "MULTIGRID DEGREES": "7,3,1",
                        "PARALMOND AGGREGATION": "SMOOTHED"})


def test_fine_operator_applications_per_iteration():
    """FPCG + p-MG with Chebyshev degree 2: per iteration one outer application and six in
    the V-cycle's fine level (pre-smoothing 2, residual 1, post-smoothing 1 + 2)."""
    e = lpg.Elliptic(MG)
    n0 = e.info("operator_applications")
    r = e.Run()
    ops = e.info("operator_applications") - n0
    assert r["converged"]
    assert 7 * r["iterations"] - 6 <= ops <= 7 * r["iterations"] + 2, (ops, r["iterations"])


def test_pmg_fp64_iterations_match_oracle():
    r = lpg.Elliptic(MG).Run()
    ro = Oracle(MG).run()
    assert r["converged"]
    assert r["iterations"] == ro["iterations"], (r["iterations"], ro["iterations"])
    assert abs(r["error"] - ro["error"]) <= 1e-6 * ro["error"]


def test_pmg_preconditioner_application_matches_oracle():
    e = lpg.Elliptic(MG)
    o = Oracle(MG)
    rng = np.random.default_rng(2)
    rh = rng.standard_normal(e.Nglobal)
    r = torch.tensor(rh, device="cuda")
    z = torch.zeros_like(r)
    e.precon(r, z)
    torch.cuda.synchronize()
    assert rel_err(z.cpu().numpy(), o.precon(rh)) < 1e-9


_PRECON_CHILD = r"""
import json, sys
import numpy as np
import torch
import libparanumal_gb300 as lpg
s = json.loads(sys.argv[1])
e = lpg.Elliptic(s)
rng = np.random.default_rng(2)
r = torch.tensor(rng.standard_normal(e.Nglobal), device="cuda")
z = torch.zeros_like(r)
e.precon(r, z)
torch.cuda.synchronize()
np.save(sys.argv[2], z.cpu().numpy())
"""


@pytest.mark.parametrize("over", [{}, {"LAMBDA": 1.0, "LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2}],
                         ids=["lambda0", "lognormal"])
def test_fp32_preconditioner_application_fused_and_separate_chebyshev(tmp_path, over):
    """The FP32 p-MG V-cycle with the Chebyshev steps on the unscaled residual that the
    operator updates in place (the default) against the same V-cycle with a separate A d
    vector (LPG_CHEB=unfused) and against the oracle's FP64 V-cycle: the two FP32 paths
    differ only in FP32 rounding order (1e-5), and both stay within FP32 accuracy of the
    FP64 preconditioner (1e-4)."""
    import json
    import os
    import subprocess
    import sys
    s = dict(MG, **{"PRECONDITIONER PRECISION": "FP32"}, **over)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = {}
    for mode in ("fused", "unfused"):
        env = dict(os.environ, PYTHONPATH=root)
        env.pop("LPG_CHEB", None)
        if mode == "unfused":
            env["LPG_CHEB"] = "unfused"
        f = tmp_path / (mode + ".npy")
        p = subprocess.run([sys.executable, "-c", _PRECON_CHILD, json.dumps(s), str(f)], env=env, cwd=root,
                           capture_output=True, text=True, timeout=600)
        assert p.returncode == 0, p.stderr[-2000:]
        out[mode] = np.load(f)
    o = Oracle(dict(MG, **over))
    zo = o.precon(np.random.default_rng(2).standard_normal(o.Ngather))
    assert rel_err(out["fused"], out["unfused"]) < 1e-5
    assert rel_err(out["fused"], zo) < 1e-4
    assert rel_err(out["unfused"], zo) < 1e-4


@pytest.mark.parametrize("over", [
    {"MULTIGRID SMOOTHER": "DAMPEDJACOBI"},
    {"MULTIGRID SMOOTHER": "DAMPEDJACOBI", "PARALMOND SMOOTHER": "DAMPEDJACOBI"},
    {"MULTIGRID SMOOTHER": "DAMPEDJACOBI", "MULTIGRID DEGREES": "7,5,3,1", "LAMBDA FIELD": "LOGNORMAL",
     "LAMBDA SEED": 2, "LAMBDA": 1.0},
], ids=["pmg", "pmg_and_amg", "7531_lognormal"])
def test_damped_jacobi_smoother_matches_oracle(over):
    """MGLevel::smoothJacobi (ellipticPreconMultiGridLevel.cpp:135-152) with the weight
    4/3/rho from the level's Arnoldi estimate (:370-383), and parCSR::smoothDampedJacobi on
    the AMG levels (parAlmondAMGSmoother.cpp): one preconditioner application against the
    oracle (1e-9), then the FPCG solve (same iterations, solution 1e-7)."""
    s = dict(MG, **over)
    e = lpg.Elliptic(s)
    o = Oracle(s)
    rh = np.random.default_rng(5).standard_normal(e.Nglobal)
    r = torch.tensor(rh, device="cuda")
    z = torch.zeros_like(r)
    e.precon(r, z)
    torch.cuda.synchronize()
    assert rel_err(z.cpu().numpy(), o.precon(rh)) < 1e-9
    res = e.Run(want_solution=True)
    ro = o.run()
    assert res["converged"]
    assert res["iterations"] == ro["iterations"], (res["iterations"], ro["iterations"])
    assert rel_err(res["xL"], ro["xL"]) < 1e-7
    # damped Jacobi is the weaker smoother: more iterations than Chebyshev on the same problem
    rc = lpg.Elliptic(dict(s, **{"MULTIGRID SMOOTHER": "CHEBYSHEV", "PARALMOND SMOOTHER": "CHEBYSHEV"})).Run()
    assert rc["iterations"] < res["iterations"]


@pytest.mark.parametrize("prec", ["FP32", "BF16GEO"])
def test_mixed_precision_preconditioner_keeps_fp64_accuracy(prec):
    s = dict(MG, **{"PRECONDITIONER PRECISION": prec})
    r = lpg.Elliptic(s).Run()
    ro = Oracle(MG).run()
    assert r["converged"]
    assert r["iterations"] <= ro["iterations"] + 3
    assert abs(r["error"] - ro["error"]) <= 0.01 * ro["error"]


@pytest.mark.parametrize("prec", ["FP64", "FP32"])
def test_double_word_outer_operator_solve(prec):
    """OPERATOR PRECISION DF64: every FP64 operator application (outer FPCG, and the FP64
    fine p-level) in double-FP32 words. The solve must behave as the FP64 method: same
    iteration count (+-1) and the oracle's discretisation error and solution norm."""
    s = dict(MG, **{"OPERATOR PRECISION": "DF64", "PRECONDITIONER PRECISION": prec})
    r = lpg.Elliptic(s).Run()
    ro = Oracle(MG).run()
    assert r["converged"]
    assert abs(r["iterations"] - ro["iterations"]) <= 1, (r["iterations"], ro["iterations"])
    assert abs(r["error"] - ro["error"]) <= 0.01 * ro["error"]
    assert abs(r["norm"] - ro["norm"]) < 1e-9 * ro["norm"]


def test_double_word_outer_operator_solve_degree5():
    """OPERATOR PRECISION DF64 at a degree without an even-odd kernel (N = 5, p-MG 5,2,1,
    FP32 p-levels): the FP64 method's iterations (+-1), error and norm."""
    base = dict(MG, **{"POLYNOMIAL DEGREE": 5, "MULTIGRID DEGREES": "5,2,1"})
    r = lpg.Elliptic(dict(base, **{"OPERATOR PRECISION": "DF64", "PRECONDITIONER PRECISION": "FP32"})).Run()
    ro = Oracle(base).run()
    assert r["converged"]
    assert abs(r["iterations"] - ro["iterations"]) <= 1, (r["iterations"], ro["iterations"])
    assert abs(r["error"] - ro["error"]) <= 0.01 * ro["error"]
    assert abs(r["norm"] - ro["norm"]) < 1e-9 * ro["norm"]


@pytest.mark.parametrize("over", [{}, {"LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2},
                                  {"LAMBDA": 0.0, "BOX BOUNDARY FLAG": -1}], ids=["jittered", "lognormal", "periodic"])
def test_semfem_preconditioner_matches_oracle(over):
    """SEMFEM (ellipticPreconSEMFEM.cpp): parAlmond AMG of the trilinear FEM matrix on the
    GLL sub-mesh, applied to the degree-N vectors."""
    s = dict(config1(), **{"BOX NX": 4, "BOX NY": 3, "BOX NZ": 3, "POLYNOMIAL DEGREE": 4, "MESH JITTER": 0.1,
                           "LAMBDA": 1.0, "LINEAR SOLVER": "PCG", "PRECONDITIONER": "SEMFEM",
                           "PARALMOND AGGREGATION": "UNSMOOTHED"})
    s.update(over)
    if over.get("BOX BOUNDARY FLAG") == -1:
        s["MESH JITTER"] = 0.0
    r = lpg.Elliptic(s).Run(want_solution=True)
    ro = Oracle(s).run()
    assert r["converged"]
    assert abs(r["iterations"] - ro["iterations"]) <= 1, (r["iterations"], ro["iterations"])
    assert rel_err(r["xL"], ro["xL"]) < 1e-7
    e = lpg.Elliptic(s)
    o = Oracle(s)
    rng = np.random.default_rng(5)
    rh = rng.standard_normal(e.Nglobal)
    z = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.precon(torch.tensor(rh, device="cuda"), z)
    torch.cuda.synchronize()
    assert rel_err(z.cpu().numpy(), o.precon(rh)) < 1e-9


@pytest.mark.parametrize("over", [{}, {"DISCRETIZATION": "IPDG"}, {"POLYNOMIAL DEGREE": 1},
                                  {"LAMBDA": 0.0, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0, "BOX NX": 4}],
                         ids=["c0", "ipdg", "c0_N1", "c0_all_neumann"])
def test_oas_preconditioner_matches_oracle(over):
    """OAS (ellipticPreconOAS.cpp) on one rank: p-multigrid of the whole mesh plus an additive
    degree-1 AMG correction."""
    s = dict(config1(), **{"BOX NX": 5, "BOX NY": 4, "BOX NZ": 3, "POLYNOMIAL DEGREE": 4, "MESH JITTER": 0.1,
                           "LAMBDA": 1.0, "LINEAR SOLVER": "PCG", "PRECONDITIONER": "OAS"})
    s.update(over)
    r = lpg.Elliptic(s).Run(want_solution=True)
    ro = Oracle(s).run()
    assert r["converged"]
    assert abs(r["iterations"] - ro["iterations"]) <= 1, (r["iterations"], ro["iterations"])
    assert rel_err(r["xL"], ro["xL"]) < 1e-7
    e, o = lpg.Elliptic(s), Oracle(s)
    rh = np.random.default_rng(9).standard_normal(e.Nglobal)
    z = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.precon(torch.tensor(rh, device="cuda"), z)
    torch.cuda.synchronize()
    assert rel_err(z.cpu().numpy(), o.precon(rh)) < 1e-9


def test_massmatrix_preconditioner_refused_for_hexahedra():
    with pytest.raises(RuntimeError, match="MASSMATRIX"):
        lpg.Elliptic(config1(**{"PRECONDITIONER": "MASSMATRIX", "LAMBDA": 1.0}))


def test_lognormal_lambda_and_gaussian_sources_solve():
    s = dict(MG, **{"LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2, "RHS FIELD": "GAUSSIAN SOURCES",
                    "RHS SEED": 3, "RHS SOURCES": 16})
    r = lpg.Elliptic(s).Run(want_solution=True)
    ro = Oracle(s).run()
    assert r["iterations"] == ro["iterations"]
    assert rel_err(r["xL"], ro["xL"]) < 1e-7
    assert abs(r["norm"] - ro["norm"]) < 1e-9 * ro["norm"]


def test_solver_level_api_and_not_converged_status():
    s = config1(**{"BOX NX": 3, "BOX NY": 3, "BOX NZ": 3})
    e = lpg.Elliptic(s)
    r = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.rhs(r)
    x = torch.zeros_like(r)
    it = e.Solve(x, r.clone(), tol=1e-8, maxit=2)
    assert it == 2
    x.zero_()
    it = e.Solve(x, r.clone(), tol=1e-8, maxit=5000)
    o = Oracle(s)
    xo, ito, _ = o.pcg(o.rhs(), tol=1e-8)
    assert it == ito
    assert rel_err(x.cpu().numpy(), xo) < 1e-8
