"""Non-blocking flexible PCG (LINEAR SOLVER = NBFPCG, linearSolverNBFPCG.cpp:72-186) on the
CUDA path against the oracle's restatement of the same recurrence: identical iteration
counts, the oracle's discretisation error and solution, and the FPCG solution."""
import pytest
import torch

import libparanumal_gb300 as lpg
from gpu_helpers import rel_err
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

JAC = {"BOX NX": 6, "BOX NY": 5, "BOX NZ": 4, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
       "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 5, "LAMBDA": 0.5, "LINEAR SOLVER": "NBFPCG",
       "PRECONDITIONER": "JACOBI", "MESH JITTER": 0.1}
MG = dict(JAC, **{"POLYNOMIAL DEGREE": 7, "PRECONDITIONER": "MULTIGRID", "MULTIGRID DEGREES": "7,3,1",
                  "PARALMOND AGGREGATION": "SMOOTHED", "LAMBDA": 0.0})


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


@pytest.mark.parametrize("settings", [JAC, MG], ids=["jacobi", "multigrid"])
def test_nbfpcg_matches_oracle(settings):
    r = lpg.Elliptic(settings).Run(want_solution=True)
    ro = Oracle(settings).run()
    assert r["converged"]
    assert r["iterations"] == ro["iterations"], (r["iterations"], ro["iterations"])
    assert abs(r["error"] - ro["error"]) <= 1e-6 * ro["error"]
    assert rel_err(r["xL"], ro["xL"]) < 1e-7


def test_nbfpcg_and_fpcg_agree():
    a = lpg.Elliptic(MG).Run(want_solution=True)
    b = lpg.Elliptic(dict(MG, **{"LINEAR SOLVER": "FPCG"})).Run(want_solution=True)
    assert abs(a["iterations"] - b["iterations"]) <= 1
    assert rel_err(a["xL"], b["xL"]) < 1e-7


def test_nbfpcg_mixed_precision_preconditioner():
    s = dict(MG, **{"PRECONDITIONER PRECISION": "FP32", "OPERATOR PRECISION": "DF64"})
    r = lpg.Elliptic(s).Run()
    ro = Oracle(MG).run()
    assert r["converged"]
    assert abs(r["iterations"] - ro["iterations"]) <= 2
    assert abs(r["error"] - ro["error"]) <= 0.01 * ro["error"]
