"""Run-to-run variation of the atomically assembled operator and of the solves built on it.

The operators assemble element contributions with atomic adds, so the order of the adds
into a shared dof, and with it the last bits of the sum, may change from one application
to the next (the reference's gather adds in a fixed order; ogsKernels.okl:86-122). These
tests bound that variation: repeated operator applications agree to a few units in the
last place, and repeated solves give the same iteration counts and solutions that agree
far below the solver tolerance, for the FP64 method and the mixed-precision one."""
import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from gpu_helpers import box, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


CFG = box(**{"BOX NX": 12, "BOX NY": 10, "BOX NZ": 9, "LAMBDA": 1.0, "LAMBDA FIELD": "LOGNORMAL",
             "LAMBDA SEED": 2, "PRECONDITIONER": "MULTIGRID", "MULTIGRID DEGREES": "7,3,1",
             "PARALMOND AGGREGATION": "SMOOTHED"})


@pytest.mark.parametrize("kind", ["FP64", "DF64", "FP32"])
def test_repeated_operator_applications_agree_to_rounding(kind):
    e = lpg.Elliptic(CFG)
    rng = np.random.default_rng(3)
    dt = torch.float32 if kind == "FP32" else torch.float64
    q = torch.tensor(rng.uniform(-1, 1, e.Nglobal), dtype=dt, device="cuda")
    outs = []
    for _ in range(4):
        Aq = torch.full_like(q, np.nan)
        {"FP64": e.Operator, "DF64": e.OperatorDF64, "FP32": e.OperatorF32}[kind](q, Aq)
        torch.cuda.synchronize()
        outs.append(Aq.cpu().numpy().astype(np.float64))
    eps = np.finfo(np.float32 if kind == "FP32" else np.float64).eps
    scale = np.abs(outs[0]).max()
    for o in outs[1:]:
        assert np.all(np.isfinite(o))
        # a reordered sum of at most 8 element contributions: a few ulps of the largest entry
        assert np.abs(o - outs[0]).max() <= 16 * eps * scale


@pytest.mark.parametrize("prec", ["FP64", "FP32"])
def test_repeated_solves_agree(prec):
    s = dict(CFG, **{"PRECONDITIONER PRECISION": prec})
    e = lpg.Elliptic(s)
    r = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.rhs(r)
    runs = []
    for _ in range(3):
        x = torch.zeros_like(r)
        it = e.Solve(x, r.clone(), tol=1e-10)   # the solve overwrites its right-hand side
        runs.append((it, x.cpu().numpy()))
    for it, x in runs[1:]:
        assert it == runs[0][0]
        assert rel_err(x, runs[0][1]) < 1e-12
