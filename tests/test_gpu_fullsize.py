"""The operator at the full benchmark sizes, through properties that do not need the
oracle (which cannot run these sizes in seconds): the 64^3 operator workload (N=7, jitter
0.1, lambda=1; 134M local nodes) and the 112^3 learned/mixed-precision mesh (lognormal
lambda; 719M local nodes, 480,048,687 dofs, geometric-factor offsets beyond 2^31).

* symmetry: q2.(A q1) = q1.(A q2) to 1e-12 relative, and q.(A q) > 0;
* linearity: A(q1 + 2 q2) = A q1 + 2 A q2 to 1e-13 of the largest entry;
* the double-FP32-word operator equals the FP64 one to 1e-12 (the FP64 bar) and the FP32
  operator to 5e-6;
* the dof count of a Dirichlet box, (n N - 1)^3.
"""
import pytest
import torch

import libparanumal_gb300 as lpg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


def box(nx, **over):
    d = {"BOX NX": nx, "BOX NY": nx, "BOX NZ": nx, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
         "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 7, "LAMBDA": 1.0, "MESH JITTER": 0.1,
         "MESH JITTER SEED": 0, "LINEAR SOLVER": "FPCG", "PRECONDITIONER": "NONE"}
    d.update(over)
    return d


def rel_max(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("nx,over", [(64, {}), (112, {"LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2})],
                         ids=["64cubed", "112cubed_lognormal"])
def test_full_size_operator_properties(nx, over):
    e = lpg.Elliptic(box(nx, **over))
    n = e.Nglobal
    assert n == (nx * 7 - 1) ** 3
    q1 = torch.empty(n, dtype=torch.float64, device="cuda")
    q2 = torch.empty_like(q1)
    e.random_vector(q1, 1)
    e.random_vector(q2, 5)
    A1, A2, A3 = torch.empty_like(q1), torch.empty_like(q1), torch.empty_like(q1)
    e.Operator(q1, A1)
    e.Operator(q2, A2)
    d12, d21 = float(torch.dot(q2, A1)), float(torch.dot(q1, A2))
    assert abs(d12 - d21) <= 1e-12 * max(abs(d12), float(torch.dot(q1, A1)))
    assert float(torch.dot(q1, A1)) > 0
    e.Operator(q1 + 2 * q2, A3)
    assert rel_max(A3, A1 + 2 * A2) < 1e-13
    del A2, A3
    dw = torch.empty_like(q1)
    e.OperatorDF64(q1, dw)
    assert rel_max(dw, A1) < 1e-12
    del dw
    q32 = q1.float()
    A32 = torch.empty_like(q32)
    e.OperatorF32(q32, A32)
    assert rel_max(A32.double(), A1) < 5e-6
    e.close()
    torch.cuda.empty_cache()
