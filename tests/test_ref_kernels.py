"""The oracle's operator against the reference's own kernels (CPU).

ellipticPartialAxHex3D (solvers/elliptic/okl/ellipticAxHex3D.okl:156-295) and the ogs
gather kernel (libs/ogs/okl/ogsKernels.okl:86-122) are translated from the reference's
OKL text by oracle/okl_translate.py with OCCA's Serial semantics, compiled with the
reference's release flags, and driven the way elliptic_t::Operator drives them on one
rank (two partial-Ax launches, then Gather(Add, Trans); ellipticOperator.cpp:29-106).
Fed the oracle's own mesh arrays, they must reproduce the oracle's partial Ax (the
kernel's AqL contract) and assembled operator to 1e-13 relative (max-norm; the two builds
may contract multiply-adds differently). This pins the oracle's Ax, which the CUDA tests
compare against at 1e-12, to the reference's own code. Skipped when neither the
reference tree nor the C file generated from it is on this machine."""
import numpy as np
import pytest

from gpu_helpers import box, rel_err
from oracle import refimpl
from oracle.oracle import Oracle

pytestmark = pytest.mark.skipif(not refimpl.available(), reason="reference kernels not built here")

CASES = [box(**{"POLYNOMIAL DEGREE": N}) for N in range(1, 9)] + [
    box(**{"POLYNOMIAL DEGREE": 5, "MESH JITTER": 0.0, "LAMBDA": 0.0, "BOX NX": 4, "BOX NY": 4, "BOX NZ": 4}),
    box(**{"POLYNOMIAL DEGREE": 3, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0}),   # periodic
    box(**{"POLYNOMIAL DEGREE": 6, "BOX BOUNDARY FLAG": 2, "LAMBDA": 0.3}),          # Neumann
    box(**{"POLYNOMIAL DEGREE": 2, "BOX NX": 1, "BOX NY": 1, "BOX NZ": 1}),          # one element
]


def ids(c):
    return "N%s_%sx%sx%s_bc%s_lam%s" % (c["POLYNOMIAL DEGREE"], c["BOX NX"], c["BOX NY"], c["BOX NZ"],
                                        c["BOX BOUNDARY FLAG"], c["LAMBDA"])


@pytest.mark.parametrize("cfg", CASES, ids=ids)
def test_oracle_operator_equals_reference_kernels(cfg):
    o = Oracle(cfg)
    r = refimpl.RefOperator.from_oracle(o, cfg["LAMBDA"])
    rng = np.random.default_rng(cfg["POLYNOMIAL DEGREE"])
    for _ in range(2):
        q = rng.uniform(-1, 1, o.Ngather)
        assert rel_err(o.partial_ax(q), r.partial_ax(q)) < 1e-13
        assert rel_err(o.operator(q), r.apply(q)) < 1e-13


def test_reference_gather_blocks_hold_at_most_512_entries():
    """Row blocks of the reference's Trans gather (ogsOperator.cpp:495-560): an N=8 box has
    dofs shared by 8 elements; the blocked gather must still give every dof's full sum."""
    cfg = box(**{"POLYNOMIAL DEGREE": 8, "BOX NX": 3, "BOX NY": 3, "BOX NZ": 3, "BOX BOUNDARY FLAG": -1})
    o = Oracle(cfg)
    r = refimpl.RefOperator.from_oracle(o, 1.0)
    # the oracle's Gather(Trans) of the reference kernel's AqL against the reference's
    # blocked gather of the same AqL (inside apply)
    q = np.random.default_rng(4).uniform(-1, 1, o.Ngather)
    assert rel_err(o.gather(r.partial_ax(q)), r.apply(q)) < 1e-14
