"""Self-consistency of the oracle's IPDG restatement (CPU): the operator is symmetric, its
Jacobi diagonal is the diagonal of the operator itself, and the discretisation error of
the manufactured sine solution converges spectrally in N, like the C0 discretisation."""
import numpy as np
import pytest

from oracle.oracle import Oracle

BASE = {"BOX NX": 3, "BOX NY": 2, "BOX NZ": 2, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
        "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 5, "LAMBDA": 0.7, "DISCRETIZATION": "IPDG",
        "LINEAR SOLVER": "PCG", "PRECONDITIONER": "JACOBI", "MESH JITTER": 0.1}


@pytest.mark.parametrize("over", [{}, {"POLYNOMIAL DEGREE": 7, "BOX BOUNDARY FLAG": -1, "MESH JITTER": 0.0},
                                  {"POLYNOMIAL DEGREE": 2, "LAMBDA FIELD": "LOGNORMAL"}],
                         ids=["dirichlet_N5", "periodic_N7", "lognormal_N2"])
def test_oracle_ipdg_operator_symmetric_and_diagonal(over):
    o = Oracle(dict(BASE, **over))
    n = o.Ngather
    rng = np.random.default_rng(1)
    a, b = rng.standard_normal(n), rng.standard_normal(n)
    Aa, Ab = o.operator(a), o.operator(b)
    assert abs(b @ Aa - a @ Ab) < 1e-11 * abs(b @ Aa)
    assert a @ Aa > 0
    d = 1.0 / o.precon(np.ones(n))
    idx = range(0, n, max(1, n // 300))
    brute = np.array([o.operator(np.eye(1, n, i).ravel())[i] for i in idx])
    assert np.abs(brute - d[list(idx)]).max() < 1e-13 * np.abs(brute).max()


def test_oracle_ipdg_error_converges_like_c0():
    errs = []
    for N in (2, 3, 4, 5):
        s = dict(BASE, **{"POLYNOMIAL DEGREE": N, "BOX NX": 3, "BOX NY": 3, "BOX NZ": 3})
        r = Oracle(s).run()
        rc = Oracle(dict(s, **{"DISCRETIZATION": "CONTINUOUS"})).run()
        errs.append(r["error"])
        assert r["error"] < 5 * rc["error"] + 1e-7
    assert all(b < 0.2 * a for a, b in zip(errs, errs[1:]))


@pytest.mark.parametrize("over", [{"POLYNOMIAL DEGREE": 1}, {"POLYNOMIAL DEGREE": 2, "BOX BOUNDARY FLAG": -1,
                                                              "MESH JITTER": 0.0, "BOX NX": 3, "BOX NY": 3},
                                  {"POLYNOMIAL DEGREE": 3, "DISCRETIZATION": "CONTINUOUS"}],
                         ids=["ipdg_N1", "ipdg_periodic_N2", "c0_N3"])
def test_oracle_assembled_matrix_equals_operator(over):
    """The explicitly assembled matrix (BuildOperatorMatrixIpdgHex3D / ...Continuous, the
    AMG's level 0) and the matrix-free operator are the same linear map (up to the 1e-8
    entry drop tolerance)."""
    o = Oracle(dict(BASE, **over))
    x = np.random.default_rng(3).standard_normal(o.Ngather)
    Ax, Mx = o.operator(x), o.matrix_apply(x)
    assert np.abs(Ax - Mx).max() < 1e-7 * np.abs(Ax).max()


def test_oracle_ipdg_with_neumann_tags_matrix(tmp_path):
    from gmsh_mesh import write_box
    f = write_box(str(tmp_path / "m.msh"), 3, 2, 2, rotate_seed=4, tags=(1, 2, 2, 1, 2, 2))
    o = Oracle(dict(BASE, **{"MESH FILE": f, "MESH JITTER": 0.0, "POLYNOMIAL DEGREE": 2}))
    x = np.random.default_rng(5).standard_normal(o.Ngather)
    Ax, Mx = o.operator(x), o.matrix_apply(x)
    assert np.abs(Ax - Mx).max() < 1e-7 * np.abs(Ax).max()
