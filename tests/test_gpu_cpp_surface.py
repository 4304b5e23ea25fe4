"""The C++ surface (include/lpg.hpp): a caller compiled against the header alone.

tests/cpp/surface_test.cpp builds an elliptic_t from a settings file, applies its Operator,
solves through linearSolver_t (the solver the settings name) with the elliptic's own
preconditioner via elliptic_t::Solve, runs a plain PCG on a user-defined operator_t (2 A)
with IdentityPrecon, gathers and scatters through an ogs_t built from the numbering's ids,
and runs elliptic_t::Run. Its outputs are compared with the oracle (CPU restatement of the
reference) on config 1 (8^3, N=5, Jacobi FPCG) and on a p-multigrid FPCG case:
operator 1e-12, iteration counts equal, solutions 1e-8, gather exact to rounding.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from gpu_helpers import rel_err
from oracle.oracle import Oracle, settings_text

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CONFIG1 = {"BOX NX": 8, "BOX NY": 8, "BOX NZ": 8, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
           "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 5, "LAMBDA": 0.0, "LINEAR SOLVER": "FPCG",
           "PRECONDITIONER": "JACOBI"}
PMG = dict(CONFIG1, **{"BOX NX": 5, "BOX NY": 4, "BOX NZ": 3, "POLYNOMIAL DEGREE": 7, "MESH JITTER": 0.1,
                       "LAMBDA": 1.0, "PRECONDITIONER": "MULTIGRID", "MULTIGRID DEGREES": "7,3,1",
                       "PARALMOND AGGREGATION": "SMOOTHED"})


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    import __graft_entry__ as g
    g.build()
    build = os.path.join(ROOT, "libparanumal_gb300", "_build")
    out = str(tmp_path_factory.mktemp("cpp") / "surface_test")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "surface_test.cpp"), "-L", build, "-llpg",
                    "-Wl,-rpath," + build, "-o", out], check=True)
    return out


@pytest.mark.parametrize("cfg", [CONFIG1, PMG], ids=["config1_jacobi_fpcg", "pmg_fpcg"])
def test_cpp_surface_matches_oracle(exe, tmp_path, cfg):
    rc = tmp_path / "s.rc"
    rc.write_text(settings_text(cfg))
    p = subprocess.run([exe, str(rc), str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    res = json.loads(p.stdout.strip().splitlines()[-1])
    o = Oracle(cfg)
    N = o.Ngather
    assert res["Nglobal"] == N and res["Ngather"] == N
    rd = lambda name: np.fromfile(str(tmp_path / name), dtype=np.float64)
    q = np.sin(0.37 * np.arange(N))
    assert rel_err(rd("Aq.bin"), o.operator(q)) < 1e-12
    xo, it, _ = o.pcg(o.rhs(), tol=1e-8)
    assert res["iterations"] == it
    assert rel_err(rd("x.bin"), xo) < 1e-8
    ro = o.run()
    assert res["run_iterations"] == ro["iterations"]
    assert abs(res["norm"] - ro["norm"]) < 1e-9 * ro["norm"]
    # plain CG on 2 A with the identity: the solution of A x = b / 2
    x2 = rd("x_twice.bin")
    assert res["iterations_twice"] > 0
    assert rel_err(2.0 * o.operator(x2), o.rhs()) < 1e-8
    v = np.cos(0.11 * np.arange(o.Nlocal))
    g = rd("gather.bin")
    assert rel_err(g, o.gather(v)) < 1e-14
    assert rel_err(rd("scatter.bin"), o.scatter(g)) < 1e-15
    assert res["caught"] == 1
