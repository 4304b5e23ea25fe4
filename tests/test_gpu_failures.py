"""Failure paths of the solve, made on the host, with no GPU fault.

* A learned smoother whose weights are NaN (host-side injection): every V-cycle's residual
  check fails, each V-cycle is redone with the plain smoother, and the solve converges in
  the plain method's iteration count to the plain solution. Garbage weights (random, huge):
  the V-cycles that do not halve the residual fall back, and the solve still converges to
  the same discrete solution.
* A NaN or Inf in the right-hand side or the initial guess: the Krylov solve stops with
  LPG_ERR_BREAKDOWN instead of iterating on NaNs (the reference's counterpart guards are
  the non-positive p.Ap / r.r checks of linearSolverPCG.cpp:93-147).
* A bounded device wait that runs out: lpg_debug_mlp_hold makes the tensor-core MLP
  kernel wait on a barrier that nothing signals for a short limit and give up, as any of
  its pipeline waits does after its limit (no copy or MMA is issued, tensor memory is
  freed). The host reads the timeout status (LPG_ERR_TIMEOUT); a learned V-cycle falls back
  to the plain smoother and the solve still converges; the context stays usable.
"""
import ctypes

import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from gpu_helpers import rel_err

pytestmark = pytest.mark.gpu

LEARN = {"BOX NX": 4, "BOX NY": 4, "BOX NZ": 4, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
         "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 7, "LAMBDA": 1.0, "LAMBDA FIELD": "LOGNORMAL",
         "LAMBDA SEED": 2, "MESH JITTER": 0.1, "MESH JITTER SEED": 0, "LINEAR SOLVER": "FPCG",
         "PRECONDITIONER": "MULTIGRID", "MULTIGRID DEGREES": "7,3,1", "PARALMOND AGGREGATION": "SMOOTHED",
         "PRECONDITIONER PRECISION": "FP32"}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)
    yield
    lpg.lib().lpg_debug_mlp_hold(0)


def _plain():
    return lpg.Elliptic(LEARN).Run(want_solution=True)


@pytest.mark.parametrize("kind", ["nan", "garbage"])
def test_bad_weights_fall_back_on_every_vcycle(kind):
    n = int(lpg.lib().lpg_mlp_param_count())
    if kind == "nan":
        w = np.full(n, np.nan, dtype=np.float32)
    else:
        w = (np.random.default_rng(1).standard_normal(n) * 1e4).astype(np.float32)
    plain = _plain()
    e = lpg.Elliptic(LEARN)
    e.set_learned_smoother(w, 0.5)
    r = e.Run(want_solution=True)
    assert r["converged"]
    assert e.info("vcycles") > 0
    if kind == "nan":
        # no learned V-cycle can pass the residual check: each is redone with the plain
        # smoother, so the preconditioner is the plain one
        assert e.info("fallbacks") == e.info("vcycles")
        assert r["iterations"] == plain["iterations"]
        assert rel_err(r["xL"], plain["xL"]) < 1e-10
    else:
        # garbage directions are scaled by the energy-optimal step, so some V-cycles may
        # still halve the residual and pass; the rest fall back, and the flexible solve
        # reaches the same discrete solution
        assert e.info("fallbacks") >= 1
        assert r["iterations"] <= plain["iterations"] + 3
        assert rel_err(r["xL"], plain["xL"]) < 1e-6


@pytest.mark.parametrize("where", ["rhs", "x0"])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_non_finite_input_stops_with_breakdown(where, bad):
    e = lpg.Elliptic(dict(LEARN, **{"PRECONDITIONER PRECISION": "FP64"}))
    r = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.rhs(r)
    x = torch.zeros_like(r)
    (r if where == "rhs" else x)[e.Nglobal // 3] = bad
    it = ctypes.c_int(-1)
    st = lpg.lib().lpg_elliptic_solve(e.h, x.data_ptr(), r.data_ptr(), 1e-8, 100, ctypes.byref(it))
    assert st == -7, (st, lpg.lib().lpg_last_error())
    assert it.value <= 1
    # the object stays usable: a clean solve afterwards converges
    e.rhs(r)
    x.zero_()
    assert e.Solve(x, r, tol=1e-8) > 0
    assert torch.isfinite(x).all()


def test_mlp_wait_limit_runs_out_and_learned_cycle_falls_back():
    L = lpg.lib()
    n = int(L.lpg_mlp_param_count())
    theta = (torch.rand(n, device="cuda", generator=torch.Generator(device="cuda").manual_seed(3)) - 0.5) * 0.1
    X = torch.randn(300, 896, device="cuda")
    Y = torch.full((300, 512), 7.0, device="cuda")
    lpg.check(L.lpg_mlp_forward_bf16(theta.data_ptr(), 300, X.data_ptr(), Y.data_ptr(), None))
    ref = Y.clone()
    # a 1 ms limit on a barrier nothing signals: the kernel gives up before any copy or MMA
    lpg.check(L.lpg_debug_mlp_hold(1_000_000))
    st = L.lpg_mlp_forward_bf16(theta.data_ptr(), 300, X.data_ptr(), Y.data_ptr(), None)
    assert st == -8, (st, L.lpg_last_error())
    assert b"timed out" in L.lpg_last_error()
    plain = _plain()
    e = lpg.Elliptic(LEARN)
    w = (theta.cpu().numpy()).astype(np.float32)
    e.set_learned_smoother(w, 0.5)
    r = e.Run(want_solution=True)
    assert r["converged"]
    assert e.info("vcycles") > 0
    assert e.info("learned_timeouts") == e.info("vcycles") == e.info("fallbacks")
    assert r["iterations"] == plain["iterations"]
    assert rel_err(r["xL"], plain["xL"]) < 1e-10
    # limit off: the kernel runs again and gives the first call's result
    lpg.check(L.lpg_debug_mlp_hold(0))
    lpg.check(L.lpg_mlp_forward_bf16(theta.data_ptr(), 300, X.data_ptr(), Y.data_ptr(), None))
    torch.cuda.synchronize()
    assert torch.equal(Y, ref)
