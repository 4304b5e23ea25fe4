"""Initial-guess strategies of the solver (CLASSIC and QR projection, EXTRAP with
minimum-norm and column-pivoted QR weights, ZERO) on a sequence of solves whose exact
solutions drift smoothly: every initial guess formed on the GPU is compared with the CPU
restatement (oracle/initial_guess.py) fed the same solution history, and the history
must make the later solves cheaper."""
import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from gpu_helpers import box, rel_err
from oracle import initial_guess as ig
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

# stopping relative to the right-hand side (not to the initial residual), so that a better
# initial guess shows as fewer iterations
BASE = box(**{"POLYNOMIAL DEGREE": 5, "BOX NX": 4, "BOX NY": 4, "BOX NZ": 3, "LINEAR SOLVER": "PCG",
              "PRECONDITIONER": "JACOBI", "LINEAR SOLVER STOPPING CRITERION": "ABS/REL-RHS-2NORM"})


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


CASES = [
    ("CLASSIC", {"INITIAL GUESS HISTORY SPACE DIMENSION": 3}, lambda: ig.Classic(3)),
    ("QR", {"INITIAL GUESS HISTORY SPACE DIMENSION": 3}, lambda: ig.RollingQR(3)),
    ("EXTRAP", {"INITIAL GUESS HISTORY SPACE DIMENSION": 3, "INITIAL GUESS EXTRAP DEGREE": 2},
     lambda: ig.Extrap(3, 2)),
    ("EXTRAP", {"INITIAL GUESS HISTORY SPACE DIMENSION": 4, "INITIAL GUESS EXTRAP DEGREE": 2,
                "INITIAL GUESS EXTRAP COEFFS METHOD": "CPQR"}, lambda: ig.Extrap(4, 2, cpqr=True)),
    ("ZERO", {}, None),
]


@pytest.mark.parametrize("strategy,extra,make_ref", CASES, ids=[c[0] + str(i) for i, c in enumerate(CASES)])
def test_initial_guess_sequence_matches_restatement(strategy, extra, make_ref):
    s = dict(BASE, **{"INITIAL GUESS STRATEGY": strategy}, **extra)
    e = lpg.Elliptic(s)
    o = Oracle(BASE)
    N = e.Nglobal
    rng = np.random.default_rng(17)
    U = [rng.uniform(-1, 1, N) for _ in range(4)]
    AU = [o.operator(u) for u in U]
    ref = make_ref() if make_ref else None
    iters = []
    for t in range(8):
        w = [1.0, 0.3 * t, 0.05 * t * t, np.sin(0.7 * t)]   # x_t = sum w_k U_k
        rhs = sum(wk * a for wk, a in zip(w, AU))
        r = torch.tensor(rhs, device="cuda")
        x0 = torch.full((N,), 5.0, dtype=torch.float64, device="cuda")
        e.initial_guess(x0, r)
        g = x0.cpu().numpy()
        if ref is None:
            assert np.all(g == 0.0)
        else:
            gref = ref.form(np.full(N, 5.0), rhs)
            if np.linalg.norm(gref) == 0.0:
                assert np.all(g == 5.0) or np.all(g == 0.0)
            else:
                assert rel_err(g, gref) < 1e-9, (t, rel_err(g, gref))
        x = torch.zeros(N, dtype=torch.float64, device="cuda")
        iters.append(e.Solve(x, r.clone(), tol=1e-8))
        torch.cuda.synchronize()
        if ref is not None:
            if strategy == "EXTRAP":
                ref.form(np.zeros(N), rhs)   # the solve formed the guess once more
            ref.update(o.operator, x.cpu().numpy())
    print(strategy, "iterations per solve:", iters, "history", e.info("ig_history"))
    if strategy != "ZERO":
        assert e.info("ig_history") >= 1
        assert min(iters[3:]) < 0.9 * iters[0], iters


LONG = [
    ("CLASSIC", {"INITIAL GUESS HISTORY SPACE DIMENSION": 10}, lambda: ig.Classic(10), 12),
    ("QR", {"INITIAL GUESS HISTORY SPACE DIMENSION": 5}, lambda: ig.RollingQR(5), 8),
    ("QR", {"INITIAL GUESS HISTORY SPACE DIMENSION": 17}, lambda: ig.RollingQR(17), 20),
    ("EXTRAP", {"INITIAL GUESS HISTORY SPACE DIMENSION": 18, "INITIAL GUESS EXTRAP DEGREE": 4},
     lambda: ig.Extrap(18, 4), 20),
]


@pytest.mark.parametrize("strategy,extra,make_ref,steps", LONG,
                         ids=["%s%d" % (c[0], c[1]["INITIAL GUESS HISTORY SPACE DIMENSION"]) for c in LONG])
def test_long_history_matches_restatement(strategy, extra, make_ref, steps):
    """History dimensions past 4 (the 8-, 16- and 32-column instances of the history
    kernels), with the rolling QR basis filled and then dropping its first column: solutions
    drawn from a 24-dimensional space, so the history directions stay independent."""
    s = dict(BASE, **{"INITIAL GUESS STRATEGY": strategy}, **extra)
    e = lpg.Elliptic(s)
    o = Oracle(BASE)
    N = e.Nglobal
    rng = np.random.default_rng(29)
    AU = [o.operator(rng.uniform(-1, 1, N)) for _ in range(24)]
    ref = make_ref()
    for t in range(steps):
        rhs = sum(np.cos(0.37 * (k + 1) * t + k) * a for k, a in enumerate(AU))
        r = torch.tensor(rhs, device="cuda")
        x0 = torch.zeros(N, dtype=torch.float64, device="cuda")
        e.initial_guess(x0, r)
        gref = ref.form(np.zeros(N), rhs)
        if np.linalg.norm(gref) > 0.0:
            err = rel_err(x0.cpu().numpy(), gref)
            assert err < 1e-9, (t, err)
        x = torch.zeros(N, dtype=torch.float64, device="cuda")
        e.Solve(x, r.clone(), tol=1e-8)
        torch.cuda.synchronize()
        if strategy == "EXTRAP":
            ref.form(np.zeros(N), rhs)
        ref.update(o.operator, x.cpu().numpy())
    assert e.info("ig_history") == min(steps, extra["INITIAL GUESS HISTORY SPACE DIMENSION"]) or strategy == "CLASSIC"


def test_bad_initial_guess_settings_are_errors():
    with pytest.raises(lpg.LPGError):
        lpg.Elliptic(dict(BASE, **{"INITIAL GUESS STRATEGY": "CLASSIC"}))          # no history dimension
    with pytest.raises(lpg.LPGError):
        lpg.Elliptic(dict(BASE, **{"INITIAL GUESS STRATEGY": "GUESS"}))
    with pytest.raises(lpg.LPGError):
        lpg.Elliptic(dict(BASE, **{"INITIAL GUESS STRATEGY": "EXTRAP",
                                   "INITIAL GUESS HISTORY SPACE DIMENSION": 2, "INITIAL GUESS EXTRAP DEGREE": 3}))
