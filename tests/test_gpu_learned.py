"""Learned fine-level smoother: the CUDA forward/backward/Adam kernels against the FP64
numpy restatement (oracle/mlp.py), BF16 tensor-core inference against FP32, training on
the plain solver's (residual, exact error) pairs, and FPCG with the learned smoother plus
per-V-cycle fallback against the plain method."""
import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from gpu_helpers import rel_err
from oracle import mlp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


def _dev(a, dtype=torch.float32):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def test_forward_backward_match_fp64_restatement():
    L = lpg.lib()
    assert L.lpg_mlp_param_count() == mlp.param_count() == 492800
    rng = np.random.default_rng(4)
    theta = mlp.glorot(2).astype(np.float32)
    B = 37
    X = rng.standard_normal((B, 896)).astype(np.float32)
    dY = rng.standard_normal((B, 512)).astype(np.float32)
    P, Xd, dYd = _dev(theta), _dev(X), _dev(dY)
    ws = torch.zeros(int(L.lpg_mlp_workspace_floats(B)), dtype=torch.float32, device="cuda")
    Y = torch.zeros((B, 512), dtype=torch.float32, device="cuda")
    lpg.check(L.lpg_mlp_forward_f32(P.data_ptr(), B, Xd.data_ptr(), ws.data_ptr(), Y.data_ptr(), None))
    G = torch.zeros_like(P)
    work = torch.zeros(2 * B * 256, dtype=torch.float32, device="cuda")
    lpg.check(L.lpg_mlp_backward_f32(P.data_ptr(), B, Xd.data_ptr(), ws.data_ptr(), dYd.data_ptr(), G.data_ptr(),
                                     work.data_ptr(), None))
    torch.cuda.synchronize()
    yref, _ = mlp.forward(theta.astype(np.float64), X.astype(np.float64))
    gref = mlp.backward(theta.astype(np.float64), X.astype(np.float64), dY.astype(np.float64))
    assert rel_err(Y.cpu().numpy(), yref) < 1e-5
    assert rel_err(G.cpu().numpy(), gref) < 1e-4
    # per-layer check so a wrong block cannot hide behind a large one
    off = 0
    for l in range(4):
        n = mlp.DIMS[l] * mlp.DIMS[l + 1] + mlp.DIMS[l + 1]
        assert rel_err(G.cpu().numpy()[off:off + n], gref[off:off + n]) < 1e-4, l
        off += n


def test_adam_step_matches_restatement():
    L = lpg.lib()
    rng = np.random.default_rng(9)
    n = 10_001
    w, g, m, v = (rng.standard_normal(n).astype(np.float32) for _ in range(4))
    v = np.abs(v)
    W, Gd, M, V = _dev(w), _dev(g), _dev(m), _dev(v)
    lpg.check(L.lpg_mlp_adam_f32(n, W.data_ptr(), Gd.data_ptr(), M.data_ptr(), V.data_ptr(), 1e-3, 3, None))
    torch.cuda.synchronize()
    wr, mr, vr = mlp.adam(w.astype(np.float64), g.astype(np.float64), m.astype(np.float64), v.astype(np.float64),
                          1e-3, 3)
    assert rel_err(W.cpu().numpy(), wr) < 1e-6
    assert rel_err(M.cpu().numpy(), mr) < 1e-6
    assert rel_err(V.cpu().numpy(), vr) < 1e-6


# 39,559 rows = 310 tiles of 128 on 152 CTAs: every CTA runs a pair of tiles (both slots of
# the two-tile kernel) and six of them a third tile alone, the last one partial
@pytest.mark.parametrize("B", [1, 130, 1000, 39559])
def test_bf16_tensor_core_inference_matches_fp32(B):
    L = lpg.lib()
    rng = np.random.default_rng(B)
    theta = mlp.glorot(5).astype(np.float32)
    X = rng.standard_normal((B, 896)).astype(np.float32)
    P, Xd = _dev(theta), _dev(X)
    Y = torch.zeros((B, 512), dtype=torch.float32, device="cuda")
    lpg.check(L.lpg_mlp_forward_bf16(P.data_ptr(), B, Xd.data_ptr(), Y.data_ptr(), None))
    torch.cuda.synchronize()
    yref, _ = mlp.forward(theta.astype(np.float64), X.astype(np.float64))
    assert rel_err(Y.cpu().numpy(), yref) < 3e-2


_MLP_CHILD = r"""
import sys
import numpy as np
import torch
import libparanumal_gb300 as lpg
from oracle import mlp
B = int(sys.argv[1])
rng = np.random.default_rng(B)
theta = torch.tensor(mlp.glorot(5).astype(np.float32), device="cuda")
X = torch.tensor(rng.standard_normal((B, 896)).astype(np.float32), device="cuda")
Y = torch.zeros((B, 512), dtype=torch.float32, device="cuda")
lpg.check(lpg.lib().lpg_mlp_forward_bf16(theta.data_ptr(), B, X.data_ptr(), Y.data_ptr(), None))
torch.cuda.synchronize()
np.save(sys.argv[2], Y.cpu().numpy())
"""


@pytest.mark.parametrize("B", [130, 39559])
def test_two_tile_mlp_kernel_equals_one_tile_kernel(tmp_path, B):
    """The tensor-core MLP with two tiles in flight per CTA (the default) against the
    one-tile kernel (LPG_MLP_TC=single): the same MMAs in the same K order and the same
    epilogue arithmetic, so the outputs are bit for bit equal."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = {}
    for mode in ("two", "single"):
        env = dict(os.environ, PYTHONPATH=root)
        env.pop("LPG_MLP_TC", None)
        if mode == "single":
            env["LPG_MLP_TC"] = "single"
        f = tmp_path / (mode + ".npy")
        p = subprocess.run([sys.executable, "-c", _MLP_CHILD, str(B), str(f)], env=env, cwd=root,
                           capture_output=True, text=True, timeout=600)
        assert p.returncode == 0, p.stderr[-2000:]
        out[mode] = np.load(f)
    assert np.all(np.isfinite(out["two"]))
    assert np.array_equal(out["two"], out["single"])


def learned_problem(nx, **over):
    d = {"BOX NX": nx, "BOX NY": nx, "BOX NZ": nx, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
         "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 7, "LAMBDA": 1.0, "LAMBDA FIELD": "LOGNORMAL",
         "LAMBDA SEED": 2, "MESH JITTER": 0.1, "MESH JITTER SEED": 0, "LINEAR SOLVER": "FPCG",
         "PRECONDITIONER": "MULTIGRID", "MULTIGRID DEGREES": "7,3,1", "PARALMOND AGGREGATION": "SMOOTHED"}
    d.update(over)
    return d


@pytest.fixture(scope="module")
def trained():
    w, hist = lpg.train_smoother(learned_problem(8), nsolves=3, samples_per_solve=400, epochs=25, batch=100,
                                 lr=1e-3, seed=11)
    return w, hist


def test_training_reduces_loss(trained):
    w, hist = trained
    assert np.all(np.isfinite(hist)) and np.all(np.isfinite(w))
    assert hist[-1] < 0.7 * hist[0], hist


@pytest.fixture(scope="module")
def trained_full():
    """The network as the benchmark trains it: 20,000 pairs from 8 plain solves on 32^3,
    40 epochs (a few seconds on the GPU)."""
    w, hist = lpg.train_smoother(learned_problem(32), nsolves=8, samples_per_solve=2500, epochs=40, batch=250,
                                 lr=1e-3, seed=7)
    return w, hist


@pytest.mark.parametrize("prec", ["FP64", "FP32"])
def test_trained_network_gains_over_the_smoother_without_it(trained_full, prec):
    """What the trained network gains over the method without it: the same V-cycle with
    the network's output zero (the damped-Jacobi part alone, energy-optimal steps, zero
    weights) needs more FPCG iterations than with the trained network (measured: 12
    without, 10 with, at 10^3 and 32^3, two steps per side). The fallback is switched off
    for both (threshold 1e30), so every V-cycle uses the smoother under test."""
    w, _ = trained_full
    s = learned_problem(10, **{"PRECONDITIONER PRECISION": prec, "LEARNED SMOOTHER STEPS": 2})
    runs = {}
    for name, weights in (("trained", w), ("without network", np.zeros_like(w))):
        e = lpg.Elliptic(s)
        e.set_learned_smoother(weights, 1e30)
        r = e.Run()
        assert r["converged"] and e.info("fallbacks") == 0
        runs[name] = r["iterations"]
    print("iterations: trained network %d, without it %d" % (runs["trained"], runs["without network"]))
    assert runs["trained"] < runs["without network"], runs


@pytest.mark.parametrize("prec", ["FP64", "FP32"])
def test_learned_smoother_solve_with_fallback(trained, prec):
    """FPCG with the learned fine smoother reaches the tolerance and the FP64 method's
    discretisation error; the V-cycle/fallback counters are consistent. The comparison of
    iterations and fallbacks with the plain method is what the network gains (or not)."""
    w, _ = trained
    # tolerance 1e-11 so that the algebraic error stays below the discretisation error
    s = learned_problem(10, **{"PRECONDITIONER PRECISION": prec, "SOLVER TOLERANCE": 1e-11})
    plain = lpg.Elliptic(s).Run()
    e = lpg.Elliptic(s)
    e.set_learned_smoother(w, 0.5)
    r = e.Run()
    vc, fb = e.info("vcycles"), e.info("fallbacks")
    print("learned smoother (%s): iterations %d vs plain %d; V-cycles %d, fallbacks %d"
          % (prec, r["iterations"], plain["iterations"], vc, fb))
    assert r["converged"]
    assert abs(r["error"] - plain["error"]) <= 0.01 * plain["error"]
    assert vc >= r["iterations"] >= 1
    assert 0 <= fb <= vc
    # with every V-cycle forced onto the fallback, the result equals the plain method's
    e2 = lpg.Elliptic(s)
    e2.set_learned_smoother(w, 0.0)
    r2 = e2.Run()
    assert e2.info("fallbacks") == e2.info("vcycles")
    assert r2["iterations"] == plain["iterations"]
    # restoring the plain smoother
    e.set_learned_smoother(None)
    assert e.Run()["iterations"] == plain["iterations"]


_CHILD = r"""
import json, sys
import numpy as np
import libparanumal_gb300 as lpg
s = json.loads(sys.argv[1])
e = lpg.Elliptic(s)
e.set_learned_smoother(np.load(sys.argv[2]), 1e30)
r = e.Run(want_solution=True)
np.save(sys.argv[3], r["xL"][::97])
print(json.dumps(dict(iterations=r["iterations"], converged=r["converged"], fallbacks=e.info("fallbacks"))))
"""


@pytest.mark.parametrize("dims,bc", [((42, 42, 42), 1), ((6, 6, 6), 2), ((5, 5, 5), -1), ((42, 42, 42), -1)],
                         ids=["dirichlet_2chunks", "neumann", "periodic", "periodic_2chunks"])
def test_lattice_correction_matches_atomic_correction(trained_full, tmp_path, dims, bc):
    """The network's correction summed per lattice node (one thread per dof over its
    element copies, LPG_LEARNED_CORRECTION=lattice) against the per-element atomic sum
    (the default), through whole FPCG solves: equal iterations and solutions equal to 1e-9
    (the two differ only in the order the copies are added). The lattice path runs the
    network in chunks of whole element layers of at most 65,536 elements and sums each
    chunk's completed lattice planes before the next: the 42^3 boxes run 37 + 5 layers (the
    shared plane waits for the second chunk; plane 0 of the periodic box, shared by the
    last and first layers, comes last)."""
    import json
    import os
    import subprocess
    import sys
    w, _ = trained_full
    wf = tmp_path / "w.npy"
    np.save(wf, w)
    s = learned_problem(dims[0], **{"BOX NY": dims[1], "BOX NZ": dims[2], "BOX BOUNDARY FLAG": bc,
                                    "PRECONDITIONER PRECISION": "FP64", "MAXIMUM ITERATIONS": 60})
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    for mode in ("lattice", "atomic"):
        env = dict(os.environ, PYTHONPATH=root)
        env.pop("LPG_LEARNED_CORRECTION", None)
        if mode == "lattice":
            env["LPG_LEARNED_CORRECTION"] = "lattice"
        out = tmp_path / (mode + ".npy")
        p = subprocess.run([sys.executable, "-c", _CHILD, json.dumps(s), str(wf), str(out)], env=env, cwd=root,
                           capture_output=True, text=True, timeout=600)
        assert p.returncode == 0, p.stderr[-2000:]
        res[mode] = json.loads(p.stdout.strip().splitlines()[-1]), np.load(out)
    (a, xa), (b, xb) = res["lattice"], res["atomic"]
    assert a["converged"] and b["converged"] and a["fallbacks"] == b["fallbacks"] == 0, (a, b)
    assert a["iterations"] == b["iterations"], (a, b)
    assert rel_err(xa, xb) < 1e-9
