"""Benchmark of the C0 hex elliptic hot path on GB300.

Workload (one step = one pass of the hot path over one batch): one assembled
screened-Poisson operator application y = A q (matrix-free sum-factorised Ax with the
gather-scatter assembly fused) on a 64x64x64 jittered hex box, N = 7 (512 GLL nodes per
element, 134,217,728 local nodes, 89,314,623 assembled dofs), lambda = 1, full per-node
geometric factors (7 FP64 values/node), q ~ U[-1,1] keyed by global lattice node id
(seed 1). Inputs (9.5 GB) exceed the 129 MB L2, so no flush is needed between steps.

value   : local GDOF/s (Nlocal / step time), device-resident inputs
e2e     : same metric through the C ABI's host-buffer operator (lpg_elliptic_operator_host):
          page-locked q in, A q out, upload + operator + download inside each timed step
          (pipelined over element chunks), timed by host wall clock
roofline: algorithmic bytes Nlocal*60 + Nglobal*16 per application over the measured
          launch time, against the measured HBM copy bandwidth
variants: the FP32, BF16-geometry and double-FP32-word operators of the same mesh (the
          preconditioner levels' and the "+DF64" solves' outer operator), CUDA-event timed
solve   : the time-to-1e-8 workloads (library Run window, setup outside): FPCG + p-MG 7->3->1
          on the 80^3 jittered box (lambda=0, manufactured sine) per preconditioner and
          operator precision, and on the 112^3 jittered box (lognormal lambda, 16 Gaussian
          sources) plain FP64 against FP32+DF64 with and without the learned fine smoother
          trained in the same run
cpu_baseline: the oracle (CPU port of the reference algorithm) on a bounded sample
--impl reference: the reference's CPU implementation on all host threads: its own partial-Ax and
          gather kernels (translated from OKL, compiled with its release flags) on the full
          64^3 workload

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--nx 64] [--N 7]
Multi-GPU (torchrun): each rank runs an independent replica of the workload
("replicas only": this path is not sharded across GPUs here); value sums all ranks
over the max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Poisson time-to-1e-8: learned+mixed vs FP64 p-MG FPCG on GB300; Ax GDOF/s, %HBM"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--nx", type=int, default=64)
    ap.add_argument("--N", type=int, default=7)
    ap.add_argument("--cpu-sample-nx", type=int, default=32)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="skip the FP32/BF16GEO/DF64 operator variants")
    ap.add_argument("--no-solves", action="store_true", help="skip the time-to-1e-8 solve blocks")
    ap.add_argument("--e2e-steps", type=int, default=12)
    ap.add_argument("--prec", default="f64", choices=["f64", "df64", "f32", "bf16g"],
                    help="operator variant timed in the Ax workload (headline: f64)")
    ap.add_argument("--solve", action="store_true", help="time-to-tolerance of the p-MG FPCG solve instead")
    ap.add_argument("--solve-precs", default="FP64,FP32,BF16GEO,FP64+DF64,FP32+DF64,BF16GEO+DF64",
                    help="preconditioner precisions; P+DF64 also runs the FP64 operator in double-FP32 words")
    ap.add_argument("--solve-reps", type=int, default=2)
    ap.add_argument("--solver", default="FPCG", choices=["FPCG", "NBFPCG", "PCG"], help="LINEAR SOLVER of --solve")
    ap.add_argument("--precon", default="MULTIGRID", choices=["MULTIGRID", "SEMFEM", "PARALMOND", "JACOBI", "OAS"],
                    help="PRECONDITIONER of --solve")
    ap.add_argument("--disc", default="CONTINUOUS", choices=["CONTINUOUS", "IPDG"], help="DISCRETIZATION of --solve")
    ap.add_argument("--learned", action="store_true", help="learned-smoother training and solve comparison")
    ap.add_argument("--mlp", action="store_true", help="learned-smoother MLP inference (lpg_mlp_forward_bf16) timing")
    ap.add_argument("--ipdg", action="store_true", help="IPDG operator (gradient + Ax) throughput")
    ap.add_argument("--sequence", action="store_true", help="repeated solves with each initial-guess strategy")
    ap.add_argument("--heat", action="store_true", help="backward-Euler time steps with each initial-guess strategy")
    ap.add_argument("--learned-pair", action="store_true", help="one plain and one learned FP32+DF64 solve")
    ap.add_argument("--gmsh", action="store_true", help="operator throughput on Gmsh meshes (lattice and random "
                    "element order) against the box")
    ap.add_argument("--weights", default="", help="--learned-pair: network weights (.npy) instead of training")
    ap.add_argument("--save-weights", default="", help="--learned-pair: write the trained weights (.npy)")
    ap.add_argument("--train-nx", type=int, default=32)
    ap.add_argument("--train-samples", type=int, default=20000)
    ap.add_argument("--train-solves", type=int, default=8)
    ap.add_argument("--train-epochs", type=int, default=40)
    ap.add_argument("--rhs", default="sine", choices=["sine", "gauss"],
                    help="learned mode: manufactured sine data or 16 Gaussian sources (seed 3)")
    ap.add_argument("--learned-steps", type=int, default=2, help="LEARNED SMOOTHER STEPS of the learned solve")
    ap.add_argument("--train-pairs", default="MIXED", choices=["MIXED", "TRAJECTORY"],
                    help="SMOOTHER TRAINING PAIRS of the training problem")
    return ap.parse_args()


def settings(nx, N):
    return {"BOX NX": nx, "BOX NY": nx, "BOX NZ": nx, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
            "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": N, "LAMBDA": 1.0, "MESH JITTER": 0.1,
            "MESH JITTER SEED": 0, "LINEAR SOLVER": "FPCG", "PRECONDITIONER": "NONE"}


def workload_name(nx, N):
    return "screened-Poisson assembled Ax, %d^3 jittered hex box, N=%d, lambda=1, FP64 geometry" % (nx, N)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid):
        self.uuid = (uuid or "").lower()
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            row = [x.strip() for x in line.split(",")]
            if not self.uuid or self.uuid in row[0].lower():
                self.rows.append(row)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_model():
    """Host CPU model name and logical core count (lscpu, else /proc/cpuinfo)."""
    name = None
    try:
        for line in subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout.splitlines():
            if line.split(":")[0].strip() == "Model name":
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"model": name, "logical_cores": os.cpu_count()}


def cpu_baseline(nx_sample, N, budget_s=12.0, nthreads=0):
    """The reference's CPU operator on a bounded sample: its own ellipticPartialAxHex3D and
    ogs gather kernels (translated from OKL, compiled with its release flags) on the oracle's
    mesh arrays, all host threads; the oracle port when those kernels are not built."""
    from oracle import refimpl
    from oracle.oracle import Oracle, threads
    import numpy as np
    o = Oracle(settings(nx_sample, N))
    nl = o.Nlocal
    host = cpu_model()
    if refimpl.available():
        r = refimpl.RefOperator.from_oracle(o, 1.0)
        del o
        q = np.random.default_rng(1).uniform(-1, 1, r.Ngather)
        t1 = r.time(q, 1, nthreads)
        reps = max(1, int(budget_s / max(t1, 1e-3)))
        t = r.time(q, reps, nthreads)
        used = nthreads if nthreads > 0 else refimpl.threads()
        return {"value": nl * reps / t / 1e9, "unit": "GDOF/s", "cores": used, "kind": "reference",
                "host": host, "build": "reference kernels translated from OKL, gcc -O3 -fopenmp -ftree-vectorize",
                "sample": "%d^3-element jittered box, N=%d, lambda=1 (%d local nodes, working set %.2f GB), "
                          "%d operator applications (ellipticPartialAxHex3D x2 + ogs Gather), %d OpenMP threads"
                          % (nx_sample, N, nl, nl * 76 / 1e9, reps, used)}
    t1 = o.time_operator(1, nthreads)
    reps = max(1, int(budget_s / max(t1, 1e-3)))
    t = o.time_operator(reps, nthreads)
    used = nthreads if nthreads > 0 else threads()
    return {"value": nl * reps / t / 1e9, "unit": "GDOF/s", "cores": used, "kind": "port", "host": host,
            "sample": "%d^3-element jittered box, N=%d, lambda=1 (%d local nodes), %d operator "
                      "applications, %d OpenMP threads" % (nx_sample, N, nl, reps, used)}


def cpu_solve_sample(nx):
    """The oracle port's FP64 p-MG FPCG solve (7->3->1, Chebyshev 2, smoothed-aggregation AMG)
    on the nx^3 jittered box, N=7, lambda=0, sine data, all host threads: wall time of its Run
    (right-hand side, solve, norms; setup outside) and iterations. kind "port": the
    reference's own solver needs OCCA, MPI and LAPACK and is not built here."""
    from oracle.oracle import Oracle, threads
    t0 = time.time()
    o = Oracle(solve_settings(nx, 7, "FP64"))
    setup = time.time() - t0
    t0 = time.time()
    r = o.run()
    return {"seconds": time.time() - t0, "iterations": r["iterations"], "error_vs_manufactured": r["error"],
            "setup_seconds": setup, "cores": threads(), "kind": "port", "host": cpu_model()}


def run_reference(a):
    """The reference's CPU implementation of the headline workload (the 64^3, N=7 operator,
    same config as the GPU arm): its own partial-Ax and gather kernels on all host threads,
    W warm-up and K timed applications, one per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    from oracle import refimpl
    from oracle.oracle import Oracle
    if not refimpl.available():
        base = cpu_baseline(a.cpu_sample_nx, a.N, budget_s=max(5.0, 2.0 * a.steps))
        value, cfg = base["value"], {"workload": workload_name(a.nx, a.N), "same_config": False}
    else:
        t0 = time.time()
        o = Oracle(settings(a.nx, a.N))
        r = refimpl.RefOperator.from_oracle(o, 1.0)
        nl = o.Nlocal
        del o
        setup = time.time() - t0
        q = np.random.default_rng(1).uniform(-1, 1, r.Ngather)
        r.time(q, max(1, a.warmup) - 1)
        t = r.time(q, a.steps)   # one more warm-up application inside, then K timed
        used = refimpl.threads()
        value = nl * a.steps / t / 1e9
        cfg = {"workload": workload_name(a.nx, a.N), "same_config": True}
        base = {"value": value, "unit": "GDOF/s", "cores": used, "kind": "reference", "host": cpu_model(),
                "build": "reference kernels translated from OKL, gcc -O3 -fopenmp -ftree-vectorize",
                "sample": "full workload: %d^3-element jittered box, N=%d, lambda=1 (%d local nodes), %d timed "
                          "operator applications (ellipticPartialAxHex3D x2 + ogs Gather), %d OpenMP threads"
                          % (a.nx, a.N, nl, a.steps, used),
                "ms_per_step": t * 1e3 / a.steps, "setup_seconds": setup}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GDOF/s",
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic", "config": cfg,
            "cpu_baseline": base, "vs_baseline": None,
            "e2e": {"value": value, "unit": "GDOF/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def max_over_ranks(ms, dist=None, device="cpu"):
    """Step time of the whole job: the slowest rank's (replicas run concurrently)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)


def job_throughput(units_per_rank, world, ms):
    """Whole-job GDOF/s: units processed by all ranks over the max-over-ranks step time."""
    return world * units_per_rank / (ms * 1e-3) / 1e9


def solve_settings(nx, N, prec, degrees="7,3,1", lam=0.0, **extra):
    d = {"BOX NX": nx, "BOX NY": nx, "BOX NZ": nx, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
         "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": N, "LAMBDA": lam, "MESH JITTER": 0.1,
         "MESH JITTER SEED": 0, "LINEAR SOLVER": "FPCG", "PRECONDITIONER": "MULTIGRID",
         "MULTIGRID DEGREES": degrees, "MULTIGRID SMOOTHER": "CHEBYSHEV",
         "MULTIGRID CHEBYSHEV DEGREE": 2, "PARALMOND AGGREGATION": "SMOOTHED",
         "PRECONDITIONER PRECISION": prec}
    d.update(extra)
    return d


def solve_variants(nx, variants, reps, law=None, learned_w=None, threshold=0.5, x_ref_name="FP64", **common):
    """Time-to-1e-8 of FPCG + p-MG (7->3->1, Chebyshev 2, smoothed-aggregation AMG on N=1) on
    an nx^3 jittered box, N=7, for each variant name: "P" or "P+DF64" (preconditioner
    precision P in FP64 / FP32 / BF16GEO; +DF64: every FP64 operator application in
    double-FP32 words), "learned+P[+DF64]" (the trained fine smoother in place of the
    fine-level Chebyshev, with per-V-cycle fallback). The solve window is the library's
    elliptic_t::Run window (after the right-hand side, to after scatter and norms;
    ellipticRun.cpp:190-221); setup is outside it. Each result: best of `reps` Runs, with
    iterations, fine-level operator applications, V-cycles and fallbacks, error against the
    manufactured solution (sine data) and the relative 2-norm difference of the local
    solution from variant `x_ref_name`'s (listed first)."""
    import numpy as np
    import torch
    import libparanumal_gb300 as lpg
    res, xref = {}, None
    for name in variants:
        learned = name.startswith("learned+")
        base, _, op = name[len("learned+") if learned else 0:].partition("+")
        extra = dict(law or {}, **common)
        if op:
            extra["OPERATOR PRECISION"] = op
        t0 = time.time()
        e = lpg.Elliptic(solve_settings(nx, 7, base, **extra))
        if learned:
            e.set_learned_smoother(learned_w, threshold)
        setup = time.time() - t0
        runs, ops = [], []
        for rep in range(reps):
            n0 = e.info("operator_applications")
            runs.append(e.Run(want_solution=(rep == 0)))
            ops.append(e.info("operator_applications") - n0)
        xL = runs[0].pop("xL")
        ib = min(range(reps), key=lambda i: runs[i]["solve_seconds"])
        best = runs[ib]
        r = {"solve_seconds": best["solve_seconds"], "solve_seconds_all": [x["solve_seconds"] for x in runs],
             "iterations": best["iterations"], "converged": best["converged"], "fine_ax": ops[ib],
             "setup_seconds": setup, "nglobal": e.Nglobal}
        if learned:
            r["vcycles"], r["fallbacks"] = e.info("vcycles"), e.info("fallbacks")
        if best["error"] >= 0:
            r["error_vs_manufactured"] = best["error"]
        if name == x_ref_name:
            xref = xL
        elif xref is not None:
            r["rel_diff_vs_%s_solution" % x_ref_name.lower()] = float(np.linalg.norm(xL - xref) / np.linalg.norm(xref))
        del xL
        res[name] = r
        e.close()
        torch.cuda.empty_cache()
    return res


def train_learned(train_nx=32, samples=20000, solves=8, epochs=40, pairs="MIXED"):
    """Learned fine smoother trained on the GPU by the library's own kernels from the plain
    p-MG FPCG of a train_nx^3 jittered box (N=7, lognormal lambda, random Gaussian-bump
    right-hand sides). Returns (weights, summary)."""
    import libparanumal_gb300 as lpg
    law = {"LAMBDA": 1.0, "LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2, "SMOOTHER TRAINING PAIRS": pairs}
    t0 = time.time()
    w, hist = lpg.train_smoother(solve_settings(train_nx, 7, "FP64", **law), nsolves=solves,
                                 samples_per_solve=samples // solves, epochs=epochs, batch=250, lr=1e-3, seed=7)
    return w, {"train_nx": train_nx, "train_samples": samples, "train_epochs": epochs, "train_pairs": pairs,
               "train_seconds": time.time() - t0, "loss_first": float(hist[0]), "loss_last": float(hist[-1])}


def run_solves(a):
    """Time-to-1e-8 of FPCG + p-MG (7->3->1, Chebyshev 2, smoothed-aggregation AMG on N=1)
    on a jittered box with the manufactured sine solution, for each preconditioner
    precision. One JSON line; setup is outside the timed window (ellipticRun.cpp:190-210).
    fine_ax counts the fine-level operator applications of the Run (right-hand-side
    lifting, outer Krylov and smoother), in any precision; rel_diff_vs_fp64_solution is the
    relative 2-norm difference of the local solution from the FP64 method's (when FP64 is
    listed first)."""
    import numpy as np
    import libparanumal_gb300 as lpg
    import __graft_entry__ as g
    g.build()
    res = {}
    x64 = None   # local solution of the FP64 method (when FP64 is the first precision)
    for prec in a.solve_precs.split(","):
        t0 = time.time()
        # "P+DF64": preconditioner precision P, FP64 operator applications in double-FP32 words
        base, _, op = prec.partition("+")
        extra = {"OPERATOR PRECISION": op} if op else {}
        extra["LINEAR SOLVER"] = a.solver
        extra["PRECONDITIONER"] = a.precon
        extra["DISCRETIZATION"] = a.disc
        e = lpg.Elliptic(solve_settings(a.nx, a.N, base, **extra))
        setup = time.time() - t0
        runs, ops = [], []
        for rep in range(a.solve_reps):
            n0 = e.info("operator_applications")
            # the first Run also returns the local solution (downloaded after the library's
            # timed window) for the comparison with the FP64 solution
            runs.append(e.Run(want_solution=(rep == 0)))
            ops.append(e.info("operator_applications") - n0)
        xL = runs[0].pop("xL")
        for r in runs[1:]:
            r.pop("xL", None)
        if prec == "FP64":
            x64 = xL
        ibest = min(range(len(runs)), key=lambda i: runs[i]["solve_seconds"])
        best = runs[ibest]
        res[prec] = {"solve_seconds": best["solve_seconds"], "iterations": best["iterations"],
                     "error_vs_manufactured": best["error"], "norm": best["norm"],
                     "converged": best["converged"], "setup_seconds": setup,
                     "fine_ax": ops[ibest], "fine_ax_per_iteration": ops[ibest] / max(1, best["iterations"]),
                     "rel_diff_vs_fp64_solution": (None if x64 is None else
                                                   float(np.linalg.norm(xL - x64) / np.linalg.norm(x64))),
                     "mg_plevels": e.info("mg_plevels"), "amg_levels": e.info("mg_amglevels"),
                     "coarse_n": e.info("coarse_n"), "nglobal": e.Nglobal}
        e.close()
    pre = "p-MG 7->3->1" if a.precon == "MULTIGRID" else a.precon
    print(json.dumps({"workload": "%s + %s time-to-1e-8, %d^3 jittered hex, N=%d, lambda=0, %s"
                      % (a.solver, pre, a.nx, a.N, a.disc), "results": res}), flush=True)


def run_learned(a):
    """Learned fine smoother (variable-coefficient screened Poisson): train on (residual, exact error)
    pairs of the plain p-MG FPCG on a 32^3 jittered box with random Gaussian-bump
    right-hand sides (lognormal lambda, N=7), then solve the nx^3 problem (manufactured
    sine data, or with --rhs gauss 16 Gaussian sources, seed 3) with the plain FP64, the
    FP32 and the learned+FP32 preconditioners, the last two also with the FP64 operator
    applications in double-FP32 words (+DF64). Each result carries the relative 2-norm
    difference of its solution from the FP64 method's. One JSON line."""
    import torch
    import libparanumal_gb300 as lpg
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)
    law = {"LAMBDA": 1.0, "LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2}
    rhs = {} if a.rhs == "sine" else {"RHS FIELD": "GAUSSIAN SOURCES", "RHS SEED": 3, "RHS SOURCES": 16}
    tlaw = dict(law, **{"SMOOTHER TRAINING PAIRS": a.train_pairs})
    t0 = time.time()
    w, hist = lpg.train_smoother(solve_settings(a.train_nx, 7, "FP64", **tlaw), nsolves=a.train_solves,
                                 samples_per_solve=a.train_samples // a.train_solves, epochs=a.train_epochs,
                                 batch=250, lr=1e-3, seed=7)
    t_train = time.time() - t0
    out = {"workload": "learned fine smoother: train %d^3, solve %d^3 jittered hex N=7 lognormal lambda, %s rhs"
                       % (a.train_nx, a.nx, "manufactured sine" if a.rhs == "sine" else "16 Gaussian sources"),
           "train_seconds": t_train, "train_samples": a.train_samples, "train_epochs": a.train_epochs,
           "train_pairs": a.train_pairs, "learned_steps": a.learned_steps,
           "loss_first": float(hist[0]), "loss_last": float(hist[-1]), "results": {}}
    x64 = None
    variants = (("FP64", "FP64", False, False), ("FP32", "FP32", False, False), ("learned+FP32", "FP32", True, False),
                ("FP32+DF64", "FP32", False, True), ("learned+FP32+DF64", "FP32", True, True))
    for name, prec, learned, dw in variants:
        t1 = time.time()
        extra = {"LEARNED SMOOTHER STEPS": a.learned_steps} if learned else {}
        if dw:
            extra["OPERATOR PRECISION"] = "DF64"
        e = lpg.Elliptic(solve_settings(a.nx, 7, prec, **law, **rhs, **extra))
        setup = time.time() - t1
        if learned:
            e.set_learned_smoother(w, 0.5)
        runs = [e.Run() for _ in range(a.solve_reps)]
        best = min(runs, key=lambda r: r["solve_seconds"])
        res = {"solve_seconds": best["solve_seconds"], "iterations": best["iterations"],
               "converged": best["converged"], "vcycles": e.info("vcycles"), "fallbacks": e.info("fallbacks"),
               "setup_seconds": setup, "nglobal": e.Nglobal}
        if a.rhs == "sine":
            res["error_vs_manufactured"] = best["error"]
        # the assembled solution of the same solve, compared with the FP64 method's
        r = torch.empty(e.Nglobal, dtype=torch.float64, device="cuda")
        x = torch.zeros_like(r)
        e.rhs(r)
        e.Solve(x, r, tol=1e-8)
        torch.cuda.synchronize()
        if x64 is None:
            x64 = x
        else:
            res["rel_diff_vs_fp64_solution"] = float((x - x64).norm() / x64.norm())
            del x
        del r
        out["results"][name] = res
        e.close()
        torch.cuda.empty_cache()
    print(json.dumps(out), flush=True)


def run_learned_pair(a):
    """One plain FP32+DF64 Run and one learned+FP32+DF64 Run (2 steps per side, fallback
    threshold 0.5) on the nx^3 jittered box, N=7, lognormal lambda, sine data -- the pair
    whose ncu launch list gives the per-component cost table. Weights: --weights PATH (a
    .npy written by --save-weights), else trained in the run on 32^3 (20,000 pairs, 40
    epochs) and written to --save-weights when given. One JSON line."""
    import numpy as np
    import torch
    import libparanumal_gb300 as lpg
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)
    if a.weights:
        w, train = np.load(a.weights), {"loaded": a.weights}
    else:
        w, train = train_learned()
        if a.save_weights:
            np.save(a.save_weights, w)
    law = {"LAMBDA": 1.0, "LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2, "OPERATOR PRECISION": "DF64"}
    out = {"workload": "plain vs learned FP32+DF64 FPCG + p-MG, %d^3 jittered hex, N=7, lognormal lambda, sine"
                       % a.nx, "training": train}
    for name, learned in (("FP32+DF64", False), ("learned+FP32+DF64", True)):
        e = lpg.Elliptic(solve_settings(a.nx, 7, "FP32", **law))
        if learned:
            e.set_learned_smoother(w, 0.5)
        r = e.Run()
        out[name] = {"iterations": r["iterations"], "solve_seconds": r["solve_seconds"], "error": r["error"],
                     "vcycles": e.info("vcycles"), "fallbacks": e.info("fallbacks")}
        e.close()
    print(json.dumps(out), flush=True)


def run_mlp(a):
    """Inference of the learned smoother's MLP through lpg_mlp_forward_bf16 (weights
    converted to BF16 inside each call) on 65,536 and 262,144 random rows: 2 warm-up and
    5 timed calls each. One JSON line; the kernel alone is seen in an ncu launch list."""
    import numpy as np
    import torch
    import libparanumal_gb300 as lpg
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)
    L = lpg.lib()
    gen = torch.Generator(device="cuda").manual_seed(3)
    theta = (torch.rand(int(L.lpg_mlp_param_count()), device="cuda", generator=gen) - 0.5) * 0.1
    res = {}
    for B in (65536, 262144):
        X = torch.randn(B, 896, device="cuda")
        Y = torch.empty(B, 512, device="cuda")
        for _ in range(2):
            lpg.check(L.lpg_mlp_forward_bf16(theta.data_ptr(), B, X.data_ptr(), Y.data_ptr(), None))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            lpg.check(L.lpg_mlp_forward_bf16(theta.data_ptr(), B, X.data_ptr(), Y.data_ptr(), None))
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 5
        res[str(B)] = {"ms_per_call_incl_weight_conversion": ms, "tflops": B * 492800 * 2 / ms / 1e9}
    print(json.dumps({"workload": "learned-smoother MLP inference, BF16 tensor cores", "results": res}), flush=True)


def run_sequence(a):
    """Repeated solves as a time stepper makes them (linearSolver_t with an initial-guess
    strategy, initialGuess.cpp): K right-hand sides r(t) = sum_k exp(-(t/1.5 - k)^2 / 2) r_k
    blending 10 Gaussian-source fields (16 sources each, seeds 3..12) of the same nx^3
    jittered box, N=7, so the data drift smoothly through a 10-dimensional space; each solve
    to 1e-8 relative to ||r|| (ABS/REL-RHS-2NORM) by FPCG + p-MG with the FP32 preconditioner
    and double-FP32 outer operator, for each INITIAL GUESS STRATEGY. Per strategy: mean
    iterations and wall time per solve over the last K-3 steps. One JSON line."""
    import math
    import torch
    import libparanumal_gb300 as lpg
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)
    base = solve_settings(a.nx, 7, "FP32", **{"OPERATOR PRECISION": "DF64",
                                              "LINEAR SOLVER STOPPING CRITERION": "ABS/REL-RHS-2NORM"})
    parts = []
    for seed in range(3, 13):
        e = lpg.Elliptic(dict(base, **{"RHS FIELD": "GAUSSIAN SOURCES", "RHS SEED": seed, "RHS SOURCES": 16}))
        r = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
        e.rhs(r)
        parts.append(r)
        e.close()
    strategies = {"ZERO": {}, "CLASSIC": {"INITIAL GUESS HISTORY SPACE DIMENSION": 8},
                  "QR": {"INITIAL GUESS HISTORY SPACE DIMENSION": 8},
                  "EXTRAP": {"INITIAL GUESS HISTORY SPACE DIMENSION": 4, "INITIAL GUESS EXTRAP DEGREE": 2,
                             "INITIAL GUESS EXTRAP COEFFS METHOD": "CPQR"}}
    res = {}
    K = max(a.steps, 6)
    for name, over in strategies.items():
        e = lpg.Elliptic(dict(base, **{"INITIAL GUESS STRATEGY": name}, **over))
        x = torch.zeros_like(parts[0])
        its, secs = [], []
        for t in range(K):
            rhs = sum(math.exp(-0.5 * (t / 1.5 - k) ** 2) * pk for k, pk in enumerate(parts))
            torch.cuda.synchronize()
            t0 = time.time()
            its.append(e.Solve(x, rhs, tol=1e-8))
            torch.cuda.synchronize()
            secs.append(time.time() - t0)
        e.close()
        res[name] = {"iterations": its, "mean_iterations_after_3": sum(its[3:]) / (K - 3),
                     "mean_seconds_after_3": sum(secs[3:]) / (K - 3)}
    print(json.dumps({"workload": "%d repeated solves, r(t) blending 10 Gaussian-source fields, %d^3 jittered "
                                  "hex, N=7, FPCG + p-MG (FP32+DF64), tol 1e-8 of ||r||" % (K, a.nx),
                      "results": res}), flush=True)


def run_heat(a):
    """A time-stepping caller (the ins velocity-solve pattern, insVelocitySolve.cpp:30-100):
    backward Euler for u_t = Laplacian u on the nx^3 jittered box, N=7, Dirichlet,
    (lambda M + K) u_{n+1} = lambda M u_n with lambda = 1/dt = 10, u_0 = the steady
    solution for 16 Gaussian sources (seed 3); each step forms lambda M u_n through lpg_elliptic_mass,
    scales it to unit norm and solves to 1e-8 of ||r|| with FPCG + p-MG (FP32
    preconditioner, double-FP32 outer operator) and one INITIAL GUESS STRATEGY. Per
    strategy: iterations per step and mean wall time per step (mass product + solve) over
    the steps after the first 3. One JSON line."""
    import torch
    import libparanumal_gb300 as lpg
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)
    lam = 10.0
    base = solve_settings(a.nx, 7, "FP32", lam=lam, **{"OPERATOR PRECISION": "DF64",
                                                       "LINEAR SOLVER STOPPING CRITERION": "ABS/REL-RHS-2NORM"})
    strategies = {"ZERO": {}, "CLASSIC": {"INITIAL GUESS HISTORY SPACE DIMENSION": 8},
                  "QR": {"INITIAL GUESS HISTORY SPACE DIMENSION": 8},
                  "EXTRAP": {"INITIAL GUESS HISTORY SPACE DIMENSION": 4, "INITIAL GUESS EXTRAP DEGREE": 2,
                             "INITIAL GUESS EXTRAP COEFFS METHOD": "CPQR"}}
    K = max(a.steps, 6)
    res = {}
    for name, over in strategies.items():
        e = lpg.Elliptic(dict(base, **{"INITIAL GUESS STRATEGY": name}, **over))
        # u_0: the steady solution for 16 Gaussian sources (seed 3), from one solve: many
        # modes, each decaying at its own rate
        steady = lpg.Elliptic(dict(base, **{"INITIAL GUESS STRATEGY": "ZERO", "RHS FIELD": "GAUSSIAN SOURCES",
                                            "RHS SEED": 3, "RHS SOURCES": 16}))
        b0 = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
        steady.rhs(b0)
        u = torch.zeros_like(b0)
        steady.Solve(u, b0, tol=1e-10)
        steady.close()
        Mu, x = torch.empty_like(u), torch.zeros_like(u)
        its, secs = [], []
        for _ in range(K):
            torch.cuda.synchronize()
            t0 = time.time()
            e.mass(u, Mu)
            # unit-norm right-hand side (the system is linear: u_{n+1} = ||b_n|| x_n), so the
            # tolerance means the same at every step while the field decays
            nb = float(Mu.norm()) * lam
            Mu.mul_(lam / nb)
            its.append(e.Solve(x, Mu, tol=1e-8))
            torch.mul(x, nb, out=u)
            torch.cuda.synchronize()
            secs.append(time.time() - t0)
        e.close()
        del u, Mu, x, b0
        torch.cuda.empty_cache()
        res[name] = {"iterations": its, "mean_iterations_after_3": sum(its[3:]) / (K - 3),
                     "mean_seconds_after_3": sum(secs[3:]) / (K - 3)}
    print(json.dumps({"workload": "backward-Euler heat steps (lambda = 1/dt = %g), %d^3 jittered hex, N=7, FPCG + "
                                  "p-MG (FP32+DF64), tol 1e-8 of ||r||, %d steps" % (lam, a.nx, K),
                      "results": res}), flush=True)


def run_ipdg(a):
    """IPDG operator throughput (DISCRETIZATION = IPDG, gradient + interior-penalty Ax) on an
    nx^3 jittered Dirichlet box at degree N: W warm-up and K timed applications on device
    vectors larger than L2, CUDA events on the library's stream, for the FP64 operator, the
    same operator in double-FP32 words (DF64) and the FP32 operator of the preconditioner
    levels. One JSON line with the algorithmic bytes of the two kernels per node and the HBM
    fraction they reach."""
    import torch
    import libparanumal_gb300 as lpg
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)
    s = dict(settings(a.nx, a.N), **{"DISCRETIZATION": "IPDG", "PRECONDITIONER": "NONE", "MESH JITTER": 0.1})
    e = lpg.Elliptic(s)
    n = e.Nglobal
    gen = torch.Generator(device="cuda").manual_seed(1)
    q = torch.rand(n, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
    Aq = torch.empty_like(q)
    stream = e.device_ptr("stream")
    torch_stream = torch.cuda.ExternalStream(stream)
    for _ in range(max(3, a.warmup)):
        e.Operator(q, Aq)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(torch_stream)
    for _ in range(a.steps):
        e.Operator(q, Aq)
    e1.record(torch_stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    # FP32 operator of the preconditioner levels (FP32 copies of vgeo/sgeo, float4 gradients)
    q32, Aq32 = q.float(), torch.empty(n, dtype=torch.float32, device="cuda")
    for _ in range(max(3, a.warmup)):
        e.OperatorF32(q32, Aq32)
    torch.cuda.synchronize()
    e0.record(torch_stream)
    for _ in range(a.steps):
        e.OperatorF32(q32, Aq32)
    e1.record(torch_stream)
    torch.cuda.synchronize()
    ms32 = e0.elapsed_time(e1) / a.steps
    # the FP64 operator in double-FP32 words (OPERATOR PRECISION DF64)
    for _ in range(max(3, a.warmup)):
        e.OperatorDF64(q, Aq)
    torch.cuda.synchronize()
    e0.record(torch_stream)
    for _ in range(a.steps):
        e.OperatorDF64(q, Aq)
    e1.record(torch_stream)
    torch.cuda.synchronize()
    msdw = e0.elapsed_time(e1) / a.steps
    Nq = a.N + 1
    Np, Nfp = Nq ** 3, Nq * Nq
    hbm, hbm_src = measured_peaks()

    def bytes_per_dof(w):                          # w = bytes of one value
        face = 6 * Nfp / Np * (5 * w + 4 + 4 * w)  # sgeo + vmapP + neighbour gradient per face node
        return (w + 10 * w + 4 * w) + (4 * w + 10 * w + face + w)   # gradient pass + Ax pass

    def line(ms_, w):
        achieved = n * bytes_per_dof(w) / (ms_ * 1e-3) / 1e9
        return {"value": n / (ms_ * 1e-3) / 1e9, "unit": "GDOF/s", "ms_per_apply": ms_,
                "bytes_per_dof": bytes_per_dof(w),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "peak_source": hbm_src,
                             "frac": achieved / hbm, "unit": "GB/s"}}

    out = {"workload": "IPDG operator (gradient + Ax), %d^3 jittered hex, N=%d" % (a.nx, a.N),
           "metric": "ipdg_operator_gdofs", "ndofs": n}
    out.update(line(ms, 8))
    out["df64"] = line(msdw, 8)
    out["fp32"] = line(ms32, 4)
    print(json.dumps(out), flush=True)


def run_gmsh(a):
    """Operator throughput on hexahedral Gmsh meshes against the box: the a.nx^3 box written
    as a Gmsh 2.2 file (shuffled node tags, randomly rotated element vertex lists, jittered
    interior vertices), once with the hexahedra in lattice order and once in random order
    (an element order without spatial locality). The FP64 operator and its FP32 /
    BF16-geometry / double-word variants are timed on each (CUDA events, W warm-up and K
    timed applications)."""
    import tempfile
    import torch
    import libparanumal_gb300 as lpg
    import __graft_entry__ as g
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from gmsh_mesh import write_box
    g.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    res = {}
    with tempfile.TemporaryDirectory() as tmp:
        meshes = {"box": None,
                  "gmsh_lattice_order": dict(shuffle_seed=1, rotate_seed=2, jitter=0.1, jitter_seed=3),
                  "gmsh_random_order": dict(shuffle_seed=1, rotate_seed=2, jitter=0.1, jitter_seed=3,
                                            element_seed=4)}
        for name, kw in meshes.items():
            st = settings(a.nx, a.N)
            if kw is not None:
                path = write_box(os.path.join(tmp, name + ".msh"), a.nx, a.nx, a.nx, **kw)
                st = {k: v for k, v in st.items() if not k.startswith("BOX N") and not k.startswith("MESH JITTER")}
                st["MESH FILE"] = path
            e = lpg.Elliptic(st)
            q = (torch.rand(e.Nglobal, dtype=torch.float64, device="cuda", generator=torch.Generator(
                device="cuda").manual_seed(1)) * 2 - 1)
            y = torch.empty_like(q)
            for _ in range(max(3, a.warmup)):
                e.Operator(q, y, sp)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(a.steps):
                e.Operator(q, y, sp)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / a.steps
            v = time_operator_variants(e, q, a, stream, sp)
            res[name] = {"elements": e.info("nelements"), "assembled_dofs": e.Nglobal,
                         "fp64_ms_per_apply": ms, "fp64_gdofs_local": e.Nlocal / (ms * 1e-3) / 1e9,
                         "variants_ms_per_apply": {k: x["ms_per_apply"] for k, x in v.items()}}
            del e
            torch.cuda.empty_cache()
    print(json.dumps({"workload": "operator on %d^3 hexahedra, N=%d, lambda=1: box against Gmsh files" % (a.nx, a.N),
                      "results": res}), flush=True)


def time_operator_variants(e, q, a, stream, sp):
    """CUDA-event time per application of the FP32, BF16-geometry and double-FP32-word
    operators of object e (the same mesh as the headline FP64 workload), with their
    algorithmic bytes per application and the achieved bandwidth."""
    import torch
    Nl, Ng = e.Nlocal, e.Nglobal
    q32 = q.float()
    y32 = torch.empty_like(q32)
    y64 = torch.empty_like(q)
    cases = {"fp32": (lambda: e.OperatorF32(q32, y32, False, sp), Nl * 32 + Ng * 8, "FP32 vectors and geometry"),
             "bf16geo": (lambda: e.OperatorF32(q32, y32, True, sp), Nl * 18 + Ng * 8,
                         "BF16 geometric factors, FP32 vectors and arithmetic"),
             "df64": (lambda: e.OperatorDF64(q, y64, sp), Nl * 60 + Ng * 16,
                      "FP64 in/out, double-FP32-word arithmetic (FP64 accuracy)")}
    out = {}
    for name, (op, nbytes, what) in cases.items():
        for _ in range(max(3, a.warmup)):
            op()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.steps):
            op()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / a.steps
        out[name] = {"arith": what, "ms_per_apply": ms, "gdofs_local": Nl / (ms * 1e-3) / 1e9,
                     "roofline": {"bound": "hbm", "unit": "GB/s", "algorithmic_bytes_per_launch": nbytes,
                                  "achieved": nbytes / (ms * 1e-3) / 1e9}}
    return out


def solve_blocks(a):
    """The time-to-1e-8 workloads, each variant timed in the library's Run window:
    (1) mixed precision: 80^3 jittered box, N=7, lambda=0, manufactured sine data, FPCG to
        1e-8 with p-MG 7->3->1 (Chebyshev 2, smoothed-aggregation AMG on N=1) whose levels
        run in FP64, FP32 or BF16-geometry FP32, the outer operator in FP64 or double-FP32 words;
    (2) learned + mixed precision at scale: 112^3 jittered box, N=7, lognormal lambda (seed 2),
        16 Gaussian sources (seed 3): plain FP64 p-MG against FP32+DF64 with and without the
        learned fine smoother, trained in this run on 32^3 (20,000 pairs, 40 epochs)."""
    t0 = time.time()
    out = {}
    out["mixed_80cubed"] = {
        "workload": "FPCG + p-MG 7->3->1 time-to-1e-8, 80^3 jittered hex, N=7, lambda=0, manufactured sine",
        "results": solve_variants(80, ["FP64", "FP32", "FP32+DF64", "BF16GEO+DF64"], a.solve_reps)}
    # the same solve at a size the CPU finishes in seconds: the oracle port's FP64 p-MG FPCG
    # (a restatement of the reference's solver, which cannot be built here) on all host
    # threads beside the GPU variants on the same 32^3 problem
    out["same_size_32cubed"] = {
        "workload": "FPCG + p-MG 7->3->1 time-to-1e-8, 32^3 jittered hex, N=7, lambda=0, manufactured sine",
        "cpu_port": cpu_solve_sample(32),
        "gpu": solve_variants(32, ["FP64", "FP32+DF64"], a.solve_reps)}
    w, train = train_learned()
    law = {"LAMBDA": 1.0, "LAMBDA FIELD": "LOGNORMAL", "LAMBDA SEED": 2,
           "RHS FIELD": "GAUSSIAN SOURCES", "RHS SEED": 3, "RHS SOURCES": 16}
    res = solve_variants(112, ["FP64", "FP32+DF64", "learned+FP32+DF64"], a.solve_reps, law=law, learned_w=w,
                         **{"LEARNED SMOOTHER STEPS": 2})
    t64 = res["FP64"]["solve_seconds"]
    out["learned_112cubed"] = {
        "workload": "FPCG + p-MG 7->3->1 time-to-1e-8, 112^3 jittered hex, N=7, lognormal lambda, 16 Gaussian sources",
        "training": train, "results": res,
        "speedup_vs_fp64": {k: t64 / v["solve_seconds"] for k, v in res.items()}}
    out["wall_seconds"] = time.time() - t0
    return out


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    if a.solve:
        return run_solves(a)
    if a.learned:
        return run_learned(a)
    if a.mlp:
        return run_mlp(a)
    if a.ipdg:
        return run_ipdg(a)
    if a.sequence:
        return run_sequence(a)
    if a.heat:
        return run_heat(a)
    if a.learned_pair:
        return run_learned_pair(a)
    if a.gmsh:
        return run_gmsh(a)
    import numpy as np
    import torch
    import libparanumal_gb300 as lpg

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import __graft_entry__ as g
    if rank == 0:
        g.build()
    if dist:
        dist.barrier()
    lpg.lib()

    t_setup = time.time()
    st = settings(a.nx, a.N)
    if a.prec == "df64":
        st["OPERATOR PRECISION"] = "DF64"   # FP64 operator interface, double-FP32 arithmetic
    e = lpg.Elliptic(st)
    Nl, Ng = e.Nlocal, e.Nglobal
    q = torch.empty(Ng, dtype=torch.float64, device="cuda")
    Aq = torch.empty_like(q)
    e.random_vector(q, 1)
    torch.cuda.synchronize()
    t_setup = time.time() - t_setup
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    if a.prec in ("f64", "df64"):
        qin, yout = q, Aq

        def op():
            e.Operator(qin, yout, sp)
    else:
        qin = q.float()
        yout = torch.empty_like(qin)
        bf = a.prec == "bf16g"

        def op():
            e.OperatorF32(qin, yout, bf, sp)

    for _ in range(a.warmup):
        op()
    torch.cuda.synchronize()

    try:
        uuid = str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        uuid = ""
    clocks = ClockSampler(uuid)
    clocks.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(a.steps):
        starts[k].record(stream)
        op()
        ends[k].record(stream)
    t1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_ms = t0.elapsed_time(t1)
    per = [s.elapsed_time(x) for s, x in zip(starts, ends)]
    launch_ms = statistics.mean(per)
    ms = max_over_ranks(total_ms / a.steps, dist, "cuda")

    # end to end through the C ABI's host-buffer operator: page-locked q in, Aq out; each
    # call uploads q, applies the operator and downloads Aq (pipelined over element
    # chunks) and returns with Aq filled, so host wall time is the step time
    prec_name = {"f64": "FP64", "df64": "FP64", "f32": "FP32", "bf16g": "BF16GEO"}[a.prec]
    qh = qin.cpu().pin_memory()
    yh = torch.empty_like(qh).pin_memory()
    for _ in range(3):
        e.OperatorHost(qh, yh, prec_name)
    dev_out = yout.cpu()
    e2e_check = float((yh - dev_out).abs().max() / dev_out.abs().max())
    if e2e_check > (1e-12 if a.prec in ("f64", "df64") else 1e-5):
        raise RuntimeError("host-buffer operator differs from the device operator: %g" % e2e_check)
    if dist:
        dist.barrier()
    t_e2e = time.perf_counter()
    for _ in range(a.e2e_steps):
        e.OperatorHost(qh, yh, prec_name)
    e2e_ms = max_over_ranks((time.perf_counter() - t_e2e) * 1e3 / a.e2e_steps, dist, "cuda")

    # the other operator variants of the same object, timed the same way (CUDA events on the
    # launching stream, inputs far above L2): the FP32 and BF16-geometry operators of the
    # preconditioner levels (the fine-level smoother and residual operator) and the FP64
    # operator in double-FP32 words (the outer operator of the "+DF64" solves)
    variants = {}
    if a.prec == "f64" and world == 1 and not a.no_variants:
        variants = time_operator_variants(e, q, a, stream, sp)

    if rank != 0:
        dist.destroy_process_group()
        return
    peak, peak_kind = measured_peaks()
    alg_bytes = {"f64": Nl * 60 + Ng * 16, "df64": Nl * 60 + Ng * 16, "f32": Nl * 32 + Ng * 8,
                 "bf16g": Nl * 18 + Ng * 8}[a.prec]
    flops = (12 * (a.N + 1) + 18) * Nl
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    # DRAM bytes per launch: the ncu capture's bytes per element (24^3 case, traffic
    # grows with the element count) times this workload's elements
    traffic = None
    tfile = os.path.join(ROOT, "profiles", {"f64": "ax_hex_f64_64cubed_N7.txt",
                                            "f32": "ax_hex_staged_f32_24cubed_N7_full.txt",
                                            "df64": "ax_hex_dw_24cubed_N7_full.txt",
                                            "bf16g": "ax_hex_staged_bf16g_24cubed_N7_full.txt"}[a.prec])
    if os.path.exists(tfile) and a.N == 7:
        for line in open(tfile):
            if line.startswith("traffic_bytes_per_element:"):
                traffic = float(line.split(":")[1].split()[0]) * a.nx ** 3
    value = job_throughput(Nl, world, ms)
    out = {
        "metric": METRIC, "value": value, "unit": "GDOF/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": a.prec, "data": "synthetic",
        "config": {"workload": workload_name(a.nx, a.N), "elements": a.nx ** 3, "N": a.N,
                   "local_nodes": Nl, "assembled_dofs": Ng, "lambda": 1.0, "jitter": 0.1,
                   "l2": "inputs %.1f GB > 129 MB L2, no flush between steps" % (alg_bytes / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "gdofs_assembled": world * Ng / (ms * 1e-3) / 1e9,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": launch_ms},
        "compute": {"arith": {"f64": "fp64", "df64": "double-fp32 words"}.get(a.prec, "fp32"),
                    "flops_per_launch": flops,
                    "achieved_tflops": flops / (launch_ms * 1e-3) / 1e12,
                    "nominal_fp64_tflops": 1.25},
        "e2e": {"value": world * Nl / (e2e_ms * 1e-3) / 1e9, "unit": "GDOF/s",
                "h2d_bytes_per_step": Ng * qin.element_size(), "d2h_bytes_per_step": Ng * qin.element_size(),
                "ms_per_step": e2e_ms,
                "api": "lpg_elliptic_operator_host%s" % ("" if a.prec in ("f64", "df64") else "_f32"),
                "host_chunks": e.info("host_chunks"), "max_rel_diff_vs_device": e2e_check},
        "gpu_launches": a.steps,
        "clocks": clk,
        "setup_seconds": t_setup,
    }
    if variants:
        for v in variants.values():
            v["roofline"]["peak"], v["roofline"]["peak_kind"] = peak, peak_kind
            v["roofline"]["frac"] = v["roofline"]["achieved"] / peak
        out["variants"] = variants
    if world == 1 and not a.no_solves and a.nx == 64 and a.N == 7:
        # free the operator workload before the solves
        del q, Aq, qin, yout
        e.close()
        torch.cuda.empty_cache()
        out["solve"] = solve_blocks(a)
    if not a.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(a.cpu_sample_nx, a.N)
    print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
