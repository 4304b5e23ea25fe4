"""Shared helpers for the GPU parity tests (the oracle is the checker)."""
import numpy as np


def box(**over):
    d = {"BOX NX": 3, "BOX NY": 2, "BOX NZ": 4, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
         "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 7, "LAMBDA": 1.0, "MESH JITTER": 0.1,
         "MESH JITTER SEED": 0, "LINEAR SOLVER": "FPCG", "PRECONDITIONER": "NONE"}
    d.update(over)
    return d


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def lattice_q(o_or_e_g2l, N, nx, ny, nz, seed=1):
    """Input vector u in [-1,1] keyed by the global lattice node id (stream 3)."""
    from oracle.oracle import u01
    g2l = o_or_e_g2l
    Nq = N + 1
    Np = Nq ** 3
    Ng = int(g2l.max()) + 1
    q = np.zeros(Ng)
    NnX, NnY = nx * N + 1, ny * N + 1
    for idx in np.nonzero(g2l >= 0)[0]:
        e, n = divmod(int(idx), Np)
        a, b, c = n % Nq, (n // Nq) % Nq, n // (Nq * Nq)
        ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
        X, Y, Z = ex * N + a, ey * N + b, ez * N + c
        q[g2l[idx]] = 2.0 * u01(seed, 3, X + Y * NnX + Z * NnX * NnY) - 1.0
    return q
