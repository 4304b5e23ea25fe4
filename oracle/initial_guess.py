"""CPU restatement of the linear solver's initial-guess strategies (test infrastructure:
only tests/ use it, as the checker of the CUDA library's strategies).

Follows include/initialGuess.hpp:38-162 and libs/linearSolver/initialGuess.cpp:
Projection::FormInitialGuess (:104-111), ClassicProjection::Update (:144-188),
RollingQRProjection::Update (:203-318, rotations from givensRotation :320-333),
Extrap::FormInitialGuess / Update / extrapCoeffs (:379-468). The minimum-norm and
column-pivoted QR solves restate linAlg_t::matrixUnderdeterminedRightSolveMinNorm / CPQR
(libs/linAlg/linAlgMatrixRightSolve.cpp:204-328): minimum-norm solution, and the basic
solution of a QR factorisation with column pivoting (largest remaining column norm,
norms within a relative 1e-10 of it counted as ties and won by the first index)."""
import math

import numpy as np


def legendre_orthonormal(j, x):
    """P_j(x) sqrt((2j+1)/2): the orthonormal Legendre basis of Vandermonde1D."""
    x = np.asarray(x, dtype=float)
    p0, p1 = np.ones_like(x), x.copy()
    if j == 0:
        return np.sqrt(0.5) * p0
    for n in range(2, j + 1):
        p0, p1 = p1, ((2 * n - 1) * x * p1 - (n - 1) * p0) / n
    return p1 * math.sqrt((2 * j + 1) / 2.0)


def _cpqr_basic(A, b):
    A = A.copy()
    b = b.copy()
    rows, cols = A.shape
    perm = list(range(cols))
    for k in range(rows):
        norms = np.array([(A[k:, j] ** 2).sum() for j in range(k, cols)])
        p = k + int(np.nonzero(norms >= norms.max() * (1.0 - 1e-10))[0][0])   # ties: first index
        if p != k:
            A[:, [k, p]] = A[:, [p, k]]
            perm[k], perm[p] = perm[p], perm[k]
        alpha = math.sqrt((A[k:, k] ** 2).sum())
        if A[k, k] > 0:
            alpha = -alpha
        v = np.zeros(rows)
        v[k:] = A[k:, k]
        v[k] -= alpha
        vv = (v[k:] ** 2).sum()
        if vv > 0:
            A[k:, k:] -= np.outer(v[k:], 2.0 * (v[k:] @ A[k:, k:]) / vv)
            b[k:] -= v[k:] * (2.0 * (v[k:] @ b[k:]) / vv)
    y = np.zeros(rows)
    for k in range(rows - 1, -1, -1):
        y[k] = (b[k] - A[k, k + 1:rows] @ y[k + 1:]) / A[k, k]
    c = np.zeros(cols)
    for k in range(rows):
        c[perm[k]] = y[k]
    return c


def extrap_coeffs(m, M, cpqr=False):
    """Weights of the last M equally spaced values, exact one step ahead for degree m."""
    if M < m + 1:
        raise ValueError("history too short for the degree")
    if M == 1:
        return np.ones(1)
    h = 2.0 / (M - 1)
    r = -1.0 + h * np.arange(M)
    A = np.array([legendre_orthonormal(j, r) for j in range(m + 1)])          # (m+1) x M
    b = np.array([float(legendre_orthonormal(j, np.array([1.0 + h]))[0]) for j in range(m + 1)])
    if cpqr:
        return _cpqr_basic(A, b)
    return A.T @ np.linalg.solve(A @ A.T, b)


def givens(a, b):
    if b != 0:
        d = 1.0 / math.hypot(a, b)
        return abs(a) * d, math.copysign(d, a) * b
    return 1.0, 0.0


class Projection:
    def __init__(self, max_dim):
        self.max_dim = max_dim
        self.B, self.X = [], []

    def form(self, x, rhs):
        if not self.B:
            return x
        a = [Bm @ rhs for Bm in self.B]
        return sum(am * Xm for am, Xm in zip(a, self.X))

    def _orthogonalise(self, bt, xt):
        acc = np.zeros(len(self.B))
        for _ in range(2):
            a = np.array([Bm @ bt for Bm in self.B])
            bt = bt - sum(am * Bm for am, Bm in zip(a, self.B))
            xt = xt - sum(am * Xm for am, Xm in zip(a, self.X))
            acc += a
        return bt, xt, acc


class Classic(Projection):
    def update(self, op, x):
        bt = op(x)
        if len(self.B) >= self.max_dim or not self.B:
            nb = np.linalg.norm(bt)
            if nb > 0:
                self.B, self.X = [bt / nb], [x / nb]
            return
        bt, xt, _ = self._orthogonalise(bt, x.copy())
        nb = np.linalg.norm(bt)
        self.B.append(bt / nb)
        self.X.append(xt / nb)


class RollingQR(Projection):
    def __init__(self, max_dim):
        super().__init__(max_dim)
        self.R = np.zeros((max_dim, max_dim))

    def update(self, op, x):
        bt = op(x)
        M = self.max_dim
        if len(self.B) == M:
            R = self.R
            R[:, :M - 1] = R[:, 1:].copy()
            R[:, M - 1] = 0.0
            B, X = [v.copy() for v in self.B], [v.copy() for v in self.X]
            for j in range(M - 1):
                c, s = givens(R[j, j], R[j + 1, j])
                rj, rj1 = R[j, j:].copy(), R[j + 1, j:].copy()
                R[j, j:], R[j + 1, j:] = c * rj + s * rj1, -s * rj + c * rj1
                B[j], B[j + 1] = c * B[j] + s * B[j + 1], -s * B[j] + c * B[j + 1]
                X[j], X[j + 1] = c * X[j] + s * X[j + 1], -s * X[j] + c * X[j + 1]
            self.B, self.X = B[:M - 1], X[:M - 1]
        if not self.B:
            nb = np.linalg.norm(bt)
            if nb > 0:
                self.B, self.X = [bt / nb], [x / nb]
                self.R[0, 0] = nb
            return
        k = len(self.B)
        nb = np.linalg.norm(bt)
        bt, xt, acc = self._orthogonalise(bt, x.copy())
        self.R[:k, k] = acc
        nbp = np.linalg.norm(bt)
        if nbp / nb > 1e-10:
            self.B.append(bt / nbp)
            self.X.append(xt / nbp)
            self.R[k, k] = nbp


class Extrap:
    def __init__(self, M, m, cpqr=False):
        extrap_coeffs(m, M, cpqr)
        self.M, self.m, self.cpqr = M, m, cpqr
        self.entry, self.shift = 0, 0
        self.H = None
        self.d = np.zeros(M)

    def form(self, x, rhs):
        if self.H is None:
            self.H = [np.zeros_like(rhs) for _ in range(self.M)]
        if self.entry < self.M:
            Mc, mc = self.M, self.m
            if self.entry != self.M - 1:
                Mc = max(1, self.entry + 1)
                mc = int(math.sqrt(Mc))
            d = np.zeros(self.M)
            if Mc == 1:
                d[self.M - 1] = 1.0
            else:
                d[self.M - Mc:] = extrap_coeffs(mc, Mc, self.cpqr)
            if self.cpqr:
                d[np.abs(d) <= 1e-14] = 0.0
            self.d = d
            self.entry += 1
        out = np.zeros_like(rhs)
        for i in range(self.M):
            if self.d[i] != 0.0:
                out = out + self.d[i] * self.H[(i + self.shift) % self.M]
        return out

    def update(self, op, x):
        self.H[self.shift] = x.copy()
        self.shift = (self.shift + 1) % self.M
