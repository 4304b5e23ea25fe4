"""CPU restatement of the VTU plot-field output (test infrastructure: only tests/ use it, as
the checker of lpg_elliptic_plot_fields).

Follows libs/mesh/meshReferenceNodesHex3D.cpp:53-63 (plot degree N+3, equispaced plot
nodes, 6*(N+3)^3 tetrahedra per element), libs/mesh/meshBasis1D.cpp (InterpolationMatrix1D
= V(r_out) V(r_in)^-1 with the orthonormal Legendre Vandermonde) and
libs/mesh/meshPlotInterpHex3D.cpp:30-100 (r, s, t contractions)."""
import numpy as np

from oracle.initial_guess import legendre_orthonormal


def gll_nodes(N):
    """GLL points of degree N: +-1 and the roots of P_N'."""
    if N == 1:
        return np.array([-1.0, 1.0])
    c = np.zeros(N + 1)
    c[N] = 1.0
    inner = np.real(np.polynomial.legendre.legroots(np.polynomial.legendre.legder(c)))
    return np.concatenate([[-1.0], np.sort(inner), [1.0]])


def interp_matrix(N, r_out):
    r_in = gll_nodes(N)
    V_in = np.array([legendre_orthonormal(j, r_in) for j in range(N + 1)]).T
    V_out = np.array([legendre_orthonormal(j, r_out) for j in range(N + 1)]).T
    return V_out @ np.linalg.inv(V_in)


def plot_interp(qL, E, N):
    """qL (E*(N+1)^3, element-major, i fastest) at the (N+4)^3 equispaced plot nodes."""
    pN = N + 3
    I = interp_matrix(N, np.linspace(-1.0, 1.0, pN + 1))
    q = np.asarray(qL).reshape(E, N + 1, N + 1, N + 1)          # [e][k][j][i]
    return np.einsum("ai,bj,ck,ekji->ecba", I, I, I, q).reshape(E, -1)


def plot_cells(N):
    return 6 * (N + 3) ** 3
