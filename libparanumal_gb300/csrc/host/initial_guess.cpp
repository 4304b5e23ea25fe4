// Initial-guess strategies (include/initialGuess.hpp:38-162, libs/linearSolver/initialGuess.cpp).
#include "initial_guess.hpp"

#include <algorithm>
#include <cmath>

namespace lpg {

namespace {

// orthonormal Legendre polynomial P_j(x) sqrt((2j+1)/2) (the basis of the reference's
// Vandermonde1D, meshBasis1D.cpp)
double legendre_orthonormal(int j, double x) {
  double p0 = 1.0, p1 = x;
  if (j == 0) return std::sqrt(0.5);
  for (int n = 2; n <= j; ++n) {
    const double p2 = ((2.0 * n - 1.0) * x * p1 - (n - 1.0) * p0) / n;
    p0 = p1;
    p1 = p2;
  }
  return p1 * std::sqrt((2.0 * j + 1.0) / 2.0);
}

// min-norm solution of A c = b, A (rows x cols) row-major with rows <= cols:
// c = A^T (A A^T)^{-1} b (Gaussian elimination with partial pivoting on A A^T)
bool min_norm_solve(int rows, int cols, const std::vector<double>& A, const std::vector<double>& b,
                    std::vector<double>& c) {
  std::vector<double> G(rows * rows, 0.0), y(b);
  for (int i = 0; i < rows; ++i)
    for (int j = 0; j < rows; ++j)
      for (int k = 0; k < cols; ++k) G[i * rows + j] += A[i * cols + k] * A[j * cols + k];
  for (int k = 0; k < rows; ++k) {
    int p = k;
    for (int i = k + 1; i < rows; ++i)
      if (std::fabs(G[i * rows + k]) > std::fabs(G[p * rows + k])) p = i;
    if (G[p * rows + k] == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < rows; ++j) std::swap(G[k * rows + j], G[p * rows + j]);
      std::swap(y[k], y[p]);
    }
    for (int i = k + 1; i < rows; ++i) {
      const double f = G[i * rows + k] / G[k * rows + k];
      for (int j = k; j < rows; ++j) G[i * rows + j] -= f * G[k * rows + j];
      y[i] -= f * y[k];
    }
  }
  for (int k = rows - 1; k >= 0; --k) {
    double v = y[k];
    for (int j = k + 1; j < rows; ++j) v -= G[k * rows + j] * y[j];
    y[k] = v / G[k * rows + k];
  }
  c.assign(cols, 0.0);
  for (int k = 0; k < cols; ++k)
    for (int i = 0; i < rows; ++i) c[k] += A[i * cols + k] * y[i];
  return true;
}

// basic solution of A c = b (rows <= cols) by Householder QR with column pivoting
// (largest remaining column norm; norms within a relative 1e-10 of the largest count as
// ties, won by the first index -- equally spaced history points give exactly tied
// columns, and a tie must not be decided by rounding): A P = Q R, c_P = [R1^{-1} Q^T b; 0]
bool cpqr_solve(int rows, int cols, std::vector<double> A, std::vector<double> b, std::vector<double>& c) {
  std::vector<int> perm(cols);
  for (int j = 0; j < cols; ++j) perm[j] = j;
  for (int k = 0; k < rows; ++k) {
    std::vector<double> nn(cols, 0.0);
    double best = 0.0;
    for (int j = k; j < cols; ++j) {
      for (int i = k; i < rows; ++i) nn[j] += A[i * cols + j] * A[i * cols + j];
      best = std::max(best, nn[j]);
    }
    int p = k;
    for (int j = k; j < cols; ++j)
      if (nn[j] >= best * (1.0 - 1e-10)) { p = j; break; }
    if (p != k) {
      for (int i = 0; i < rows; ++i) std::swap(A[i * cols + k], A[i * cols + p]);
      std::swap(perm[k], perm[p]);
    }
    // Householder reflector of column k below the diagonal
    double alpha = 0.0;
    for (int i = k; i < rows; ++i) alpha += A[i * cols + k] * A[i * cols + k];
    alpha = std::sqrt(alpha);
    if (alpha == 0.0) return false;
    if (A[k * cols + k] > 0) alpha = -alpha;
    std::vector<double> v(rows, 0.0);
    for (int i = k; i < rows; ++i) v[i] = A[i * cols + k];
    v[k] -= alpha;
    double vv = 0.0;
    for (int i = k; i < rows; ++i) vv += v[i] * v[i];
    if (vv > 0) {
      for (int j = k; j < cols; ++j) {
        double d = 0.0;
        for (int i = k; i < rows; ++i) d += v[i] * A[i * cols + j];
        d = 2.0 * d / vv;
        for (int i = k; i < rows; ++i) A[i * cols + j] -= d * v[i];
      }
      double d = 0.0;
      for (int i = k; i < rows; ++i) d += v[i] * b[i];
      d = 2.0 * d / vv;
      for (int i = k; i < rows; ++i) b[i] -= d * v[i];
    }
  }
  std::vector<double> y(rows);
  for (int k = rows - 1; k >= 0; --k) {
    double v = b[k];
    for (int j = k + 1; j < rows; ++j) v -= A[k * cols + j] * y[j];
    if (A[k * cols + k] == 0.0) return false;
    y[k] = v / A[k * cols + k];
  }
  c.assign(cols, 0.0);
  for (int k = 0; k < rows; ++k) c[perm[k]] = y[k];
  return true;
}

// Givens rotation zeroing b in [a; b] (RollingQRProjection::givensRotation)
void givens(double a, double b, double& c, double& s) {
  if (b != 0) {
    const double d = 1.0 / std::hypot(a, b);
    c = std::fabs(a) * d;
    s = std::copysign(d, a) * b;
  } else {
    c = 1.0;
    s = 0.0;
  }
}

struct NoGuess : InitialGuess {
  int form(double*, const double*, cudaStream_t) override { return LPG_OK; }
  int update(Elliptic*, const double*, cudaStream_t) override { return LPG_OK; }
};

struct ZeroGuess : InitialGuess {
  int64_t N;
  explicit ZeroGuess(int64_t n) : N(n) {}
  int form(double* x, const double*, cudaStream_t s) override {
    LPG_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * N, s));
    return LPG_OK;
  }
  int update(Elliptic*, const double*, cudaStream_t) override { return LPG_OK; }
};

// history space of right-hand sides B (orthonormal) and matching solutions X
struct Projection : InitialGuess {
  Platform* plat;
  int64_t N;
  int maxDim, curDim = 0;
  DevBuf<double> btilde, xtilde, B, X, partials;
  std::vector<double> part;
  int history() const override { return curDim; }

  Projection(Platform* p, int64_t n, int m) : plat(p), N(n), maxDim(m) {}
  int init() {
    int rc;
    if ((rc = btilde.alloc(N)) || (rc = xtilde.alloc(N)) || (rc = B.alloc(N * maxDim)) || (rc = X.alloc(N * maxDim)) ||
        (rc = partials.alloc((int64_t)kMaxHistory * kMultiDotBlocks)))
      return rc;
    return LPG_OK;
  }
  // alphas[m] = B_m . v for m < curDim (block sums added on the host in block order)
  int inner(const double* v, HistCoeffs& alphas, cudaStream_t s) {
    int nb = 0, rc;
    if ((rc = multi_dot(N, curDim, v, B.p, partials.p, &nb, s))) return rc;
    part.resize((size_t)curDim * nb);
    if (curDim > 0) {
      LPG_CUDA_TRY(cudaMemcpyAsync(part.data(), partials.p, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s));
      LPG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    for (int m = 0; m < kMaxHistory; ++m) alphas.v[m] = 0.0;
    for (int m = 0; m < curDim; ++m)
      for (int b = 0; b < nb; ++b) alphas.v[m] += part[(size_t)m * nb + b];
    return LPG_OK;
  }
  double norm(const double* v) {
    double r = 0;
    if (plat->norm2sq(N, v, r)) return -1;
    return std::sqrt(r);
  }
  int store(int slot, double scale, const double* b, const double* x, cudaStream_t s) {
    int rc;
    if ((rc = axpy<double>(N, scale, b, 0.0, B.p + (int64_t)slot * N, s))) return rc;
    return axpy<double>(N, scale, x, 0.0, X.p + (int64_t)slot * N, s);
  }
  // x = sum_m (B_m . rhs) X_m (Projection::FormInitialGuess)
  int form(double* x, const double* rhs, cudaStream_t s) override {
    if (curDim == 0) return LPG_OK;
    HistCoeffs a;
    int rc;
    if ((rc = inner(rhs, a, s))) return rc;
    return combine(N, curDim, nullptr, 1.0, a, X.p, x, s);
  }
  // btilde, xtilde -= sum (B_m . btilde) (B_m, X_m), twice; alphas of both passes summed
  int orthogonalise(cudaStream_t s, double* rcol) {
    int rc;
    for (int pass = 0; pass < 2; ++pass) {
      HistCoeffs a;
      if ((rc = inner(btilde.p, a, s))) return rc;
      if ((rc = combine(N, curDim, btilde.p, -1.0, a, B.p, btilde.p, s)) ||
          (rc = combine(N, curDim, xtilde.p, -1.0, a, X.p, xtilde.p, s)))
        return rc;
      if (rcol)
        for (int i = 0; i < curDim; ++i) rcol[i] += a.v[i];
    }
    return LPG_OK;
  }
};

struct Classic : Projection {
  using Projection::Projection;
  // ClassicProjection::Update (initialGuess.cpp:144-188)
  int update(Elliptic* el, const double* x, cudaStream_t s) override {
    int rc;
    if ((rc = el->Operator(x, btilde.p, s))) return rc;
    if (curDim >= maxDim || curDim == 0) {
      const double nb = norm(btilde.p);
      if (nb < 0) return LPG_ERR_CUDA;
      if (nb > 0) {
        if ((rc = store(0, 1.0 / nb, btilde.p, x, s))) return rc;
        curDim = 1;
      }
      return LPG_OK;
    }
    LPG_CUDA_TRY(cudaMemcpyAsync(xtilde.p, x, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
    if ((rc = orthogonalise(s, nullptr))) return rc;
    const double nb = norm(btilde.p);
    if (nb < 0) return LPG_ERR_CUDA;
    if ((rc = store(curDim, 1.0 / nb, btilde.p, xtilde.p, s))) return rc;
    ++curDim;
    return LPG_OK;
  }
};

struct RollingQR : Projection {
  std::vector<double> R;   // maxDim x maxDim, row-major
  RollingQR(Platform* p, int64_t n, int m) : Projection(p, n, m), R((size_t)m * m, 0.0) {}
  // RollingQRProjection::Update (initialGuess.cpp:203-318)
  int update(Elliptic* el, const double* x, cudaStream_t s) override {
    int rc;
    if ((rc = el->Operator(x, btilde.p, s))) return rc;
    const int M = maxDim;
    if (curDim == M) {
      // drop the first column of R, restore the triangle with Givens rotations and
      // apply the same rotations to the columns of B and X
      for (int j = 0; j < M; ++j) {
        for (int i = 0; i < M - 1; ++i) R[j * M + i] = R[j * M + i + 1];
        R[j * M + M - 1] = 0.0;
      }
      HistCoeffs cs, sn;
      for (int j = 0; j < M - 1; ++j) {
        double c = 0, sv = 0;
        givens(R[j * M + j], R[(j + 1) * M + j], c, sv);
        cs.v[j] = c;
        sn.v[j] = sv;
        for (int i = j; i < M; ++i) {
          const double a = R[j * M + i], b = R[(j + 1) * M + i];
          R[j * M + i] = c * a + sv * b;
          R[(j + 1) * M + i] = -sv * a + c * b;
        }
      }
      if ((rc = givens_columns(N, M, cs, sn, B.p, X.p, s))) return rc;
      --curDim;
    }
    if (curDim == 0) {
      const double nb = norm(btilde.p);
      if (nb < 0) return LPG_ERR_CUDA;
      if (nb > 0) {
        if ((rc = store(0, 1.0 / nb, btilde.p, x, s))) return rc;
        R[0] = nb;
        curDim = 1;
      }
      return LPG_OK;
    }
    LPG_CUDA_TRY(cudaMemcpyAsync(xtilde.p, x, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
    const double nb = norm(btilde.p);
    if (nb < 0) return LPG_ERR_CUDA;
    std::vector<double> col(kMaxHistory, 0.0);
    if ((rc = orthogonalise(s, col.data()))) return rc;
    for (int i = 0; i < curDim; ++i) R[i * M + curDim] = col[i];
    const double nbp = norm(btilde.p);
    if (nbp < 0) return LPG_ERR_CUDA;
    // keep the new direction only if it is not (numerically) in the span already
    if (nbp / nb > 1.0e-10) {
      if ((rc = store(curDim, 1.0 / nbp, btilde.p, xtilde.p, s))) return rc;
      R[curDim * M + curDim] = nbp;
      ++curDim;
    }
    return LPG_OK;
  }
};

struct Extrapolation : InitialGuess {
  int64_t N;
  int M, m;
  bool cpqr;
  int entry = 0, shift = 0;
  DevBuf<double> H;     // M solutions, ring buffer
  HistCoeffs d{};
  Extrapolation(int64_t n, int hist, int deg, bool qr) : N(n), M(hist), m(deg), cpqr(qr) {}
  int history() const override { return std::min(entry, M); }
  int init(cudaStream_t s) {
    std::vector<double> c;
    int rc;
    if ((rc = extrap_coeffs(m, M, cpqr, c))) return rc;
    if ((rc = H.alloc(N * M))) return rc;
    LPG_CUDA_TRY(cudaMemsetAsync(H.p, 0, sizeof(double) * N * M, s));
    return LPG_OK;
  }
  // Extrap::FormInitialGuess (initialGuess.cpp:379-430): while the history fills, the
  // weights use the M' = entry + 1 solutions there are, degree floor(sqrt(M'))
  int form(double* x, const double*, cudaStream_t s) override {
    if (entry < M) {
      int Mc = M, mc = m;
      if (entry != M - 1) {
        Mc = std::max(1, entry + 1);
        mc = (int)std::sqrt((double)Mc);
      }
      for (int i = 0; i < kMaxHistory; ++i) d.v[i] = 0.0;
      if (Mc == 1) {
        d.v[M - 1] = 1.0;
      } else {
        std::vector<double> c;
        int rc;
        if ((rc = extrap_coeffs(mc, Mc, cpqr, c))) return rc;
        for (int i = 0; i < Mc; ++i) d.v[M - Mc + i] = c[i];
      }
      if (cpqr)
        for (int i = 0; i < M; ++i)
          if (std::fabs(d.v[i]) <= 1e-14) d.v[i] = 0.0;
      ++entry;
    }
    return extrap(N, M, shift, d, H.p, x, s);
  }
  int update(Elliptic*, const double* x, cudaStream_t s) override {
    LPG_CUDA_TRY(cudaMemcpyAsync(H.p + (int64_t)shift * N, x, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
    shift = (shift + 1) % M;
    return LPG_OK;
  }
};

}  // namespace

int extrap_coeffs(int m, int M, bool cpqr, std::vector<double>& c) {
  if (M < 1 || m < 0 || M > kMaxHistory)
    return set_error(LPG_ERR_SETTINGS, "extrapolation: history dimension must be 1.." + std::to_string(kMaxHistory));
  if (M < m + 1)
    return set_error(LPG_ERR_SETTINGS, "Extrapolation space dimension (" + std::to_string(M) +
                                           ") too low for degree (" + std::to_string(m) + ")");
  if (M == 1) {
    c.assign(1, 1.0);
    return LPG_OK;
  }
  // V^T c = b with V[i][j] = P_j(r_i), r_i = -1 + i h, b_j = P_j(1 + h), h = 2/(M-1)
  const double h = 2.0 / (M - 1);
  const int rows = m + 1, cols = M;
  std::vector<double> A((size_t)rows * cols), b(rows);
  for (int j = 0; j < rows; ++j) {
    for (int i = 0; i < cols; ++i) A[(size_t)j * cols + i] = legendre_orthonormal(j, -1.0 + i * h);
    b[j] = legendre_orthonormal(j, 1.0 + h);
  }
  const bool ok = cpqr ? cpqr_solve(rows, cols, A, b, c) : min_norm_solve(rows, cols, A, b, c);
  if (!ok) return set_error(LPG_ERR_INVALID, "extrapolation: singular system");
  return LPG_OK;
}

std::unique_ptr<InitialGuess> make_initial_guess(const Settings& S, Platform* plat, int64_t N, int* status) {
  *status = LPG_OK;
  const std::string kind = S.get("INITIAL GUESS STRATEGY", "NONE");
  if (kind == "NONE") return std::make_unique<NoGuess>();
  if (kind == "ZERO") return std::make_unique<ZeroGuess>(N);
  const int dim = S.geti("INITIAL GUESS HISTORY SPACE DIMENSION", -1);
  if (dim < 1 || dim > kMaxHistory) {
    *status = set_error(LPG_ERR_SETTINGS, "INITIAL GUESS HISTORY SPACE DIMENSION must be 1.." +
                                              std::to_string(kMaxHistory) + " for strategy " + kind);
    return nullptr;
  }
  if (kind == "CLASSIC" || kind == "QR") {
    std::unique_ptr<Projection> p;
    if (kind == "CLASSIC") p = std::make_unique<Classic>(plat, N, dim);
    else p = std::make_unique<RollingQR>(plat, N, dim);
    if ((*status = p->init())) return nullptr;
    return p;
  }
  if (kind == "EXTRAP") {
    const int deg = S.geti("INITIAL GUESS EXTRAP DEGREE", -1);
    const std::string method = S.get("INITIAL GUESS EXTRAP COEFFS METHOD", "MINNORM");
    if (method != "MINNORM" && method != "CPQR") {
      *status = set_error(LPG_ERR_SETTINGS, "INITIAL GUESS EXTRAP COEFFS METHOD must be MINNORM or CPQR");
      return nullptr;
    }
    auto e = std::make_unique<Extrapolation>(N, dim, deg, method == "CPQR");
    if ((*status = e->init(plat->stream))) return nullptr;
    return e;
  }
  *status = set_error(LPG_ERR_SETTINGS, "INITIAL GUESS STRATEGY must be NONE, ZERO, CLASSIC, QR or EXTRAP");
  return nullptr;
}

}  // namespace lpg
