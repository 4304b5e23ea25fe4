// p-multigrid V-cycle over a parAlmond-style smoothed-aggregation AMG coarse hierarchy.
//
// p-levels (matrix-free, device): ellipticPreconMultiGrid.cpp:31-154 and
// ellipticPreconMultiGridLevel.cpp:30-473 (Chebyshev / damped Jacobi smoothing,
// weighted restriction, prolongation, Arnoldi estimate of rho(D^{-1}A) from a drand48
// start vector). The p-levels run in FP64, FP32, or FP32 with BF16 geometric factors.
// AMG levels (assembled CSR, FP64): parAlmondAMGSetup.cpp:35-144 (setup on the host,
// as in the reference), parAlmondVcycle.cpp:34-60, parAlmondAMGSmoother.cpp:35-160,
// parAlmondCoarseExact.cpp:35-227 (dense inverse of the <= 1000-row base level).
// The drand48 stream is seeded with 0 and consumed in the reference's order: p-level
// Arnoldi vectors, then per AMG level the Arnoldi vector and the MIS-2 priorities.
#include "objects.hpp"
#include "learned.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace lpg {

// ================================================================ host sparse matrices
struct HCSR {
  int64_t n = 0, m = 0;
  std::vector<int64_t> rs;
  std::vector<int32_t> cols;
  std::vector<double> vals;
  int64_t nnz() const { return (int64_t)cols.size(); }
};

static void spmv_host(const HCSR& A, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < A.n; ++i) {
    double s = 0;
    for (int64_t j = A.rs[i]; j < A.rs[i + 1]; ++j) s += A.vals[j] * x[A.cols[j]];
    y[i] = s;
  }
}

static HCSR transpose(const HCSR& A) {
  HCSR T;
  T.n = A.m;
  T.m = A.n;
  T.rs.assign(T.n + 1, 0);
  for (int32_t c : A.cols) T.rs[c + 1]++;
  for (int64_t i = 0; i < T.n; ++i) T.rs[i + 1] += T.rs[i];
  T.cols.resize(A.nnz());
  T.vals.resize(A.nnz());
  std::vector<int64_t> pos(T.rs.begin(), T.rs.end() - 1);
  for (int64_t i = 0; i < A.n; ++i)
    for (int64_t j = A.rs[i]; j < A.rs[i + 1]; ++j) {
      const int64_t p = pos[A.cols[j]]++;
      T.cols[p] = (int32_t)i;
      T.vals[p] = A.vals[j];
    }
  return T;
}

// C = A B by rows with a dense accumulator; columns of each row sorted.
static HCSR spmm(const HCSR& A, const HCSR& B) {
  HCSR C;
  C.n = A.n;
  C.m = B.m;
  C.rs.assign(A.n + 1, 0);
  int nth = 1;
#ifdef _OPENMP
  nth = omp_get_max_threads();
#endif
  std::vector<std::vector<int32_t>> pc(nth);
  std::vector<std::vector<double>> pv(nth);
  std::vector<int64_t> chunkStart(nth + 1, 0);
  std::vector<int64_t> rowCount(A.n, 0);
#pragma omp parallel
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    const int64_t lo = A.n * t / nth, hi = A.n * (t + 1) / nth;
    std::vector<double> acc(B.m, 0.0);
    std::vector<int32_t> mark(B.m, -1), list;
    for (int64_t i = lo; i < hi; ++i) {
      list.clear();
      for (int64_t j = A.rs[i]; j < A.rs[i + 1]; ++j) {
        const int32_t k = A.cols[j];
        const double a = A.vals[j];
        for (int64_t jj = B.rs[k]; jj < B.rs[k + 1]; ++jj) {
          const int32_t c = B.cols[jj];
          if (mark[c] != (int32_t)i) { mark[c] = (int32_t)i; acc[c] = 0.0; list.push_back(c); }
          acc[c] += a * B.vals[jj];
        }
      }
      std::sort(list.begin(), list.end());
      for (int32_t c : list) { pc[t].push_back(c); pv[t].push_back(acc[c]); }
      rowCount[i] = (int64_t)list.size();
    }
  }
  for (int64_t i = 0; i < A.n; ++i) C.rs[i + 1] = C.rs[i] + rowCount[i];
  C.cols.reserve(C.rs[A.n]);
  C.vals.reserve(C.rs[A.n]);
  for (int t = 0; t < nth; ++t) {
    C.cols.insert(C.cols.end(), pc[t].begin(), pc[t].end());
    C.vals.insert(C.vals.end(), pv[t].begin(), pv[t].end());
  }
  return C;
}

// ================================================================ device CSR
struct DCSR {
  int64_t n = 0, m = 0;
  DevBuf<int64_t> rs;
  DevBuf<int32_t> cols;
  DevBuf<double> vals;
  int upload(const HCSR& A, cudaStream_t s) {
    n = A.n;
    m = A.m;
    int rc;
    if ((rc = rs.alloc(n + 1)) || (rc = rs.upload(A.rs.data(), n + 1, s))) return rc;
    if (A.nnz() > 0) {
      if ((rc = cols.alloc(A.nnz())) || (rc = cols.upload(A.cols.data(), A.nnz(), s))) return rc;
      if ((rc = vals.alloc(A.nnz())) || (rc = vals.upload(A.vals.data(), A.nnz(), s))) return rc;
    }
    return LPG_OK;
  }
};

// ================================================================ AMG setup (host)
struct ALevel {
  HCSR A, P, R;
  DCSR dA, dP, dR;
  std::vector<double> diagA, diagInv;
  DevBuf<double> dDiagInv;
  double rho = 0, lambda0 = 0, lambda1 = 0, jlambda = 0;
  DevBuf<double> rhs, x, res, s1, s2, s3;
};

// parCSR::rhoDinvA (parAlmondparCSR.cpp:351-440): 10-step Arnoldi on D^{-1}A on the host.
static double rho_dinv_a(const HCSR& A, const std::vector<double>& diagInv, Rand48& rng) {
  const int64_t N = A.n;
  int k = 10;
  if (k > N) k = (int)N;
  std::vector<double> H(k * k, 0.0);
  std::vector<std::vector<double>> V(k + 1, std::vector<double>(N));
  std::vector<double> Vx(N);
  for (int64_t n = 0; n < N; ++n) Vx[n] = rng.next();
  double nrm = 0;
  for (int64_t n = 0; n < N; ++n) nrm += Vx[n] * Vx[n];
  nrm = std::sqrt(nrm);
  for (int64_t n = 0; n < N; ++n) V[0][n] = Vx[n] * (1.0 / nrm);
  for (int j = 0; j < k; ++j) {
    spmv_host(A, V[j].data(), V[j + 1].data());
    for (int64_t n = 0; n < N; ++n) V[j + 1][n] *= diagInv[n];
    for (int i = 0; i <= j; ++i) {
      double hij = 0;
      for (int64_t n = 0; n < N; ++n) hij += V[i][n] * V[j + 1][n];
      for (int64_t n = 0; n < N; ++n) V[j + 1][n] += -hij * V[i][n];
      H[i + j * k] = hij;
    }
    if (j + 1 < k) {
      double nj = 0;
      for (int64_t n = 0; n < N; ++n) nj += V[j + 1][n] * V[j + 1][n];
      nj = std::sqrt(nj);
      H[j + 1 + j * k] = nj;
      for (int64_t n = 0; n < N; ++n) V[j + 1][n] *= (1. / nj);
    }
  }
  return hessenberg_spectral_radius(k, H);
}

static void diag_setup(ALevel& L, Rand48& rng) {
  const int64_t N = L.A.n;
  L.diagA.assign(N, 0.0);
  L.diagInv.assign(N, 0.0);
  for (int64_t i = 0; i < N; ++i)
    for (int64_t j = L.A.rs[i]; j < L.A.rs[i + 1]; ++j)
      if (L.A.cols[j] == i) L.diagA[i] = L.A.vals[j];
  for (int64_t i = 0; i < N; ++i) L.diagInv[i] = (L.diagA[i] != 0.0) ? 1.0 / L.diagA[i] : 0.0;
  L.rho = rho_dinv_a(L.A, L.diagInv, rng);
}

static bool custom_less(int smax, double rmax, int64_t imax, int s, double r, int64_t i) {
  if (s > smax) return true;
  if (smax > s) return false;
  if (r > rmax) return true;
  if (rmax > r) return false;
  return i > imax;
}

// Strength of connection (parAlmondStrongGraph.cpp) and distance-2 maximal independent
// set aggregation (parAlmondFormAggregates.cpp:54-251).
static int64_t form_aggregates(const ALevel& L, double theta, bool rugeStuben, std::vector<int64_t>& F2C, Rand48& rng) {
  const HCSR& A = L.A;
  const int64_t N = A.n;
  std::vector<int64_t> Crs(N + 1, 0);
  std::vector<int64_t> Ccols;
  Ccols.reserve(A.nnz());
  for (int64_t i = 0; i < N; ++i) {
    if (rugeStuben) {
      const int sign = (L.diagA[i] >= 0) ? 1 : -1;
      double maxOD = 0;
      for (int64_t jj = A.rs[i]; jj < A.rs[i + 1]; ++jj) {
        if (A.cols[jj] == i) continue;
        const double OD = -sign * A.vals[jj];
        if (OD > maxOD) maxOD = OD;
      }
      for (int64_t jj = A.rs[i]; jj < A.rs[i + 1]; ++jj) {
        const int64_t col = A.cols[jj];
        if (col == i) { Ccols.push_back(col); continue; }
        if (-sign * A.vals[jj] > theta * maxOD) Ccols.push_back(col);
      }
    } else {
      const double Aii = std::fabs(L.diagA[i]);
      for (int64_t jj = A.rs[i]; jj < A.rs[i + 1]; ++jj) {
        const int64_t col = A.cols[jj];
        if (col == i) { Ccols.push_back(col); continue; }
        const double Ajj = std::fabs(L.diagA[col]);
        if (std::fabs(A.vals[jj]) > theta * std::sqrt(Aii * Ajj)) Ccols.push_back(col);
      }
    }
    Crs[i + 1] = (int64_t)Ccols.size();
  }
  std::vector<double> rands(N), Tr(N);
  std::vector<int> states(N, 0), Ts(N);
  std::vector<int64_t> Ti(N), Tc(N);
  for (int64_t i = 0; i < N; ++i) rands[i] = rng.next();
  std::vector<int> colCnt(N, 0);
  for (int64_t c : Ccols) colCnt[c]++;
  for (int64_t i = 0; i < N; ++i) rands[i] += colCnt[i];
  for (;;) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
      int smax = states[i];
      double rmax = rands[i];
      int64_t imax = i;
      if (smax != 1)
        for (int64_t jj = Crs[i]; jj < Crs[i + 1]; ++jj) {
          const int64_t col = Ccols[jj];
          if (col == i) continue;
          if (custom_less(smax, rmax, imax, states[col], rands[col], col)) { smax = states[col]; rmax = rands[col]; imax = col; }
        }
      Ts[i] = smax; Tr[i] = rmax; Ti[i] = imax;
    }
    int64_t undecided = 0;
#pragma omp parallel for schedule(static) reduction(+ : undecided)
    for (int64_t i = 0; i < N; ++i) {
      int smax = Ts[i];
      double rmax = Tr[i];
      int64_t imax = Ti[i];
      for (int64_t jj = Crs[i]; jj < Crs[i + 1]; ++jj) {
        const int64_t col = Ccols[jj];
        if (col == i) continue;
        if (custom_less(smax, rmax, imax, Ts[col], Tr[col], Ti[col])) { smax = Ts[col]; rmax = Tr[col]; imax = Ti[col]; }
      }
      if (states[i] == 0 && imax == i) states[i] = 1;
      if (states[i] == 0 && smax == 1) states[i] = -1;
      if (states[i] == 0) undecided++;
    }
    if (undecided == 0) break;
  }
  int64_t numAggs = 0;
  F2C.assign(N, -1);
  for (int64_t i = 0; i < N; ++i)
    if (states[i] == 1) F2C[i] = numAggs++;
  // first neighbours: the pass reads F2C of MIS nodes only, so it is order independent
  for (int64_t i = 0; i < N; ++i) {
    int smax = states[i];
    double rmax = rands[i];
    int64_t imax = i, cmax = F2C[i];
    if (smax != 1)
      for (int64_t jj = Crs[i]; jj < Crs[i + 1]; ++jj) {
        const int64_t col = Ccols[jj];
        if (col == i) continue;
        if (custom_less(smax, rmax, imax, states[col], rands[col], col)) {
          smax = states[col]; rmax = rands[col]; imax = col; cmax = F2C[col];
        }
      }
    Ts[i] = smax; Tr[i] = rmax; Ti[i] = imax; Tc[i] = cmax;
    if (F2C[i] == -1 && smax == 1 && cmax > -1) F2C[i] = cmax;
  }
  std::vector<int64_t> F2Cnew(F2C);
  for (int64_t i = 0; i < N; ++i) {
    int smax = Ts[i];
    double rmax = Tr[i];
    int64_t imax = Ti[i], cmax = Tc[i];
    for (int64_t jj = Crs[i]; jj < Crs[i + 1]; ++jj) {
      const int64_t col = Ccols[jj];
      if (col == i) continue;
      if (custom_less(smax, rmax, imax, Ts[col], Tr[col], Ti[col])) { smax = Ts[col]; rmax = Tr[col]; imax = Ti[col]; cmax = Tc[col]; }
    }
    if (F2Cnew[i] == -1 && smax == 1 && cmax > -1) F2Cnew[i] = cmax;
  }
  F2C.swap(F2Cnew);
  return numAggs;
}

// coarsenAmgLevel (parAlmondCoarsenLevel.cpp:33-84)
static int amg_coarsen(ALevel& L, ALevel& Lc, std::vector<double>& nullv, double theta, bool rs, bool unsmoothed,
                       Rand48& rng) {
  const int64_t N = L.A.n;
  std::vector<int64_t> F2C;
  const int64_t Nc = form_aggregates(L, theta, rs, F2C, rng);
  for (int64_t i = 0; i < N; ++i)
    if (F2C[i] < 0) return set_error(LPG_ERR_INVALID, "AMG: unaggregated row");
  // tentative prolongator with normalised columns (parAlmondTentativeProlongator.cpp:33-94)
  HCSR T;
  T.n = N; T.m = Nc;
  T.rs.resize(N + 1);
  T.cols.resize(N);
  T.vals.resize(N);
  for (int64_t i = 0; i <= N; ++i) T.rs[i] = i;
  std::vector<double> cn(Nc, 0.0);
  for (int64_t i = 0; i < N; ++i) { T.cols[i] = (int32_t)F2C[i]; T.vals[i] = nullv[i]; cn[F2C[i]] += nullv[i] * nullv[i]; }
  for (int64_t c = 0; c < Nc; ++c) cn[c] = std::sqrt(cn[c]);
  for (int64_t i = 0; i < N; ++i) T.vals[i] /= cn[T.cols[i]];
  nullv.assign(cn.begin(), cn.end());
  if (!unsmoothed) {
    // P = (I - omega D^{-1} A) T, omega = 4/3/rho (parAlmondSmoothPrologator.cpp:33-301)
    // Row i: the entry of T followed by the row's A entries mapped to aggregates, stably
    // sorted by column and merged; rows are independent, so they are built in parallel
    // (same sums, in the same order, as one stable sort of all entries).
    const double omega = (4. / 3.) / L.rho;
    HCSR P;
    P.n = N; P.m = Nc;
    P.rs.assign(N + 1, 0);
    std::vector<int64_t> start(N + 1, 0);
    for (int64_t i = 0; i < N; ++i) start[i + 1] = start[i] + 1 + (L.A.rs[i + 1] - L.A.rs[i]);
    std::vector<int32_t> pc(start[N]);
    std::vector<double> pv(start[N]);
#pragma omp parallel
    {
      std::vector<std::pair<int32_t, double>> row;
#pragma omp for schedule(dynamic, 4096)
      for (int64_t i = 0; i < N; ++i) {
        row.clear();
        row.emplace_back((int32_t)T.cols[i], T.vals[i]);
        const double invDi = 1.0 / L.diagA[i];
        for (int64_t j = L.A.rs[i]; j < L.A.rs[i + 1]; ++j) {
          const int32_t col = L.A.cols[j];
          row.emplace_back((int32_t)T.cols[col], -omega * invDi * L.A.vals[j] * T.vals[col]);
        }
        std::stable_sort(row.begin(), row.end(),
                         [](const std::pair<int32_t, double>& x, const std::pair<int32_t, double>& y) {
                           return x.first < y.first;
                         });
        int64_t k = start[i];
        for (size_t q = 0; q < row.size(); ++q) {
          if (k > start[i] && pc[k - 1] == row[q].first) { pv[k - 1] += row[q].second; continue; }
          pc[k] = row[q].first; pv[k] = row[q].second; ++k;
        }
        P.rs[i + 1] = k - start[i];
      }
    }
    for (int64_t i = 0; i < N; ++i) P.rs[i + 1] += P.rs[i];
    P.cols.resize(P.rs[N]);
    P.vals.resize(P.rs[N]);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
      const int64_t n = P.rs[i + 1] - P.rs[i];
      std::copy(pc.begin() + start[i], pc.begin() + start[i] + n, P.cols.begin() + P.rs[i]);
      std::copy(pv.begin() + start[i], pv.begin() + start[i] + n, P.vals.begin() + P.rs[i]);
    }
    L.P = std::move(P);
  } else {
    L.P = T;
  }
  L.R = transpose(L.P);
  HCSR AP = spmm(L.A, L.P);
  Lc.A = spmm(L.R, AP);
  diag_setup(Lc, rng);
  return LPG_OK;
}

// dense inverse by LU with partial pivoting (row-major, in place)
static int dense_inverse(int64_t n, std::vector<double>& A) {
  std::vector<double> LU(A);
  std::vector<int64_t> piv(n);
  for (int64_t k = 0; k < n; ++k) {
    int64_t p = k;
    double amax = std::fabs(LU[k * n + k]);
    for (int64_t i = k + 1; i < n; ++i)
      if (std::fabs(LU[i * n + k]) > amax) { amax = std::fabs(LU[i * n + k]); p = i; }
    piv[k] = p;
    if (amax == 0.0) return set_error(LPG_ERR_INVALID, "AMG coarse matrix is singular");
    if (p != k)
      for (int64_t j = 0; j < n; ++j) std::swap(LU[k * n + j], LU[p * n + j]);
    const double inv = 1.0 / LU[k * n + k];
#pragma omp parallel for schedule(static)
    for (int64_t i = k + 1; i < n; ++i) {
      const double l = LU[i * n + k] * inv;
      LU[i * n + k] = l;
      if (l != 0.0)
        for (int64_t j = k + 1; j < n; ++j) LU[i * n + j] -= l * LU[k * n + j];
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < n; ++j) {
    std::vector<double> col(n, 0.0);
    col[j] = 1.0;
    for (int64_t k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(col[k], col[piv[k]]);
    for (int64_t i = 0; i < n; ++i) {
      double s = col[i];
      for (int64_t q = 0; q < i; ++q) s -= LU[i * n + q] * col[q];
      col[i] = s;
    }
    for (int64_t i = n - 1; i >= 0; --i) {
      double s = col[i];
      for (int64_t q = i + 1; q < n; ++q) s -= LU[i * n + q] * col[q];
      col[i] = s / LU[i * n + i];
    }
    for (int64_t i = 0; i < n; ++i) A[i * n + j] = col[i];
  }
  return LPG_OK;
}

// ================================================================ p-level
struct PLevel {
  Elliptic* el = nullptr;
  Elliptic* elC = nullptr;
  int Nf = 0, Nc = 0;
  double lambda0 = 0, lambda1 = 0;
  DevBuf<double> invDiag64, P64;
  DevBuf<float> invDiag32, P32;
  DevBuf<double> rhs64, x64, res64;  // this level's vectors (levels > 0 own rhs/x)
  DevBuf<float> rhs32, x32, res32;
};

class MultiGrid : public Precon {
 public:
  Platform* plat = nullptr;
  Elliptic* fine = nullptr;
  MGOptions opt;
  std::vector<std::unique_ptr<Elliptic>> owned;
  std::vector<std::unique_ptr<PLevel>> p;
  std::vector<std::unique_ptr<ALevel>> a;
  DevBuf<double> coarseInv;
  int64_t coarseN = 0;
  // smoother scratch (largest p-level)
  DevBuf<double> s64[3];
  DevBuf<float> s32[3];
  // coarse vectors of the last p-level, FP64 view for the AMG hierarchy
  DevBuf<double> aRhs0, aX0;
  DevBuf<float> in32, out32;

  // learned fine-level smoother; per fine dof: lcoef = weight / diag (the network
  // correction's scaling) and ljac = (4/3/rho) / diag (its damped-Jacobi part), FP64 and FP32
  LearnedSmoother* learned = nullptr;
  BoxNumbering box{};
  double threshold = 0.5;
  int64_t nFallback = 0, nVcycle = 0, nTimeout = 0;
  DevBuf<double> lcoef64, ljac64;
  DevBuf<float> lcoef32, ljac32;

  int levels_p() const override { return (int)p.size(); }
  int levels_amg() const override { return (int)a.size(); }
  int64_t coarse_n() const override { return coarseN; }
  int64_t fallbacks() const override { return nFallback; }
  int64_t learned_timeouts() const override { return nTimeout; }
  int64_t vcycles() const override { return nVcycle; }
  double fine_rho() const override {
    if (p.empty()) return 0;
    return opt.smoother == 0 ? p[0]->lambda1 : (4.0 / 3.0) / p[0]->lambda0;
  }
  int set_learned(LearnedSmoother* L, const BoxNumbering& b, double thr) override {
    if (p.empty()) return set_error(LPG_ERR_UNSUPPORTED, "a learned smoother needs at least one p-level");
    if (fine->mesh.N != 7) return set_error(LPG_ERR_UNSUPPORTED, "the learned smoother is defined for N = 7");
    learned = L;
    box = b;
    threshold = thr;
    nFallback = nVcycle = nTimeout = 0;
    if (!L) return LPG_OK;
    // 1/diag of the fine level (the damped-Jacobi smoother stores it pre-scaled by 4/3/rho)
    PLevel& F = *p[0];
    const int64_t N = fine->Nglobal;
    const double unscale = (opt.smoother == 1) ? 1.0 / F.lambda0 : 1.0;
    const double jw = fine_rho() > 0 ? (4.0 / 3.0) / fine_rho() : 0.0;
    cudaStream_t s = plat->stream;
    int rc;
    if ((rc = lcoef64.alloc(N)) || (rc = ljac64.alloc(N)) || (rc = lcoef32.alloc(N)) || (rc = ljac32.alloc(N)))
      return rc;
    if ((rc = amxpy<double>(N, unscale, F.invDiag64.p, fine->weightG.p, 0.0, lcoef64.p, s)) ||
        (rc = axpy<double>(N, unscale * jw, F.invDiag64.p, 0.0, ljac64.p, s)) ||
        (rc = convert<double, float>(N, lcoef64.p, lcoef32.p, s)) || (rc = convert<double, float>(N, ljac64.p, ljac32.p, s)))
      return rc;
    LPG_CUDA_TRY(cudaStreamSynchronize(s));
    return LPG_OK;
  }

  int setup(Elliptic* el, const MeshConfig& c, const MGOptions& o);
  int apply(const double* r, double* z, cudaStream_t s) override;
  int apply_mixed(const double* r, double* z, const float** z32, cudaStream_t s) override;
  uint64_t rngAfter = 0;   // state of the random stream when setup finished

 private:
  bool f32() const { return opt.prec != Prec::F64; }
  template <typename T> T* vec(DevBuf<double>& d, DevBuf<float>& f);
  template <typename T> int op(Elliptic* el, const T* q, T* Aq, cudaStream_t s);
  template <typename T> int residual(Elliptic* el, const T* RHS, const T* X, T* RES, cudaStream_t s);
  template <typename T> int smooth(PLevel& L, const T* r, T* x, bool xIsZero, cudaStream_t s);
  template <typename T> int vcycle_p(int k, const T* rhs, T* x, cudaStream_t s);
  template <typename T> int coarse_correct(int k, const T* RES, T* X, cudaStream_t s);
  template <typename T> int vcycle_learned(const T* rhs, T* x, cudaStream_t s);
  template <typename T> int dot_host(int64_t n, const T* x, const T* y, double& out, cudaStream_t s);
  int vcycle_a(int k, const double* rhs, double* x, cudaStream_t s);
  int smooth_a(ALevel& L, const double* b, double* x, bool xIsZero, cudaStream_t s);
  int setup_amg(Elliptic* el, Rand48& rng);
};

template <> double* MultiGrid::vec<double>(DevBuf<double>& d, DevBuf<float>&) { return d.p; }
template <> float* MultiGrid::vec<float>(DevBuf<double>&, DevBuf<float>& f) { return f.p; }

template <>
int MultiGrid::op<double>(Elliptic* el, const double* q, double* Aq, cudaStream_t s) {
  return el->Operator(q, Aq, s);
}
template <>
int MultiGrid::op<float>(Elliptic* el, const float* q, float* Aq, cudaStream_t s) {
  return el->OperatorF32(q, Aq, opt.prec, s);
}

// RES = RHS - A X. The C0 FP32 operator assembles straight into a copy of RHS with the
// sign of the contributions flipped (one copy instead of a memset and an axpy pass).
template <>
int MultiGrid::residual<double>(Elliptic* el, const double* RHS, const double* X, double* RES, cudaStream_t s) {
  int rc;
  if ((rc = el->Operator(X, RES, s))) return rc;
  return axpy<double>(el->Nglobal, 1.0, RHS, -1.0, RES, s);
}
template <>
int MultiGrid::residual<float>(Elliptic* el, const float* RHS, const float* X, float* RES, cudaStream_t s) {
  int rc;
  if (el->ipdg) {
    if ((rc = el->OperatorF32(X, RES, opt.prec, s))) return rc;
    return axpy<float>(el->Nglobal, 1.f, RHS, -1.f, RES, s);
  }
  LPG_CUDA_TRY(cudaMemcpyAsync(RES, RHS, sizeof(float) * el->Nglobal, cudaMemcpyDeviceToDevice, s));
  return el->OperatorF32(X, RES, opt.prec, s, -1.f);
}

// ---------------------------------------------------------------- p-level smoothing
// LPG_CHEB=unfused (a tuning override): the FP32 Chebyshev steps with a separate A d vector
static bool cheb_unfused() {
  static const bool v = [] {
    const char* e = std::getenv("LPG_CHEB");
    return e && !std::strcmp(e, "unfused");
  }();
  return v;
}

template <typename T>
int MultiGrid::smooth(PLevel& L, const T* r, T* X, bool xIsZero, cudaStream_t s) {
  const int64_t N = L.el->Nglobal;
  T* invDiag = vec<T>(L.invDiag64, L.invDiag32);
  T* RES = vec<T>(s64[0], s32[0]);
  T* Ad = vec<T>(s64[1], s32[1]);
  T* d = vec<T>(s64[2], s32[2]);
  int rc;
  if (opt.smoother == 1) {  // damped Jacobi, invDiag pre-scaled by 4/3/rho
    if (xIsZero) return amxpy<T>(N, T(1), invDiag, r, T(0), X, s);
    if ((rc = op<T>(L.el, X, RES, s))) return rc;
    if ((rc = axpy<T>(N, T(1), r, T(-1), RES, s))) return rc;
    return amxpy<T>(N, T(1), invDiag, RES, T(1), X, s);
  }
  const double theta = 0.5 * (L.lambda1 + L.lambda0);
  const double delta = 0.5 * (L.lambda1 - L.lambda0);
  const double invTheta = 1.0 / theta;
  const double sigma = theta / delta;
  double rho_n = 1. / sigma, rho_np1;
  // same recurrence as the reference's loop (x += d before each application of A, and
  // once at the end), with each x += d fused into the pass that produced d
  if (!xIsZero && (rc = op<T>(L.el, X, RES, s))) return rc;
  // FP32 C0 levels: the smoother keeps the unscaled residual u = r - A x, which the
  // operator updates in place (u -= A d, assembled straight into it): no A d vector and no
  // memset of it, and each step pass reads 4 vectors and writes 2 instead of 5 and 3
  const bool fused = std::is_same<T, float>::value && !L.el->ipdg && !cheb_unfused();
  bool started = false;
  if constexpr (std::is_same<T, float>::value) {
    if (fused) {
      if ((rc = cheb_start_u<T>(N, invDiag, r, xIsZero ? nullptr : RES, RES, d, X, (T)invTheta, xIsZero, s)))
        return rc;
      started = true;
    }
  }
  if (!started && (rc = cheb_start<T>(N, invDiag, r, xIsZero ? nullptr : RES, RES, d, X, (T)invTheta, xIsZero, s)))
    return rc;
  for (int k = 0; k < opt.chebDegree; ++k) {
    rho_np1 = 1.0 / (2. * sigma - rho_n);
    const double rhoDivDelta = 2.0 * rho_np1 / delta;
    const bool last = (k == opt.chebDegree - 1);   // the last step's res and d are not read again
    if constexpr (std::is_same<T, float>::value) {
      if (fused) {
        if ((rc = L.el->OperatorF32(d, RES, opt.prec, s, -1.f))) return rc;
        if ((rc = cheb_step_u<T>(N, invDiag, RES, d, X, (T)(rho_np1 * rho_n), (T)rhoDivDelta, s, last))) return rc;
        rho_n = rho_np1;
        continue;
      }
    }
    if ((rc = op<T>(L.el, d, Ad, s))) return rc;
    if ((rc = cheb_step<T>(N, invDiag, Ad, RES, d, X, (T)(rho_np1 * rho_n), (T)rhoDivDelta, s, last))) return rc;
    rho_n = rho_np1;
  }
  return LPG_OK;
}

template <typename T>
int MultiGrid::vcycle_p(int k, const T* RHS, T* X, cudaStream_t s) {
  PLevel& L = *p[k];
  const int64_t N = L.el->Nglobal;
  T* RES = vec<T>(L.res64, L.res32);
  int rc;
  if ((rc = smooth<T>(L, RHS, X, true, s))) return rc;
  if ((rc = residual<T>(L.el, RHS, X, RES, s))) return rc;
  if ((rc = coarse_correct<T>(k, RES, X, s))) return rc;
  return smooth<T>(L, RHS, X, false, s);
}

// X += P (coarse-level V-cycle of the restricted residual RES)
template <typename T>
int MultiGrid::coarse_correct(int k, const T* RES, T* X, cudaStream_t s) {
  PLevel& L = *p[k];
  int rc;
  const bool last = (k + 1 == (int)p.size());
  T* weight = vec<T>(L.el->weightG, L.el->weightG32);
  const T* P = vec<T>(L.P64, L.P32);
  if (!last) {
    T* rhsC = vec<T>(p[k + 1]->rhs64, p[k + 1]->rhs32);
    T* xC = vec<T>(p[k + 1]->x64, p[k + 1]->x32);
    if ((rc = pmg_coarsen<T>(L.Nf, L.Nc, L.el->mesh.E, L.el->g2l.p, weight, RES, P, L.elC->g2l.p, rhsC,
                             L.elC->Nglobal, s)))
      return rc;
    if ((rc = vcycle_p<T>(k + 1, rhsC, xC, s))) return rc;
    if ((rc = pmg_prolongate_map<T>(L.Nf, L.Nc, L.el->mesh.E, L.elC->g2l.p, xC, P, L.el->g2l.p, L.el->owner.p,
                                    X, s)))
      return rc;
  } else {
    // coarse space of the last p-level = level 0 of the FP64 AMG hierarchy
    const int64_t NC = L.elC->Nglobal;
    const T* xCT = nullptr;
    if constexpr (std::is_same<T, double>::value) {
      if ((rc = pmg_coarsen<T>(L.Nf, L.Nc, L.el->mesh.E, L.el->g2l.p, weight, RES, P, L.elC->g2l.p, aRhs0.p, NC,
                               s)))
        return rc;
      if ((rc = vcycle_a(0, aRhs0.p, aX0.p, s))) return rc;
      xCT = aX0.p;
    } else {
      if ((rc = pmg_coarsen<T>(L.Nf, L.Nc, L.el->mesh.E, L.el->g2l.p, weight, RES, P, L.elC->g2l.p, in32.p, NC,
                               s)))
        return rc;
      if ((rc = convert<float, double>(NC, in32.p, aRhs0.p, s))) return rc;
      if ((rc = vcycle_a(0, aRhs0.p, aX0.p, s))) return rc;
      if ((rc = convert<double, float>(NC, aX0.p, out32.p, s))) return rc;
      xCT = out32.p;
    }
    if ((rc = pmg_prolongate_map<T>(L.Nf, L.Nc, L.el->mesh.E, L.elC->g2l.p, xCT, P, L.el->g2l.p, L.el->owner.p, X,
                                    s)))
      return rc;
  }
  return LPG_OK;
}

template <typename T>
int MultiGrid::dot_host(int64_t n, const T* x, const T* y, double& out, cudaStream_t s) {
  int rc;
  if constexpr (std::is_same<T, double>::value) rc = dot(n, x, y, plat->scalars.p + 2, plat->partials.p, s);
  else rc = dot_f32(n, x, y, plat->scalars.p + 2, plat->partials.p, s);
  if (rc) return rc;
  LPG_CUDA_TRY(cudaMemcpyAsync(plat->hostScalars + 2, plat->scalars.p + 2, sizeof(double), cudaMemcpyDeviceToHost, s));
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  out = plat->hostScalars[2];
  return LPG_OK;
}

// V-cycle whose fine-level smoother is S(r) = (4/3/rho) D^{-1} r + L(r), a damped-Jacobi
// step plus the learned element-local correction L. A smoothing step takes c = S(RES)
// with the energy-optimal step w = (c.RES)/(c.Ac) (w = 0 if c.Ac <= 0): X += w c,
// RES -= w A c. Pre- and post-smoothing are opt.learnedSteps such steps around the
// coarse correction (X = 0, RES = RHS at the start). If the V-cycle leaves
// ||RHS - A X|| > threshold ||RHS||, it is redone with the plain smoother (fallback),
// and the fallback is counted.
template <typename T>
int MultiGrid::vcycle_learned(const T* RHS, T* X, cudaStream_t s) {
  PLevel& L = *p[0];
  Elliptic* el = L.el;
  const int64_t N = el->Nglobal, E = el->mesh.E;
  T* RES = vec<T>(L.res64, L.res32);
  T* AD = vec<T>(s64[1], s32[1]);
  T* D = vec<T>(s64[2], s32[2]);
  const T* coef = vec<T>(lcoef64, lcoef32);
  const T* jac = vec<T>(ljac64, ljac32);
  int rc;
  // floor of the element scales: kScaleFloor x the RMS of the V-cycle's right-hand side
  double bb;
  if ((rc = dot_host<T>(N, RHS, RHS, bb, s))) return rc;
  const float sfloor = (float)(LearnedSmoother::kScaleFloor * std::sqrt(bb / (double)std::max<int64_t>(N, 1)));
  auto smooth_step = [&]() -> int {
    int r;
    // c = (4/3/rho) D^{-1} RES + network correction; AD = A c
    if ((r = amxpy<T>(N, T(1), jac, RES, T(0), D, s))) return r;
    if ((r = learned->apply<T>(box, E, el->g2l.p, RES, coef, D, N, sfloor, s))) return r;
    if ((r = op<T>(el, D, AD, s))) return r;
    // w = (c.RES)/(c.Ac) from one two-product pass; X += w c, RES -= w A c in one pass,
    // which reads the two products from device memory (no host round trip per step)
    if ((r = dot2<T>(N, D, RES, AD, plat->scalars.p + 2, plat->partials.p, s))) return r;
    return update2_dev<T>(N, plat->scalars.p + 2, D, AD, X, RES, s);
  };
  // a tensor-core pipeline timeout inside the network (LPG_ERR_TIMEOUT) abandons the
  // learned attempt: the V-cycle is redone with the plain smoother and counted
  auto learned_part = [&]() -> int {
    int r;
    if ((r = learned->clear_tc(s))) return r;
    LPG_CUDA_TRY(cudaMemsetAsync(X, 0, sizeof(T) * N, s));
    LPG_CUDA_TRY(cudaMemcpyAsync(RES, RHS, sizeof(T) * N, cudaMemcpyDeviceToDevice, s));
    for (int k = 0; k < opt.learnedSteps; ++k)
      if ((r = smooth_step())) return r;
    if ((r = coarse_correct<T>(0, RES, X, s))) return r;
    if ((r = residual<T>(el, RHS, X, RES, s))) return r;
    for (int k = 0; k < opt.learnedSteps; ++k)
      if ((r = smooth_step())) return r;
    // the network's tensor-core status, once per V-cycle (a timeout discards the V-cycle)
    return learned->check_tc(s);
  };
  rc = learned_part();
  if (rc == LPG_ERR_TIMEOUT) {
    nVcycle++;
    nFallback++;
    nTimeout++;
    return vcycle_p<T>(0, RHS, X, s);
  }
  if (rc) return rc;
  // residual reduction of this V-cycle
  double rr;
  if ((rc = dot_host<T>(N, RES, RES, rr, s))) return rc;
  nVcycle++;
  if (!(rr <= threshold * threshold * bb)) {
    nFallback++;
    return vcycle_p<T>(0, RHS, X, s);
  }
  return LPG_OK;
}

// ---------------------------------------------------------------- AMG V-cycle (device)
int MultiGrid::smooth_a(ALevel& L, const double* b, double* x, bool xIsZero, cudaStream_t s) {
  const int64_t N = L.A.n;
  int rc;
  if (opt.amgSmoother == 1) {
    if (xIsZero) return amxpy<double>(N, L.jlambda, L.dDiagInv.p, b, 0.0, x, s);
    // d = lambda D^{-1}(b - A x); x += d
    if ((rc = csr_cheb_residual(N, L.dA.rs.p, L.dA.cols.p, L.dA.vals.p, 0.0, 1.0, L.dDiagInv.p, b, x, L.s1.p, s)))
      return rc;
    return axpy<double>(N, L.jlambda, L.s1.p, 1.0, x, s);
  }
  const double theta = 0.5 * (L.lambda1 + L.lambda0);
  const double delta = 0.5 * (L.lambda1 - L.lambda0);
  const double invTheta = 1.0 / theta;
  const double sigma = theta / delta;
  double rho_n = 1. / sigma, rho_np1;
  double* d = L.s1.p;
  double* r = L.s2.p;
  if (xIsZero) {
    if ((rc = csr_cheb_start(N, invTheta, L.dDiagInv.p, b, r, d, x, s))) return rc;
  } else {
    if ((rc = csr_cheb_residual(N, L.dA.rs.p, L.dA.cols.p, L.dA.vals.p, 0.0, 1.0, L.dDiagInv.p, b, x, r, s))) return rc;
    if ((rc = csr_cheb_update(N, 0.0, invTheta, opt.amgChebDegree == 0, r, d, x, s))) return rc;
  }
  for (int k = 0; k < opt.amgChebDegree; ++k) {
    if ((rc = csr_cheb_residual(N, L.dA.rs.p, L.dA.cols.p, L.dA.vals.p, 1.0, 0.0, L.dDiagInv.p, b, d, r, s))) return rc;
    rho_np1 = 1.0 / (2. * sigma - rho_n);
    if ((rc = csr_cheb_update(N, rho_np1 * rho_n, 2.0 * rho_np1 / delta, k == opt.amgChebDegree - 1, r, d, x, s)))
      return rc;
    rho_n = rho_np1;
  }
  return LPG_OK;
}

int MultiGrid::vcycle_a(int k, const double* RHS, double* X, cudaStream_t s) {
  if (k == (int)a.size() - 1) return gemv(coarseN, coarseInv.p, RHS, X, s);
  ALevel& L = *a[k];
  ALevel& C = *a[k + 1];
  const int64_t N = L.A.n;
  int rc;
  if ((rc = smooth_a(L, RHS, X, true, s))) return rc;
  if ((rc = csr_spmv(N, L.dA.rs.p, L.dA.cols.p, L.dA.vals.p, -1.0, X, 0.0, L.res.p, s))) return rc;
  if ((rc = axpy<double>(N, 1.0, RHS, 1.0, L.res.p, s))) return rc;
  if ((rc = csr_spmv(L.R.n, L.dR.rs.p, L.dR.cols.p, L.dR.vals.p, 1.0, L.res.p, 0.0, C.rhs.p, s))) return rc;
  if ((rc = vcycle_a(k + 1, C.rhs.p, C.x.p, s))) return rc;
  if ((rc = csr_spmv(N, L.dP.rs.p, L.dP.cols.p, L.dP.vals.p, 1.0, C.x.p, 1.0, X, s))) return rc;
  return smooth_a(L, RHS, X, false, s);
}

int MultiGrid::apply(const double* r, double* z, cudaStream_t s) {
  int rc;
  if (p.empty()) {
    rc = vcycle_a(0, r, z, s);
  } else if (!f32()) {
    rc = learned ? vcycle_learned<double>(r, z, s) : vcycle_p<double>(0, r, z, s);
  } else {
    const int64_t N = fine->Nglobal;
    PLevel& L0 = *p[0];
    if ((rc = convert<double, float>(N, r, L0.rhs32.p, s))) return rc;
    if (learned) rc = vcycle_learned<float>(L0.rhs32.p, L0.x32.p, s);
    else rc = vcycle_p<float>(0, L0.rhs32.p, L0.x32.p, s);
    if (rc) return rc;
    rc = convert<float, double>(N, L0.x32.p, z, s);
  }
  if (rc) return rc;
  if (fine->allNeumann) {  // ZeroMean (ellipticZeroMean.cpp:29-37)
    if ((rc = sum(fine->Nglobal, z, plat->scalars.p + 1, plat->partials.p, s))) return rc;
    rc = add_scalar(fine->Nglobal, plat->scalars.p + 1, -fine->allNeumannScale * fine->allNeumannScale, z, s);
  }
  return rc;
}

// FP32 p-levels: the V-cycle's FP32 result is handed to the Krylov loop as it is (no FP64
// copy); all-Neumann problems take the FP64 path, whose zero-mean step works on z
int MultiGrid::apply_mixed(const double* r, double* z, const float** z32, cudaStream_t s) {
  *z32 = nullptr;
  if (p.empty() || !f32() || fine->allNeumann) return apply(r, z, s);
  const int64_t N = fine->Nglobal;
  PLevel& L0 = *p[0];
  int rc;
  if ((rc = convert<double, float>(N, r, L0.rhs32.p, s))) return rc;
  if (learned) rc = vcycle_learned<float>(L0.rhs32.p, L0.x32.p, s);
  else rc = vcycle_p<float>(0, L0.rhs32.p, L0.x32.p, s);
  if (rc) return rc;
  *z32 = L0.x32.p;
  return LPG_OK;
}

// ---------------------------------------------------------------- setup
// LPG_SETUP_TIMES=1 prints the host setup phases of the AMG hierarchy to stderr
static void setup_time(const char* what, double& t0, int64_t a = -1, int64_t b = -1) {
  static const bool on = std::getenv("LPG_SETUP_TIMES") != nullptr;
  const double t = omp_get_wtime();
  if (on) std::fprintf(stderr, "[lpg setup] %-22s %8.3f s  %lld %lld\n", what, t - t0, (long long)a, (long long)b);
  t0 = t;
}

int MultiGrid::setup_amg(Elliptic* el, Rand48& rng) {
  cudaStream_t s = plat->stream;
  double t0 = omp_get_wtime();
  auto L0 = std::make_unique<ALevel>();
  int rc = el->BuildMatrix(L0->A.rs, L0->A.cols, L0->A.vals, s);
  if (rc) return rc;
  L0->A.n = L0->A.m = el->Nglobal;
  setup_time("matrix", t0, L0->A.n, L0->A.nnz());
  diag_setup(*L0, rng);
  setup_time("level 0 smoother", t0);
  a.push_back(std::move(L0));
  const int64_t Nrows = a[0]->A.n;
  std::vector<double> nullv(Nrows, 1.0 / std::sqrt((double)Nrows));
  const int64_t target = 1000;
  int64_t globalSize = Nrows;
  double theta = opt.amgRugeStuben ? 0.5 : 0.08;
  if (globalSize > target) {
    for (;;) {
      ALevel& L = *a.back();
      if (opt.amgSmoother == 1) L.jlambda = (4. / 3.) / L.rho;
      else { L.lambda1 = L.rho; L.lambda0 = L.rho / 10.; }
      auto Lc = std::make_unique<ALevel>();
      if ((rc = amg_coarsen(L, *Lc, nullv, theta, opt.amgRugeStuben, opt.amgUnsmoothed, rng))) return rc;
      setup_time("coarsen", t0, Lc->A.n, Lc->A.nnz());
      a.push_back(std::move(Lc));
      if (!opt.amgRugeStuben) theta /= 2;
      const int64_t coarseSize = a.back()->A.n;
      if (coarseSize <= target || globalSize < 2 * coarseSize) break;
      globalSize = coarseSize;
    }
  }
  // exact coarse solver: dense inverse (+ null-space penalty for all-Neumann problems)
  ALevel& B = *a.back();
  coarseN = B.A.n;
  std::vector<double> dense(coarseN * coarseN, 0.0);
  for (int64_t i = 0; i < coarseN; ++i)
    for (int64_t j = B.A.rs[i]; j < B.A.rs[i + 1]; ++j) dense[i * coarseN + B.A.cols[j]] = B.A.vals[j];
  if (el->allNeumann)
    for (int64_t i = 0; i < coarseN; ++i)
      for (int64_t j = 0; j < coarseN; ++j) dense[i * coarseN + j] += nullv[i] * nullv[j];
  if ((rc = dense_inverse(coarseN, dense))) return rc;
  setup_time("coarse inverse", t0, coarseN);
  if ((rc = coarseInv.alloc(coarseN * coarseN)) || (rc = coarseInv.upload(dense.data(), coarseN * coarseN, s))) return rc;
  // device copies and work vectors
  for (size_t k = 0; k < a.size(); ++k) {
    ALevel& L = *a[k];
    const int64_t n = L.A.n;
    if ((rc = L.rhs.alloc(n)) || (rc = L.x.alloc(n)) || (rc = L.res.alloc(n)) || (rc = L.s1.alloc(n)) ||
        (rc = L.s2.alloc(n)))
      return rc;
    if (k + 1 < a.size()) {
      if ((rc = L.dA.upload(L.A, s)) || (rc = L.dP.upload(L.P, s)) || (rc = L.dR.upload(L.R, s))) return rc;
      if ((rc = L.dDiagInv.alloc(n)) || (rc = L.dDiagInv.upload(L.diagInv.data(), n, s))) return rc;
    }
  }
  return LPG_OK;
}

int MultiGrid::setup(Elliptic* el, const MeshConfig& c, const MGOptions& o) {
  fine = el;
  plat = el->plat;
  opt = o;
  cudaStream_t s = plat->stream;
  Rand48 rng;
  rng.seed(0);  // srand48(rank) in buildParAlmondKernels (parAlmondKernels.cpp:55-58)
  if (o.rngGiven) rng.x = o.rngState;
  int rc;
  struct SaveRng {
    uint64_t& out;
    Rand48& r;
    ~SaveRng() { out = r.x; }
  } saveRng{rngAfter, rng};
  if (o.amgOnly) {
    if (o.semfem) {
      // SEMFEMPrecon (ellipticPreconSEMFEM.cpp:56-247, hexahedra): parAlmond on the
      // low-order matrix, applied to the degree-N vectors directly
      auto fem = std::make_unique<Elliptic>();
      if ((rc = fem->setup_semfem(*el, s))) return rc;
      rc = setup_amg(fem.get(), rng);
      fem.reset();   // the AMG levels own their matrices; the sub-mesh is no longer needed
      return rc;
    }
    if ((rc = setup_amg(el, rng))) return rc;
    return LPG_OK;
  }
  const std::vector<int>& deg = o.degrees;
  Elliptic* cur = el;
  size_t maxN = 0;
  for (size_t l = 0; l + 1 < deg.size(); ++l) {
    auto L = std::make_unique<PLevel>();
    L->el = cur;
    L->Nf = deg[l];
    L->Nc = deg[l + 1];
    const int64_t N = cur->Nglobal;
    maxN = std::max<size_t>(maxN, (size_t)N);
    // smoother setup (SetupSmoother, ellipticPreconMultiGridLevel.cpp:345-383)
    DevBuf<double> diag;
    if ((rc = diag.alloc(N)) || (rc = cur->BuildDiagonal(diag.p, s))) return rc;
    if ((rc = L->invDiag64.alloc(N)) || (rc = inverse_f64(N, diag.p, L->invDiag64.p, s))) return rc;
    {
      // maxEigSmoothAx (ellipticPreconMultiGridLevel.cpp:393-473), FP64 on the device
      int k = 10;
      if (k > N) k = (int)N;
      std::vector<double> H(k * k, 0.0), Vx(N);
      for (int64_t i = 0; i < N; ++i) Vx[i] = rng.next();
      std::vector<std::unique_ptr<DevBuf<double>>> V;
      for (int i = 0; i <= k; ++i) {
        V.push_back(std::make_unique<DevBuf<double>>());
        if ((rc = V.back()->alloc(N))) return rc;
      }
      DevBuf<double> AVx;
      if ((rc = AVx.alloc(N)) || (rc = AVx.upload(Vx.data(), N, s))) return rc;
      double nrm2;
      if ((rc = plat->norm2sq(N, AVx.p, nrm2))) return rc;
      if ((rc = axpy<double>(N, 1. / std::sqrt(nrm2), AVx.p, 0.0, V[0]->p, s))) return rc;
      for (int j = 0; j < k; ++j) {
        if ((rc = cur->Operator(V[j]->p, AVx.p, s))) return rc;
        if ((rc = amxpy<double>(N, 1.0, L->invDiag64.p, AVx.p, 0.0, V[j + 1]->p, s))) return rc;
        for (int i = 0; i <= j; ++i) {
          double hij;
          if ((rc = plat->dot(N, V[i]->p, V[j + 1]->p, hij))) return rc;
          if ((rc = axpy<double>(N, -hij, V[i]->p, 1.0, V[j + 1]->p, s))) return rc;
          H[i + j * k] = hij;
        }
        if (j + 1 < k) {
          double nj2;
          if ((rc = plat->norm2sq(N, V[j + 1]->p, nj2))) return rc;
          const double nj = std::sqrt(nj2);
          if ((rc = axpy<double>(N, 0.0, V[j + 1]->p, 1.0 / nj, V[j + 1]->p, s))) return rc;
          H[j + 1 + j * k] = nj;
        }
      }
      const double rho = hessenberg_spectral_radius(k, H);
      if (o.smoother == 0) {
        L->lambda1 = rho;
        L->lambda0 = rho / 10.;
      } else {
        L->lambda0 = (4. / 3.) / rho;
        if ((rc = axpy<double>(N, 0.0, L->invDiag64.p, L->lambda0, L->invDiag64.p, s))) return rc;
      }
    }
    std::vector<double> P;
    gll_interpolation(L->Nc, L->Nf, P);
    if ((rc = L->P64.alloc((int64_t)P.size())) || (rc = L->P64.upload(P.data(), (int64_t)P.size(), s))) return rc;
    // next (coarser) level
    auto next = std::make_unique<Elliptic>();
    if ((rc = next->setup(plat, c, L->Nc, el->lambda, el->hasLambdaE ? &el->lambdaE_h : nullptr, s))) return rc;
    L->elC = next.get();
    cur = next.get();
    owned.push_back(std::move(next));
    p.push_back(std::move(L));
  }
  if ((rc = setup_amg(cur, rng))) return rc;
  // work vectors and reduced-precision copies
  const int64_t NC = cur->Nglobal;
  if ((rc = aRhs0.alloc(NC)) || (rc = aX0.alloc(NC))) return rc;
  for (size_t k = 0; k < p.size(); ++k) {
    PLevel& L = *p[k];
    const int64_t N = L.el->Nglobal;
    if (!f32()) {
      if ((rc = L.res64.alloc(N))) return rc;
      if (k > 0 && ((rc = L.rhs64.alloc(N)) || (rc = L.x64.alloc(N)))) return rc;
    } else {
      if ((rc = L.el->make_f32(opt.prec == Prec::BF16G, s))) return rc;
      if ((rc = L.res32.alloc(N)) || (rc = L.rhs32.alloc(N)) || (rc = L.x32.alloc(N))) return rc;
      if ((rc = L.invDiag32.alloc(N)) || (rc = convert<double, float>(N, L.invDiag64.p, L.invDiag32.p, s))) return rc;
      if ((rc = L.P32.alloc(L.P64.n)) || (rc = convert<double, float>(L.P64.n, L.P64.p, L.P32.p, s))) return rc;
      if (k > 0) L.invDiag64.release();  // the fine level keeps FP64 1/diag for a learned smoother
    }
  }
  if (f32()) {
    if ((rc = in32.alloc(NC)) || (rc = out32.alloc(NC))) return rc;
    for (int i = 0; i < 3; ++i)
      if ((rc = s32[i].alloc((int64_t)maxN))) return rc;
  } else {
    for (int i = 0; i < 3; ++i)
      if ((rc = s64[i].alloc((int64_t)maxN))) return rc;
  }
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  return LPG_OK;
}

std::unique_ptr<Precon> make_multigrid(Elliptic* el, const MeshConfig& c, const MGOptions& o, int* status) {
  auto mg = std::make_unique<MultiGrid>();
  *status = mg->setup(el, c, o);
  if (*status) return nullptr;
  return mg;
}

// ================================================================ OAS
// OASPrecon (ellipticPreconOAS.cpp:30-223) on one rank: the one-ring patch is the whole
// mesh, so the patch solve is this problem's p-multigrid V-cycle; the coarse problem is the
// degree-1 problem with its own AMG (set up after the patch hierarchy on the same random
// stream), reached by a direct N -> 1 transfer and added to the patch solution.
class OASPrecon : public Precon {
 public:
  Elliptic* el = nullptr;
  std::unique_ptr<MultiGrid> patch;
  std::unique_ptr<Elliptic> elC;
  std::unique_ptr<MultiGrid> coarse;
  DevBuf<double> P64, rC, zC;

  int levels_p() const override { return patch ? patch->levels_p() : 0; }
  int levels_amg() const override { return coarse ? coarse->levels_amg() : 0; }
  int64_t coarse_n() const override { return coarse ? coarse->coarse_n() : 0; }

  int setup(Elliptic* e, const MeshConfig& c, const MGOptions& o) {
    el = e;
    cudaStream_t s = e->plat->stream;
    const int N = e->mesh.N;
    int rc;
    MGOptions oc = o;
    oc.amgOnly = true;
    oc.semfem = false;
    oc.prec = Prec::F64;
    if (N > 1) {
      patch = std::make_unique<MultiGrid>();
      MGOptions op = o;
      op.amgOnly = false;
      op.semfem = false;
      if ((rc = patch->setup(e, c, op))) return rc;
      oc.rngGiven = true;
      oc.rngState = patch->rngAfter;
      elC = std::make_unique<Elliptic>();
      if ((rc = elC->setup(e->plat, c, 1, e->lambda, e->hasLambdaE ? &e->lambdaE_h : nullptr, s))) return rc;
      coarse = std::make_unique<MultiGrid>();
      if ((rc = coarse->setup(elC.get(), c, oc))) return rc;
      std::vector<double> P;
      gll_interpolation(1, N, P);
      if ((rc = P64.alloc((int64_t)P.size())) || (rc = P64.upload(P.data(), (int64_t)P.size(), s))) return rc;
      if ((rc = rC.alloc(elC->Nglobal)) || (rc = zC.alloc(elC->Nglobal))) return rc;
    } else {
      coarse = std::make_unique<MultiGrid>();
      if ((rc = coarse->setup(e, c, oc))) return rc;
    }
    LPG_CUDA_TRY(cudaStreamSynchronize(s));
    return LPG_OK;
  }

  int apply(const double* r, double* z, cudaStream_t s) override {
    if (!patch) return coarse->apply(r, z, s);
    int rc;
    const int N = el->mesh.N;
    const int64_t E = el->mesh.E;
    if ((rc = patch->apply(r, z, s))) return rc;
    if ((rc = pmg_coarsen<double>(N, 1, E, el->g2l.p, el->weightG.p, r, P64.p, elC->g2l.p, rC.p, elC->Nglobal, s)))
      return rc;
    if ((rc = coarse->apply(rC.p, zC.p, s))) return rc;
    if ((rc = pmg_prolongate_map<double>(N, 1, E, elC->g2l.p, zC.p, P64.p, el->g2l.p, el->owner.p, z, s))) return rc;
    if (el->allNeumann) {
      Platform* plat = el->plat;
      if ((rc = sum(el->Nglobal, z, plat->scalars.p + 1, plat->partials.p, s))) return rc;
      rc = add_scalar(el->Nglobal, plat->scalars.p + 1, -el->allNeumannScale * el->allNeumannScale, z, s);
    }
    return rc;
  }
};

std::unique_ptr<Precon> make_oas(Elliptic* el, const MeshConfig& c, const MGOptions& o, int* status) {
  auto p = std::make_unique<OASPrecon>();
  *status = p->setup(el, c, o);
  if (*status) return nullptr;
  return p;
}

// ================================================================ Identity / Jacobi
class IdentityPrecon : public Precon {
 public:
  Elliptic* el;
  explicit IdentityPrecon(Elliptic* e) : el(e) {}
  int apply(const double* r, double* z, cudaStream_t s) override {
    LPG_CUDA_TRY(cudaMemcpyAsync(z, r, sizeof(double) * el->Nglobal, cudaMemcpyDeviceToDevice, s));
    return LPG_OK;
  }
};

class JacobiPrecon : public Precon {
 public:
  Elliptic* el;
  DevBuf<double> invDiag;
  explicit JacobiPrecon(Elliptic* e) : el(e) {}
  int apply(const double* r, double* z, cudaStream_t s) override {
    int rc = amxpy<double>(el->Nglobal, 1.0, invDiag.p, r, 0.0, z, s);
    if (rc) return rc;
    if (el->allNeumann) {
      Platform* plat = el->plat;
      if ((rc = sum(el->Nglobal, z, plat->scalars.p + 1, plat->partials.p, s))) return rc;
      rc = add_scalar(el->Nglobal, plat->scalars.p + 1, -el->allNeumannScale * el->allNeumannScale, z, s);
    }
    return rc;
  }
};

std::unique_ptr<Precon> make_identity(Elliptic* el) { return std::make_unique<IdentityPrecon>(el); }

std::unique_ptr<Precon> make_jacobi(Elliptic* el, int* status) {
  auto j = std::make_unique<JacobiPrecon>(el);
  DevBuf<double> diag;
  cudaStream_t s = el->plat->stream;
  int rc;
  if ((rc = diag.alloc(el->Nglobal)) || (rc = el->BuildDiagonal(diag.p, s)) || (rc = j->invDiag.alloc(el->Nglobal)) ||
      (rc = inverse_f64(el->Nglobal, diag.p, j->invDiag.p, s))) {
    *status = rc;
    return nullptr;
  }
  *status = LPG_OK;
  return j;
}

}  // namespace lpg
