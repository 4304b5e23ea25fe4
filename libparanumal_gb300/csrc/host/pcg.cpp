// (Flexible) preconditioned conjugate gradients: pcg::Solve / pcg::UpdatePCG
// (libs/linearSolver/linearSolverPCG.cpp:67-171). Vector updates and reductions run
// on the device; each inner product is copied to the host once, as the reference does,
// because the host decides alpha, beta and convergence.
#include "objects.hpp"

#include <algorithm>
#include <cmath>

namespace lpg {

int PCGWork::ensure(int64_t n) {
  if (p.n == n) return LPG_OK;
  int rc;
  if ((rc = p.alloc(n)) || (rc = z.alloc(n)) || (rc = Ax.alloc(n)) || (rc = Ap.alloc(n))) return rc;
  LPG_CUDA_TRY(cudaMemset(p.p, 0, sizeof(double) * n));
  LPG_CUDA_TRY(cudaMemset(Ap.p, 0, sizeof(double) * n));
  return LPG_OK;
}

int pcg_solve(Platform* plat, Elliptic* el, Precon* pc, PCGWork& w, bool flexible, bool stopRhs, double* x,
              double* r, double tol, int maxit, PCGResult& res) {
  const int64_t N = el->Nglobal;
  cudaStream_t s = plat->stream;
  int rc = w.ensure(N);
  if (rc) return rc;
  LPG_CUDA_TRY(cudaMemsetAsync(w.Ap.p, 0, sizeof(double) * N, s));
  double rdotz1 = 0, rdotz2 = 0, alpha = 0, beta = 0, pAp = 0, rdotr0 = 0, TOL = 0;
  if (stopRhs) {
    double nb2;
    if ((rc = plat->norm2sq(N, r, nb2))) return rc;
    TOL = std::max(tol * tol * nb2, tol * tol);
  }
  if ((rc = el->Operator(x, w.Ax.p, s))) return rc;
  if ((rc = axpy<double>(N, -1.0, w.Ax.p, 1.0, r, s))) return rc;
  if ((rc = plat->norm2sq(N, r, rdotr0))) return rc;
  if (!stopRhs) TOL = std::max(tol * tol * rdotr0, tol * tol);
  int iter;
  res.breakdown = false;
  for (iter = 0; iter < maxit; ++iter) {
    if ((iter == 0 && rdotr0 == 0.0) || (iter > 0 && rdotr0 <= TOL)) break;
    if ((rc = pc->apply(r, w.z.p, s))) return rc;
    rdotz2 = rdotz1;
    if ((rc = plat->dot(N, r, w.z.p, rdotz1))) return rc;
    if (flexible) {
      double zdotAp;
      if ((rc = plat->dot(N, w.z.p, w.Ap.p, zdotAp))) return rc;
      beta = (iter == 0) ? 0.0 : -alpha * zdotAp / rdotz2;
    } else {
      beta = (iter == 0) ? 0.0 : rdotz1 / rdotz2;
    }
    if ((rc = axpy<double>(N, 1.0, w.z.p, beta, w.p.p, s))) return rc;
    if ((rc = el->Operator(w.p.p, w.Ap.p, s))) return rc;
    if ((rc = plat->dot(N, w.p.p, w.Ap.p, pAp))) return rc;
    if (!(pAp > 0.0) || !std::isfinite(pAp)) { res.breakdown = true; break; }
    alpha = rdotz1 / pAp;
    if ((rc = pcg_update(N, alpha, w.p.p, w.Ap.p, x, r, plat->scalars.p, plat->partials.p, s))) return rc;
    LPG_CUDA_TRY(cudaMemcpyAsync(plat->hostScalars, plat->scalars.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    LPG_CUDA_TRY(cudaStreamSynchronize(s));
    rdotr0 = plat->hostScalars[0];
    if (!std::isfinite(rdotr0)) { res.breakdown = true; ++iter; break; }
  }
  res.iters = iter;
  res.rdotr = rdotr0;
  return LPG_OK;
}

std::vector<int> degree_schedule(int N, const std::string& coarsening, const std::vector<int>& explicitList) {
  std::vector<int> deg;
  if (!explicitList.empty()) {
    deg = explicitList;
    if (deg.front() != N) deg.insert(deg.begin(), N);
    if (deg.back() != 1) deg.push_back(1);
    return deg;
  }
  int Nf = N, Nc = N, NpFine = (N + 1) * (N + 1) * (N + 1), NpCoarse = NpFine;
  deg.push_back(N);
  while (Nc > 1) {
    if (coarsening == "ALLDEGREES") Nc = Nf - 1;
    else if (coarsening == "HALFDEGREES") Nc = std::max(1, (Nf + 1) / 2);
    else
      while (NpCoarse > NpFine / 2 && Nc > 1) { Nc--; NpCoarse = (Nc + 1) * (Nc + 1) * (Nc + 1); }
    NpCoarse = (Nc + 1) * (Nc + 1) * (Nc + 1);
    deg.push_back(Nc);
    Nf = Nc;
    NpFine = NpCoarse;
  }
  return deg;
}

}  // namespace lpg
