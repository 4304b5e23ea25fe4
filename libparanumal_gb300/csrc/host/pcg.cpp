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
  // a NaN or Inf in the right-hand side or the initial guess: stop before iterating on it
  if (!std::isfinite(rdotr0) || !std::isfinite(TOL)) {
    res.breakdown = true;
    res.iters = 0;
    res.rdotr = rdotr0;
    return LPG_OK;
  }
  for (iter = 0; iter < maxit; ++iter) {
    if ((iter == 0 && rdotr0 == 0.0) || (iter > 0 && rdotr0 <= TOL)) break;
    const float* z32 = nullptr;
    if ((rc = pc->apply_mixed(r, w.z.p, &z32, s))) return rc;
    rdotz2 = rdotz1;
    double zdotAp = 0;
    if (z32) {
      // FP32 preconditioner output: r.z and z.Ap in one pass, z widened exactly to FP64
      if ((rc = dot2_mixed(N, z32, r, w.Ap.p, plat->scalars.p + 4, plat->partials.p, s))) return rc;
      LPG_CUDA_TRY(cudaMemcpyAsync(plat->hostScalars + 4, plat->scalars.p + 4, 2 * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
      LPG_CUDA_TRY(cudaStreamSynchronize(s));
      rdotz1 = plat->hostScalars[4];
      zdotAp = plat->hostScalars[5];
    } else {
      if ((rc = plat->dot(N, r, w.z.p, rdotz1))) return rc;
      if (flexible && (rc = plat->dot(N, w.z.p, w.Ap.p, zdotAp))) return rc;
    }
    if (flexible) beta = (iter == 0) ? 0.0 : -alpha * zdotAp / rdotz2;
    else beta = (iter == 0) ? 0.0 : rdotz1 / rdotz2;
    if (z32) rc = direction_mixed(N, z32, beta, w.p.p, s);
    else rc = axpy<double>(N, 1.0, w.z.p, beta, w.p.p, s);
    if (rc) return rc;
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

int NBWork::ensure(int64_t n) {
  if (u.n == n) return LPG_OK;
  int rc;
  if ((rc = u.alloc(n)) || (rc = p.alloc(n)) || (rc = w.alloc(n)) || (rc = this->n.alloc(n)) || (rc = m.alloc(n)) ||
      (rc = s.alloc(n)) || (rc = z.alloc(n)) || (rc = q.alloc(n)) || (rc = Ax.alloc(n)) || (rc = partials.alloc(4 * 1024)))
    return rc;
  host.resize(4 * 1024);
  return LPG_OK;
}

// sums of the k block partial arrays, in block order (update0/1NBFPCG's host loop)
static int nb_sums(NBWork& w, int k, int nb, cudaStream_t s, double* out) {
  LPG_CUDA_TRY(cudaMemcpyAsync(w.host.data(), w.partials.p, sizeof(double) * k * nb, cudaMemcpyDeviceToHost, s));
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  for (int j = 0; j < k; ++j) {
    double t = w.host[(size_t)j * nb];
    for (int b = 1; b < nb; ++b) t += w.host[(size_t)j * nb + b];
    out[j] = t;
  }
  return LPG_OK;
}

int nbfpcg_solve(Platform* plat, Elliptic* el, Precon* pc, NBWork& w, double* x, double* r, double tol, int maxit,
                 PCGResult& res) {
  const int64_t N = el->Nglobal;
  cudaStream_t s = plat->stream;
  int rc, nb = 0;
  if ((rc = w.ensure(N))) return rc;
  const size_t bytes = sizeof(double) * N;
  if ((rc = el->Operator(x, w.Ax.p, s)) || (rc = axpy<double>(N, -1.0, w.Ax.p, 1.0, r, s))) return rc;
  if ((rc = pc->apply(r, w.u.p, s))) return rc;
  LPG_CUDA_TRY(cudaMemcpyAsync(w.p.p, w.u.p, bytes, cudaMemcpyDeviceToDevice, s));
  if ((rc = el->Operator(w.p.p, w.w.p, s))) return rc;
  double d3[3];
  if ((rc = nb_dots3(N, w.u.p, r, w.w.p, w.partials.p, &nb, s)) || (rc = nb_sums(w, 3, nb, s, d3))) return rc;
  if ((rc = pc->apply(w.w.p, w.m.p, s)) || (rc = el->Operator(w.m.p, w.n.p, s))) return rc;
  LPG_CUDA_TRY(cudaMemcpyAsync(w.s.p, w.w.p, bytes, cudaMemcpyDeviceToDevice, s));
  LPG_CUDA_TRY(cudaMemcpyAsync(w.q.p, w.m.p, bytes, cudaMemcpyDeviceToDevice, s));
  LPG_CUDA_TRY(cudaMemcpyAsync(w.z.p, w.n.p, bytes, cudaMemcpyDeviceToDevice, s));
  double gamma0 = d3[0], delta0 = d3[1], rdotr0 = d3[2];
  double eta0 = delta0, alpha0 = gamma0 / eta0, beta0 = 0.0;
  const double TOL = std::max(tol * tol * rdotr0, tol * tol);
  int iter;
  res.breakdown = false;
  if (!std::isfinite(rdotr0) || !std::isfinite(alpha0)) {
    res.breakdown = true;
    res.iters = 0;
    res.rdotr = rdotr0;
    return LPG_OK;
  }
  for (iter = 0; iter < maxit; ++iter) {
    if (rdotr0 <= TOL) break;
    double d4[4];
    // x += a p, r -= a s, u -= a q, w -= a z, n = w - r, with the four inner products
    if ((rc = nb_update(N, alpha0, w.p.p, w.s.p, w.q.p, w.z.p, x, r, w.u.p, w.w.p, w.n.p, w.partials.p, &nb, s)))
      return rc;
    if ((rc = pc->apply(w.n.p, w.m.p, s))) return rc;                             // m = M (w - r)
    if ((rc = axpy<double>(N, 1.0, w.u.p, 1.0, w.m.p, s))) return rc;            // m += u
    if ((rc = el->Operator(w.m.p, w.n.p, s))) return rc;                          // n = A m
    if ((rc = nb_sums(w, 4, nb, s, d4))) return rc;
    gamma0 = d4[0];
    beta0 = -d4[1] / eta0;
    delta0 = d4[2];
    rdotr0 = d4[3];
    if ((rc = nb_directions(N, beta0, w.u.p, w.w.p, w.m.p, w.n.p, w.p.p, w.s.p, w.q.p, w.z.p, s))) return rc;
    eta0 = delta0 - beta0 * beta0 * eta0;
    alpha0 = gamma0 / eta0;
    if (!std::isfinite(rdotr0) || !std::isfinite(alpha0)) { res.breakdown = true; ++iter; break; }
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
