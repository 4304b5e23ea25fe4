// Learned fine-level smoother (no reference counterpart): training-data generation by
// the plain solver, MLP training with the project's own forward/backward/Adam kernels,
// and inference with BF16 tensor-core tiles.
//
// Training samples: random Gaussian-bump right-hand sides b on a training mesh; the
// exact error e = A^{-1} b of the zero initial guess comes from the plain p-MG FPCG solve
// to 1e-10; each sampled element contributes (its normalised residual block and face
// traces, D .* e restricted to it / s_e).
#include "learned.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "../mlp.hpp"

namespace lpg {

int LearnedSmoother::load(const float* hostParams, cudaStream_t s) {
  int rc;
  if ((rc = params.alloc(kMlpParams)) || (rc = params.upload(hostParams, kMlpParams, s))) return rc;
  MLPParams P = MLPParams::view(params.p);
  const int dims[5] = {kMlpIn, kMlpHidden, kMlpHidden, kMlpHidden, kMlpOut};
  for (int l = 0; l < 4; ++l) {
    if ((rc = Wt[l].alloc((int64_t)dims[l] * dims[l + 1]))) return rc;
    if ((rc = transpose_to_bf16(dims[l], dims[l + 1], P.W[l], Wt[l].p, s))) return rc;
  }
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  ready = true;
  return LPG_OK;
}

int LearnedSmoother::ensure_chunk(int64_t rows) {
  if (chunk >= rows) return LPG_OK;
  int rc;
  if ((rc = X.alloc(rows * kMlpIn)) || (rc = H0.alloc(rows * kMlpHidden)) || (rc = H1.alloc(rows * kMlpHidden)) ||
      (rc = out.alloc(rows * kMlpOut)) || (rc = scale.alloc(rows)))
    return rc;
  chunk = rows;
  return LPG_OK;
}

// z = average over shared nodes of s_e * invDiag .* MLP(features(r))
template <typename T>
int LearnedSmoother::apply(const BoxNumbering& b, int64_t E, const int32_t* g2l, const T* r, const double* invDiag,
                           const double* weight, T* z, int64_t Nglobal, cudaStream_t s) {
  if (!ready) return set_error(LPG_ERR_INVALID, "learned smoother has no weights");
  const int Np = (b.N + 1) * (b.N + 1) * (b.N + 1);
  int rc;
  const int64_t C = std::min<int64_t>(E, kChunk);
  if ((rc = ensure_chunk(C))) return rc;
  LPG_CUDA_TRY(cudaMemsetAsync(z, 0, sizeof(T) * Nglobal, s));
  MLPParams P = MLPParams::view(params.p);
  for (int64_t e0 = 0; e0 < E; e0 += C) {
    const int64_t n = std::min<int64_t>(C, E - e0);
    if ((rc = element_features<T, __nv_bfloat16>(b, E, e0, n, g2l, r, X.p, scale.p, s))) return rc;
    if ((rc = bf16_linear((int)n, kMlpHidden, kMlpIn, X.p, Wt[0].p, P.b[0], true, true, H0.p, s))) return rc;
    if ((rc = bf16_linear((int)n, kMlpHidden, kMlpHidden, H0.p, Wt[1].p, P.b[1], true, true, H1.p, s))) return rc;
    if ((rc = bf16_linear((int)n, kMlpHidden, kMlpHidden, H1.p, Wt[2].p, P.b[2], true, true, H0.p, s))) return rc;
    if ((rc = bf16_linear((int)n, kMlpOut, kMlpHidden, H0.p, Wt[3].p, P.b[3], false, false, out.p, s))) return rc;
    if ((rc = apply_correction<T>(Np, n, e0, g2l, out.p, scale.p, invDiag, weight, z, s))) return rc;
  }
  return LPG_OK;
}
template int LearnedSmoother::apply<double>(const BoxNumbering&, int64_t, const int32_t*, const double*, const double*,
                                            const double*, double*, int64_t, cudaStream_t);
template int LearnedSmoother::apply<float>(const BoxNumbering&, int64_t, const int32_t*, const float*, const double*,
                                           const double*, float*, int64_t, cudaStream_t);

// ---------------------------------------------------------------- training
int train_smoother(Platform* plat, Elliptic* el, Precon* plainMG, const BoxNumbering& b, const TrainOptions& o,
                   std::vector<float>& weights, std::vector<float>& lossHistory) {
  cudaStream_t s = plat->stream;
  const int64_t E = el->mesh.E, Ng = el->Nglobal, Np = el->mesh.Np;
  if (Np != 512) return set_error(LPG_ERR_UNSUPPORTED, "learned smoother needs POLYNOMIAL DEGREE 7");
  int rc;
  // inverse diagonal of the assembled operator
  DevBuf<double> invDiag;
  if ((rc = invDiag.alloc(Ng)) || (rc = el->BuildDiagonal(invDiag.p, s)) || (rc = inverse_f64(Ng, invDiag.p, invDiag.p, s)))
    return rc;
  const int64_t total = (int64_t)o.nsolves * o.samplesPerSolve;
  DevBuf<float> Xtr, Ttr;
  if ((rc = Xtr.alloc(total * kMlpIn)) || (rc = Ttr.alloc(total * kMlpOut))) return rc;
  DevBuf<float> Xall, scaleAll;
  if ((rc = Xall.alloc(E * kMlpIn)) || (rc = scaleAll.alloc(E))) return rc;
  DevBuf<double> rhs, x, r;
  DevBuf<int32_t> elems;
  DevBuf<float> scaleSel;
  if ((rc = rhs.alloc(Ng)) || (rc = x.alloc(Ng)) || (rc = r.alloc(Ng)) || (rc = elems.alloc(o.samplesPerSolve)) ||
      (rc = scaleSel.alloc(o.samplesPerSolve)))
    return rc;
  Rand48 rng;
  rng.seed((long)(o.seed & 0x7fffffff));
  PCGWork work;
  const MeshConfig& c = el->mesh.cfg;
  for (int sidx = 0; sidx < o.nsolves; ++sidx) {
    // random Gaussian-bump right-hand side: o.bumps bumps, centres U(domain), widths
    // U[0.05,0.2], signed unit amplitudes (sign by the sample stream)
    std::vector<double> src(4 * o.bumps);
    std::vector<double> sign(o.bumps);
    for (int k = 0; k < o.bumps; ++k) {
      src[4 * k + 0] = -c.dimx / 2 + c.dimx * rng.next();
      src[4 * k + 1] = -c.dimy / 2 + c.dimy * rng.next();
      src[4 * k + 2] = -c.dimz / 2 + c.dimz * rng.next();
      src[4 * k + 3] = 0.05 + 0.15 * rng.next();
      sign[k] = (rng.next() < 0.5) ? -1.0 : 1.0;
    }
    // signed bumps: split into positive and negative source sets and combine
    DevBuf<double> rhsNeg;
    if ((rc = rhsNeg.alloc(Ng))) return rc;
    for (int pass = 0; pass < 2; ++pass) {
      std::vector<double> sel;
      for (int k = 0; k < o.bumps; ++k)
        if ((sign[k] > 0) == (pass == 0)) sel.insert(sel.end(), src.begin() + 4 * k, src.begin() + 4 * k + 4);
      el->rhsKind = 1;
      el->sources = sel;
      if (sel.empty()) {
        LPG_CUDA_TRY(cudaMemsetAsync(pass == 0 ? rhs.p : rhsNeg.p, 0, sizeof(double) * Ng, s));
        continue;
      }
      if ((rc = el->sources_d.alloc((int64_t)sel.size())) || (rc = el->sources_d.upload(sel.data(), (int64_t)sel.size(), s)))
        return rc;
      if ((rc = el->BuildRhs(pass == 0 ? rhs.p : rhsNeg.p, s))) return rc;
    }
    if ((rc = axpy<double>(Ng, -1.0, rhsNeg.p, 1.0, rhs.p, s))) return rc;
    // exact error of the zero guess: e = A^{-1} b by the plain p-MG FPCG
    LPG_CUDA_TRY(cudaMemsetAsync(x.p, 0, sizeof(double) * Ng, s));
    LPG_CUDA_TRY(cudaMemcpyAsync(r.p, rhs.p, sizeof(double) * Ng, cudaMemcpyDeviceToDevice, s));
    PCGResult res;
    if ((rc = pcg_solve(plat, el, plainMG, work, true, false, x.p, r.p, o.solveTol, 500, res))) return rc;
    // features of every element for residual b, then a random subset of elements
    if ((rc = element_features<double, float>(b, E, 0, E, el->g2l.p, rhs.p, Xall.p, scaleAll.p, s))) return rc;
    std::vector<int32_t> pick(o.samplesPerSolve);
    for (int i = 0; i < o.samplesPerSolve; ++i) pick[i] = (int32_t)std::min<int64_t>(E - 1, (int64_t)(rng.next() * E));
    if ((rc = elems.upload(pick.data(), o.samplesPerSolve, s))) return rc;
    const int64_t base = (int64_t)sidx * o.samplesPerSolve;
    if ((rc = gather_rows(o.samplesPerSolve, elems.p, Xall.p, Xtr.p + base * kMlpIn, s))) return rc;
    std::vector<float> scHost(E), sel(o.samplesPerSolve);
    if ((rc = scaleAll.download(scHost.data(), E, s))) return rc;
    for (int i = 0; i < o.samplesPerSolve; ++i) sel[i] = scHost[pick[i]];
    if ((rc = scaleSel.upload(sel.data(), o.samplesPerSolve, s))) return rc;
    if ((rc = training_targets((int)Np, o.samplesPerSolve, elems.p, el->g2l.p, x.p, invDiag.p, scaleSel.p,
                               Ttr.p + base * kMlpOut, s)))
      return rc;
  }
  // initial parameters: Glorot-uniform weights, zero biases (seeded)
  std::vector<float> w0(kMlpParams, 0.f);
  {
    const int dims[5] = {kMlpIn, kMlpHidden, kMlpHidden, kMlpHidden, kMlpOut};
    int64_t off = 0;
    for (int l = 0; l < 4; ++l) {
      const double a = std::sqrt(6.0 / (dims[l] + dims[l + 1]));
      for (int64_t i = 0; i < (int64_t)dims[l] * dims[l + 1]; ++i) w0[off + i] = (float)((2 * rng.next() - 1) * a);
      off += (int64_t)dims[l] * dims[l + 1] + dims[l + 1];
    }
  }
  DevBuf<float> W, G, M1, M2, acts, w0buf, w1buf, Y, dY, loss;
  const int B = o.batch;
  if ((rc = W.alloc(kMlpParams)) || (rc = G.alloc(kMlpParams)) || (rc = M1.alloc(kMlpParams)) ||
      (rc = M2.alloc(kMlpParams)) || (rc = acts.alloc(MLPActs::floats(B))) || (rc = w0buf.alloc((int64_t)B * kMlpHidden)) ||
      (rc = w1buf.alloc((int64_t)B * kMlpHidden)) || (rc = dY.alloc((int64_t)B * kMlpOut)) || (rc = loss.alloc(1)))
    return rc;
  if ((rc = W.upload(w0.data(), kMlpParams, s))) return rc;
  LPG_CUDA_TRY(cudaMemsetAsync(M1.p, 0, sizeof(float) * kMlpParams, s));
  LPG_CUDA_TRY(cudaMemsetAsync(M2.p, 0, sizeof(float) * kMlpParams, s));
  MLPParams P = MLPParams::view(W.p), Gp = MLPParams::view(G.p);
  MLPActs A = MLPActs::view(acts.p, B);
  lossHistory.clear();
  int step = 0;
  const int64_t nb = total / B;
  for (int ep = 0; ep < o.epochs; ++ep) {
    double epLoss = 0;
    for (int64_t bi = 0; bi < nb; ++bi) {
      const float* Xb = Xtr.p + bi * B * kMlpIn;
      const float* Tb = Ttr.p + bi * B * kMlpOut;
      if ((rc = mlp_forward_f32(P, B, Xb, A, s))) return rc;
      if ((rc = mse_loss((int64_t)B * kMlpOut, B, A.A[3], Tb, dY.p, loss.p, s))) return rc;
      if ((rc = mlp_backward_f32(P, B, Xb, A, dY.p, Gp, w0buf.p, w1buf.p, s))) return rc;
      if ((rc = adam_step(kMlpParams, W.p, G.p, M1.p, M2.p, o.lr, ++step, s))) return rc;
      float lh;
      if ((rc = loss.download(&lh, 1, s))) return rc;
      epLoss += lh;
    }
    lossHistory.push_back((float)(epLoss / std::max<int64_t>(nb, 1)));
  }
  weights.resize(kMlpParams);
  return W.download(weights.data(), kMlpParams, s);
}

}  // namespace lpg
