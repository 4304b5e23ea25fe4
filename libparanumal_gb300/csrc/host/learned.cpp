// Learned fine-level smoother (no reference counterpart): training-data generation by
// the plain solver, MLP training with the project's own forward/backward/Adam kernels,
// and inference with BF16 tensor-core tiles.
//
// Training samples: random Gaussian-bump right-hand sides b on a training mesh. The plain
// p-MG FPCG solve to 1e-10 gives x*; re-running it for k = 1..3 iterations gives the
// residual r_k and the exact error e_k = x* - x_k of the plain solver's iterate. Each
// sampled element contributes (its normalised residual block and face traces of r_k,
// D .* e_k restricted to it / s_e). Residuals from the iteration are dominated by the
// high-frequency content a smoother has to remove. With SMOOTHER TRAINING PAIRS = MIXED
// (default) every second sample set is synthetic instead: a random error e (lattice
// noise after 0, 2 or 6 damped-Jacobi sweeps) and r = A e, which widens the residual
// distribution toward what the post-smoothing step sees after a coarse correction.
#include "learned.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "../mlp.hpp"

namespace lpg {

int LearnedSmoother::load(const float* hostParams, cudaStream_t s) {
  int rc;
  if ((rc = params.alloc(kMlpParams)) || (rc = params.upload(hostParams, kMlpParams, s))) return rc;
  if ((rc = red.alloc(1)) || (rc = partials.alloc(kReducePartials)) || (rc = tcErr.alloc(1))) return rc;
  LPG_CUDA_TRY(cudaMemsetAsync(tcErr.p, 0, sizeof(int), s));
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

// dst (rows x 512) = MLP(X (rows x 896)): the fused tcgen05 kernel, or with
// LPG_MLP_TC=off (a tuning override) the per-layer mma.sync kernels
int LearnedSmoother::forward_bf16(int64_t rows, float* dst, cudaStream_t s) {
  static const bool layered = [] {
    const char* e = std::getenv("LPG_MLP_TC");
    return e && !std::strcmp(e, "off");
  }();
  MLPParams P = MLPParams::view(params.p);
  int rc;
  if (!layered) {
    const __nv_bfloat16* w[4] = {Wt[0].p, Wt[1].p, Wt[2].p, Wt[3].p};
    const float* bias[4] = {P.b[0], P.b[1], P.b[2], P.b[3]};
    return mlp_forward_tc(rows, X.p, w, bias, dst, tcErr.p, s);
  }
  if ((rc = bf16_linear((int)rows, kMlpHidden, kMlpIn, X.p, Wt[0].p, P.b[0], true, true, H0.p, s))) return rc;
  if ((rc = bf16_linear((int)rows, kMlpHidden, kMlpHidden, H0.p, Wt[1].p, P.b[1], true, true, H1.p, s))) return rc;
  if ((rc = bf16_linear((int)rows, kMlpHidden, kMlpHidden, H1.p, Wt[2].p, P.b[2], true, true, H0.p, s))) return rc;
  return bf16_linear((int)rows, kMlpOut, kMlpHidden, H0.p, Wt[3].p, P.b[3], false, false, dst, s);
}

// the tensor-core pipeline's timeout flag (waits for the stream)
int LearnedSmoother::check_tc(cudaStream_t s) {
  int code = 0;
  int rc = tcErr.download(&code, 1, s);
  if (rc) return rc;
  if (code) return set_error(LPG_ERR_TIMEOUT, "MLP tensor-core pipeline timed out (code " + std::to_string(code) + ")");
  return LPG_OK;
}

int LearnedSmoother::clear_tc(cudaStream_t s) {
  LPG_CUDA_TRY(cudaMemsetAsync(tcErr.p, 0, sizeof(int), s));
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

// z += average over shared nodes of s_e * invDiag .* MLP(features(r))
template <typename T>
int LearnedSmoother::apply(const BoxNumbering& b, int64_t E, const int32_t* g2l, const T* r, const T* coef, T* z,
                           int64_t Nglobal, float sfloor, cudaStream_t s) {
  (void)Nglobal;
  if (!ready) return set_error(LPG_ERR_INVALID, "learned smoother has no weights");
  if (E != (int64_t)b.nx * b.ny * b.nz) return set_error(LPG_ERR_INVALID, "learned smoother: box element count");
  const int Np = (b.N + 1) * (b.N + 1) * (b.N + 1);
  int rc;
  const int64_t C = std::min<int64_t>(E, kChunk);
  if ((rc = ensure_chunk(C))) return rc;
  static const bool atomic = [] {
    const char* e = std::getenv("LPG_LEARNED_CORRECTION");
    return !(e && !std::strcmp(e, "lattice"));
  }();
  if (atomic) {
    for (int64_t e0 = 0; e0 < E; e0 += C) {
      const int64_t n = std::min<int64_t>(C, E - e0);
      if ((rc = element_features<T, __nv_bfloat16>(b, E, e0, n, g2l, r, X.p, scale.p, sfloor, s))) return rc;
      if ((rc = forward_bf16(n, out.p, s))) return rc;
      if ((rc = apply_correction<T>(Np, n, e0, g2l, out.p, scale.p, coef, z, s))) return rc;
    }
    return LPG_OK;
  }
  // chunks of whole element layers; after each chunk the lattice planes whose copies are
  // all computed are summed while the chunk's outputs are still in L2: element layers
  // [z0, z1) complete planes z0*N .. z1*N - 1 (the top plane waits for the next layer; the
  // last chunk also takes plane nz*N, or plane 0 of a periodic box)
  const int64_t layer = (int64_t)b.nx * b.ny;
  const int64_t LC = std::min<int64_t>(E, std::max<int64_t>(1, kChunk / layer) * layer);
  if (LC > chunk && (rc = ensure_chunk(LC))) return rc;
  if (allRows < E) {
    if ((rc = outAll.alloc(E * kMlpOut)) || (rc = scaleAll.alloc(E))) return rc;
    allRows = E;
  }
  for (int64_t e0 = 0; e0 < E; e0 += LC) {
    const int64_t n = std::min<int64_t>(LC, E - e0);
    if ((rc = element_features<T, __nv_bfloat16>(b, E, e0, n, g2l, r, X.p, scaleAll.p + e0, sfloor, s))) return rc;
    if ((rc = forward_bf16(n, outAll.p + e0 * kMlpOut, s))) return rc;
    const int z0 = (int)(e0 / layer), z1 = (int)((e0 + n) / layer);
    const bool last = (z1 == b.nz);
    const int Zb = (b.periodic && z0 == 0) ? 1 : z0 * b.N;
    const int Ze = z1 * b.N + ((last && !b.periodic) ? 1 : 0);
    if ((rc = lattice_correction<T>(b, g2l, outAll.p, scaleAll.p, coef, z, Zb, Ze, s))) return rc;
    if (last && b.periodic && (rc = lattice_correction<T>(b, g2l, outAll.p, scaleAll.p, coef, z, 0, 1, s))) return rc;
  }
  return LPG_OK;
}
template int LearnedSmoother::apply<double>(const BoxNumbering&, int64_t, const int32_t*, const double*, const double*,
                                            double*, int64_t, float, cudaStream_t);
template int LearnedSmoother::apply<float>(const BoxNumbering&, int64_t, const int32_t*, const float*, const float*,
                                           float*, int64_t, float, cudaStream_t);

// ---------------------------------------------------------------- training
double lastKeptFraction = 0;

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
  // the smoother is w D^{-1} r + network correction with the reference's damped-Jacobi
  // weight w = 4/3/rho (rho of D^{-1}A on the finest level); the network learns the rest
  const double jacobiW = plainMG->fine_rho() > 0 ? (4.0 / 3.0) / plainMG->fine_rho() : 0.0;
  DevBuf<float> Xtr, Ttr;
  if ((rc = Xtr.alloc(total * kMlpIn)) || (rc = Ttr.alloc(total * kMlpOut))) return rc;
  DevBuf<float> Xall, scaleAll;
  if ((rc = Xall.alloc(E * kMlpIn)) || (rc = scaleAll.alloc(E))) return rc;
  DevBuf<double> rhs, x, r, xstar;
  DevBuf<int32_t> elems;
  DevBuf<float> Tall;
  double keptFraction = 0;
  if ((rc = xstar.alloc(Ng)) || (rc = Tall.alloc(E * kMlpOut))) return rc;
  // 1D modal low-pass on the GLL nodes: F = V diag(degree <= 3) V^{-1}, V[i][m] = P_m(x_i)
  DevBuf<double> lowpass;
  {
    const int Nq = el->mesh.Nq;
    const std::vector<double>& xg = el->mesh.r1d;
    std::vector<double> V(Nq * Nq), Vi(Nq * Nq, 0.0), F(Nq * Nq, 0.0);
    for (int i = 0; i < Nq; ++i) {
      double p0 = 1, p1 = xg[i];
      V[i * Nq + 0] = 1;
      if (Nq > 1) V[i * Nq + 1] = xg[i];
      for (int m = 2; m < Nq; ++m) {
        const double p2 = ((2 * m - 1) * xg[i] * p1 - (m - 1) * p0) / m;
        V[i * Nq + m] = p2;
        p0 = p1;
        p1 = p2;
      }
    }
    // Gauss-Jordan inverse of V (Nq <= 9)
    std::vector<double> Aug(V);
    for (int i = 0; i < Nq; ++i) Vi[i * Nq + i] = 1;
    for (int c = 0; c < Nq; ++c) {
      int piv = c;
      for (int r2 = c + 1; r2 < Nq; ++r2)
        if (std::fabs(Aug[r2 * Nq + c]) > std::fabs(Aug[piv * Nq + c])) piv = r2;
      for (int j = 0; j < Nq; ++j) { std::swap(Aug[c * Nq + j], Aug[piv * Nq + j]); std::swap(Vi[c * Nq + j], Vi[piv * Nq + j]); }
      const double d = Aug[c * Nq + c];
      for (int j = 0; j < Nq; ++j) { Aug[c * Nq + j] /= d; Vi[c * Nq + j] /= d; }
      for (int r2 = 0; r2 < Nq; ++r2) {
        if (r2 == c) continue;
        const double f = Aug[r2 * Nq + c];
        for (int j = 0; j < Nq; ++j) { Aug[r2 * Nq + j] -= f * Aug[c * Nq + j]; Vi[r2 * Nq + j] -= f * Vi[c * Nq + j]; }
      }
    }
    for (int i = 0; i < Nq; ++i)
      for (int j = 0; j < Nq; ++j)
        for (int m = 0; m <= std::min(3, Nq - 1); ++m) F[i * Nq + j] += V[i * Nq + m] * Vi[m * Nq + j];
    if ((rc = lowpass.alloc(Nq * Nq)) || (rc = lowpass.upload(F.data(), Nq * Nq, s))) return rc;
  }
  DevBuf<float> scaleSel;
  if ((rc = rhs.alloc(Ng)) || (rc = x.alloc(Ng)) || (rc = r.alloc(Ng)) || (rc = elems.alloc(o.samplesPerSolve)) ||
      (rc = scaleSel.alloc(o.samplesPerSolve)))
    return rc;
  Rand48 rng;
  rng.seed((long)(o.seed & 0x7fffffff));
  PCGWork work;
  const MeshConfig& c = el->mesh.cfg;
  for (int sidx = 0; sidx < o.nsolves; ++sidx) {
    if (o.synthetic && (sidx % 2 == 1)) {
      // synthetic pair: e = lattice noise after m damped-Jacobi sweeps (m = 0, 2, 6 gives
      // rough to smoother errors), r = A e; x holds e
      static const int sweeps[3] = {0, 2, 6};
      const int m = sweeps[(sidx / 2) % 3];
      if ((rc = lattice_random(b, Ng, el->owner.p, o.seed * 1000003ULL + (uint64_t)sidx, x.p, s))) return rc;
      for (int j = 0; j < m; ++j) {
        if ((rc = el->Operator(x.p, r.p, s))) return rc;
        if ((rc = amxpy<double>(Ng, -2.0 / 3.0, invDiag.p, r.p, 1.0, x.p, s))) return rc;
      }
      if ((rc = el->Operator(x.p, r.p, s))) return rc;
    } else {
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
      // converged solution x* of the plain p-MG FPCG
      LPG_CUDA_TRY(cudaMemsetAsync(xstar.p, 0, sizeof(double) * Ng, s));
      LPG_CUDA_TRY(cudaMemcpyAsync(r.p, rhs.p, sizeof(double) * Ng, cudaMemcpyDeviceToDevice, s));
      PCGResult res;
      if ((rc = pcg_solve(plat, el, plainMG, work, true, false, xstar.p, r.p, o.solveTol, 500, res))) return rc;
      // a (residual, exact error) pair of the plain solver's trajectory: after k iterations
      // the residual is r_k and the exact error is x* - x_k (the FPCG run is deterministic)
      const int kIter = 1 + (sidx % 3);
      LPG_CUDA_TRY(cudaMemsetAsync(x.p, 0, sizeof(double) * Ng, s));
      LPG_CUDA_TRY(cudaMemcpyAsync(r.p, rhs.p, sizeof(double) * Ng, cudaMemcpyDeviceToDevice, s));
      if ((rc = pcg_solve(plat, el, plainMG, work, true, false, x.p, r.p, 0.0, kIter, res))) return rc;
      if ((rc = axpy<double>(Ng, 1.0, xstar.p, -1.0, x.p, s))) return rc;  // x := x* - x_k
    }
    // features of every element for residual r_k (scales floored at kScaleFloor x RMS),
    // then a random subset of the elements whose residual is not negligible
    double bb;
    if ((rc = plat->norm2sq(Ng, r.p, bb))) return rc;
    const double rms = std::sqrt(bb / (double)Ng);
    if ((rc = element_features<double, float>(b, E, 0, E, el->g2l.p, r.p, Xall.p, scaleAll.p,
                                              (float)(LearnedSmoother::kScaleFloor * rms), s)))
      return rc;
    std::vector<float> scHost(E), sel(o.samplesPerSolve);
    if ((rc = scaleAll.download(scHost.data(), E, s))) return rc;
    // targets of every element: the share of the exact error e_k outside the coarse
    // (degree <= 3) space on each element -- what the fine-level smoother is responsible
    // for; the remainder is the coarse levels' share
    if ((rc = highpass_targets(el->mesh.Nq, E, el->g2l.p, x.p, invDiag.p, scaleAll.p, lowpass.p, Tall.p, s))) return rc;
    std::vector<int32_t> cand;
    for (int64_t e2 = 0; e2 < E; ++e2)
      if (scHost[e2] >= 1e-2 * rms) cand.push_back((int32_t)e2);
    keptFraction += (double)cand.size() / (double)E / o.nsolves;
    if (cand.empty()) return set_error(LPG_ERR_INVALID, "smoother training: right-hand side is zero");
    std::vector<int32_t> pick(o.samplesPerSolve);
    for (int i = 0; i < o.samplesPerSolve; ++i)
      pick[i] = cand[std::min<size_t>(cand.size() - 1, (size_t)(rng.next() * cand.size()))];
    if ((rc = elems.upload(pick.data(), o.samplesPerSolve, s))) return rc;
    const int64_t base = (int64_t)sidx * o.samplesPerSolve;
    if ((rc = gather_rows(o.samplesPerSolve, elems.p, Xall.p, Xtr.p + base * kMlpIn, s))) return rc;
    (void)sel;
    (void)scaleSel;
    // rows of the selected elements (the target rows have kMlpOut = 512 entries)
    {
      std::vector<float> Th(E * kMlpOut), Ts((int64_t)o.samplesPerSolve * kMlpOut);
      if ((rc = Tall.download(Th.data(), E * kMlpOut, s))) return rc;
      for (int i = 0; i < o.samplesPerSolve; ++i)
        std::memcpy(Ts.data() + (int64_t)i * kMlpOut, Th.data() + (int64_t)pick[i] * kMlpOut, sizeof(float) * kMlpOut);
      LPG_CUDA_TRY(cudaMemcpyAsync(Ttr.p + base * kMlpOut, Ts.data(), sizeof(float) * Ts.size(), cudaMemcpyHostToDevice, s));
      LPG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    // the damped-Jacobi part w D^{-1} r is applied outside the network: in network
    // output units (divided by invDiag s_e) it is w times the normalised residual input
    if (jacobiW > 0 && (rc = subtract_inputs(o.samplesPerSolve, (float)jacobiW, Xtr.p + base * kMlpIn,
                                             Ttr.p + base * kMlpOut, s)))
      return rc;
  }
  lastKeptFraction = keptFraction;
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
  // minibatches: a fresh random permutation of all samples every epoch (the samples are
  // stored grouped by sample set); learning rate with cosine decay to 5 % of o.lr
  DevBuf<int32_t> perm;
  DevBuf<float> Xb, Tb;
  if ((rc = perm.alloc(total)) || (rc = Xb.alloc((int64_t)B * kMlpIn)) || (rc = Tb.alloc((int64_t)B * kMlpOut))) return rc;
  std::vector<int32_t> order(total);
  for (int64_t i = 0; i < total; ++i) order[i] = (int32_t)i;
  const int64_t totalSteps = std::max<int64_t>(1, (int64_t)o.epochs * nb);
  for (int ep = 0; ep < o.epochs; ++ep) {
    for (int64_t i = total - 1; i > 0; --i) std::swap(order[i], order[(int64_t)(rng.next() * (double)(i + 1)) % (i + 1)]);
    if ((rc = perm.upload(order.data(), total, s))) return rc;
    double epLoss = 0;
    for (int64_t bi = 0; bi < nb; ++bi) {
      if ((rc = gather_rows_w(B, kMlpIn, perm.p + bi * B, Xtr.p, Xb.p, s)) ||
          (rc = gather_rows_w(B, kMlpOut, perm.p + bi * B, Ttr.p, Tb.p, s)))
        return rc;
      const double frac = (double)step / (double)totalSteps;
      const float lr = (float)(o.lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(3.14159265358979323846 * frac))));
      if ((rc = mlp_forward_f32(P, B, Xb.p, A, s))) return rc;
      if ((rc = mse_loss((int64_t)B * kMlpOut, B, A.A[3], Tb.p, dY.p, loss.p, s))) return rc;
      if ((rc = mlp_backward_f32(P, B, Xb.p, A, dY.p, Gp, w0buf.p, w1buf.p, s))) return rc;
      if ((rc = adam_step(kMlpParams, W.p, G.p, M1.p, M2.p, lr, ++step, s))) return rc;
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
