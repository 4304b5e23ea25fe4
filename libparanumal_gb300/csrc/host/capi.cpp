// extern "C" boundary: solver objects (elliptic_t built from .rc settings) and the
// kernel entry points for gather-scatter and vector operations. No C++ exception
// crosses this boundary; every function returns an LPG status.
#include "objects.hpp"
#include "initial_guess.hpp"
#include "learned.hpp"
#include "../mlp.hpp"

#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <sstream>

using namespace lpg;

struct lpg_elliptic {
  Settings settings;
  Platform plat;
  MeshConfig mcfg;
  std::unique_ptr<Elliptic> el;
  std::unique_ptr<Precon> precon;
  PCGWork work;
  std::unique_ptr<LearnedSmoother> learned;
  std::unique_ptr<InitialGuess> ig;
  bool flexible = false, stopRhs = false, nonblocking = false;
  NBWork nbwork;
  double tol = 1e-8;
  int maxit = 5000;
  DevBuf<double> q_in, Aq_out, x, r, xL, norms;
};

namespace {

#define LPG_GUARD_BEGIN try {
#define LPG_GUARD_END                                                          \
  }                                                                            \
  catch (const std::bad_alloc&) { return set_error(LPG_ERR_ALLOC, "host allocation failed"); } \
  catch (const std::exception& ex) { return set_error(LPG_ERR_INVALID, ex.what()); }            \
  catch (...) { return set_error(LPG_ERR_INVALID, "unknown exception"); }

// Library-owned reduction scratch per device (partial sums of the two-stage reductions).
std::mutex g_scratch_mu;
double* g_scratch[64] = {nullptr};

int reduction_scratch(double** out) {
  int dev = 0;
  LPG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(LPG_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, sizeof(double) * kReducePartials);
    if (e != cudaSuccess) return set_error(LPG_ERR_ALLOC, std::string("reduction scratch: ") + cudaGetErrorString(e));
    g_scratch[dev] = (double*)p;
  }
  *out = g_scratch[dev];
  return LPG_OK;
}

std::vector<int> parse_int_list(const std::string& v) {
  std::vector<int> out;
  std::string cur;
  for (char ch : v + ",") {
    if (ch >= '0' && ch <= '9') cur += ch;
    else if (!cur.empty()) { out.push_back(std::atoi(cur.c_str())); cur.clear(); }
  }
  return out;
}

int build(lpg_elliptic* h) {
  Settings& S = h->settings;
  if (S.geti("ELEMENT TYPE", 12) != 12 || S.geti("MESH DIMENSION", 3) != 3)
    return set_error(LPG_ERR_UNSUPPORTED, "only hexahedra (ELEMENT TYPE 12, MESH DIMENSION 3) are supported");
  const std::string disc = S.get("DISCRETIZATION", "CONTINUOUS");
  if (disc != "CONTINUOUS" && disc != "IPDG")
    return set_error(LPG_ERR_SETTINGS, "DISCRETIZATION must be CONTINUOUS or IPDG");
  MeshConfig& c = h->mcfg;
  c.ipdg = (disc == "IPDG");
  c.nx = S.geti("BOX GLOBAL NX", 0) > 0 ? S.geti("BOX GLOBAL NX", 0) : S.geti("BOX NX", 10);
  c.ny = S.geti("BOX GLOBAL NY", 0) > 0 ? S.geti("BOX GLOBAL NY", 0) : S.geti("BOX NY", 10);
  c.nz = S.geti("BOX GLOBAL NZ", 0) > 0 ? S.geti("BOX GLOBAL NZ", 0) : S.geti("BOX NZ", 10);
  c.dimx = S.getd("BOX DIMX", 10);
  c.dimy = S.getd("BOX DIMY", 10);
  c.dimz = S.getd("BOX DIMZ", 10);
  c.bcflag = S.geti("BOX BOUNDARY FLAG", 1);
  c.jitter = S.getd("MESH JITTER", 0.0);
  c.jitterSeed = (uint64_t)std::strtoull(S.get("MESH JITTER SEED", "0").c_str(), nullptr, 10);
  const std::string meshFile = S.get("MESH FILE", "BOX");
  if (meshFile != "BOX") {
    // hexahedral Gmsh mesh (mesh_t::ReadGmshHex3D); boundary tags 1 Dirichlet, 2 Neumann
    auto f = std::make_shared<HexMeshData>();
    int rcm = read_gmsh_hex(meshFile, *f);
    if (rcm) return rcm;
    if (S.get("RHS FIELD", "SINE") != "SINE")
      return set_error(LPG_ERR_UNSUPPORTED, "a MESH FILE mesh supports RHS FIELD = SINE only");
    if (c.jitter != 0.0) return set_error(LPG_ERR_UNSUPPORTED, "MESH JITTER applies to BOX meshes only");
    c.file = f;
  }
  const int N = S.geti("POLYNOMIAL DEGREE", 4);
  const double lambda = S.getd("LAMBDA", 1.0);
  const int64_t E = c.is_box() ? (int64_t)c.nx * c.ny * c.nz : c.file->E;
  std::vector<double> lamE;
  const bool lognormal = S.is("LAMBDA FIELD", "LOGNORMAL");
  if (lognormal) {
    // lambda_e = exp(z), z ~ N(0,1) by Box-Muller on hashed uniforms keyed by element id
    const uint64_t seed = (uint64_t)std::strtoull(S.get("LAMBDA SEED", "2").c_str(), nullptr, 10);
    lamE.resize(E);
    for (int64_t e = 0; e < E; ++e) {
      const double u1 = 1.0 - hash_u01(seed, 4, (uint64_t)e);
      const double u2 = hash_u01(seed, 5, (uint64_t)e);
      lamE[e] = std::exp(std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2));
    }
  }
  int rc;
  if ((rc = h->plat.init())) return rc;
  h->el = std::make_unique<Elliptic>();
  if ((rc = h->el->setup(&h->plat, c, N, lambda, lognormal ? &lamE : nullptr, h->plat.stream))) return rc;
  Elliptic* el = h->el.get();
  const std::string opPrec = S.get("OPERATOR PRECISION", "FP64");
  if (opPrec != "FP64" && opPrec != "DF64") return set_error(LPG_ERR_SETTINGS, "OPERATOR PRECISION must be FP64 or DF64");
  el->opDW = (opPrec == "DF64");
  // right-hand side data
  const std::string rhsField = S.get("RHS FIELD", "SINE");
  if (rhsField == "GAUSSIAN SOURCES") {
    el->rhsKind = 1;
    const uint64_t seed = (uint64_t)std::strtoull(S.get("RHS SEED", "3").c_str(), nullptr, 10);
    const int ns = S.geti("RHS SOURCES", 16);
    el->sources.resize(4 * ns);
    for (int k = 0; k < ns; ++k) {
      el->sources[4 * k + 0] = -c.dimx / 2 + c.dimx * hash_u01(seed, 6, (uint64_t)k);
      el->sources[4 * k + 1] = -c.dimy / 2 + c.dimy * hash_u01(seed, 7, (uint64_t)k);
      el->sources[4 * k + 2] = -c.dimz / 2 + c.dimz * hash_u01(seed, 8, (uint64_t)k);
      el->sources[4 * k + 3] = 0.05 + 0.15 * hash_u01(seed, 9, (uint64_t)k);
    }
    if ((rc = el->sources_d.alloc(4 * ns)) || (rc = el->sources_d.upload(el->sources.data(), 4 * ns, h->plat.stream)))
      return rc;
  } else if (rhsField != "SINE") {
    return set_error(LPG_ERR_SETTINGS, "RHS FIELD must be SINE or GAUSSIAN SOURCES");
  }
  // linear solver
  const std::string ls = S.get("LINEAR SOLVER", "PCG");
  if (ls != "PCG" && ls != "FPCG" && ls != "NBFPCG")
    return set_error(LPG_ERR_UNSUPPORTED, "LINEAR SOLVER must be PCG, FPCG or NBFPCG");
  h->flexible = (ls == "FPCG");
  h->nonblocking = (ls == "NBFPCG");
  h->stopRhs = S.is("LINEAR SOLVER STOPPING CRITERION", "ABS/REL-RHS-2NORM");
  h->tol = S.getd("SOLVER TOLERANCE", 1e-8);
  h->maxit = S.geti("MAXIMUM ITERATIONS", 5000);
  // preconditioner
  const std::string pre = S.get("PRECONDITIONER", "NONE");
  if (pre == "NONE") h->precon = make_identity(el);
  else if (pre == "JACOBI") h->precon = make_jacobi(el, &rc);
  else if (pre == "MASSMATRIX")   // MassMatrixPrecon refuses hexahedra (ellipticPreconMassMatrix.cpp:34-35)
    return set_error(LPG_ERR_UNSUPPORTED, "MASSMATRIX preconditioner is only available for triangle and "
                                          "tetrahedra elements. Use JACOBI instead.");
  else if (c.ipdg && pre == "SEMFEM")
    return set_error(LPG_ERR_UNSUPPORTED, "SEMFEM is supported for CONTINUOUS only");
  else if (c.ipdg && pre != "NONE" && pre != "JACOBI" && S.get("PRECONDITIONER PRECISION", "FP64") == "BF16GEO")
    return set_error(LPG_ERR_UNSUPPORTED, "IPDG multigrid runs in FP64 or FP32 (PRECONDITIONER PRECISION)");
  else if (pre == "MULTIGRID" || pre == "PARALMOND" || pre == "SEMFEM" || pre == "OAS") {
    MGOptions o;
    o.amgOnly = (pre == "PARALMOND" || pre == "SEMFEM");
    o.semfem = (pre == "SEMFEM");
    o.degrees = degree_schedule(N, S.get("MULTIGRID COARSENING", "HALFDOFS"), parse_int_list(S.get("MULTIGRID DEGREES", "")));
    o.smoother = S.is("MULTIGRID SMOOTHER", "DAMPEDJACOBI") ? 1 : 0;
    o.chebDegree = S.geti("MULTIGRID CHEBYSHEV DEGREE", 2);
    const std::string prec = S.get("PRECONDITIONER PRECISION", "FP64");
    if (prec == "FP64") o.prec = Prec::F64;
    else if (prec == "FP32") o.prec = Prec::F32;
    else if (prec == "BF16GEO") o.prec = Prec::BF16G;
    else return set_error(LPG_ERR_SETTINGS, "PRECONDITIONER PRECISION must be FP64, FP32 or BF16GEO");
    o.amgSmoother = S.is("PARALMOND SMOOTHER", "DAMPEDJACOBI") ? 1 : 0;
    o.amgChebDegree = S.geti("PARALMOND CHEBYSHEV DEGREE", 2);
    o.amgUnsmoothed = S.is("PARALMOND AGGREGATION", "UNSMOOTHED");
    o.amgRugeStuben = S.is("PARALMOND STRENGTH", "RUGESTUBEN");
    o.learnedSteps = S.geti("LEARNED SMOOTHER STEPS", 2);
    if (o.learnedSteps < 1 || o.learnedSteps > 8)
      return set_error(LPG_ERR_SETTINGS, "LEARNED SMOOTHER STEPS must be 1..8");
    if (S.get("PARALMOND CYCLE", "VCYCLE") != "VCYCLE")
      return set_error(LPG_ERR_UNSUPPORTED, "PARALMOND CYCLE must be VCYCLE");
    h->precon = (pre == "OAS") ? make_oas(el, c, o, &rc) : make_multigrid(el, c, o, &rc);
  } else {
    return set_error(LPG_ERR_UNSUPPORTED,
                     "PRECONDITIONER must be NONE, JACOBI, MULTIGRID, PARALMOND, SEMFEM or OAS");
  }
  if (rc) return rc;
  if (!h->precon) return set_error(LPG_ERR_INVALID, "preconditioner setup failed");
  const int64_t Ng = el->Nglobal;
  if ((rc = h->q_in.alloc(Ng)) || (rc = h->Aq_out.alloc(Ng)) || (rc = h->x.alloc(Ng)) || (rc = h->r.alloc(Ng)) ||
      (rc = h->norms.alloc(2)))
    return rc;
  if ((rc = h->work.ensure(Ng))) return rc;
  h->ig = make_initial_guess(S, &h->plat, Ng, &rc);
  if (rc) return rc;
  LPG_CUDA_TRY(cudaStreamSynchronize(h->plat.stream));
  return LPG_OK;
}

cudaStream_t pick(lpg_elliptic* h, void* stream) {
  return stream ? (cudaStream_t)stream : h->plat.stream;
}

}  // namespace

// ================================================================ misc
extern "C" const char* lpg_version(void) { return "libparanumal_gb300 0.1 (sm_103a)"; }

extern "C" int lpg_device_malloc(void** ptr, uint64_t bytes) {
  if (!ptr) return set_error(LPG_ERR_INVALID, "null ptr");
  LPG_CUDA_TRY(cudaMalloc(ptr, bytes));
  return LPG_OK;
}
extern "C" int lpg_set_device(int device) {
  LPG_CUDA_TRY(cudaSetDevice(device));
  return LPG_OK;
}
extern "C" int lpg_memcpy_d2d(void* dst, const void* src, uint64_t bytes, void* stream) {
  LPG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return LPG_OK;
}
extern "C" int lpg_device_free(void* ptr) {
  LPG_CUDA_TRY(cudaFree(ptr));
  return LPG_OK;
}
extern "C" int lpg_memcpy_h2d(void* dst, const void* src, uint64_t bytes, void* stream) {
  LPG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  return LPG_OK;
}
extern "C" int lpg_memcpy_d2h(void* dst, const void* src, uint64_t bytes, void* stream) {
  LPG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  return LPG_OK;
}
extern "C" int lpg_stream_sync(void* stream) {
  LPG_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return LPG_OK;
}

// ================================================================ kernel entry points
extern "C" int lpg_ogs_gather_add_f64(int64_t Nlocal, const int32_t* g2l, const double* v, double* gv, int64_t Nglobal,
                                      void* stream) {
  if (Nlocal < 0 || Nglobal < 0 || (Nlocal > 0 && (!g2l || !v)) || (Nglobal > 0 && !gv))
    return set_error(LPG_ERR_INVALID, "ogs gather: bad arguments");
  return gather_add<double>(Nlocal, g2l, v, gv, Nglobal, true, (cudaStream_t)stream);
}
extern "C" int lpg_ogs_gather_owner_f64(int64_t Nglobal, const int32_t* owner, const double* v, double* gv, void* stream) {
  if (Nglobal < 0 || (Nglobal > 0 && (!owner || !v || !gv))) return set_error(LPG_ERR_INVALID, "ogs gather: bad arguments");
  return gather_owner<double>(Nglobal, owner, v, gv, (cudaStream_t)stream);
}
extern "C" int lpg_ogs_scatter_f64(int64_t Nlocal, const int32_t* g2l, const double* gv, double* v, void* stream) {
  if (Nlocal < 0 || (Nlocal > 0 && (!g2l || !gv || !v))) return set_error(LPG_ERR_INVALID, "ogs scatter: bad arguments");
  return scatter<double>(Nlocal, g2l, gv, v, (cudaStream_t)stream);
}
extern "C" int lpg_axpy_f64(int64_t N, double alpha, const double* x, double beta, double* y, void* stream) {
  if (N < 0 || (N > 0 && (!x || !y))) return set_error(LPG_ERR_INVALID, "axpy: bad arguments");
  return axpy<double>(N, alpha, x, beta, y, (cudaStream_t)stream);
}
extern "C" int lpg_amxpy_f64(int64_t N, double alpha, const double* x, const double* y, double beta, double* z,
                             void* stream) {
  if (N < 0 || (N > 0 && (!x || !y || !z))) return set_error(LPG_ERR_INVALID, "amxpy: bad arguments");
  return amxpy<double>(N, alpha, x, y, beta, z, (cudaStream_t)stream);
}
extern "C" int lpg_dot_f64(int64_t N, const double* x, const double* y, double* result_dev, void* stream) {
  if (N < 0 || !result_dev || (N > 0 && (!x || !y))) return set_error(LPG_ERR_INVALID, "dot: bad arguments");
  double* scratch;
  int rc = reduction_scratch(&scratch);
  if (rc) return rc;
  return dot(N, x, y, result_dev, scratch, (cudaStream_t)stream);
}
extern "C" int lpg_norm2sq_f64(int64_t N, const double* x, double* result_dev, void* stream) {
  return lpg_dot_f64(N, x, x, result_dev, stream);
}
extern "C" int lpg_pcg_update_f64(int64_t N, double alpha, const double* p, const double* Ap, double* x, double* r,
                                  double* result_dev, void* stream) {
  if (N < 0 || !result_dev || (N > 0 && (!p || !Ap || !x || !r))) return set_error(LPG_ERR_INVALID, "pcg update: bad arguments");
  double* scratch;
  int rc = reduction_scratch(&scratch);
  if (rc) return rc;
  return pcg_update(N, alpha, p, Ap, x, r, result_dev, scratch, (cudaStream_t)stream);
}

extern "C" int lpg_norm2_f64(int64_t N, const double* x, double* result_dev, void* stream) {
  if (N < 0 || !result_dev || (N > 0 && !x)) return set_error(LPG_ERR_INVALID, "norm2: bad arguments");
  double* scratch;
  int rc = reduction_scratch(&scratch);
  if (rc) return rc;
  return norm2(N, x, result_dev, scratch, (cudaStream_t)stream);
}
extern "C" int lpg_halo_pack_f64(int64_t n, const int32_t* idx, const double* v, double* buf, void* stream) {
  if (n < 0 || (n > 0 && (!idx || !v || !buf))) return set_error(LPG_ERR_INVALID, "halo pack: bad arguments");
  return halo_pack(n, idx, v, buf, (cudaStream_t)stream);
}
extern "C" int lpg_halo_unpack_add_f64(int64_t n, const int32_t* idx, const double* buf, double* v, void* stream) {
  if (n < 0 || (n > 0 && (!idx || !v || !buf))) return set_error(LPG_ERR_INVALID, "halo unpack: bad arguments");
  return halo_unpack_add(n, idx, buf, v, (cudaStream_t)stream);
}
extern "C" int lpg_jacobi_f64(int64_t N, const double* invDiag, const double* r, double* z, void* stream) {
  if (N < 0 || (N > 0 && (!invDiag || !r || !z))) return set_error(LPG_ERR_INVALID, "jacobi: bad arguments");
  return amxpy<double>(N, 1.0, invDiag, r, 0.0, z, (cudaStream_t)stream);
}

// p-multigrid transfers and Chebyshev passes, FP64 and FP32 (the preconditioner levels'
// precision)
template <typename T>
static int restrict_entry(int Nf, int Nc, int64_t E, const int32_t* g2lF, const T* weightF, const T* rF, const T* P,
                          const int32_t* g2lC, T* rC, int64_t NglobalC, void* stream) {
  if (Nf < 1 || Nf > 8 || Nc < 1 || Nc > Nf || E < 0 || NglobalC < 0 ||
      (E > 0 && (!g2lF || !weightF || !rF || !P || !g2lC)) || (NglobalC > 0 && !rC))
    return set_error(LPG_ERR_INVALID, "pmg restrict: bad arguments (1 <= Nc <= Nf <= 8)");
  return pmg_coarsen<T>(Nf, Nc, E, g2lF, weightF, rF, P, g2lC, rC, NglobalC, (cudaStream_t)stream);
}
template <typename T>
static int prolong_entry(int Nf, int Nc, int64_t E, const int32_t* g2lC, const T* xC, const T* P,
                         const int32_t* g2lF, const int32_t* ownerF, T* xF, void* stream) {
  if (Nf < 1 || Nf > 8 || Nc < 1 || Nc > Nf || E < 0 || (E > 0 && (!g2lC || !xC || !P || !g2lF || !ownerF || !xF)))
    return set_error(LPG_ERR_INVALID, "pmg prolong: bad arguments (1 <= Nc <= Nf <= 8)");
  return pmg_prolongate_map<T>(Nf, Nc, E, g2lC, xC, P, g2lF, ownerF, xF, (cudaStream_t)stream);
}
extern "C" int lpg_pmg_restrict_f64(int Nf, int Nc, int64_t E, const int32_t* g2lF, const double* weightF,
                                    const double* rF, const double* P, const int32_t* g2lC, double* rC,
                                    int64_t NglobalC, void* stream) {
  return restrict_entry<double>(Nf, Nc, E, g2lF, weightF, rF, P, g2lC, rC, NglobalC, stream);
}
extern "C" int lpg_pmg_restrict_f32(int Nf, int Nc, int64_t E, const int32_t* g2lF, const float* weightF,
                                    const float* rF, const float* P, const int32_t* g2lC, float* rC,
                                    int64_t NglobalC, void* stream) {
  return restrict_entry<float>(Nf, Nc, E, g2lF, weightF, rF, P, g2lC, rC, NglobalC, stream);
}
extern "C" int lpg_pmg_prolong_add_f64(int Nf, int Nc, int64_t E, const int32_t* g2lC, const double* xC,
                                       const double* P, const int32_t* g2lF, const int32_t* ownerF, double* xF,
                                       void* stream) {
  return prolong_entry<double>(Nf, Nc, E, g2lC, xC, P, g2lF, ownerF, xF, stream);
}
extern "C" int lpg_pmg_prolong_add_f32(int Nf, int Nc, int64_t E, const int32_t* g2lC, const float* xC,
                                       const float* P, const int32_t* g2lF, const int32_t* ownerF, float* xF,
                                       void* stream) {
  return prolong_entry<float>(Nf, Nc, E, g2lC, xC, P, g2lF, ownerF, xF, stream);
}
template <typename T>
static int cheb_start_entry(int64_t N, const T* invDiag, const T* r, const T* Ax, T* res, T* d, T* x, T invTheta,
                            int xIsZero, void* stream) {
  if (N < 0 || (N > 0 && (!invDiag || !r || !res || !d || !x || (!xIsZero && !Ax))))
    return set_error(LPG_ERR_INVALID, "cheb start: bad arguments");
  return cheb_start<T>(N, invDiag, r, xIsZero ? nullptr : Ax, res, d, x, invTheta, xIsZero != 0,
                       (cudaStream_t)stream);
}
template <typename T>
static int cheb_step_entry(int64_t N, const T* invDiag, const T* Ad, T* res, T* d, T* x, T a, T b, void* stream) {
  if (N < 0 || (N > 0 && (!invDiag || !Ad || !res || !d || !x))) return set_error(LPG_ERR_INVALID, "cheb step: bad arguments");
  return cheb_step<T>(N, invDiag, Ad, res, d, x, a, b, (cudaStream_t)stream);
}
extern "C" int lpg_cheb_start_f64(int64_t N, const double* invDiag, const double* r, const double* Ax, double* res,
                                  double* d, double* x, double invTheta, int xIsZero, void* stream) {
  return cheb_start_entry<double>(N, invDiag, r, Ax, res, d, x, invTheta, xIsZero, stream);
}
extern "C" int lpg_cheb_start_f32(int64_t N, const float* invDiag, const float* r, const float* Ax, float* res,
                                  float* d, float* x, float invTheta, int xIsZero, void* stream) {
  return cheb_start_entry<float>(N, invDiag, r, Ax, res, d, x, invTheta, xIsZero, stream);
}
extern "C" int lpg_cheb_update_f64(int64_t N, const double* invDiag, const double* Ad, double* res, double* d,
                                   double* x, double a, double b, void* stream) {
  return cheb_step_entry<double>(N, invDiag, Ad, res, d, x, a, b, stream);
}
extern "C" int lpg_cheb_update_f32(int64_t N, const float* invDiag, const float* Ad, float* res, float* d, float* x,
                                   float a, float b, void* stream) {
  return cheb_step_entry<float>(N, invDiag, Ad, res, d, x, a, b, stream);
}

// parAlmond level kernels (CSR: int64 row starts, int32 columns, FP64 values)
static bool csr_ok(int64_t n, const int64_t* rs, const int32_t* cols, const double* vals) {
  return n >= 0 && (n == 0 || (rs && cols && vals));
}
extern "C" int lpg_csr_spmv_f64(int64_t Nrows, const int64_t* rowStarts, const int32_t* cols, const double* vals,
                                double alpha, const double* x, double beta, double* y, void* stream) {
  if (!csr_ok(Nrows, rowStarts, cols, vals) || (Nrows > 0 && (!x || !y)))
    return set_error(LPG_ERR_INVALID, "csr spmv: bad arguments");
  return csr_spmv(Nrows, rowStarts, cols, vals, alpha, x, beta, y, (cudaStream_t)stream);
}
extern "C" int lpg_csr_cheb_start_f64(int64_t N, double invTheta, const double* diagInv, const double* b, double* r,
                                      double* d, double* x, void* stream) {
  if (N < 0 || (N > 0 && (!diagInv || !b || !r || !d || !x))) return set_error(LPG_ERR_INVALID, "csr cheb start: bad arguments");
  return csr_cheb_start(N, invTheta, diagInv, b, r, d, x, (cudaStream_t)stream);
}
extern "C" int lpg_csr_cheb_residual_f64(int64_t N, const int64_t* rowStarts, const int32_t* cols, const double* vals,
                                         double alpha, double beta, const double* diagInv, const double* b,
                                         const double* x, double* r, void* stream) {
  if (!csr_ok(N, rowStarts, cols, vals) || (N > 0 && (!diagInv || !b || !x || !r)))
    return set_error(LPG_ERR_INVALID, "csr cheb residual: bad arguments");
  return csr_cheb_residual(N, rowStarts, cols, vals, alpha, beta, diagInv, b, x, r, (cudaStream_t)stream);
}
extern "C" int lpg_csr_cheb_update_f64(int64_t N, double a, double b, int lastIt, const double* r, double* d,
                                       double* x, void* stream) {
  if (N < 0 || (N > 0 && (!r || !d || !x))) return set_error(LPG_ERR_INVALID, "csr cheb update: bad arguments");
  return csr_cheb_update(N, a, b, lastIt, r, d, x, (cudaStream_t)stream);
}
extern "C" int lpg_gemv_f64(int64_t n, const double* A, const double* x, double* y, void* stream) {
  if (n < 0 || (n > 0 && (!A || !x || !y))) return set_error(LPG_ERR_INVALID, "gemv: bad arguments");
  return gemv(n, A, x, y, (cudaStream_t)stream);
}

// ================================================================ solver objects
extern "C" int lpg_elliptic_create(const char* settings, lpg_elliptic** out) {
  if (!settings || !out) return set_error(LPG_ERR_INVALID, "null argument");
  *out = nullptr;
  LPG_GUARD_BEGIN
  auto h = std::make_unique<lpg_elliptic>();
  int rc = h->settings.parse(settings);
  if (rc) return rc;
  if ((rc = build(h.get()))) return rc;
  *out = h.release();
  return LPG_OK;
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_destroy(lpg_elliptic* e) {
  LPG_GUARD_BEGIN
  delete e;
  return LPG_OK;
  LPG_GUARD_END
}

extern "C" int64_t lpg_elliptic_info(const lpg_elliptic* e, int what) {
  if (!e || !e->el) return -1;
  switch (what) {
    case LPG_INFO_NELEMENTS: return e->el->mesh.E;
    case LPG_INFO_NP: return e->el->mesh.Np;
    case LPG_INFO_NGLOBAL: return e->el->Nglobal;
    case LPG_INFO_NLOCAL: return e->el->Nlocal;
    case LPG_INFO_N: return e->el->mesh.N;
    case LPG_INFO_ALLNEUMANN: return e->el->allNeumann ? 1 : 0;
    case LPG_INFO_MG_PLEVELS: return e->precon ? e->precon->levels_p() : 0;
    case LPG_INFO_MG_AMGLEVELS: return e->precon ? e->precon->levels_amg() : 0;
    case LPG_INFO_COARSE_N: return e->precon ? e->precon->coarse_n() : 0;
    case LPG_INFO_DEVICE_BYTES: return device_bytes_in_use();
    case LPG_INFO_VCYCLES: return e->precon ? e->precon->vcycles() : 0;
    case LPG_INFO_FALLBACKS: return e->precon ? e->precon->fallbacks() : 0;
    case LPG_INFO_HOST_CHUNKS: return e->el->pipe ? e->el->pipe->K : 0;
    case LPG_INFO_IG_HISTORY: return e->ig ? e->ig->history() : 0;
    case LPG_INFO_OPERATOR_APPLICATIONS: return e->el->nOps;
    case LPG_INFO_LEARNED_TIMEOUTS: return e->precon ? e->precon->learned_timeouts() : 0;
    case LPG_INFO_MORTON_ORDER: return e->el->elemOrder.p ? 1 : 0;
    default: return -1;
  }
}

extern "C" int lpg_elliptic_get(const lpg_elliptic* e, const char* name, void* host_out, uint64_t bytes) {
  if (!e || !name || !host_out) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  Elliptic* el = e->el.get();
  cudaStream_t s = e->plat.stream;
  const std::string n(name);
  const int64_t E = el->mesh.E, Np = el->mesh.Np;
  auto need = [&](uint64_t b) { return bytes < b ? set_error(LPG_ERR_INVALID, "output buffer too small") : LPG_OK; };
  int rc;
  if (n == "GlobalToLocal") {
    if ((rc = need(sizeof(int32_t) * el->Nlocal))) return rc;
    return el->g2l.download((int32_t*)host_out, el->Nlocal, s);
  }
  if (n == "ownerLocal") {
    if ((rc = need(sizeof(int32_t) * el->Nglobal))) return rc;
    return el->owner.download((int32_t*)host_out, el->Nglobal, s);
  }
  if (n == "weightG") {
    if ((rc = need(sizeof(double) * el->Nglobal))) return rc;
    return el->weightG.download((double*)host_out, el->Nglobal, s);
  }
  if (n == "D") {
    if ((rc = need(sizeof(double) * el->mesh.D.size()))) return rc;
    std::memcpy(host_out, el->mesh.D.data(), sizeof(double) * el->mesh.D.size());
    return LPG_OK;
  }
  if (n == "lambdaE") {
    if (!el->hasLambdaE) return set_error(LPG_ERR_INVALID, "no lambda field");
    if ((rc = need(sizeof(double) * E))) return rc;
    std::memcpy(host_out, el->lambdaE_h.data(), sizeof(double) * E);
    return LPG_OK;
  }
  if (n == "ggeo" || n == "wJ" || n == "geo") {
    std::vector<double> geo(E * 7 * Np);
    if ((rc = el->mesh.geo.download(geo.data(), E * 7 * Np, s))) return rc;
    double* out = (double*)host_out;
    if (n == "geo") {
      if ((rc = need(sizeof(double) * E * 7 * Np))) return rc;
      std::memcpy(out, geo.data(), sizeof(double) * E * 7 * Np);
    } else if (n == "ggeo") {
      if ((rc = need(sizeof(double) * E * 6 * Np))) return rc;
      for (int64_t e2 = 0; e2 < E; ++e2) std::memcpy(out + e2 * 6 * Np, geo.data() + e2 * 7 * Np, sizeof(double) * 6 * Np);
    } else {
      if ((rc = need(sizeof(double) * E * Np))) return rc;
      for (int64_t e2 = 0; e2 < E; ++e2) std::memcpy(out + e2 * Np, geo.data() + e2 * 7 * Np + 6 * Np, sizeof(double) * Np);
    }
    return LPG_OK;
  }
  if (n == "invDiag") {
    if ((rc = need(sizeof(double) * el->Nglobal))) return rc;
    DevBuf<double> d;
    if ((rc = d.alloc(el->Nglobal)) || (rc = el->BuildDiagonal(d.p, s)) || (rc = inverse_f64(el->Nglobal, d.p, d.p, s)))
      return rc;
    return d.download((double*)host_out, el->Nglobal, s);
  }
  return set_error(LPG_ERR_INVALID, "unknown array name: " + n);
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_device_ptr(const lpg_elliptic* e, const char* name, void** ptr) {
  if (!e || !name || !ptr) return set_error(LPG_ERR_INVALID, "null argument");
  const std::string n(name);
  if (n == "q_in") *ptr = e->q_in.p;
  else if (n == "Aq_out") *ptr = e->Aq_out.p;
  else if (n == "x") *ptr = e->x.p;
  else if (n == "r") *ptr = e->r.p;
  else if (n == "GlobalToLocal") *ptr = e->el->g2l.p;
  else if (n == "geo") *ptr = e->el->mesh.geo.p;
  else if (n == "D") *ptr = e->el->mesh.D_d.p;
  else if (n == "stream") *ptr = (void*)e->plat.stream;
  else return set_error(LPG_ERR_INVALID, "unknown device pointer name: " + n);
  return LPG_OK;
}

extern "C" int lpg_elliptic_random_vector(lpg_elliptic* e, uint64_t seed, double* q, void* stream) {
  if (!e || !q) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  const MeshConfig& c = e->mcfg;
  if (!c.is_box() || c.ipdg)
    return set_error(LPG_ERR_UNSUPPORTED, "random lattice vectors need MESH FILE = BOX and CONTINUOUS");
  BoxNumbering b{c.nx, c.ny, c.nz, e->el->mesh.N, c.bcflag == -1 ? 1 : 0, c.bcflag == 1 ? 1 : 0};
  return lattice_random(b, e->el->Nglobal, e->el->owner.p, seed, q, pick(e, stream));
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_operator(lpg_elliptic* e, const double* q, double* Aq, void* stream) {
  if (!e || !q || !Aq) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  return e->el->Operator(q, Aq, pick(e, stream));
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_operator_df64(lpg_elliptic* e, const double* q, double* Aq, void* stream) {
  if (!e || !q || !Aq) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  return e->el->OperatorDW(q, Aq, pick(e, stream));
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_operator_f32(lpg_elliptic* e, const float* q, float* Aq, int bf16geo, void* stream) {
  if (!e || !q || !Aq) return set_error(LPG_ERR_INVALID, "null argument");
  if (e->el->ipdg && bf16geo) return set_error(LPG_ERR_UNSUPPORTED, "BF16 geometry is defined for CONTINUOUS only");
  LPG_GUARD_BEGIN
  cudaStream_t s = pick(e, stream);
  int rc = e->el->make_f32(bf16geo != 0, s);
  if (rc) return rc;
  return e->el->OperatorF32(q, Aq, bf16geo ? Prec::BF16G : Prec::F32, s);
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_operator_host(lpg_elliptic* e, const double* q_host, double* Aq_host) {
  if (!e || !q_host || !Aq_host) return set_error(LPG_ERR_INVALID, "null argument");
  if (e->el->ipdg) return set_error(LPG_ERR_UNSUPPORTED, "the host-buffer operator is CONTINUOUS only");
  LPG_GUARD_BEGIN
  return e->el->OperatorHost(q_host, Aq_host, e->plat.stream);
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_operator_host_f32(lpg_elliptic* e, const float* q_host, float* Aq_host, int bf16geo) {
  if (!e || !q_host || !Aq_host) return set_error(LPG_ERR_INVALID, "null argument");
  if (e->el->ipdg) return set_error(LPG_ERR_UNSUPPORTED, "the host-buffer operator is CONTINUOUS only");
  LPG_GUARD_BEGIN
  cudaStream_t s = e->plat.stream;
  int rc = e->el->make_f32(bf16geo != 0, s);
  if (rc) return rc;
  return e->el->OperatorHostF32(q_host, Aq_host, bf16geo ? Prec::BF16G : Prec::F32, s);
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_precon(lpg_elliptic* e, const double* r, double* z, void* stream) {
  if (!e || !r || !z) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  cudaStream_t s = pick(e, stream);
  if (s != e->plat.stream) {
    // the preconditioner's scratch lives on the object's stream: order the work
    LPG_CUDA_TRY(cudaStreamSynchronize(s));
    int rc = e->precon->apply(r, z, e->plat.stream);
    if (rc) return rc;
    LPG_CUDA_TRY(cudaStreamSynchronize(e->plat.stream));
    return LPG_OK;
  }
  return e->precon->apply(r, z, s);
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_zero_mean(lpg_elliptic* e, double* q, void* stream) {
  if (!e || !q) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  Elliptic* el = e->el.get();
  if (!el->allNeumann) return LPG_OK;
  cudaStream_t s = stream ? (cudaStream_t)stream : e->plat.stream;
  int rc;
  if ((rc = sum(el->Nglobal, q, e->plat.scalars.p + 1, e->plat.partials.p, s))) return rc;
  return add_scalar(el->Nglobal, e->plat.scalars.p + 1, -el->allNeumannScale * el->allNeumannScale, q, s);
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_mass(lpg_elliptic* e, const double* u, double* Mu, void* stream) {
  if (!e || !u || !Mu) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  Elliptic* el = e->el.get();
  if (el->ipdg) return set_error(LPG_ERR_UNSUPPORTED, "mass product: CONTINUOUS discretisation only");
  cudaStream_t s = stream ? (cudaStream_t)stream : e->plat.stream;
  return mass_apply(el->mesh.N, el->mesh.E, el->mesh.geo.p, el->g2l.p, u, Mu, el->Nglobal, s);
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_rhs(lpg_elliptic* e, double* r, void* stream) {
  if (!e || !r) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  (void)stream;
  return e->el->BuildRhs(r, e->plat.stream);
  LPG_GUARD_END
}

static int solve_impl(lpg_elliptic* e, double* x, double* r, double tol, int maxit, int* iters) {
  Elliptic* el = e->el.get();
  cudaStream_t s = e->plat.stream;
  int rc;
  if (el->allNeumann) {  // elliptic_t::Solve removes the mean of r (ellipticSolve.cpp:33-34)
    if ((rc = sum(el->Nglobal, r, e->plat.scalars.p + 1, e->plat.partials.p, s))) return rc;
    if ((rc = add_scalar(el->Nglobal, e->plat.scalars.p + 1, -el->allNeumannScale * el->allNeumannScale, r, s))) return rc;
  }
  // linearSolver_t::Solve (linearSolver.cpp:30-43): initial guess from the history,
  // solve, then the new solution goes into the history
  if ((rc = e->ig->form(x, r, s))) return rc;
  PCGResult res;
  if (e->nonblocking) rc = nbfpcg_solve(&e->plat, el, e->precon.get(), e->nbwork, x, r, tol, maxit, res);
  else rc = pcg_solve(&e->plat, el, e->precon.get(), e->work, e->flexible, e->stopRhs, x, r, tol, maxit, res);
  if (rc) return rc;
  if (iters) *iters = res.iters;
  if (!res.breakdown && (rc = e->ig->update(el, x, s))) return rc;
  if (res.breakdown) return set_error(LPG_ERR_BREAKDOWN, "(F)PCG breakdown: non-positive p.Ap or non-finite residual");
  if (res.iters >= maxit) return set_error(LPG_ERR_NOT_CONVERGED, "(F)PCG reached the iteration limit");
  return LPG_OK;
}

extern "C" int lpg_elliptic_initial_guess(lpg_elliptic* e, double* x, const double* rhs, void* stream) {
  if (!e || !x || !rhs) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  cudaStream_t s = pick(e, stream);
  int rc = e->ig->form(x, rhs, s);
  if (rc) return rc;
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  return LPG_OK;
  LPG_GUARD_END
}

extern "C" int lpg_extrap_coeffs(int degree, int history, int cpqr, double* coeffs_out) {
  if (!coeffs_out) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  std::vector<double> c;
  const int rc = extrap_coeffs(degree, history, cpqr != 0, c);
  if (rc) return rc;
  std::memcpy(coeffs_out, c.data(), sizeof(double) * c.size());
  return LPG_OK;
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_solve(lpg_elliptic* e, double* x, double* r, double tol, int maxit, int* iters) {
  if (!e || !x || !r) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  return solve_impl(e, x, r, tol, maxit, iters);
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_run(lpg_elliptic* e, double* xL_host, int* iters, double* norm, double* err,
                                double* solve_seconds) {
  if (!e) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  Elliptic* el = e->el.get();
  cudaStream_t s = e->plat.stream;
  int rc;
  if ((rc = el->BuildRhs(e->r.p, s))) return rc;
  LPG_CUDA_TRY(cudaMemsetAsync(e->x.p, 0, sizeof(double) * el->Nglobal, s));
  if (!e->xL.p && (rc = e->xL.alloc(el->Nlocal))) return rc;
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  const auto t0 = std::chrono::steady_clock::now();
  int it = 0;
  rc = solve_impl(e, e->x.p, e->r.p, e->tol, e->maxit, &it);
  if (rc && rc != LPG_ERR_NOT_CONVERGED) return rc;
  const int solveStatus = rc;
  if ((rc = scatter<double>(el->Nlocal, el->g2l.p, e->x.p, e->xL.p, s))) return rc;
  if ((rc = solution_norms(el->mesh.N, el->mesh.E, el->mesh.EX.p, el->mesh.EY.p, el->mesh.EZ.p, el->mesh.r1d_d.p,
                           el->mesh.geo.p, el->g2l.p, el->rhsKind, e->xL.p, e->norms.p, s)))
    return rc;
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  const auto t1 = std::chrono::steady_clock::now();
  double nrm[2];
  if ((rc = e->norms.download(nrm, 2, s))) return rc;
  if (iters) *iters = it;
  if (norm) *norm = std::sqrt(nrm[0]);
  if (err) *err = (el->rhsKind == 0) ? std::sqrt(nrm[1]) : -1.0;
  if (solve_seconds) *solve_seconds = std::chrono::duration<double>(t1 - t0).count();
  if (xL_host && (rc = e->xL.download(xL_host, el->Nlocal, s))) return rc;
  if (e->settings.is("OUTPUT TO FILE", "TRUE")) {
    const std::string name = e->settings.get("OUTPUT FILE NAME", "elliptic") + "_0000.vtu";
    if ((rc = el->PlotFields(e->xL.p, name, s))) return rc;
  }
  return solveStatus;
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_plot_fields(lpg_elliptic* e, const double* qL, const char* file_name) {
  if (!e || !qL || !file_name) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  return e->el->PlotFields(qL, file_name, e->plat.stream);
  LPG_GUARD_END
}

// ================================================================ Gmsh meshes (host only)
extern "C" int lpg_hex_mesh_info(const char* path, int64_t* nelements, int64_t* nnodes, int64_t* nboundary_faces) {
  if (!path) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  HexMeshData m;
  const int rc = read_gmsh_hex(path, m);
  if (rc) return rc;
  if (nelements) *nelements = m.E;
  if (nnodes) *nnodes = m.Nnodes;
  if (nboundary_faces) *nboundary_faces = (int64_t)m.binfo.size() / 5;
  return LPG_OK;
  LPG_GUARD_END
}

extern "C" int lpg_hex_mesh_numbering(const char* path, int N, int32_t* global_to_local, int64_t* nglobal) {
  if (!path) return set_error(LPG_ERR_INVALID, "null argument");
  if (N < 1 || N > 8) return set_error(LPG_ERR_UNSUPPORTED, "POLYNOMIAL DEGREE must be 1..8");
  LPG_GUARD_BEGIN
  HexMeshData m;
  int rc = read_gmsh_hex(path, m);
  if (rc) return rc;
  std::vector<double> r1d, w1d;
  gll_nodes_weights(N, r1d, w1d);
  HexNumbering num;
  if ((rc = number_hex_nodes(m, N, r1d, num))) return rc;
  if (global_to_local) std::memcpy(global_to_local, num.g2l.data(), sizeof(int32_t) * num.g2l.size());
  if (nglobal) *nglobal = num.Nglobal;
  return LPG_OK;
  LPG_GUARD_END
}

// ================================================================ learned smoother
extern "C" int64_t lpg_mlp_param_count(void) { return kMlpParams; }
extern "C" int64_t lpg_mlp_workspace_floats(int64_t B) { return B > 0 ? MLPActs::floats(B) : 0; }

extern "C" int lpg_mlp_forward_f32(const float* params, int64_t B, const float* X, float* workspace, float* Y,
                                   void* stream) {
  if (!params || !X || !workspace || !Y || B <= 0 || B > INT32_MAX)
    return set_error(LPG_ERR_INVALID, "mlp forward: bad arguments");
  LPG_GUARD_BEGIN
  cudaStream_t s = (cudaStream_t)stream;
  MLPParams P = MLPParams::view(const_cast<float*>(params));
  MLPActs A = MLPActs::view(workspace, B);
  int rc = mlp_forward_f32(P, (int)B, X, A, s);
  if (rc) return rc;
  LPG_CUDA_TRY(cudaMemcpyAsync(Y, A.A[3], sizeof(float) * B * kMlpOut, cudaMemcpyDeviceToDevice, s));
  return LPG_OK;
  LPG_GUARD_END
}

extern "C" int lpg_mlp_backward_f32(const float* params, int64_t B, const float* X, const float* workspace,
                                    const float* dY, float* grads, float* work, void* stream) {
  if (!params || !X || !workspace || !dY || !grads || !work || B <= 0 || B > INT32_MAX)
    return set_error(LPG_ERR_INVALID, "mlp backward: bad arguments");
  LPG_GUARD_BEGIN
  MLPParams P = MLPParams::view(const_cast<float*>(params));
  MLPParams G = MLPParams::view(grads);
  MLPActs A = MLPActs::view(const_cast<float*>(workspace), B);
  return mlp_backward_f32(P, (int)B, X, A, dY, G, work, work + B * kMlpHidden, (cudaStream_t)stream);
  LPG_GUARD_END
}

extern "C" int lpg_mlp_adam_f32(int64_t n, float* w, const float* g, float* m, float* v, float lr, int step,
                                void* stream) {
  if (n < 0 || (n > 0 && (!w || !g || !m || !v)) || step < 1) return set_error(LPG_ERR_INVALID, "adam: bad arguments");
  return adam_step(n, w, g, m, v, lr, step, (cudaStream_t)stream);
}

extern "C" int lpg_mlp_forward_bf16(const float* params, int64_t B, const float* X, float* Y, void* stream) {
  if (!params || !X || !Y || B <= 0 || B > INT32_MAX) return set_error(LPG_ERR_INVALID, "mlp bf16 forward: bad arguments");
  LPG_GUARD_BEGIN
  cudaStream_t s = (cudaStream_t)stream;
  LearnedSmoother L;
  int rc;
  std::vector<float> host(kMlpParams);
  LPG_CUDA_TRY(cudaMemcpyAsync(host.data(), params, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, s));
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  if ((rc = L.load(host.data(), s)) || (rc = L.ensure_chunk(B))) return rc;
  if ((rc = convert<float, __nv_bfloat16>(B * kMlpIn, X, L.X.p, s))) return rc;
  if ((rc = L.forward_bf16(B, L.out.p, s))) return rc;
  LPG_CUDA_TRY(cudaMemcpyAsync(Y, L.out.p, sizeof(float) * B * kMlpOut, cudaMemcpyDeviceToDevice, s));
  if ((rc = L.check_tc(s))) return rc;
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  return LPG_OK;
  LPG_GUARD_END
}

extern "C" int lpg_debug_mlp_hold(uint64_t ns) {
  mlp_tc_set_hold((unsigned long long)ns);
  return LPG_OK;
}

extern "C" int lpg_smoother_train(const char* settings, int nsolves, int samples_per_solve, int epochs, int batch,
                                  float lr, uint64_t seed, float* weights_host, float* loss_history_host) {
  if (!settings || !weights_host || nsolves < 1 || samples_per_solve < 1 || epochs < 1 || batch < 1 ||
      (int64_t)nsolves * samples_per_solve < batch)
    return set_error(LPG_ERR_INVALID, "smoother train: bad arguments");
  LPG_GUARD_BEGIN
  lpg_elliptic* e = nullptr;
  int rc = lpg_elliptic_create(settings, &e);
  if (rc) return rc;
  std::unique_ptr<lpg_elliptic> owner(e);
  if (e->precon->levels_p() < 1 || e->settings.get("PRECONDITIONER", "") != "MULTIGRID")
    return set_error(LPG_ERR_INVALID, "smoother train: PRECONDITIONER must be MULTIGRID");
  const MeshConfig& c = e->mcfg;
  if (!c.is_box()) return set_error(LPG_ERR_UNSUPPORTED, "smoother training needs MESH FILE = BOX");
  BoxNumbering b{c.nx, c.ny, c.nz, e->el->mesh.N, c.bcflag == -1 ? 1 : 0, c.bcflag == 1 ? 1 : 0};
  TrainOptions o;
  o.nsolves = nsolves;
  o.samplesPerSolve = samples_per_solve;
  o.epochs = epochs;
  o.batch = batch;
  o.lr = lr;
  o.seed = seed;
  const std::string pairs = e->settings.get("SMOOTHER TRAINING PAIRS", "MIXED");
  if (pairs != "MIXED" && pairs != "TRAJECTORY")
    return set_error(LPG_ERR_SETTINGS, "SMOOTHER TRAINING PAIRS must be MIXED or TRAJECTORY");
  o.synthetic = (pairs == "MIXED");
  std::vector<float> w, hist;
  if ((rc = train_smoother(&e->plat, e->el.get(), e->precon.get(), b, o, w, hist))) return rc;
  std::memcpy(weights_host, w.data(), sizeof(float) * w.size());
  if (loss_history_host) std::memcpy(loss_history_host, hist.data(), sizeof(float) * hist.size());
  return LPG_OK;
  LPG_GUARD_END
}

extern "C" int lpg_elliptic_set_learned_smoother(lpg_elliptic* e, const float* weights_host, double threshold) {
  if (!e) return set_error(LPG_ERR_INVALID, "null argument");
  LPG_GUARD_BEGIN
  const MeshConfig& c = e->mcfg;
  if (!c.is_box() && weights_host) return set_error(LPG_ERR_UNSUPPORTED, "the learned smoother needs MESH FILE = BOX");
  BoxNumbering b{c.nx, c.ny, c.nz, e->el->mesh.N, c.bcflag == -1 ? 1 : 0, c.bcflag == 1 ? 1 : 0};
  if (!weights_host) {
    int rc = e->precon->set_learned(nullptr, b, threshold);
    e->learned.reset();
    return rc;
  }
  auto L = std::make_unique<LearnedSmoother>();
  int rc = L->load(weights_host, e->plat.stream);
  if (rc) return rc;
  if ((rc = e->precon->set_learned(L.get(), b, threshold))) return rc;
  e->learned = std::move(L);
  return LPG_OK;
  LPG_GUARD_END
}
