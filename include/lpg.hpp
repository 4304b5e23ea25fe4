/*
 * libparanumal_gb300: C++ surface of the C0 hexahedral elliptic path with the shapes of
 * libParanumal's classes, header-only over the C ABI in lpg.h (no CUDA headers needed).
 *
 *   libp::deviceMemory<T>, libp::memory<T>   include/memory.hpp:35-345 (ref-counted, +offset slices)
 *   libp::settings_t, libp::platform_t, libp::comm_t
 *   libp::operator_t                          include/operator.hpp:35-40
 *   libp::precon_t, libp::IdentityPrecon      include/precon.hpp:36-69
 *   libp::linearSolver_t + LinearSolver::pcg / fpcg
 *                                             include/linearSolver.hpp:41-96, libs/linearSolver/linearSolverPCG.cpp:35-171
 *   libp::ogs::ogs_t                          include/ogs.hpp:179-345 (one rank, k = 1, Add)
 *   libp::elliptic_t                          solvers/elliptic/elliptic.hpp:110-169
 *
 * Errors: a non-zero status from the C ABI becomes a libp::exception carrying the status
 * and lpg_last_error()'s text, as LIBP_ABORT throws libp::exception (include/utils.hpp:57-76).
 * Paths above are relative to the libParanumal source tree.
 *
 * Differences from the reference, by design of this library:
 *   - one rank: comm_t is a placeholder and halo exchanges are absent;
 *   - elliptic_t::Setup builds its mesh from the settings (BOX or Gmsh MESH FILE) instead of
 *     taking a mesh_t; its preconditioner is the one the settings name and lives on the GPU;
 *   - the Krylov solvers below are generic over operator_t (any operator and preconditioner
 *     object) and run their vector work through the library's BLAS-1 kernels;
 *     elliptic_t::Solve uses them as the reference's does.
 */
#ifndef LPG_HPP
#define LPG_HPP

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdint>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lpg.h"

namespace libp {

typedef double dfloat;
typedef int dlong;
typedef long long hlong;

class exception : public std::runtime_error {
 public:
  exception(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status, const char* where) {
  if (status != LPG_OK) {
    const char* msg = lpg_last_error();
    throw exception(status, std::string(where) + ": " + (msg ? msg : ""));
  }
}

/* host array: memory<T> (include/memory.hpp:35-285), contiguous, shallow-copied handle */
template <typename T>
class memory {
 public:
  memory() = default;
  explicit memory(size_t n) { malloc(n); }
  void malloc(size_t n) { data_ = std::make_shared<std::vector<T>>(n); }
  void calloc(size_t n) { data_ = std::make_shared<std::vector<T>>(n, T(0)); }
  size_t length() const { return data_ ? data_->size() : 0; }
  T* ptr() { return data_ ? data_->data() : nullptr; }
  const T* ptr() const { return data_ ? data_->data() : nullptr; }
  T& operator[](size_t i) { return (*data_)[i]; }
  const T& operator[](size_t i) const { return (*data_)[i]; }

 private:
  std::shared_ptr<std::vector<T>> data_;
};

/* device array: deviceMemory<T> (include/memory.hpp:289-345). Copies share the buffer;
 * o + k is a slice starting k entries in. */
template <typename T>
class deviceMemory {
 public:
  deviceMemory() = default;
  /* a view of device memory owned elsewhere (no free) */
  deviceMemory(T* ptr, size_t n) : base_(std::shared_ptr<void>(static_cast<void*>(ptr), [](void*) {})), n_(n) {}

  static deviceMemory alloc(size_t n) {
    void* p = nullptr;
    check(lpg_device_malloc(&p, sizeof(T) * (n ? n : 1)), "deviceMemory::malloc");
    deviceMemory m;
    m.base_ = std::shared_ptr<void>(p, [](void* q) { lpg_device_free(q); });
    m.n_ = n;
    return m;
  }

  size_t length() const { return n_; }
  T* ptr() const { return base_ ? static_cast<T*>(base_.get()) + off_ : nullptr; }
  bool isInitialized() const { return base_ != nullptr; }

  deviceMemory operator+(ptrdiff_t k) const {
    deviceMemory m = *this;
    m.off_ += k;
    m.n_ -= k;
    return m;
  }

  void copyFrom(const T* host, size_t n, size_t offset = 0) {
    check(lpg_memcpy_h2d(ptr() + offset, host, sizeof(T) * n, nullptr), "deviceMemory::copyFrom");
    check(lpg_stream_sync(nullptr), "deviceMemory::copyFrom");
  }
  void copyFrom(const memory<T>& h) { copyFrom(h.ptr(), h.length()); }
  void copyFrom(const deviceMemory<T>& d, size_t n) {
    check(lpg_memcpy_d2d(ptr(), d.ptr(), sizeof(T) * n, nullptr), "deviceMemory::copyFrom");
  }
  void copyTo(T* host, size_t n, size_t offset = 0) const {
    check(lpg_memcpy_d2h(host, ptr() + offset, sizeof(T) * n, nullptr), "deviceMemory::copyTo");
    check(lpg_stream_sync(nullptr), "deviceMemory::copyTo");
  }
  void copyTo(memory<T>& h) const { copyTo(h.ptr(), h.length()); }

 private:
  std::shared_ptr<void> base_;
  size_t off_ = 0, n_ = 0;
};

/* settings_t (include/settings.hpp): keys and values, rendered in the .rc format */
class settings_t {
 public:
  void changeSetting(const std::string& key, const std::string& value) { kv_[key] = value; }
  template <typename V>
  void changeSetting(const std::string& key, const V& value) {
    std::ostringstream os;
    os << value;
    kv_[key] = os.str();
  }
  std::string getSetting(const std::string& key) const {
    auto it = kv_.find(key);
    return it == kv_.end() ? std::string() : it->second;
  }
  bool compareSetting(const std::string& key, const std::string& value) const { return getSetting(key) == value; }
  /* reads the .rc format: "[KEY]" lines, each followed by its value line */
  void parse(const std::string& text) {
    std::istringstream in(text);
    std::string line, key;
    while (std::getline(in, line)) {
      const size_t a = line.find_first_not_of(" \t\r"), b = line.find_last_not_of(" \t\r");
      if (a == std::string::npos) continue;
      line = line.substr(a, b - a + 1);
      if (line.front() == '[' && line.back() == ']') key = line.substr(1, line.size() - 2);
      else if (!key.empty()) { kv_[key] = line; key.clear(); }
    }
  }
  std::string rc() const {
    std::string s;
    for (const auto& kv : kv_) s += "[" + kv.first + "]\n" + kv.second + "\n\n";
    return s;
  }

 private:
  std::map<std::string, std::string> kv_;
};

struct comm_t {};   // one rank

/* platform_t (include/platform.hpp): the device and its allocations */
class platform_t {
 public:
  platform_t() = default;
  explicit platform_t(const settings_t& s) {
    const std::string d = s.getSetting("DEVICE NUMBER");
    if (!d.empty()) check(lpg_set_device(std::stoi(d)), "platform_t");
  }
  template <typename T>
  deviceMemory<T> malloc(size_t n) const { return deviceMemory<T>::alloc(n); }
  template <typename T>
  deviceMemory<T> malloc(const memory<T>& h) const {
    deviceMemory<T> d = deviceMemory<T>::alloc(h.length());
    d.copyFrom(h);
    return d;
  }
  void finish() const { check(lpg_stream_sync(nullptr), "platform_t::finish"); }
};

/* operator_t (include/operator.hpp:35-40) */
class operator_t {
 public:
  virtual ~operator_t() = default;
  virtual void Operator(deviceMemory<dfloat>& /*o_r*/, deviceMemory<dfloat>& /*o_Mr*/) {
    throw exception(LPG_ERR_UNSUPPORTED, "Operator not implemented in this object");
  }
};

/* precon_t (include/precon.hpp:36-56) */
class precon_t : public operator_t {
 public:
  void Operator(deviceMemory<dfloat>& o_r, deviceMemory<dfloat>& o_Mr) override {
    if (!precon) throw exception(LPG_ERR_INVALID, "Precon not initialized");
    precon->Operator(o_r, o_Mr);
  }
  template <class Precon, class... Args>
  void Setup(Args&&... args) {
    precon = std::make_shared<Precon>(args...);
  }

 private:
  std::shared_ptr<operator_t> precon;
};

/* IdentityPrecon (include/precon.hpp:59-69) */
class IdentityPrecon : public operator_t {
 public:
  explicit IdentityPrecon(dlong n) : N(n) {}
  void Operator(deviceMemory<dfloat>& o_r, deviceMemory<dfloat>& o_Mr) override { o_Mr.copyFrom(o_r, N); }

 private:
  dlong N;
};

namespace LinearSolver {

/* linearSolverBase_t (include/linearSolver.hpp:79-96) */
class linearSolverBase_t {
 public:
  platform_t platform;
  settings_t settings;
  comm_t comm;
  dlong N, Nhalo;
  linearSolverBase_t(dlong n, dlong nhalo, platform_t& p, settings_t& s, comm_t c)
      : platform(p), settings(s), comm(c), N(n), Nhalo(nhalo) {}
  virtual ~linearSolverBase_t() = default;
  virtual int Solve(operator_t& linearOperator, operator_t& precon, deviceMemory<dfloat>& o_x,
                    deviceMemory<dfloat>& o_rhs, const dfloat tol, const int MAXIT, const int verbose) = 0;
};

/* pcg / flexible pcg (libs/linearSolver/linearSolverPCG.cpp:35-171): o_rhs holds the
 * right-hand side and is overwritten by the residual; o_x holds the initial guess and is
 * overwritten by the solution. Stops at ||r||^2 <= max(tol^2 ||r0||^2, tol^2). Returns the
 * iteration count. A non-positive or non-finite p.Ap or a non-finite residual throws with
 * LPG_ERR_BREAKDOWN. */
class pcg : public linearSolverBase_t {
 public:
  pcg(dlong n, dlong nhalo, platform_t& p, settings_t& s, comm_t c, bool flex = false)
      : linearSolverBase_t(n, nhalo, p, s, c), flexible(flex) {
    const size_t len = (size_t)N + Nhalo;
    o_p = deviceMemory<dfloat>::alloc(len);
    o_z = deviceMemory<dfloat>::alloc(len);
    o_Ax = deviceMemory<dfloat>::alloc(len);
    o_Ap = deviceMemory<dfloat>::alloc(len);
    o_scalar = deviceMemory<dfloat>::alloc(1);
  }

  int Solve(operator_t& A, operator_t& M, deviceMemory<dfloat>& o_x, deviceMemory<dfloat>& o_r, const dfloat tol,
            const int MAXIT, const int verbose) override {
    // r = b - A x
    A.Operator(o_x, o_Ax);
    check(lpg_axpy_f64(N, -1.0, o_Ax.ptr(), 1.0, o_r.ptr(), nullptr), "pcg");
    dfloat rdotr = dot(o_r, o_r);
    if (!std::isfinite(rdotr)) throw exception(LPG_ERR_BREAKDOWN, "pcg: non-finite initial residual");
    const dfloat TOL = std::max(tol * tol * rdotr, tol * tol);
    check(lpg_axpy_f64(N, 0.0, o_Ax.ptr(), 0.0, o_p.ptr(), nullptr), "pcg");   // p = 0
    check(lpg_axpy_f64(N, 0.0, o_Ax.ptr(), 0.0, o_Ap.ptr(), nullptr), "pcg");  // Ap = 0
    dfloat rdotz1 = 0, rdotz2 = 0, alpha = 0, beta = 0;
    int iter = 0;
    for (iter = 0; iter < MAXIT; ++iter) {
      if ((iter == 0 && rdotr == 0.0) || (iter > 0 && rdotr <= TOL)) break;
      M.Operator(o_r, o_z);
      rdotz2 = rdotz1;
      rdotz1 = dot(o_r, o_z);
      if (flexible) {
        const dfloat zdotAp = dot(o_z, o_Ap);
        beta = (iter == 0) ? 0.0 : -alpha * zdotAp / rdotz2;
      } else {
        beta = (iter == 0) ? 0.0 : rdotz1 / rdotz2;
      }
      check(lpg_axpy_f64(N, 1.0, o_z.ptr(), beta, o_p.ptr(), nullptr), "pcg");   // p = z + beta p
      A.Operator(o_p, o_Ap);
      const dfloat pAp = dot(o_p, o_Ap);
      if (!(pAp > 0.0) || !std::isfinite(pAp)) throw exception(LPG_ERR_BREAKDOWN, "pcg: non-positive p.Ap");
      alpha = rdotz1 / pAp;
      // x += alpha p; r -= alpha Ap; r.r (linearSolverUpdatePCG.okl)
      check(lpg_pcg_update_f64(N, alpha, o_p.ptr(), o_Ap.ptr(), o_x.ptr(), o_r.ptr(), o_scalar.ptr(), nullptr),
            "pcg");
      rdotr = scalar();
      if (!std::isfinite(rdotr)) throw exception(LPG_ERR_BREAKDOWN, "pcg: non-finite residual");
      if (verbose) std::printf("iter=%05d pAp=%.4e norm(r)=%.4e\n", iter + 1, pAp, std::sqrt(rdotr));
    }
    return iter;
  }

 private:
  bool flexible;
  deviceMemory<dfloat> o_p, o_z, o_Ax, o_Ap, o_scalar;
  dfloat scalar() {
    dfloat v = 0;
    o_scalar.copyTo(&v, 1);
    return v;
  }
  dfloat dot(const deviceMemory<dfloat>& a, const deviceMemory<dfloat>& b) {
    check(lpg_dot_f64(N, a.ptr(), b.ptr(), o_scalar.ptr(), nullptr), "pcg: dot");
    return scalar();
  }
};

/* fpcg: flexible PCG (LINEAR SOLVER = FPCG), beta = -alpha (z.Ap) / (r.z)_old */
class fpcg : public pcg {
 public:
  fpcg(dlong n, dlong nhalo, platform_t& p, settings_t& s, comm_t c) : pcg(n, nhalo, p, s, c, true) {}
};

}  // namespace LinearSolver

/* linearSolver_t (include/linearSolver.hpp:41-73) */
class linearSolver_t {
 public:
  template <class Solver, class... Args>
  void Setup(Args&&... args) {
    ls = std::make_shared<Solver>(args...);
  }
  int Solve(operator_t& linearOperator, operator_t& precon, deviceMemory<dfloat>& o_x, deviceMemory<dfloat>& o_rhs,
            const dfloat tol, const int MAXIT, const int verbose) {
    if (!ls) throw exception(LPG_ERR_INVALID, "LinearSolver not initialized");
    return ls->Solve(linearOperator, precon, o_x, o_rhs, tol, MAXIT, verbose);
  }

 private:
  std::shared_ptr<LinearSolver::linearSolverBase_t> ls;
};

namespace ogs {

typedef enum { Add, Mul, Max, Min } Op;
typedef enum { Sym, NoTrans, Trans } Transpose;
typedef enum { Auto, Pairwise, CrystalRouter, AllToAll } Method;
typedef enum { Signed, Unsigned } Kind;

/* ogs_t (include/ogs.hpp:179-345) on one rank: ids[n] = 0 marks a node that takes no part
 * (masked); nodes with equal |ids| form one group, numbered in order of first appearance
 * (the single-rank order of ogsSetup.cpp). A negative id flags a copy: NoTrans gathers take
 * each group's first unflagged copy. Double data, k = 1, Op = Add. */
class ogs_t {
 public:
  dlong N = 0;
  dlong Ngather = 0;

  void Setup(const dlong _N, memory<hlong> ids, comm_t, const Kind kind, const Method, const bool unique,
             const bool, platform_t& platform) {
    N = _N;
    std::map<hlong, dlong> gid;
    memory<dlong> g2l(N > 0 ? N : 1);
    for (dlong n = 0; n < N; ++n) {
      const hlong id = ids[n];
      if (id == 0) { g2l[n] = -1; continue; }
      const hlong key = id < 0 ? -id : id;
      auto it = gid.find(key);
      if (it == gid.end()) it = gid.emplace(key, (dlong)gid.size()).first;
      g2l[n] = it->second;
    }
    Ngather = (dlong)gid.size();
    memory<dlong> owner(Ngather > 0 ? Ngather : 1);
    for (dlong g = 0; g < Ngather; ++g) owner[g] = -1;
    for (dlong n = 0; n < N; ++n)   // first unflagged copy, else the first copy
      if (g2l[n] >= 0 && (owner[g2l[n]] < 0 || (ids[owner[g2l[n]]] < 0 && ids[n] > 0))) owner[g2l[n]] = n;
    (void)kind;
    (void)unique;
    o_g2l = platform.malloc(g2l);
    o_owner = platform.malloc(owner);
    GlobalToLocal = g2l;
  }

  /* GlobalToLocal (ogs.hpp:195): assembled index per node, -1 where masked */
  void SetupGlobalToLocalMapping(memory<dlong> out) const {
    for (dlong n = 0; n < N; ++n) out[n] = GlobalToLocal[n];
  }

  void Gather(deviceMemory<dfloat> o_gv, deviceMemory<dfloat> o_v, const int k, const Op op, const Transpose trans) {
    need(k, op);
    if (trans == Trans)
      check(lpg_ogs_gather_add_f64(N, o_g2l.ptr(), o_v.ptr(), o_gv.ptr(), Ngather, nullptr), "ogs Gather");
    else
      check(lpg_ogs_gather_owner_f64(Ngather, o_owner.ptr(), o_v.ptr(), o_gv.ptr(), nullptr), "ogs Gather");
  }
  void Scatter(deviceMemory<dfloat> o_v, deviceMemory<dfloat> o_gv, const int k, const Transpose trans) {
    if (k != 1) throw exception(LPG_ERR_UNSUPPORTED, "ogs Scatter: k must be 1");
    if (trans == Trans) throw exception(LPG_ERR_UNSUPPORTED, "ogs Scatter: Trans is not provided");
    check(lpg_ogs_scatter_f64(N, o_g2l.ptr(), o_gv.ptr(), o_v.ptr(), nullptr), "ogs Scatter");
  }
  /* v = Scatter(Gather(v, Trans)) (GatherScatter with Sym) */
  void GatherScatter(deviceMemory<dfloat> o_v, const int k, const Op op, const Transpose) {
    need(k, op);
    if (!o_gs.isInitialized() || o_gs.length() < (size_t)Ngather) o_gs = deviceMemory<dfloat>::alloc(Ngather);
    Gather(o_gs, o_v, k, op, Trans);
    Scatter(o_v, o_gs, k, NoTrans);
  }

 private:
  memory<dlong> GlobalToLocal;
  deviceMemory<dlong> o_g2l, o_owner;
  deviceMemory<dfloat> o_gs;
  static void need(int k, Op op) {
    if (k != 1 || op != Add) throw exception(LPG_ERR_UNSUPPORTED, "ogs: k = 1 and Op = Add only");
  }
};

}  // namespace ogs

class elliptic_t;

/* the preconditioner an elliptic_t's settings name ([PRECONDITIONER] JACOBI, MULTIGRID,
 * PARALMOND, SEMFEM, OAS or NONE), applied on the GPU: z = M^{-1} r */
class EllipticPrecon : public operator_t {
 public:
  explicit EllipticPrecon(lpg_elliptic* h) : h_(h) {}
  void Operator(deviceMemory<dfloat>& o_r, deviceMemory<dfloat>& o_Mr) override {
    check(lpg_elliptic_precon(h_, o_r.ptr(), o_Mr.ptr(), nullptr), "precon Operator");
  }

 private:
  lpg_elliptic* h_;
};

/* elliptic_t (solvers/elliptic/elliptic.hpp:110-169) */
class elliptic_t : public operator_t {
 public:
  platform_t platform;
  settings_t settings;
  precon_t precon;
  dlong Nglobal = 0;   // assembled dofs (the vectors Operator and Solve take)
  hlong Nlocal = 0;    // local nodes E * Np
  int allNeumann = 0;

  elliptic_t() = default;
  elliptic_t(platform_t& p, settings_t& s) { Setup(p, s); }

  /* builds mesh, geometry, numbering and preconditioner from the settings */
  void Setup(platform_t& p, settings_t& s) {
    platform = p;
    settings = s;
    lpg_elliptic* h = nullptr;
    check(lpg_elliptic_create(s.rc().c_str(), &h), "elliptic_t::Setup");
    h_ = std::shared_ptr<lpg_elliptic>(h, [](lpg_elliptic* q) { lpg_elliptic_destroy(q); });
    Nglobal = (dlong)lpg_elliptic_info(h, LPG_INFO_NGLOBAL);
    Nlocal = (hlong)lpg_elliptic_info(h, LPG_INFO_NLOCAL);
    allNeumann = (int)lpg_elliptic_info(h, LPG_INFO_ALLNEUMANN);
    precon.Setup<EllipticPrecon>(h);
  }

  /* elliptic_t::Operator (ellipticOperator.cpp:29-106) */
  void Operator(deviceMemory<dfloat>& o_q, deviceMemory<dfloat>& o_Aq) override {
    check(lpg_elliptic_operator(h_.get(), o_q.ptr(), o_Aq.ptr(), nullptr), "elliptic_t::Operator");
  }

  /* elliptic_t::Solve (ellipticSolve.cpp:29-39) */
  int Solve(linearSolver_t& linearSolver, deviceMemory<dfloat>& o_x, deviceMemory<dfloat>& o_r, const dfloat tol,
            const int MAXIT, const int verbose) {
    if (allNeumann) ZeroMean(o_r);
    return linearSolver.Solve(*this, precon, o_x, o_r, tol, MAXIT, verbose);
  }

  /* elliptic_t::ZeroMean (ellipticZeroMean.cpp:29-37) */
  void ZeroMean(deviceMemory<dfloat>& o_q) {
    check(lpg_elliptic_zero_mean(h_.get(), o_q.ptr(), nullptr), "elliptic_t::ZeroMean");
  }

  /* the assembled right-hand side of Run (forcing, Dirichlet lifting, Gather(Trans)) */
  void BuildRhs(deviceMemory<dfloat>& o_r) {
    check(lpg_elliptic_rhs(h_.get(), o_r.ptr(), nullptr), "elliptic_t::BuildRhs");
  }

  /* elliptic_t::BuildOperatorDiagonal (ellipticBuildOperatorDiagonal.cpp:29-80): the
   * assembled diagonal of A (Nglobal entries) */
  void BuildOperatorDiagonal(memory<dfloat>& diagA) {
    memory<dfloat> inv(Nglobal);
    check(lpg_elliptic_get(h_.get(), "invDiag", inv.ptr(), sizeof(dfloat) * Nglobal), "BuildOperatorDiagonal");
    diagA.malloc(Nglobal);
    for (dlong n = 0; n < Nglobal; ++n) diagA[n] = inv[n] != 0.0 ? 1.0 / inv[n] : 0.0;
  }

  struct RunResult {
    int iterations;
    dfloat norm, error, solveSeconds;
  };
  /* elliptic_t::Run (ellipticRun.cpp:30-248): rhs, timed solve, scatter + AddBC, norms;
   * xL (Nlocal entries) receives the local solution when given */
  RunResult Run(memory<dfloat>* xL = nullptr) {
    RunResult r{};
    if (xL) xL->malloc((size_t)Nlocal);
    const int st = lpg_elliptic_run(h_.get(), xL ? xL->ptr() : nullptr, &r.iterations, &r.norm, &r.error,
                                    &r.solveSeconds);
    if (st != LPG_OK && st != LPG_ERR_NOT_CONVERGED) check(st, "elliptic_t::Run");
    return r;
  }

  /* GlobalToLocal of the assembled numbering (int32 per local node, -1 masked) */
  memory<dlong> GlobalToLocal() const {
    memory<dlong> g(Nlocal);
    check(lpg_elliptic_get(h_.get(), "GlobalToLocal", g.ptr(), sizeof(dlong) * Nlocal), "GlobalToLocal");
    return g;
  }

  lpg_elliptic* handle() const { return h_.get(); }

 private:
  std::shared_ptr<lpg_elliptic> h_;
};

}  // namespace libp

#endif
