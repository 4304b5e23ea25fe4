// Host-side objects mirroring the reference's class surface for the C0 hex path:
// settings_t, platform_t, mesh_t, ogs (masked, Signed + unique), elliptic_t, precon_t
// (Identity / Jacobi / MultiGrid with p-levels and parAlmond AMG levels) and the
// (flexible) PCG linear solver. Device arrays live in HBM; host code orchestrates.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../lpg_internal.hpp"
#include "../lpg_errors.hpp"
#include "hexmesh.hpp"

namespace lpg {

int set_error(int status, const std::string& msg);

// ---------------------------------------------------------------- settings_t
// Parses the reference's .rc format: "[KEY]" lines followed by a value line.
struct Settings {
  std::map<std::string, std::string> kv;
  int parse(const std::string& text);      // LPG_OK or LPG_ERR_SETTINGS
  std::string get(const std::string& k, const std::string& def) const;
  int geti(const std::string& k, int def) const;
  double getd(const std::string& k, double def) const;
  bool is(const std::string& k, const std::string& v) const { return get(k, "") == v; }
};

// ---------------------------------------------------------------- device buffers
template <typename T>
struct DevBuf {
  T* p = nullptr;
  int64_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  int alloc(int64_t count);
  int upload(const T* host, int64_t count, cudaStream_t s);
  int download(T* host, int64_t count, cudaStream_t s) const;
  void release();
  int64_t bytes() const { return n * (int64_t)sizeof(T); }
};

int64_t device_bytes_in_use();

// ---------------------------------------------------------------- drand48 stream
struct Rand48 {
  uint64_t x = 0;
  void seed(long s) { x = (((uint64_t)(uint32_t)s) << 16) | 0x330EULL; }
  double next() {
    x = (0x5DEECE66DULL * x + 0xBULL) & ((1ULL << 48) - 1);
    return (double)x * (1.0 / 281474976710656.0);
  }
};

uint64_t splitmix64(uint64_t x);
double hash_u01(uint64_t seed, uint64_t stream, uint64_t key);

// ---------------------------------------------------------------- 1D basis
void gll_nodes_weights(int N, std::vector<double>& x, std::vector<double>& w);
void gll_derivative(int N, const std::vector<double>& x, std::vector<double>& D);
// Interpolation from GLL(Nc) to GLL(Nf): P[i*(Nc+1)+m] = l_m(x_i)
void gll_interpolation(int Nc, int Nf, std::vector<double>& P);
double hessenberg_spectral_radius(int k, const std::vector<double>& Hcolmajor);

// ---------------------------------------------------------------- platform_t
struct Platform {
  cudaStream_t stream = nullptr;
  DevBuf<double> partials;   // reduction partial sums
  DevBuf<double> scalars;    // device scalars for reductions
  double* hostScalars = nullptr;  // pinned mirror
  int init();
  ~Platform();
  // blocking reductions (one device->host copy per call, as linAlg.cpp:172-185)
  int dot(int64_t n, const double* x, const double* y, double& out);
  int norm2sq(int64_t n, const double* x, double& out) { return dot(n, x, x, out); }
  int sum(int64_t n, const double* x, double& out);
};

// ---------------------------------------------------------------- mesh_t (one degree)
struct MeshConfig {
  int nx = 10, ny = 10, nz = 10;
  double dimx = 10, dimy = 10, dimz = 10;
  int bcflag = 1;
  double jitter = 0.0;
  uint64_t jitterSeed = 0;
  // MESH FILE: a hexahedral mesh read from a Gmsh file (the box fields are then unused)
  std::shared_ptr<const HexMeshData> file;
  bool is_box() const { return !file; }
  // DISCRETIZATION = IPDG (every level of a hierarchy shares it)
  bool ipdg = false;
};

struct Mesh {
  MeshConfig cfg;
  int N = 0, Nq = 0, Np = 0;
  int64_t E = 0;
  std::vector<double> r1d, w1d, D;
  DevBuf<double> EX, EY, EZ;      // [E][8]
  DevBuf<double> D_d, r1d_d, w1d_d;
  DevBuf<double> geo;             // [E][7][Np] FP64
  DevBuf<float> geo32, D32;       // FP32 copies (preconditioner)
  DevBuf<__nv_bfloat16> geo16;    // BF16 copy
  DevBuf<float2> geoDW;           // double-word (hi, lo) copy for the double-word operator
  int setup(const MeshConfig& c, int N, cudaStream_t s);
  // E, N, r1d, w1d, D set: upload vertices, reference data, geometric factors
  int setup_vertices(const std::vector<double>& ex, const std::vector<double>& ey, const std::vector<double>& ez,
                     cudaStream_t s);
  int make_f32(cudaStream_t s);
  int make_bf16(cudaStream_t s);
  int make_dw(cudaStream_t s);
};

// ---------------------------------------------------------------- elliptic_t
enum class Prec { F64 = 0, F32 = 1, BF16G = 2 };

// Copy/compute pipeline of the host-buffer operator. Elements are cut into K chunks in
// element order; chunk c reads assembled entries [0, inEnd[c]) and, once it has run,
// entries [0, outEnd[c]) of the result are final (no later chunk touches them). With
// the box numbering (entries grouped by owner element, owner = smallest element holding
// the node) both are long prefixes, so the upload of q, the chunks' operator launches
// and the download of Aq overlap on three streams.
struct PipeSplit {
  std::vector<int64_t> e0;          // K+1 chunk boundaries (elements)
  std::vector<int64_t> inEnd, outEnd;
};
struct HostPipe {
  int K = 0;
  // native: the FP64 kernel's chunks, ending on whole waves of that kernel (its time bounds
  // the pipeline); even: equal chunks, for the double-word and FP32 pipelines, which the
  // copies bound
  PipeSplit native, even;
  cudaStream_t h2d = nullptr, d2h = nullptr;
  std::vector<cudaEvent_t> inReady, chunkDone;
  DevBuf<double> q, Aq;
  DevBuf<float> q32, Aq32;
  ~HostPipe();
};

struct Elliptic {
  Platform* plat = nullptr;
  Mesh mesh;
  double lambda = 0;
  bool hasLambdaE = false;
  std::vector<double> lambdaE_h;
  DevBuf<double> lambdaE;
  DevBuf<float> lambdaE32;
  int64_t Nglobal = 0, Nlocal = 0;
  bool allNeumann = false;
  bool hasDirichlet = false;       // some nodes are masked (Dirichlet data lifted into the rhs)
  double allNeumannScale = 1;
  DevBuf<int32_t> g2l, owner;
  // C0 meshes read from a file: the elements in Morton order of their centroids, the order
  // in which the operators visit them (storage keeps the file's order); empty for boxes,
  // whose lattice order already keeps neighbours together
  DevBuf<int32_t> elemOrder;
  DevBuf<double> weightG;
  DevBuf<float> weightG32;
  int rhsKind = 0;                 // 0 sine, 1 Gaussian sources
  std::vector<double> sources;     // nsources*4
  DevBuf<double> sources_d;
  // Neumann boundary data (CONTINUOUS): local nodes on Neumann-type boundary faces and, per
  // node, the mask of those faces
  DevBuf<int32_t> neuNode, neuMask;
  int64_t neuCount = 0;
  int set_neumann_nodes(const std::vector<int32_t>& node, const std::vector<int32_t>& mask, cudaStream_t s);
  // IPDG: unknowns are the local nodes (GlobalToLocal is the identity); face data
  bool ipdg = false;
  double tau = 0;
  DevBuf<double> vgeo, sgeo, g4;
  DevBuf<float> vgeo32, sgeo32, g4_32;  // FP32 copies and gradient scratch (preconditioner levels)
  DevBuf<float2> vgeoDW, sgeoDW;        // (hi, lo) copies for OPERATOR PRECISION DF64
  DevBuf<float> g8;                     // double-word gradients, 8 floats per node
  int OperatorIpdgDW(const double* q, double* Aq, cudaStream_t s);
  int64_t nOps = 0;   // applications through Operator and OperatorF32 (any precision)
  DevBuf<int32_t> vmapP;
  DevBuf<int> EToB;
  std::vector<int64_t> EToE_h;     // element neighbours (host), for the matrix probing
  int setup_ipdg(const MeshConfig& c, int N, const std::vector<double>* lamE, cudaStream_t s);
  int BuildMatrixIpdg(std::vector<int64_t>& rowStarts, std::vector<int32_t>& cols, std::vector<double>& vals,
                      cudaStream_t s);
  IpdgArgs ipdg_args() const;

  int setup(Platform* p, const MeshConfig& c, int N, double lambda, const std::vector<double>* lamE,
            cudaStream_t s);
  int setup_file(const MeshConfig& c, int N, const std::vector<double>* lamE, cudaStream_t s);
  int morton_element_order(const HexMeshData& hm, cudaStream_t s);
  // VTU file of the local field qL (E*Np, device)
  int PlotFields(const double* qL, const std::string& fileName, cudaStream_t s);
  int finish_setup(const std::vector<double>* lamE, cudaStream_t s);
  // low-order problem on the GLL sub-mesh of `sem` sharing its numbering (SEMFEM)
  int setup_semfem(const Elliptic& sem, cudaStream_t s);
  int make_f32(bool bf16, cudaStream_t s);
  // OPERATOR PRECISION: FP64 (default) or DF64 (double-FP32 words on the FP32 pipe,
  // FP64-accurate) for every FP64 operator application of this object
  bool opDW = false;
  int Operator(const double* q, double* Aq, cudaStream_t s);
  int OperatorDW(const double* q, double* Aq, cudaStream_t s);
  // accumulate = 0: Aq = A q; otherwise Aq += accumulate * A q (C0 only)
  // accumulate != 0: Aq += accumulate * A q (C0 only)
  int OperatorF32(const float* q, float* Aq, Prec prec, cudaStream_t s, float accumulate = 0.f);
  // Aq = A q with host buffers (page-locked for overlap); returns when Aq is filled
  std::unique_ptr<HostPipe> pipe;
  int BuildPipe(cudaStream_t s);
  int OperatorHost(const double* qHost, double* AqHost, cudaStream_t s);
  int OperatorHostF32(const float* qHost, float* AqHost, Prec prec, cudaStream_t s);
  int BuildDiagonal(double* diagG, cudaStream_t s);   // assembled diag(A)
  int BuildRhs(double* r, cudaStream_t s);            // forcing + lifting, gathered
  // host copy of the assembled N-degree stiffness (+lambda mass), COO sorted (row, col)
  // assembled operator matrix (CSR: Nglobal+1 row starts, sorted columns)
  int BuildMatrix(std::vector<int64_t>& rowStarts, std::vector<int32_t>& cols, std::vector<double>& vals,
                  cudaStream_t s);
};

// ---------------------------------------------------------------- preconditioners
struct LearnedSmoother;

struct Precon {
  virtual ~Precon() = default;
  virtual int apply(const double* r, double* z, cudaStream_t s) = 0;
  // z = M^{-1} r for a Krylov loop that can take the result in FP32: a preconditioner
  // that computes in FP32 sets *z32 to its FP32 result (valid until its next application)
  // and leaves z unwritten; otherwise *z32 = nullptr and z is written as by apply
  virtual int apply_mixed(const double* r, double* z, const float** z32, cudaStream_t s) {
    *z32 = nullptr;
    return apply(r, z, s);
  }
  virtual int levels_p() const { return 0; }
  virtual int levels_amg() const { return 0; }
  virtual int64_t coarse_n() const { return 0; }
  // learned fine-level smoother with per-V-cycle fallback to the plain smoother when the
  // V-cycle reduces the residual by less than `threshold` (ratio above it)
  virtual int set_learned(LearnedSmoother*, const BoxNumbering&, double /*threshold*/) {
    return set_error(LPG_ERR_UNSUPPORTED, "a learned smoother needs PRECONDITIONER = MULTIGRID");
  }
  virtual int64_t fallbacks() const { return 0; }
  virtual int64_t learned_timeouts() const { return 0; }
  // spectral radius estimate of D^{-1} A on the finest p-level (0 without p-levels)
  virtual double fine_rho() const { return 0; }
  virtual int64_t vcycles() const { return 0; }
};

std::unique_ptr<Precon> make_identity(Elliptic* el);
std::unique_ptr<Precon> make_jacobi(Elliptic* el, int* status);
struct MGOptions {
  std::vector<int> degrees;       // fine..1
  int smoother = 0;               // 0 Chebyshev, 1 damped Jacobi
  int chebDegree = 2;
  Prec prec = Prec::F64;
  int amgSmoother = 0;
  int amgChebDegree = 2;
  bool amgUnsmoothed = false;
  bool amgRugeStuben = false;
  bool amgOnly = false;           // PARALMOND: AMG on the fine matrix
  bool semfem = false;            // SEMFEM: AMG on the low-order matrix of the GLL sub-mesh
  // random stream of the setup: a fresh srand48(0) unless a state is handed over (OAS builds
  // its coarse AMG after the patch hierarchy on one stream)
  bool rngGiven = false;
  uint64_t rngState = 0;
  int learnedSteps = 2;           // learned smoothing steps before and after the coarse correction
};
std::unique_ptr<Precon> make_multigrid(Elliptic* el, const MeshConfig& c, const MGOptions& o, int* status);
// OAS (ellipticPreconOAS.cpp) on one rank: p-multigrid of the problem plus an additive
// degree-1 AMG correction
std::unique_ptr<Precon> make_oas(Elliptic* el, const MeshConfig& c, const MGOptions& o, int* status);

// ---------------------------------------------------------------- linear solver
struct PCGResult {
  int iters = 0;
  double rdotr = 0;
  bool breakdown = false;
};
struct PCGWork {
  DevBuf<double> p, z, Ax, Ap;
  int ensure(int64_t n);
};
int pcg_solve(Platform* plat, Elliptic* el, Precon* pc, PCGWork& w, bool flexible, bool stopRhs,
              double* x, double* r, double tol, int maxit, PCGResult& res);
// non-blocking flexible PCG (linearSolverNBFPCG.cpp:72-186): fused update + 4 inner
// products per iteration; stopping criterion relative to the initial residual
struct NBWork {
  DevBuf<double> u, p, w, n, m, s, z, q, Ax, partials;
  std::vector<double> host;
  int ensure(int64_t n);
};
int nbfpcg_solve(Platform* plat, Elliptic* el, Precon* pc, NBWork& w, double* x, double* r, double tol, int maxit,
                 PCGResult& res);

// degree schedule of the p-multigrid hierarchy (ellipticPreconMultiGrid.cpp:49-84)
std::vector<int> degree_schedule(int N, const std::string& coarsening, const std::vector<int>& explicitList);

}  // namespace lpg
