// Internal (C++) interfaces between the host objects and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>

namespace lpg {


// ---------------------------------------------------------------- operator
enum class AxMode { Assemble, AccumulateAssembled, PartialLocal, LocalInSubtract };

template <typename T, typename G>
struct AxArgs {
  int N = 0;
  int64_t Nelements = 0;
  const int32_t* elementList = nullptr;
  const int32_t* g2l = nullptr;
  const G* ggeo = nullptr;
  int64_t geoStride = 0;
  const G* wJ = nullptr;
  int64_t wJStride = 0;
  const T* D = nullptr;
  T lambda = 0;
  const T* lambdaE = nullptr;
  const T* q = nullptr;
  T* out = nullptr;
  int64_t Nglobal = 0;
  // assembled modes: out += outScale * A q (FP32 kernels only; FP64 requires 1). With
  // out preset to b and outScale = -1 an AccumulateAssembled launch leaves the residual
  // b - A q without a separate vector pass.
  T outScale = T(1);
};

template <typename T, typename G>
int ax_hex(const AxArgs<T, G>& a, AxMode mode, cudaStream_t s);
// Assembled operator in double-FP32 ("double-word") arithmetic: FP64 q and Aq, geometric
// factors pre-split into (hi, lo) float pairs ([e][7][Np] float2), N = 1..8 (even-odd
// kernels for N = 3 and 7).
int ax_hex_dw(const AxArgs<double, float2>& a, cudaStream_t s);
// elements covered by one full wave (every SM at the kernel's occupancy) of the assembled
// FP64 (dw = false; mass = the instantiation with the lambda term) or double-word operator
// kernel at degree N; 1 where not known
int ax_wave_elements(int N, bool dw, bool mass);
// FP64 -> (hi, lo) float pairs (hi = x rounded to FP32, lo = x - hi rounded to FP32)
int split_to_float2(int64_t n, const double* x, float2* y, cudaStream_t s);

// ---------------------------------------------------------------- setup kernels
// Geometric factors of trilinear hexahedra from their 8 vertices
// (meshPhysicalNodesHex3D.cpp + meshGeometricFactorsHex3D.cpp), packed [e][7][Np]:
// G00,G01,G02,G11,G12,G22,wJ. Counts nodes with J < 1e-12 into *badCount (device).
int geometric_factors(int N, int64_t E, const double* EX, const double* EY, const double* EZ,
                      const double* D, const double* r1d, const double* w1d, double* geo,
                      int* badCount, cudaStream_t s);

// Box-mesh numbering (closed form of ConnectNodes + ogs ordering): GlobalToLocal per
// local node, ownerLocal per dof and multiplicity per dof.
struct BoxNumbering {
  int nx, ny, nz, N;
  int periodic;       // BOX BOUNDARY FLAG == -1
  int dirichlet;      // faces are Dirichlet (flag 1)
};
int box_numbering(const BoxNumbering& b, const int64_t* elemBase, int32_t* g2l, int32_t* owner,
                  int32_t* mult, int64_t Nglobal, cudaStream_t s);

// q[g] = 2u-1 with u keyed by (seed, global lattice node id of dof g): the input
// vector of the operator-throughput workload, independent of numbering and partition.
int lattice_random(const BoxNumbering& b, int64_t Nglobal, const int32_t* owner, uint64_t seed, double* q,
                   cudaStream_t s);

// Right-hand side forcing * wJ per local node and Dirichlet data g at masked nodes.
struct RhsSpec {
  int kind;            // 0 sine, 1 Gaussian sources
  int nsources;
  const double* src;   // nsources * 4: cx, cy, cz, w (device)
};
int rhs_local(int N, int64_t E, const double* EX, const double* EY, const double* EZ,
              const double* r1d, const double* geo, const double* lambdaE, double lambda,
              const int32_t* g2l, RhsSpec spec, double* rL, double* gL, cudaStream_t s);
// rL[node[t]] -= Neumann data terms of the faces in faceMask[t] (sine data file)
int neumann_flux(int N, int64_t count, const int32_t* node, const int32_t* faceMask, const double* EX,
                 const double* EY, const double* EZ, const double* r1d, const double* w1d, double* rL,
                 cudaStream_t s);
// Solution norm / error: sum of wJ*xL^2 and wJ*(xL-u)^2 (u manufactured, sine only) into
// out[0], out[1] (device). xL gets Dirichlet data at masked nodes.
int solution_norms(int N, int64_t E, const double* EX, const double* EY, const double* EZ,
                   const double* r1d, const double* geo, const int32_t* g2l, int kind, double* xL,
                   double* out, cudaStream_t s);
// Operator diagonal per local node (ellipticBuildOperatorDiagonal.cpp:998-1057).
int operator_diagonal_local(int N, int64_t E, const double* geo, const double* D, double lambda,
                            const double* lambdaE, const int32_t* g2l, double rankBoost,
                            double* diagL, cudaStream_t s);
// Assembled diagonal mass product Mu = Gather(Trans)(wJ .* Scatter(u)) (Mu overwritten).
int mass_apply(int N, int64_t E, const double* geo, const int32_t* g2l, const double* u, double* Mu, int64_t Nglobal,
               cudaStream_t s);
// Per element: smallest (lo) and largest (hi) assembled index among its unmasked nodes.
int element_dof_range(int N, int64_t E, const int32_t* g2l, int32_t* lo, int32_t* hi, cudaStream_t s);

// ---------------------------------------------------------------- ogs + vectors
template <typename T>
int gather_add(int64_t Nlocal, const int32_t* g2l, const T* v, T* gv, int64_t Nglobal, bool zero,
               cudaStream_t s);
template <typename T>
int gather_owner(int64_t Nglobal, const int32_t* owner, const T* v, T* gv, cudaStream_t s);
template <typename T>
int scatter(int64_t Nlocal, const int32_t* g2l, const T* gv, T* v, cudaStream_t s);

// y = a x + b y (b == 0 ignores y)
template <typename T> int axpy(int64_t N, T a, const T* x, T b, T* y, cudaStream_t s);
// z = a x.*y + b z
template <typename T> int amxpy(int64_t N, T a, const T* x, const T* y, T b, T* z, cudaStream_t s);
template <typename T> int fill(int64_t N, T v, T* x, cudaStream_t s);
template <typename Tin, typename Tout> int convert(int64_t N, const Tin* x, Tout* y, cudaStream_t s);
int inverse_in_place(int64_t N, double* x, cudaStream_t s);   // x = 1/x where x > 0 else 0
int inverse_f64(int64_t N, const double* x, double* y, cudaStream_t s);  // y = 1/x
int multiplicity_to_weight(int64_t N, const int32_t* mult, double* w, cudaStream_t s);  // w = 1/mult

// Deterministic two-stage reductions into a device scalar; `partials` holds
// kReducePartials doubles.
constexpr int kReducePartials = 1024;
int reduction_blocks(int64_t N);  // stage-1 CTAs (= partial sums) used for N entries
int dot(int64_t N, const double* x, const double* y, double* out, double* partials, cudaStream_t s);
int dot_f32(int64_t N, const float* x, const float* y, double* out, double* partials, cudaStream_t s);
int sum(int64_t N, const double* x, double* out, double* partials, cudaStream_t s);
int norm2(int64_t N, const double* x, double* out, double* partials, cudaStream_t s);   // sqrt(x.x)
// out2[0] = x.y, out2[1] = x.z in one pass (partials: kReducePartials doubles)
template <typename T>
int dot2(int64_t N, const T* x, const T* y, const T* z, double* out2, double* partials, cudaStream_t s);
// x += a p; r -= a q
template <typename T> int update2(int64_t N, T a, const T* p, const T* q, T* x, T* r, cudaStream_t s);
// update2 with a = sc[0] / sc[1] from device memory (0 when sc[1] <= 0 or not finite)
template <typename T> int update2_dev(int64_t N, const double* sc, const T* p, const T* q, T* x, T* r, cudaStream_t s);
// FPCG with an FP32 preconditioner output z: out2 = (r.z, z.Ap) in FP64, and p = z + beta p
int dot2_mixed(int64_t N, const float* z, const double* r, const double* Ap, double* out2, double* partials,
               cudaStream_t s);
int direction_mixed(int64_t N, const float* z, double beta, double* p, cudaStream_t s);
// halo exchange halves: buf[i] = v[idx[i]]; v[idx[i]] += buf[i]
int halo_pack(int64_t n, const int32_t* idx, const double* v, double* buf, cudaStream_t s);
int halo_unpack_add(int64_t n, const int32_t* idx, const double* buf, double* v, cudaStream_t s);
int pcg_update(int64_t N, double alpha, const double* p, const double* Ap, double* x, double* r,
               double* out, double* partials, cudaStream_t s);
int add_scalar(int64_t N, const double* scalarDev, double scale, double* x, cudaStream_t s);

// Chebyshev smoother vector updates (ellipticPreconMultiGridLevel.cpp:154-206)
template <typename T>
int cheb_update(int64_t N, const T* invDiag, const T* Ad, T* res, T* d, T a, T b, cudaStream_t s);
// fused passes: start (res = invDiag (r - Ax) or invDiag r; d = invTheta res; x = d or x += d)
// and step (res -= invDiag Ad; d = a d + b res; x += d)
template <typename T>
int cheb_start(int64_t N, const T* invDiag, const T* r, const T* Ax, T* res, T* d, T* x, T invTheta, bool xIsZero,
               cudaStream_t s);
template <typename T>
int cheb_step(int64_t N, const T* invDiag, const T* Ad, T* res, T* d, T* x, T a, T b, cudaStream_t s,
              bool last = false);
// the same on the unscaled residual u = r - A x, which the operator updates in place
// (u -= A d): start u = r - Ax (or r), d = invTheta invDiag u, x = d or x += d; step
// d = a d + b invDiag u, x += d (last: d not written)
template <typename T>
int cheb_start_u(int64_t N, const T* invDiag, const T* r, const T* Ax, T* u, T* d, T* x, T invTheta, bool xIsZero,
                 cudaStream_t s);
template <typename T>
int cheb_step_u(int64_t N, const T* invDiag, const T* u, T* d, T* x, T a, T b, cudaStream_t s, bool last = false);

// ---------------------------------------------------------------- p-multigrid transfers
// xC = assembled sum over coarse copies of P^T (weightF .* xF) per element (xC overwritten)
template <typename T>
int pmg_coarsen(int Nf, int Nc, int64_t E, const int32_t* g2lF, const T* weightF, const T* xF,
                const T* P, const int32_t* g2lC, T* xC, int64_t NglobalC, cudaStream_t s);
// xF += owning-copy value of P xC per element
template <typename T>
int pmg_prolongate_map(int Nf, int Nc, int64_t E, const int32_t* g2lC, const T* xC, const T* P,
                       const int32_t* g2lF, const int32_t* ownerF, T* xF, cudaStream_t s);

// ---------------------------------------------------------------- initial-guess history
constexpr int kMaxHistory = 32;        // history space dimension limit
constexpr int kMultiDotBlocks = 1024;  // partial sums per history vector
struct HistCoeffs {
  double v[kMaxHistory];
};
// partials[m * nblocks + b] (m < k): block shares of Q_m . x; *nblocks set
int multi_dot(int64_t N, int k, const double* x, const double* Q, double* partials, int* nblocks, cudaStream_t s);
// out = u + beta sum_m c[m] Q_m (u may be null = 0; out may alias u)
int combine(int64_t N, int k, const double* u, double beta, const HistCoeffs& c, const double* Q, double* out,
            cudaStream_t s);
// rotations i = 0..dim-2 on column pairs (i, i+1) of Q and U, then column dim-1 = 0
int givens_columns(int64_t N, int dim, const HistCoeffs& c, const HistCoeffs& sn, double* Q, double* U, cudaStream_t s);
// x = sum_i d[i] H_{(i + shift) % nh}
int extrap(int64_t N, int nh, int shift, const HistCoeffs& d, const double* H, double* x, cudaStream_t s);

// ---------------------------------------------------------------- NBFPCG passes
// partials[k * nb + b] (nb <= 1024 blocks, *nb set): u.r, u.w, r.r
int nb_dots3(int64_t N, const double* u, const double* r, const double* w, double* partials, int* nb, cudaStream_t s);
// x += a p; r -= a s; u -= a q; w -= a z; nv = w - r; partials: u.r, u.s, u.w, r.r
int nb_update(int64_t N, double a, const double* p, const double* sv, const double* q, const double* z, double* x,
              double* r, double* u, double* w, double* nv, double* partials, int* nb, cudaStream_t s);
// p = u + beta p; s = w + beta s; q = m + beta q; z = nv + beta z
int nb_directions(int64_t N, double beta, const double* u, const double* w, double* m, const double* nv, double* p,
                  double* sv, double* q, double* z, cudaStream_t s);

// ---------------------------------------------------------------- IPDG
// Interior-penalty DG operator pieces (DISCRETIZATION = IPDG); unknowns are the E*Np
// local nodes. vgeo [e][10][Np] (rx..tz, JW), sgeo [e][5][6 Nfp] (nx, ny, nz, WsJ, hinv),
// vmapP [e][6][Nfp] (neighbour volume node), EToB [e][6], g4 [E*Np] gradient scratch.
struct IpdgArgs {
  int N = 0;
  int64_t E = 0;
  const double *EX = nullptr, *EY = nullptr, *EZ = nullptr, *D = nullptr, *r1d = nullptr, *w1d = nullptr;
  double *vgeo = nullptr, *sgeo = nullptr, *hfac = nullptr;
  const int32_t* vmapP = nullptr;
  const int* EToB = nullptr;
  double lambda = 0, tau = 0;
  const double* lambdaE = nullptr;
  const double* q = nullptr;
  double4_32a* g4 = nullptr;
  double* out = nullptr;
};
// the operator on FP32 copies of vgeo, sgeo, D and lambdaE (preconditioner levels)
struct IpdgArgsF32 {
  int N = 0;
  int64_t E = 0;
  const float *vgeo = nullptr, *sgeo = nullptr, *D = nullptr;
  const int32_t* vmapP = nullptr;
  const int* EToB = nullptr;
  float lambda = 0, tau = 0;
  const float* lambdaE = nullptr;
  const float* q = nullptr;
  float4* g4 = nullptr;
  float* out = nullptr;
};
int ipdg_operator_f32(const IpdgArgsF32& a, cudaStream_t s);
// the FP64 operator in double-FP32 words (OPERATOR PRECISION DF64): vgeo and sgeo split
// into (hi, lo) pairs, gradients as 2 float4 per node, q and out FP64
struct IpdgArgsDW {
  int N = 0;
  int64_t E = 0;
  const float2 *vgeo = nullptr, *sgeo = nullptr;
  const double* D = nullptr;
  const int32_t* vmapP = nullptr;
  const int* EToB = nullptr;
  double lambda = 0, tau = 0;
  const double* lambdaE = nullptr;
  const double* q = nullptr;
  float4* g8 = nullptr;
  double* out = nullptr;
};
int ipdg_operator_dw(const IpdgArgsDW& a, cudaStream_t s);
// vgeo, sgeo (hfac = scratch [E][6 Nfp]); mapP = paired face node of each face node
int ipdg_geometry(const IpdgArgs& a, const int32_t* mapP, cudaStream_t s);
int ipdg_operator(const IpdgArgs& a, cudaStream_t s);   // out = A q (q, g4 scratch)
int ipdg_rhs_bc(const IpdgArgs& a, cudaStream_t s);     // out -= boundary data terms
int ipdg_diagonal(const IpdgArgs& a, cudaStream_t s);   // out = diag(A)

// ---------------------------------------------------------------- plot output
// out[e][4][(N+4)^3] = x, y, z (trilinear image of the vertices) and qL interpolated by I
// ((N+4) x (N+1), row-major) at the equispaced plot points pr (N+4 values), for E elements
int plot_interp(int N, int64_t E, const double* I, const double* pr, const double* qL, const double* EX,
                const double* EY, const double* EZ, double* out, cudaStream_t s);

// ---------------------------------------------------------------- sparse / dense
// y = alpha A x + beta y (CSR, FP64)
int csr_spmv(int64_t Nrows, const int64_t* rowStarts, const int32_t* cols, const double* vals,
             double alpha, const double* x, double beta, double* y, cudaStream_t s);
// Chebyshev CSR pieces (parAlmond okl/SmoothChebyshev.okl)
int csr_cheb_start(int64_t N, double invTheta, const double* diagInv, const double* b, double* r,
                   double* d, double* x, cudaStream_t s);
int csr_cheb_residual(int64_t N, const int64_t* rowStarts, const int32_t* cols, const double* vals,
                      double alpha, double beta, const double* diagInv, const double* b,
                      const double* x, double* r, cudaStream_t s);
int csr_cheb_update(int64_t N, double a, double b, int lastIt, const double* r, double* d,
                    double* x, cudaStream_t s);
// dense y = A x, A row-major n x n
int gemv(int64_t n, const double* A, const double* x, double* y, cudaStream_t s);

}  // namespace lpg
