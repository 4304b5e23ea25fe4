/*
 * libparanumal_gb300: C ABI of the GB300 (sm_103a) C0 hexahedral elliptic path.
 *
 * Two levels:
 *   1. kernel entry points: device pointers, explicit sizes, a cudaStream_t passed
 *      as void*; each returns an int status (LPG_OK = 0, negative on error, text by
 *      lpg_last_error()). They never allocate unless stated.
 *   2. solver objects: an elliptic_t built from a settings text in the reference's
 *      .rc format, with Operator / precon / Solve / Run entry points.
 *
 * Every entry point cites the reference interface it replaces (paths are relative
 * to the libParanumal source tree). No C++ exception crosses this boundary.
 */
#ifndef LPG_H
#define LPG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
#define LPG_OK 0
#define LPG_ERR_INVALID (-1)       /* bad argument */
#define LPG_ERR_CUDA (-2)          /* CUDA runtime error */
#define LPG_ERR_UNSUPPORTED (-3)   /* e.g. polynomial degree outside 1..8 */
#define LPG_ERR_NOT_CONVERGED (-4) /* solver hit MAXIT */
#define LPG_ERR_ALLOC (-5)         /* device allocation failed */
#define LPG_ERR_SETTINGS (-6)      /* unknown or malformed setting */
#define LPG_ERR_BREAKDOWN (-7)     /* NaN/Inf or non-positive curvature in (F)PCG */
#define LPG_ERR_TIMEOUT (-8)       /* a bounded wait inside a device pipeline ran out */

/* Replaces LIBP_ABORT's message (include/utils.hpp:57-76): text of the last error on
 * this thread. */
const char *lpg_last_error(void);
const char *lpg_version(void);

/* Device memory helpers for callers without a CUDA runtime of their own
 * (platform_t::malloc / memory copies, include/platform.hpp:163-205). */
int lpg_device_malloc(void **ptr, uint64_t bytes);
int lpg_device_free(void *ptr);
int lpg_memcpy_h2d(void *dst, const void *src, uint64_t bytes, void *stream);
int lpg_memcpy_d2h(void *dst, const void *src, uint64_t bytes, void *stream);
int lpg_memcpy_d2d(void *dst, const void *src, uint64_t bytes, void *stream);
/* platform_t's DEVICE NUMBER (libs/core/platformDeviceConfig.cpp:80-100): makes `device` current for the
 * calling thread; later objects and kernels use it. */
int lpg_set_device(int device);
int lpg_stream_sync(void *stream);

/* ------------------------------------------------------------------ operator kernels */
/*
 * Matrix-free screened-Poisson operator on hexahedra with fused assembly:
 *   Aq[g] = sum over local copies n of g of ( D^T G D q_e + lambda_e wJ q_e )[n]
 * Replaces ellipticPartialAxHex3D (solvers/elliptic/okl/ellipticAxHex3D.okl:156-295)
 * followed by ogsMasked.Gather(Aq, AqL, Add, Trans) (solvers/elliptic/src/ellipticOperator.cpp:29-106).
 *   N              polynomial degree, 1..8
 *   Nelements      elements to process; elementList (int32, may be NULL = 0..Nelements-1)
 *   GlobalToLocal  int32 per local node (E*Np): assembled dof index or -1 (masked)
 *   ggeo, wJ       geometric factors: ggeo[e*geoStride + c*Np + n] for c = G00,G01,G02,G11,G12,G22
 *                  and wJ[e*wJStride + n]. The reference layout is geoStride = 6*Np, wJStride = Np;
 *                  the packed layout used by this library's own objects is geoStride = wJStride = 7*Np
 *                  with wJ = ggeo + 6*Np.
 *   D              (N+1)^2 derivative matrix, row-major, D[i*Nq+j] = l_j'(r_i)
 *   lambda         scalar; lambdaE (per element, may be NULL) overrides it
 *   q              assembled input (Nglobal); Aq assembled output (Nglobal), overwritten
 * _f64: FP64 storage and arithmetic. _f32: FP32 vectors and geometry. _bf16g: BF16
 * geometric factors with FP32 vectors and FP32 accumulation.
 */
int lpg_ax_hex_f64(int N, int64_t Nelements, const int32_t *elementList, const int32_t *GlobalToLocal,
                   const double *ggeo, int64_t geoStride, const double *wJ, int64_t wJStride,
                   const double *D, double lambda, const double *lambdaE,
                   const double *q, double *Aq, int64_t Nglobal, void *stream);
int lpg_ax_hex_f32(int N, int64_t Nelements, const int32_t *elementList, const int32_t *GlobalToLocal,
                   const float *ggeo, int64_t geoStride, const float *wJ, int64_t wJStride,
                   const float *D, float lambda, const float *lambdaE,
                   const float *q, float *Aq, int64_t Nglobal, void *stream);
int lpg_ax_hex_bf16g(int N, int64_t Nelements, const int32_t *elementList, const int32_t *GlobalToLocal,
                     const void *ggeo_bf16, int64_t geoStride, const void *wJ_bf16, int64_t wJStride,
                     const float *D, float lambda, const float *lambdaE,
                     const float *q, float *Aq, int64_t Nglobal, void *stream);

/* Unassembled variant with the reference kernel's exact contract: writes the local
 * result AqL[e*Np + n] for the listed elements (ellipticAxHex3D.okl:156-295). */
int lpg_partial_ax_hex_f64(int N, int64_t Nelements, const int32_t *elementList,
                           const int32_t *GlobalToLocal, const double *ggeo, int64_t geoStride,
                           const double *wJ, int64_t wJStride, const double *D, double lambda,
                           const double *lambdaE, const double *q, double *AqL, void *stream);

/* ------------------------------------------------------------------ gather-scatter */
/* ogs_t::Gather(gv, v, 1, Add, Trans) (libs/ogs/ogs.cpp:213-285): gv[g] = sum of v over
 * copies; overwrites gv. Uses GlobalToLocal (-1 entries skipped). */
int lpg_ogs_gather_add_f64(int64_t Nlocal, const int32_t *GlobalToLocal, const double *v,
                           double *gv, int64_t Nglobal, void *stream);
/* ogs_t::Gather(gv, v, 1, Add, NoTrans): one copy per dof, picked by ownerLocal[g]. */
int lpg_ogs_gather_owner_f64(int64_t Nglobal, const int32_t *ownerLocal, const double *v, double *gv,
                             void *stream);
/* ogs_t::Scatter(v, gv, 1, NoTrans) (libs/ogs/ogs.cpp:287-330): v[n] = gv[GlobalToLocal[n]],
 * masked nodes set to 0. */
int lpg_ogs_scatter_f64(int64_t Nlocal, const int32_t *GlobalToLocal, const double *gv, double *v,
                        void *stream);

/* ------------------------------------------------------------------ vector kernels */
/* linAlg_t (include/linAlg.hpp:37-208; libs/linAlg/okl/linAlg*.okl). Reductions write their
 * result to a device scalar (no host synchronisation); partial sums use a
 * library-owned scratch buffer allocated on first use. */
int lpg_axpy_f64(int64_t N, double alpha, const double *x, double beta, double *y, void *stream);
int lpg_amxpy_f64(int64_t N, double alpha, const double *x, const double *y, double beta, double *z,
                  void *stream);
int lpg_dot_f64(int64_t N, const double *x, const double *y, double *result_dev, void *stream);
int lpg_norm2sq_f64(int64_t N, const double *x, double *result_dev, void *stream);
/* No counterpart in the reference. Same result as lpg_dot_f64, but allocates nothing:
 * for callers that cannot let a library call cudaMalloc -- host frameworks that own all
 * device memory through their own pool, and latency-sensitive loops where cudaMalloc /
 * cudaFree would synchronise the device. The partial sums live in a fixed 8 KB device
 * array (1024 doubles) that every GPU loading the library holds until exit. The first
 * call on each device looks up that array's address (with the device current) and should
 * come before any stream capture. N must be 0..2^40; larger N fails with LPG_ERR_INVALID.
 * All calls share the array, so calls that overlap on the GPU race. */
int lpg_dot_f64_noalloc(int64_t N, const double *x, const double *y, double *result_dev, void *stream);
/* linearSolverUpdatePCG.okl:29-75 + pcg::UpdatePCG (linearSolverPCG.cpp:153-171):
 * x += alpha p; r -= alpha Ap; result_dev = r.r */
int lpg_pcg_update_f64(int64_t N, double alpha, const double *p, const double *Ap, double *x, double *r,
                       double *result_dev, void *stream);

/* linAlg_t::norm2 (libs/linAlg/linAlg.cpp:154-167): result_dev = sqrt(x.x). */
int lpg_norm2_f64(int64_t N, const double *x, double *result_dev, void *stream);
/* JacobiPrecon::Operator (solvers/elliptic/src/ellipticPreconJacobi.cpp:42-):
 * z = invDiag .* r. */
int lpg_jacobi_f64(int64_t N, const double *invDiag, const double *r, double *z, void *stream);

/* ------------------------------------------------------------------ partition and halo */
/* Element partition of a box mesh into `nranks` slabs of whole element layers along z, for
 * callers that split the operator across ranks (one process per GPU) as elliptic_t::Operator
 * does with MPI (solvers/elliptic/src/ellipticOperator.cpp:29-106; halo_t, include/ogs.hpp:
 * 347-400). Rank r gets NZ/P (+1 for r < NZ%P) layers, the per-rank count of
 * meshSetupBoxHex3D.cpp:63-69 applied to z: the element range [e0, e1) of the single-rank
 * order. Host only (no GPU). info (6 entries) gets e0, e1, the number of dofs the rank owns,
 * the number of local dofs (owned first, then halo, each in global lattice order: the plane
 * shared with rank r+1 is owned by r), and the lengths of the `below` and `above` lists.
 * The arrays may be NULL (sizes only): global_to_local ((e1-e0)*(N+1)^3: local dof or -1 for
 * a masked node, for lpg_ax_hex_f64 on the rank's elements), below / above (the rank's
 * local indices of the plane shared with rank r-1 / r+1, in that plane's lattice order, so
 * rank r's `above` pairs entry by entry with rank r+1's `below`), lattice (global lattice
 * id X + NX*(Y + NY*Z) of each local dof, NX = nx*N+1, ...). bcflag 1 (Dirichlet: boundary
 * lattice nodes masked) or 2 (Neumann); periodic boxes are not partitioned. */
int lpg_box_partition(int nx, int ny, int nz, int N, int bcflag, int nranks, int rank, int64_t *info,
                      int32_t *global_to_local, int32_t *below, int32_t *above, int64_t *lattice);
/* The two device halves of a halo exchange (ogs extract kernel, libs/ogs/okl/ogsKernels.okl:167-;
 * the exchange itself -- MPI, NCCL -- is the caller's): pack buf[i] = v[idx[i]] before
 * sending, unpack_add v[idx[i]] += buf[i] for what was received. After every rank has
 * assembled its elements' contributions to its local dofs, exchanging at each shared plane
 * gives both ranks the full sums there. */
int lpg_halo_pack_f64(int64_t n, const int32_t *idx, const double *v, double *buf, void *stream);
int lpg_halo_unpack_add_f64(int64_t n, const int32_t *idx, const double *buf, double *v, void *stream);

/* ------------------------------------------------------------------ p-multigrid level kernels */
/* MGLevel::coarsen (solvers/elliptic/src/ellipticPreconMultiGridLevel.cpp:41-82 with
 * ellipticPartialPreconCoarsenHex3D, okl/ellipticPreconCoarsenHex3D.okl:209-294): per element,
 * the fine local values weightF .* rF (scattered by g2lF, masked nodes 0) are restricted by
 * P^T in each direction and assembled into rC (NglobalC, overwritten) through g2lC.
 * P is the (Nf+1) x (Nc+1) GLL interpolation matrix, row-major (P[i*(Nc+1)+j] = l_j(r_i)). */
int lpg_pmg_restrict_f64(int Nf, int Nc, int64_t E, const int32_t *g2lF, const double *weightF,
                         const double *rF, const double *P, const int32_t *g2lC, double *rC,
                         int64_t NglobalC, void *stream);
int lpg_pmg_restrict_f32(int Nf, int Nc, int64_t E, const int32_t *g2lF, const float *weightF,
                         const float *rF, const float *P, const int32_t *g2lC, float *rC,
                         int64_t NglobalC, void *stream);
/* MGLevel::prolongate (ellipticPreconMultiGridLevel.cpp:84-125 with
 * ellipticPartialPreconProlongateHex3D, okl/ellipticPreconProlongateHex3D.okl:216-301):
 * xF += P xC, element by element; each fine dof is written once, by its owning local copy
 * (ownerF[g] = the first local node of dof g, as lpg_elliptic_get("ownerLocal") returns). */
int lpg_pmg_prolong_add_f64(int Nf, int Nc, int64_t E, const int32_t *g2lC, const double *xC,
                            const double *P, const int32_t *g2lF, const int32_t *ownerF, double *xF,
                            void *stream);
int lpg_pmg_prolong_add_f32(int Nf, int Nc, int64_t E, const int32_t *g2lC, const float *xC,
                            const float *P, const int32_t *g2lF, const int32_t *ownerF, float *xF,
                            void *stream);
/* MGLevel::smoothChebyshev (ellipticPreconMultiGridLevel.cpp:154-206) as two fused passes.
 * start: res = invDiag .* (r - Ax) (xIsZero: res = invDiag .* r, Ax unused);
 *        d = invTheta res; x = d (xIsZero) or x += d.
 * update (one Chebyshev step after Ad = A d): res -= invDiag .* Ad; d = a d + b res; x += d. */
int lpg_cheb_start_f64(int64_t N, const double *invDiag, const double *r, const double *Ax, double *res,
                       double *d, double *x, double invTheta, int xIsZero, void *stream);
int lpg_cheb_start_f32(int64_t N, const float *invDiag, const float *r, const float *Ax, float *res,
                       float *d, float *x, float invTheta, int xIsZero, void *stream);
int lpg_cheb_update_f64(int64_t N, const double *invDiag, const double *Ad, double *res, double *d,
                        double *x, double a, double b, void *stream);
int lpg_cheb_update_f32(int64_t N, const float *invDiag, const float *Ad, float *res, float *d, float *x,
                        float a, float b, void *stream);

/* ------------------------------------------------------------------ parAlmond level kernels */
/* CSR matrices: int64 row starts (Nrows+1), int32 columns, FP64 values.
 * parCSR::SpMV (libs/parAlmond/parAlmondparCSR.cpp:99-140, okl/SpMVcsr.okl):
 * y = alpha A x + beta y (beta = 0 ignores y). */
int lpg_csr_spmv_f64(int64_t Nrows, const int64_t *rowStarts, const int32_t *cols, const double *vals,
                     double alpha, const double *x, double beta, double *y, void *stream);
/* parCSR::smoothChebyshev (libs/parAlmond/parAlmondAMGSmoother.cpp:68-160, okl/SmoothChebyshev.okl:30-167):
 * start (x = 0): r = diagInv .* b; d = invTheta r; x = d.
 * residual: r = alpha r + diagInv .* (beta b - A x).
 * update: d = a d + b r; x += d (lastIt: d is not stored). */
int lpg_csr_cheb_start_f64(int64_t N, double invTheta, const double *diagInv, const double *b, double *r,
                           double *d, double *x, void *stream);
int lpg_csr_cheb_residual_f64(int64_t N, const int64_t *rowStarts, const int32_t *cols, const double *vals,
                              double alpha, double beta, const double *diagInv, const double *b,
                              const double *x, double *r, void *stream);
int lpg_csr_cheb_update_f64(int64_t N, double a, double b, int lastIt, const double *r, double *d, double *x,
                            void *stream);
/* exactSolver_t::solve (libs/parAlmond/parAlmondCoarseExact.cpp:35-60, okl/dGEMV.okl):
 * y = A x with the dense n x n inverse A, row-major. */
int lpg_gemv_f64(int64_t n, const double *A, const double *x, double *y, void *stream);

/* ------------------------------------------------------------------ solver objects */
/* elliptic_t (solvers/elliptic/elliptic.hpp:56-170) built from settings in the
 * reference's .rc format ([KEY] newline value): the reference's keys for this path
 * (ellipticSettings.cpp, parAlmondSettings.cpp, meshSettings.cpp, initialGuess.cpp) plus
 * the additions documented beside their entry points; unknown keys fail with
 * LPG_ERR_SETTINGS, as the reference aborts
 * (solvers/elliptic/src/ellipticSettings.cpp:144-146). */
typedef struct lpg_elliptic lpg_elliptic;

int lpg_elliptic_create(const char *settings, lpg_elliptic **out);
int lpg_elliptic_destroy(lpg_elliptic *e);

#define LPG_INFO_NELEMENTS 0
#define LPG_INFO_NP 1
#define LPG_INFO_NGLOBAL 2
#define LPG_INFO_NLOCAL 3
#define LPG_INFO_N 4
#define LPG_INFO_ALLNEUMANN 5
#define LPG_INFO_MG_PLEVELS 6
#define LPG_INFO_MG_AMGLEVELS 7
#define LPG_INFO_COARSE_N 8
#define LPG_INFO_DEVICE_BYTES 9
#define LPG_INFO_VCYCLES 10        /* V-cycles run with the learned fine smoother */
#define LPG_INFO_FALLBACKS 11      /* of those, redone with the plain smoother */
#define LPG_INFO_HOST_CHUNKS 12    /* element chunks of the host-buffer operator (0 before its first call) */
#define LPG_INFO_IG_HISTORY 13     /* current dimension of the initial-guess history */
#define LPG_INFO_OPERATOR_APPLICATIONS 14 /* fine-level operator applications (FP64, double-word
                                             and FP32) since creation: outer Krylov, smoother,
                                             residual and setup applications */
#define LPG_INFO_LEARNED_TIMEOUTS 15 /* learned V-cycles redone with the plain smoother because the
                                        network's tensor-core pipeline reported a timeout */
#define LPG_INFO_MORTON_ORDER 16   /* 1 if the operators visit the elements of a mesh file in Morton
                                      order of their centroids (the file's order had no locality) */
int64_t lpg_elliptic_info(const lpg_elliptic *e, int what);

/* Copy a named setup array to host memory: "GlobalToLocal" (int32), "ownerLocal" (int32),
 * "ggeo" (E*6*Np double, reference layout), "wJ", "D", "weightG", "lambdaE", "invDiag". */
int lpg_elliptic_get(const lpg_elliptic *e, const char *name, void *host_out, uint64_t bytes);

/* Device pointers owned by the object (valid until destroy): "q_in", "Aq_out", "x", "r"
 * are FP64 vectors of length Nglobal usable as scratch by the caller. */
int lpg_elliptic_device_ptr(const lpg_elliptic *e, const char *name, void **ptr);

/* Seeded input vector with no reference counterpart (the reference's tests use
 * manufactured data only): q[g] = 2u-1, u uniform in [0,1) keyed by (seed, global
 * lattice node id of dof g), so the vector does not depend on numbering or partition. */
int lpg_elliptic_random_vector(lpg_elliptic *e, uint64_t seed, double *q, void *stream);

/* elliptic_t::Operator (ellipticOperator.cpp:29-106): Aq = A q, device pointers (Nglobal). */
int lpg_elliptic_operator(lpg_elliptic *e, const double *q, double *Aq, void *stream);
/* Reduced-precision operator of the same object (no reference counterpart; the
 * reference is FP64 only): FP32 vectors, FP32 (bf16geo = 0) or BF16 (bf16geo = 1)
 * geometric factors, FP32 arithmetic. The reduced-precision copies of the geometric
 * factors are made on first use. DISCRETIZATION = IPDG: FP32 volume and surface factors
 * (bf16geo must be 0). */
int lpg_elliptic_operator_f32(lpg_elliptic *e, const float *q, float *Aq, int bf16geo, void *stream);
/* The same operator (device vectors, FP64 in and out) computed in double-FP32 words on
 * the FP32 pipe -- no reference counterpart. 48-bit significands; agrees with the FP64
 * operator to about 1e-14 relative (sums with absolute error ~2^-48 of the magnitudes
 * summed); inputs below 2^-74 in magnitude lose the low word. Any N (CONTINUOUS and
 * IPDG). The setting
 * [OPERATOR PRECISION] DF64 makes every FP64 operator application of the object use it. */
int lpg_elliptic_operator_df64(lpg_elliptic *e, const double *q, double *Aq, void *stream);
/* elliptic_t::Operator (ellipticOperator.cpp:29-106) on HOST arrays, as the OCCA Serial
 * backend's operator takes them: Aq_host = A q_host (Nglobal entries each), returning
 * when Aq_host is filled. The upload of q, the operator and the download of Aq are
 * pipelined over element chunks on the object's stream and two copy streams; overlap
 * needs page-locked buffers (pageable ones give the same result, copied serially).
 * Device work vectors are allocated on the first call. Calls on one object must not
 * overlap. */
int lpg_elliptic_operator_host(lpg_elliptic *e, const double *q_host, double *Aq_host);
/* The same with FP32 vectors and FP32 (bf16geo = 0) or BF16 (bf16geo = 1) geometric
 * factors (no reference counterpart). */
int lpg_elliptic_operator_host_f32(lpg_elliptic *e, const float *q_host, float *Aq_host, int bf16geo);
/* precon_t::Operator (include/precon.hpp:36-56): z = M^{-1} r, device pointers. */
int lpg_elliptic_precon(lpg_elliptic *e, const double *r, double *z, void *stream);
/* elliptic_t::Solve (ellipticSolve.cpp:29-39): (F)PCG on device vectors x (initial
 * guess, overwritten) and r (right-hand side, overwritten by the residual).
 * Returns the iteration count in *iters. */
int lpg_elliptic_solve(lpg_elliptic *e, double *x, double *r, double tol, int maxit, int *iters);
/* elliptic_t::ZeroMean (ellipticZeroMean.cpp:29-37): removes the mean of the assembled
 * vector q (Nglobal, device) when the problem has the constant null space (all-Neumann
 * boundaries with lambda = 0); otherwise a no-op. */
int lpg_elliptic_zero_mean(lpg_elliptic *e, double *q, void *stream);
/* The assembled (diagonal GLL) mass product Mu = Gather(Trans)(wJ .* Scatter(u)) of
 * device vectors of length Nglobal (CONTINUOUS only): the lambda M u_old term that
 * time-stepping callers of the screened-Poisson solve add to their right-hand side, as the
 * ins velocity solve does (solvers/ins/src/insVelocitySolve.cpp:30-100: velocityRhsKernel
 * forms RHS = MM RHS / nu + boundary data and the elliptic lambda is gamma / nu). */
int lpg_elliptic_mass(lpg_elliptic *e, const double *u, double *Mu, void *stream);
/* The assembled right-hand side of elliptic_t::Run (forcing, Dirichlet lifting,
 * Gather(Trans)) into a device vector r (Nglobal). */
int lpg_elliptic_rhs(lpg_elliptic *e, double *r, void *stream);
/* Initial-guess strategies of linearSolver_t (include/initialGuess.hpp:38-162), chosen by
 * [INITIAL GUESS STRATEGY] NONE (default) | ZERO | CLASSIC | QR | EXTRAP with
 * [INITIAL GUESS HISTORY SPACE DIMENSION] (1..32), [INITIAL GUESS EXTRAP DEGREE] and
 * [INITIAL GUESS EXTRAP COEFFS METHOD] MINNORM | CPQR. lpg_elliptic_solve forms the initial
 * guess from the history before the solve and adds the solution afterwards
 * (linearSolver.cpp:30-43). lpg_elliptic_initial_guess only forms it
 * (initialGuessStrategy_t::FormInitialGuess): x (Nglobal, device) from rhs (device). */
int lpg_elliptic_initial_guess(lpg_elliptic *e, double *x, const double *rhs, void *stream);
/* Extrapolation weights (Extrap::extrapCoeffs, initialGuess.cpp:440-468): coeffs_out gets
 * `history` weights of the last `history` equally spaced solutions, exact one step ahead
 * for polynomials of degree `degree`; cpqr = 0 minimum-norm, 1 column-pivoted QR basic
 * solution. Host only. */
int lpg_extrap_coeffs(int degree, int history, int cpqr, double *coeffs_out);
/* elliptic_t::Run (ellipticRun.cpp:30-248): rhs, timed solve, scatter + AddBC, then the
 * mass-weighted solution norm and, for manufactured data, the error norm.
 * xL_host (Nlocal doubles) may be NULL; solve_seconds is the wall time of the solve.
 * With [OUTPUT TO FILE] = TRUE the solution is also written to
 * <OUTPUT FILE NAME>_0000.vtu (ellipticRun.cpp:223-235). */
int lpg_elliptic_run(lpg_elliptic *e, double *xL_host, int *iters, double *norm, double *err,
                     double *solve_seconds);
/* elliptic_t::PlotFields (ellipticPlotFields.cpp:30-140): ASCII VTU UnstructuredGrid of the
 * local field qL (Nlocal doubles, device) interpolated to the equispaced degree-(N+3) plot
 * nodes of every element, each plot cube split into 6 tetrahedra (VTK type 10). */
int lpg_elliptic_plot_fields(lpg_elliptic *e, const double *qL, const char *file_name);

/* ------------------------------------------------------------------ Gmsh meshes */
/* [MESH FILE] = <path> (instead of BOX) reads a Gmsh 2.2 ASCII hexahedral mesh
 * (mesh_t::ReadGmshHex3D, meshReadGmshHex3D.cpp:33-170): type-5 hexahedra in file order,
 * type-3 quadrilaterals as boundary faces whose physical tag is the boundary flag
 * (1 Dirichlet, 2 Neumann). Both functions below are host only (no GPU needed).
 * lpg_hex_mesh_info: element, node and tagged boundary-face counts. */
int lpg_hex_mesh_info(const char *path, int64_t *nelements, int64_t *nnodes, int64_t *nboundary_faces);
/* GlobalToLocal of the degree-N nodes of the mesh in `path` (mesh_t::ConnectNodes,
 * meshConnectNodes.cpp:32-117, with the single-rank ogs ordering, ogsSetup.cpp:408-432):
 * global_to_local gets nelements*(N+1)^3 entries (assembled dof, or -1 for Dirichlet
 * nodes) unless NULL; nglobal gets the number of assembled dofs. */
int lpg_hex_mesh_numbering(const char *path, int N, int32_t *global_to_local, int64_t *nglobal);

/* ------------------------------------------------------------------ learned smoother */
/* No reference counterpart. Element-local MLP
 * 896 -> 256 -> 256 -> 256 -> 512 with GELU (tanh form) after the hidden layers; input =
 * the element's 512 residual values and 6 x 64 face-neighbour traces divided by the
 * element residual RMS s_e; the network's correction is s_e * invDiag * output,
 * averaged over shared nodes. As fine-level smoother it is added to a damped-Jacobi
 * step (4/3/rho) invDiag * r, and each smoothing correction c is taken with the
 * energy-optimal step (c.r)/(c.Ac). Parameter vector (FP32, lpg_mlp_param_count() = 492800):
 * W0 (896x256 row-major), b0, W1 (256x256), b1, W2 (256x256), b2, W3 (256x512), b3. */
int64_t lpg_mlp_param_count(void);
/* floats of the activation workspace for a batch of B rows */
int64_t lpg_mlp_workspace_floats(int64_t B);
/* FP32 forward: Y (B x 512) = MLP(X (B x 896)); workspace keeps the activations for the
 * backward pass. */
int lpg_mlp_forward_f32(const float *params, int64_t B, const float *X, float *workspace, float *Y, void *stream);
/* FP32 backward of the forward above: grads (param layout) of sum(dY . Y); work holds
 * 2 x B x 256 floats. */
int lpg_mlp_backward_f32(const float *params, int64_t B, const float *X, const float *workspace, const float *dY,
                         float *grads, float *work, void *stream);
/* Adam step (b1 0.9, b2 0.999, eps 1e-8; step counts from 1). */
int lpg_mlp_adam_f32(int64_t n, float *w, const float *g, float *m, float *v, float lr, int step, void *stream);
/* Inference path: BF16 tensor-core layers (FP32 accumulate) with BF16 activations and an
 * FP32 output layer. Allocates its temporaries. */
int lpg_mlp_forward_bf16(const float *params, int64_t B, const float *X, float *Y, void *stream);
/* Trains the network on (residual, exact error) pairs from the plain p-MG FPCG solver of
 * the problem in `settings` (N = 7, PRECONDITIONER = MULTIGRID) on random Gaussian-bump
 * right-hand sides; with [SMOOTHER TRAINING PAIRS] MIXED (default; TRAJECTORY turns it
 * off) every second sample set is a synthetic pair (random error e, r = A e). Targets are
 * the error outside the element's degree <= 3 modal space minus the damped-Jacobi part.
 * weights_host gets lpg_mlp_param_count() floats, loss_history_host (may be NULL) the
 * mean training loss of each epoch. */
int lpg_smoother_train(const char *settings, int nsolves, int samples_per_solve, int epochs, int batch, float lr,
                       uint64_t seed, float *weights_host, float *loss_history_host);
/* Replaces the fine-level Chebyshev smoother of e's multigrid preconditioner by the
 * damped-Jacobi + network smoother with these weights (BF16 inference); a V-cycle whose
 * residual ratio ||r - A z|| / ||r|| exceeds `threshold` (e.g. 0.5) is redone with the
 * plain smoother. weights_host = NULL restores the plain smoother. */
int lpg_elliptic_set_learned_smoother(lpg_elliptic *e, const float *weights_host, double threshold);
/* Diagnostics (no reference counterpart): every following launch of the fused tensor-core
 * MLP kernel first waits up to `ns` nanoseconds on a barrier that nothing signals, then
 * gives up the way any of its bounded pipeline waits does -- records a timeout, issues no
 * copy or MMA, frees its tensor memory and returns. The caller sees LPG_ERR_TIMEOUT from
 * lpg_mlp_forward_bf16, and a learned V-cycle falls back to the plain smoother. 0 (the
 * default) turns it off. Exists so the timeout path can be tested without a GPU fault. */
int lpg_debug_mlp_hold(uint64_t ns);

#ifdef __cplusplus
}
#endif
#endif
