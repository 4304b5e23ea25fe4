/*
 * Oracle (test infrastructure only): settings parsing, RNG streams, 1D GLL basis
 * and the small dense linear algebra the reference takes from LAPACK.
 *
 * Follows libs/mesh/meshBasis1D.cpp:34-370 (JacobiP, GradJacobiP, JacobiGQ,
 * JacobiGLL with mass-lumped weights, Dmatrix1D = Vr/V, InterpolationMatrix1D).
 * LAPACK stand-ins: dgetrf/dgetri (libs/linAlg/linAlgMatrixInverse.cpp:29-54),
 * dgesv right-solve (libs/linAlg/linAlgMatrixRightSolve.cpp:29-253), dgeev
 * eigenvalues (libs/linAlg/linAlgMatrixEig.cpp:29-124). The reference pins no
 * LAPACK version; these restatements agree with it to rounding.
 */
#include "orc_internal.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>

/* ---------------------------------------------------------------- RNG */

uint64_t orc_splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* Uniform [0,1) keyed by (seed, stream, key): order- and partition-independent. */
double orc_u01(uint64_t seed, uint64_t stream, uint64_t key) {
  uint64_t h = orc_splitmix64(orc_splitmix64(seed ^ (stream << 56)) + key);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

/* POSIX drand48: X_{n+1} = (a X_n + c) mod 2^48, srand48(s) sets X = (s<<16)+0x330E.
 * The reference seeds it with srand48(rank) (libs/parAlmond/parAlmondKernels.cpp:55-58). */
void orc_srand48(orc_rand48 *r, long seed) {
  r->x = (((uint64_t)(uint32_t)seed) << 16) | 0x330EULL;
}
double orc_drand48(orc_rand48 *r) {
  r->x = (0x5DEECE66DULL * r->x + 0xBULL) & ((1ULL << 48) - 1);
  return (double)r->x * (1.0 / 281474976710656.0);
}

/* ---------------------------------------------------------------- settings */

static void trim(char *s) {
  size_t n = strlen(s);
  while (n && isspace((unsigned char)s[n - 1])) s[--n] = 0;
  size_t i = 0;
  while (s[i] && isspace((unsigned char)s[i])) i++;
  if (i) memmove(s, s + i, strlen(s + i) + 1);
}

static int parse_list(const char *v, int *out, int maxn) {
  int n = 0;
  const char *p = v;
  while (*p && n < maxn) {
    while (*p && !isdigit((unsigned char)*p)) p++;
    if (!*p) break;
    out[n++] = (int)strtol(p, (char **)&p, 10);
  }
  return n;
}

static int set_key(orc_settings *s, const char *key, const char *val) {
#define IS(k) (strcmp(key, k) == 0)
#define V(v) (strcmp(val, v) == 0)
  if (IS("BOX NX")) s->nx = atoi(val);
  else if (IS("BOX NY")) s->ny = atoi(val);
  else if (IS("BOX NZ")) s->nz = atoi(val);
  else if (IS("BOX DIMX")) s->dimx = atof(val);
  else if (IS("BOX DIMY")) s->dimy = atof(val);
  else if (IS("BOX DIMZ")) s->dimz = atof(val);
  else if (IS("BOX BOUNDARY FLAG")) s->bcflag = atoi(val);
  else if (IS("POLYNOMIAL DEGREE")) s->N = atoi(val);
  else if (IS("LAMBDA")) s->lambda = atof(val);
  else if (IS("LAMBDA FIELD")) s->lambda_field = V("LOGNORMAL") ? 1 : 0;
  else if (IS("LAMBDA SEED")) s->lambda_seed = strtoull(val, 0, 10);
  else if (IS("MESH JITTER")) s->jitter = atof(val);
  else if (IS("MESH JITTER SEED")) s->jitter_seed = strtoull(val, 0, 10);
  else if (IS("RHS FIELD")) s->rhs = V("GAUSSIAN SOURCES") ? ORC_RHS_GAUSSIAN_SOURCES : V("GAUSSIAN BUMPS") ? ORC_RHS_BUMPS : ORC_RHS_SINE;
  else if (IS("RHS SEED")) s->rhs_seed = strtoull(val, 0, 10);
  else if (IS("RHS SOURCES")) s->nsources = atoi(val);
  else if (IS("LINEAR SOLVER")) s->solver = V("NBFPCG") ? ORC_NBFPCG : V("FPCG") ? ORC_FPCG : ORC_PCG;
  else if (IS("LINEAR SOLVER STOPPING CRITERION")) s->stop_rhs = V("ABS/REL-RHS-2NORM");
  else if (IS("PRECONDITIONER")) s->precon = V("JACOBI") ? ORC_PRE_JACOBI : V("MULTIGRID") ? ORC_PRE_MULTIGRID : V("PARALMOND") ? ORC_PRE_PARALMOND : V("SEMFEM") ? ORC_PRE_SEMFEM : V("OAS") ? ORC_PRE_OAS : ORC_PRE_NONE;
  else if (IS("MULTIGRID COARSENING")) s->mg_coarsening = V("ALLDEGREES") ? ORC_MG_ALLDEGREES : V("HALFDEGREES") ? ORC_MG_HALFDEGREES : ORC_MG_HALFDOFS;
  else if (IS("MULTIGRID DEGREES")) { s->mg_ndeg = parse_list(val, s->mg_degrees, 16); if (s->mg_ndeg > 0) s->mg_coarsening = ORC_MG_LIST; }
  else if (IS("MULTIGRID SMOOTHER")) s->mg_smoother = V("DAMPEDJACOBI") ? ORC_SMOOTH_JACOBI : ORC_SMOOTH_CHEBYSHEV;
  else if (IS("MULTIGRID CHEBYSHEV DEGREE")) s->mg_cheb_degree = atoi(val);
  else if (IS("PARALMOND STRENGTH")) s->amg_strength_rs = V("RUGESTUBEN");
  else if (IS("PARALMOND AGGREGATION")) s->amg_unsmoothed = V("UNSMOOTHED");
  else if (IS("PARALMOND SMOOTHER")) s->amg_smoother = V("DAMPEDJACOBI") ? ORC_SMOOTH_JACOBI : ORC_SMOOTH_CHEBYSHEV;
  else if (IS("PARALMOND CHEBYSHEV DEGREE")) s->amg_cheb_degree = atoi(val);
  else if (IS("SOLVER TOLERANCE")) s->tol = atof(val);
  else if (IS("MAXIMUM ITERATIONS")) s->maxit = atoi(val);
  /* keys accepted and ignored (fixed by this path or not relevant on the CPU) */
  else if (IS("MESH FILE")) {
    if (strcmp(val, "BOX") == 0) s->mesh_file[0] = 0;
    else snprintf(s->mesh_file, sizeof(s->mesh_file), "%s", val);
  }
  else if (IS("DISCRETIZATION")) {
    if (V("IPDG")) s->ipdg = 1;
    else if (V("CONTINUOUS")) s->ipdg = 0;
    else return -1;
  }
  else if (IS("FORMAT") || IS("DATA FILE") || IS("MESH DIMENSION") ||
           IS("ELEMENT TYPE") || IS("THREAD MODEL") || IS("PLATFORM NUMBER") ||
           IS("DEVICE NUMBER") || IS("PARALMOND CYCLE") ||
           IS("OUTPUT TO FILE") || IS("VERBOSE") || IS("ELEMENT MAP") ||
           IS("PRECONDITIONER PRECISION") || IS("FINE SMOOTHER") || IS("OUTPUT FILE NAME"))
    ;
  else return -1;
  return 0;
#undef IS
#undef V
}

int orc_parse_settings(const char *text, orc_settings *s) {
  memset(s, 0, sizeof(*s));
  /* defaults: ellipticSettings.cpp:40-98, meshSettings.cpp:35-90, parAlmondSettings.cpp:33-60 */
  s->nx = s->ny = s->nz = 10;
  s->dimx = s->dimy = s->dimz = 10.0;
  s->bcflag = 1;
  s->N = 4;
  s->lambda = 1.0;
  s->jitter_seed = 0;
  s->lambda_seed = 2;
  s->rhs_seed = 3;
  s->nsources = 16;
  s->solver = ORC_PCG;
  s->precon = ORC_PRE_NONE;
  s->mg_coarsening = ORC_MG_HALFDOFS;
  s->mg_smoother = ORC_SMOOTH_CHEBYSHEV;
  s->mg_cheb_degree = 2;
  s->amg_smoother = ORC_SMOOTH_CHEBYSHEV;
  s->amg_cheb_degree = 2;
  s->tol = 1.0e-8;
  s->maxit = 5000;

  char *buf = strdup(text);
  char key[256] = {0};
  int havekey = 0;
  int rc = 0;
  for (char *line = strtok(buf, "\n"); line; line = strtok(NULL, "\n")) {
    char tmp[1024];
    strncpy(tmp, line, sizeof(tmp) - 1);
    tmp[sizeof(tmp) - 1] = 0;
    char *hash = strchr(tmp, '#');
    if (hash) *hash = 0;
    trim(tmp);
    if (!tmp[0]) continue;
    if (tmp[0] == '[') {
      char *e = strchr(tmp, ']');
      if (!e) { rc = -1; break; }
      *e = 0;
      snprintf(key, sizeof(key), "%.255s", tmp + 1);
      trim(key);
      havekey = 1;
    } else if (havekey) {
      if (set_key(s, key, tmp) != 0) { rc = -2; fprintf(stderr, "oracle: unknown setting [%s]\n", key); }
      havekey = 0;
    }
  }
  free(buf);
  return rc;
}

/* ---------------------------------------------------------------- 1D basis */

double orc_jacobiP(double a, double alpha, double beta, int N) {
  /* orthonormal Jacobi polynomial by the three-term recurrence (meshBasis1D.cpp:189-220) */
  double gamma0 = pow(2.0, alpha + beta + 1) / (alpha + beta + 1) * tgamma(1 + alpha) *
                  tgamma(1 + beta) / tgamma(1 + alpha + beta);
  double p0 = 1.0 / sqrt(gamma0);
  if (N == 0) return p0;
  double gamma1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * gamma0;
  double p1 = ((alpha + beta + 2) * a / 2 + (alpha - beta) / 2) / sqrt(gamma1);
  if (N == 1) return p1;
  double pm1 = p0, pc = p1;
  double aold = 2 / (2 + alpha + beta) * sqrt((alpha + 1.) * (beta + 1.) / (alpha + beta + 3.));
  for (int i = 1; i <= N - 1; ++i) {
    double h1 = 2. * i + alpha + beta;
    double anew = 2. / (h1 + 2.) * sqrt((i + 1.) * (i + 1. + alpha + beta) * (i + 1 + alpha) *
                                        (i + 1 + beta) / (h1 + 1) / (h1 + 3));
    double bnew = -(alpha * alpha - beta * beta) / h1 / (h1 + 2);
    double pn = 1. / anew * (-aold * pm1 + (a - bnew) * pc);
    aold = anew;
    pm1 = pc;
    pc = pn;
  }
  return pc;
}

double orc_gradJacobiP(double a, double alpha, double beta, int N) {
  if (N <= 0) return 0.0;
  return sqrt(N * (N + alpha + beta + 1.)) * orc_jacobiP(a, alpha + 1.0, beta + 1.0, N - 1);
}

/* Gauss-Jacobi nodes as eigenvalues of the symmetric recurrence matrix (meshBasis1D.cpp:285-347). */
void orc_jacobiGQ(double alpha, double beta, int N, double *x) {
  if (N == 0) { x[0] = (alpha - beta) / (alpha + beta + 2); return; }
  int n1 = N + 1;
  double *J = (double *)calloc((size_t)n1 * n1, sizeof(double));
  for (int n = 0; n <= N; ++n) {
    double h1 = 2 * n + alpha + beta;
    J[n * n1 + n] += -0.5 * (alpha * alpha - beta * beta) / ((h1 + 2) * h1) * 2;
    if (n < N) {
      double v = (2. / (h1 + 2.)) * sqrt((n + 1) * (n + 1 + alpha + beta) * (n + 1 + alpha) *
                                         (n + 1 + beta) / ((h1 + 1) * (h1 + 3)));
      J[n * n1 + n + 1] += v;
      J[(n + 1) * n1 + n] += v;
    }
  }
  if (alpha + beta < 10 * 2.220446049250313e-16) J[0] = 0;
  orc_sym_eigenvalues(n1, J, x);
  /* ascending order */
  for (int i = 0; i < n1; ++i)
    for (int j = i + 1; j < n1; ++j)
      if (x[i] > x[j]) { double t = x[i]; x[i] = x[j]; x[j] = t; }
  free(J);
}

static void vandermonde1D(int N, int npts, const double *r, double *V) {
  for (int n = 0; n < npts; ++n)
    for (int i = 0; i <= N; ++i) V[n * (N + 1) + i] = orc_jacobiP(r[n], 0, 0, i);
}

void orc_jacobiGLL(int N, double *x, double *w) {
  x[0] = -1.0;
  x[N] = 1.0;
  if (N > 1) orc_jacobiGQ(1, 1, N - 2, x + 1);
  if (!w) return;
  /* mass-lumped weights: row sums of inv(V V^T) (meshBasis1D.cpp:263-283, 100-115) */
  int Nq = N + 1;
  double *V = (double *)malloc(sizeof(double) * Nq * Nq);
  double *M = (double *)malloc(sizeof(double) * Nq * Nq);
  vandermonde1D(N, Nq, x, V);
  for (int n = 0; n < Nq; ++n)
    for (int m = 0; m < Nq; ++m) {
      double res = 0;
      for (int i = 0; i < Nq; ++i) res += V[n * Nq + i] * V[m * Nq + i];
      M[n * Nq + m] = res;
    }
  orc_matrix_inverse(Nq, M);
  for (int n = 0; n < Nq; ++n) {
    double res = 0;
    for (int m = 0; m < Nq; ++m) res += M[n * Nq + m];
    w[n] = res;
  }
  free(V);
  free(M);
}

void orc_dmatrix1D(int N, const double *r, double *D) {
  int Nq = N + 1;
  double *V = (double *)malloc(sizeof(double) * Nq * Nq);
  double *Vr = (double *)malloc(sizeof(double) * Nq * Nq);
  vandermonde1D(N, Nq, r, V);
  for (int n = 0; n < Nq; ++n)
    for (int i = 0; i < Nq; ++i) Vr[n * Nq + i] = orc_gradJacobiP(r[n], 0, 0, i);
  orc_right_solve(Nq, Nq, Vr, Nq, V, D);
  free(V);
  free(Vr);
}

void orc_interp1D(int N, const double *rin, int Nout, const double *rout, double *I) {
  int Nq = N + 1;
  double *Vin = (double *)malloc(sizeof(double) * Nq * Nq);
  double *Vout = (double *)malloc(sizeof(double) * Nout * Nq);
  vandermonde1D(N, Nq, rin, Vin);
  vandermonde1D(N, Nout, rout, Vout);
  orc_right_solve(Nout, Nq, Vout, Nq, Vin, I);
  free(Vin);
  free(Vout);
}

/* ---------------------------------------------------------------- dense LA */

/* LU with partial pivoting; returns 0 on success. A row-major n x n, piv length n. */
static int lu_factor(int n, double *A, int *piv) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    double amax = fabs(A[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (fabs(A[i * n + k]) > amax) { amax = fabs(A[i * n + k]); p = i; }
    piv[k] = p;
    if (amax == 0.0) return -1;
    if (p != k)
      for (int j = 0; j < n; ++j) { double t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
    double inv = 1.0 / A[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      double l = A[i * n + k] * inv;
      A[i * n + k] = l;
      if (l != 0.0)
        for (int j = k + 1; j < n; ++j) A[i * n + j] -= l * A[k * n + j];
    }
  }
  return 0;
}

static void lu_solve(int n, const double *LU, const int *piv, double *b) {
  for (int k = 0; k < n; ++k)
    if (piv[k] != k) { double t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int j = 0; j < i; ++j) s -= LU[i * n + j] * b[j];
    b[i] = s;
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= LU[i * n + j] * b[j];
    b[i] = s / LU[i * n + i];
  }
}

int orc_matrix_inverse(int n, double *A) {
  double *LU = (double *)malloc(sizeof(double) * (size_t)n * n);
  int *piv = (int *)malloc(sizeof(int) * n);
  double *col = (double *)malloc(sizeof(double) * n);
  memcpy(LU, A, sizeof(double) * (size_t)n * n);
  int rc = lu_factor(n, LU, piv);
  if (rc == 0) {
    for (int j = 0; j < n; ++j) {
      for (int i = 0; i < n; ++i) col[i] = (i == j) ? 1.0 : 0.0;
      lu_solve(n, LU, piv, col);
      for (int i = 0; i < n; ++i) A[i * n + j] = col[i];
    }
  }
  free(LU);
  free(piv);
  free(col);
  return rc;
}

/* C (nrA x nB) = A (nrA x ncA) / B (nB x nB): solve C B = A, i.e. B^T C^T = A^T. */
int orc_right_solve(int nrA, int ncA, const double *A, int nB, const double *B, double *C) {
  if (ncA != nB) return -1;
  double *BT = (double *)malloc(sizeof(double) * nB * nB);
  int *piv = (int *)malloc(sizeof(int) * nB);
  double *rhs = (double *)malloc(sizeof(double) * nB);
  for (int i = 0; i < nB; ++i)
    for (int j = 0; j < nB; ++j) BT[i * nB + j] = B[j * nB + i];
  int rc = lu_factor(nB, BT, piv);
  if (rc == 0) {
    for (int r = 0; r < nrA; ++r) {
      for (int j = 0; j < nB; ++j) rhs[j] = A[r * ncA + j];
      lu_solve(nB, BT, piv, rhs);
      for (int j = 0; j < nB; ++j) C[r * nB + j] = rhs[j];
    }
  }
  free(BT);
  free(piv);
  free(rhs);
  return rc;
}

/* Cyclic Jacobi rotations for a small symmetric matrix (GLL nodes only, n <= 16). */
void orc_sym_eigenvalues(int n, double *A, double *w) {
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
    if (off < 1e-300) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = A[p * n + q];
        if (apq == 0.0) continue;
        double app = A[p * n + p], aqq = A[q * n + q];
        double theta = (aqq - app) / (2 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
        double c = 1 / sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {
          double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = A[i * n + i];
}

/* Eigenvalues of a real upper-Hessenberg matrix by Francis double-shift QR sweeps
 * with 3x3 Householder reflectors and deflation on negligible sub-diagonals
 * (the textbook implicit double-shift QR). Input is column-major, as the
 * reference's Arnoldi Hessenberg H[i + j*k] (ellipticPreconMultiGridLevel.cpp:441-458). */
void orc_hessenberg_eigenvalues(int n, const double *Hc, double *wr, double *wi) {
  double *A = (double *)malloc(sizeof(double) * n * n);
#define AA(i, j) A[(i) * n + (j)]
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) AA(i, j) = (j >= i - 1) ? Hc[i + j * n] : 0.0;
  int hi = n - 1, iter = 0;
  const double eps = 2.220446049250313e-16;
  while (hi >= 0) {
    if (hi == 0) { wr[0] = AA(0, 0); wi[0] = 0; hi--; continue; }
    int l = hi;
    while (l > 0) {
      double sc = fabs(AA(l - 1, l - 1)) + fabs(AA(l, l));
      if (sc == 0.0) sc = 1.0;
      if (fabs(AA(l, l - 1)) <= eps * sc) { AA(l, l - 1) = 0.0; break; }
      l--;
    }
    if (l == hi) { wr[hi] = AA(hi, hi); wi[hi] = 0; hi--; iter = 0; continue; }
    if (l == hi - 1) {
      double a = AA(hi - 1, hi - 1), b = AA(hi - 1, hi), c = AA(hi, hi - 1), d = AA(hi, hi);
      double p = 0.5 * (a - d), disc = p * p + b * c, m = 0.5 * (a + d);
      if (disc >= 0) {
        double sq = sqrt(disc);
        double z = p + (p >= 0 ? sq : -sq);
        double e1 = d + z;
        double e2 = (z != 0.0) ? d - b * c / z : d;
        wr[hi - 1] = e1; wr[hi] = e2; wi[hi - 1] = wi[hi] = 0;
      } else {
        double sq = sqrt(-disc);
        wr[hi - 1] = wr[hi] = m; wi[hi - 1] = sq; wi[hi] = -sq;
      }
      hi -= 2; iter = 0;
      continue;
    }
    if (iter > 300) { /* give up: report diagonal */
      for (int i = l; i <= hi; ++i) { wr[i] = AA(i, i); wi[i] = 0; }
      hi = l - 1; iter = 0; continue;
    }
    double s, t;
    if (iter > 0 && iter % 11 == 0) { /* exceptional shift */
      double e = fabs(AA(hi, hi - 1)) + fabs(AA(hi - 1, hi - 2));
      s = 1.5 * e; t = e * e;
    } else {
      s = AA(hi - 1, hi - 1) + AA(hi, hi);
      t = AA(hi - 1, hi - 1) * AA(hi, hi) - AA(hi - 1, hi) * AA(hi, hi - 1);
    }
    double x = AA(l, l) * AA(l, l) + AA(l, l + 1) * AA(l + 1, l) - s * AA(l, l) + t;
    double y = AA(l + 1, l) * (AA(l, l) + AA(l + 1, l + 1) - s);
    double z = AA(l + 1, l) * AA(l + 2, l + 1);
    for (int k = l; k <= hi - 2; ++k) {
      double nv = sqrt(x * x + y * y + z * z);
      if (nv != 0.0) {
        double alpha = (x >= 0) ? -nv : nv;
        double u0 = x - alpha, u1 = y, u2 = z;
        double uu = u0 * u0 + u1 * u1 + u2 * u2;
        if (uu != 0.0) {
          double beta = 2.0 / uu;
          int c0 = (k > l) ? k - 1 : l;
          for (int j = c0; j <= hi; ++j) {
            double dot = u0 * AA(k, j) + u1 * AA(k + 1, j) + u2 * AA(k + 2, j);
            dot *= beta;
            AA(k, j) -= dot * u0; AA(k + 1, j) -= dot * u1; AA(k + 2, j) -= dot * u2;
          }
          int r1 = (k + 3 < hi) ? k + 3 : hi;
          for (int i = l; i <= r1; ++i) {
            double dot = u0 * AA(i, k) + u1 * AA(i, k + 1) + u2 * AA(i, k + 2);
            dot *= beta;
            AA(i, k) -= dot * u0; AA(i, k + 1) -= dot * u1; AA(i, k + 2) -= dot * u2;
          }
        }
      }
      x = AA(k + 1, k);
      y = AA(k + 2, k);
      z = (k < hi - 2) ? AA(k + 3, k) : 0.0;
    }
    /* final 2x2 Givens rotation on rows/cols hi-1, hi */
    {
      int k = hi - 1;
      double r = hypot(x, y);
      if (r != 0.0) {
        double c = x / r, sn = y / r;
        int c0 = (k > l) ? k - 1 : l;
        for (int j = c0; j <= hi; ++j) {
          double a1 = AA(k, j), a2 = AA(k + 1, j);
          AA(k, j) = c * a1 + sn * a2;
          AA(k + 1, j) = -sn * a1 + c * a2;
        }
        for (int i = l; i <= hi; ++i) {
          double a1 = AA(i, k), a2 = AA(i, k + 1);
          AA(i, k) = c * a1 + sn * a2;
          AA(i, k + 1) = -sn * a1 + c * a2;
        }
      }
    }
    iter++;
  }
#undef AA
  free(A);
}
