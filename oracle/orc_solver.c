/*
 * Oracle (test infrastructure only): element operators, preconditioners and the
 * (flexible) PCG driver of the reference's C0 hex elliptic solve, on the CPU.
 *
 * Follows:
 *   solvers/elliptic/okl/ellipticAxHex3D.okl:156-295          partial Ax (same loop order)
 *   solvers/elliptic/src/ellipticOperator.cpp:29-106          Ax + ogs Gather(Add, Trans)
 *   solvers/elliptic/okl/ellipticRhsHex3D.okl:28-51, data/ellipticSine3D.h:27-51
 *   solvers/elliptic/okl/ellipticRhsBCHex3D.okl:60-290         Dirichlet lifting
 *   solvers/elliptic/okl/ellipticAddBCHex3D.okl:27-47
 *   solvers/elliptic/src/ellipticRun.cpp:30-248                driver, Solution norm
 *   libs/linearSolver/linearSolverPCG.cpp:35-171               PCG / FPCG
 *   solvers/elliptic/src/ellipticBuildOperatorDiagonal.cpp:998-1057
 *   solvers/elliptic/src/ellipticPreconJacobi.cpp:30-51
 *   solvers/elliptic/src/ellipticPreconMultiGrid.cpp:31-154    p-MG hierarchy
 *   solvers/elliptic/src/ellipticPreconMultiGridLevel.cpp:30-473 level ops, Chebyshev, Arnoldi
 *   solvers/elliptic/okl/ellipticPreconCoarsenHex3D.okl:209-294, ellipticPreconProlongateHex3D.okl:216-301
 *   solvers/elliptic/src/ellipticBuildOperatorMatrixContinuous.cpp:697-880
 *   libs/parAlmond/parAlmond*.cpp                                       AMG setup / V-cycle / exact coarse solve
 */
#include "orc_internal.h"
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif



/* ================================================================ element operators */

static void partial_ax_element(const orc_mesh *m, hlong e, double lambda, const int *G2L,
                               const double *q, const double *qLocal, double *AqL) {
  const int Nq = m->Nq, Np = m->Np;
  const double *D = m->D;
  double r_q[16][16][16];
  double r_Aq[16][16][16];
  double s_q[16][16], s_Gqr[16][16], s_Gqs[16][16];
  double r_qt[16][16], r_Gqt[16][16], r_Auk[16][16];
  double G00[16][16], G01[16][16], G02[16][16], G11[16][16], G12[16][16], G22[16][16], GwJ[16][16];
  for (int j = 0; j < Nq; ++j)
    for (int i = 0; i < Nq; ++i)
      for (int k = 0; k < Nq; ++k) {
        const hlong id = e * Np + i + j * Nq + k * Nq * Nq;
        if (qLocal) r_q[j][i][k] = qLocal[id];
        else {
          const int g = G2L[id];
          r_q[j][i][k] = (g != -1) ? q[g] : 0.0;
        }
        r_Aq[j][i][k] = 0.0;
      }
  for (int k = 0; k < Nq; ++k) {
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        const hlong gb = e * 6 * Np + k * Nq * Nq + j * Nq + i;
        G00[j][i] = m->ggeo[gb + 0 * Np]; G01[j][i] = m->ggeo[gb + 1 * Np]; G02[j][i] = m->ggeo[gb + 2 * Np];
        G11[j][i] = m->ggeo[gb + 3 * Np]; G12[j][i] = m->ggeo[gb + 4 * Np]; G22[j][i] = m->ggeo[gb + 5 * Np];
        GwJ[j][i] = m->wJ[e * Np + k * Nq * Nq + j * Nq + i];
      }
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        s_q[j][i] = r_q[j][i][k];
        double qt = 0;
        for (int mm = 0; mm < Nq; ++mm) qt += D[k * Nq + mm] * r_q[j][i][mm];
        r_qt[j][i] = qt;
      }
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        double qr = 0, qs = 0;
        for (int mm = 0; mm < Nq; ++mm) {
          qr += D[i * Nq + mm] * s_q[j][mm];
          qs += D[j * Nq + mm] * s_q[mm][i];
        }
        s_Gqs[j][i] = (G01[j][i] * qr + G11[j][i] * qs + G12[j][i] * r_qt[j][i]);
        s_Gqr[j][i] = (G00[j][i] * qr + G01[j][i] * qs + G02[j][i] * r_qt[j][i]);
        r_Gqt[j][i] = (G02[j][i] * qr + G12[j][i] * qs + G22[j][i] * r_qt[j][i]);
        r_Auk[j][i] = GwJ[j][i] * lambda * r_q[j][i][k];
      }
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        double auk = r_Auk[j][i];
        for (int mm = 0; mm < Nq; ++mm) {
          auk += D[mm * Nq + j] * s_Gqs[mm][i];
          r_Aq[j][i][mm] += D[k * Nq + mm] * r_Gqt[j][i];
          auk += D[mm * Nq + i] * s_Gqr[j][mm];
        }
        r_Aq[j][i][k] += auk;
      }
  }
  for (int j = 0; j < Nq; ++j)
    for (int i = 0; i < Nq; ++i)
      for (int k = 0; k < Nq; ++k) AqL[e * Np + k * Nq * Nq + j * Nq + i] = r_Aq[j][i][k];
}

static inline double elem_lambda(const orc_elliptic *el, hlong e) {
  return el->lambdaE ? el->lambdaE[e] : el->lambda;
}

void orc_partial_ax(const orc_elliptic *el, const double *q, double *AqL) {
  const orc_mesh *m = el->mesh;
#pragma omp parallel for schedule(static)
  for (hlong e = 0; e < m->Nelements; ++e)
    partial_ax_element(m, e, elem_lambda(el, e), el->ogs.GlobalToLocal, q, NULL, AqL);
}

static void local_ax(const orc_elliptic *el, const double *qL, double *AqL) {
  const orc_mesh *m = el->mesh;
#pragma omp parallel for schedule(static)
  for (hlong e = 0; e < m->Nelements; ++e)
    partial_ax_element(m, e, elem_lambda(el, e), NULL, NULL, qL, AqL);
}

static double *g_scratchL = NULL;
static hlong g_scratchN = 0;
static double *scratchL(hlong n) {
  if (n > g_scratchN) { free(g_scratchL); g_scratchL = (double *)malloc(sizeof(double) * n); g_scratchN = n; }
  return g_scratchL;
}

void orc_operator(const orc_elliptic *el, const double *q, double *Aq) {
  if (el->ipdg) { orc_ipdg_operator(el, q, Aq); return; }
  double *AqL = scratchL(el->ogs.Nlocal);
  orc_partial_ax(el, q, AqL);
  orc_gather_trans(&el->ogs, AqL, Aq);
}

void orc_build_diagonal(const orc_elliptic *el, double *diagA) {
  if (el->ipdg) { orc_ipdg_diagonal(el, diagA); return; }
  const orc_mesh *m = el->mesh;
  const int Nq = m->Nq, Np = m->Np;
  const double *D = m->D;
  double *AL = (double *)malloc(sizeof(double) * el->ogs.Nlocal);
#pragma omp parallel for
  for (hlong e = 0; e < m->Nelements; ++e) {
    const double lam = elem_lambda(el, e);
    for (int nz = 0; nz < Nq; nz++)
      for (int ny = 0; ny < Nq; ny++)
        for (int nx = 0; nx < Nq; nx++) {
          const int idn = nx + ny * Nq + nz * Nq * Nq;
          const hlong base = e * Np * 6;
          double a;
          if (el->mapB[e * Np + idn] != 1) {
            a = 0;
            a += 2 * m->ggeo[base + idn + 1 * Np] * D[nx + nx * Nq] * D[ny + ny * Nq];
            a += 2 * m->ggeo[base + idn + 2 * Np] * D[nx + nx * Nq] * D[nz + nz * Nq];
            a += 2 * m->ggeo[base + idn + 4 * Np] * D[ny + ny * Nq] * D[nz + nz * Nq];
            for (int k = 0; k < Nq; k++) {
              const int iid = k + ny * Nq + nz * Nq * Nq;
              a += m->ggeo[base + iid + 0 * Np] * D[nx + k * Nq] * D[nx + k * Nq];
            }
            for (int k = 0; k < Nq; k++) {
              const int iid = nx + k * Nq + nz * Nq * Nq;
              a += m->ggeo[base + iid + 3 * Np] * D[ny + k * Nq] * D[ny + k * Nq];
            }
            for (int k = 0; k < Nq; k++) {
              const int iid = nx + ny * Nq + k * Nq * Nq;
              a += m->ggeo[base + iid + 5 * Np] * D[nz + k * Nq] * D[nz + k * Nq];
            }
            a += m->wJ[e * Np + idn] * lam;
          } else {
            a = 1;
          }
          AL[e * Np + idn] = a;
        }
    if (el->allNeumann)
      for (int n = 0; n < Np; ++n)
        if (el->mapB[n + e * Np] != 1) AL[e * Np + n] += el->allNeumannScale * el->allNeumannScale;
  }
  orc_gather_trans(&el->ogs, AL, diagA);
  free(AL);
}

/* ================================================================ vectors */

static double dot(hlong n, const double *a, const double *b) {
  double s = 0;
#pragma omp parallel for reduction(+ : s)
  for (hlong i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
/* y = a x + b y */
static void axpy(hlong n, double a, const double *x, double b, double *y) {
#pragma omp parallel for
  for (hlong i = 0; i < n; ++i) y[i] = a * x[i] + b * y[i];
}
/* z = a x.*y + b z */
static void amxpy(hlong n, double a, const double *x, const double *y, double b, double *z) {
#pragma omp parallel for
  for (hlong i = 0; i < n; ++i) z[i] = a * x[i] * y[i] + b * z[i];
}
static double *dalloc(hlong n) { return (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

static void zero_mean(const orc_elliptic *el, double *q) {
  const hlong n = el->ogs.Ngather;
  double s = 0;
  for (hlong i = 0; i < n; ++i) s += q[i];
  s *= el->allNeumannScale * el->allNeumannScale;
  for (hlong i = 0; i < n; ++i) q[i] -= s;
}

/* ================================================================ sparse matrices (single rank) */

typedef struct { hlong row, col; double val; } orc_nz;

typedef struct {
  hlong Nrows, Ncols, nnz;
  hlong *rowStarts, *cols;
  double *vals;
} orc_csr;

static int cmp_nz(const void *a, const void *b) {
  const orc_nz *x = (const orc_nz *)a, *y = (const orc_nz *)b;
  if (x->row != y->row) return x->row < y->row ? -1 : 1;
  if (x->col != y->col) return x->col < y->col ? -1 : 1;
  return 0;
}

/* sort, merge duplicates, build CSR (parCSR(parCOO) with one rank) */
static orc_csr csr_from_coo(hlong Nrows, hlong Ncols, orc_nz *e, hlong n) {
  qsort(e, (size_t)n, sizeof(orc_nz), cmp_nz);
  hlong cnt = 0;
  for (hlong i = 0; i < n; ++i) {
    if (cnt > 0 && e[cnt - 1].row == e[i].row && e[cnt - 1].col == e[i].col) e[cnt - 1].val += e[i].val;
    else e[cnt++] = e[i];
  }
  orc_csr A;
  A.Nrows = Nrows; A.Ncols = Ncols; A.nnz = cnt;
  A.rowStarts = (hlong *)calloc(Nrows + 1, sizeof(hlong));
  A.cols = (hlong *)malloc(sizeof(hlong) * (cnt + 1));
  A.vals = (double *)malloc(sizeof(double) * (cnt + 1));
  for (hlong i = 0; i < cnt; ++i) {
    A.rowStarts[e[i].row + 1]++;
    A.cols[i] = e[i].col;
    A.vals[i] = e[i].val;
  }
  for (hlong r = 0; r < Nrows; ++r) A.rowStarts[r + 1] += A.rowStarts[r];
  return A;
}

static void csr_free(orc_csr *A) { free(A->rowStarts); free(A->cols); free(A->vals); memset(A, 0, sizeof(*A)); }

/* y = alpha A x + beta y */
static void csr_spmv(const orc_csr *A, double alpha, const double *x, double beta, double *y) {
#pragma omp parallel for
  for (hlong i = 0; i < A->Nrows; ++i) {
    double r = 0;
    for (hlong j = A->rowStarts[i]; j < A->rowStarts[i + 1]; ++j) r += A->vals[j] * x[A->cols[j]];
    y[i] = (beta != 0.0) ? alpha * r + beta * y[i] : alpha * r;
  }
}

static orc_csr csr_transpose(const orc_csr *A) {
  orc_nz *e = (orc_nz *)malloc(sizeof(orc_nz) * (A->nnz + 1));
  hlong c = 0;
  for (hlong i = 0; i < A->Nrows; ++i)
    for (hlong j = A->rowStarts[i]; j < A->rowStarts[i + 1]; ++j) { e[c].row = A->cols[j]; e[c].col = i; e[c].val = A->vals[j]; c++; }
  orc_csr T = csr_from_coo(A->Ncols, A->Nrows, e, c);
  free(e);
  return T;
}

static orc_csr csr_spmm(const orc_csr *A, const orc_csr *B) {
  hlong cap = 0;
  for (hlong i = 0; i < A->Nrows; ++i)
    for (hlong j = A->rowStarts[i]; j < A->rowStarts[i + 1]; ++j) {
      hlong c = A->cols[j];
      cap += B->rowStarts[c + 1] - B->rowStarts[c];
    }
  orc_nz *e = (orc_nz *)malloc(sizeof(orc_nz) * (cap + 1));
  hlong n = 0;
  for (hlong i = 0; i < A->Nrows; ++i)
    for (hlong j = A->rowStarts[i]; j < A->rowStarts[i + 1]; ++j) {
      const hlong c = A->cols[j];
      for (hlong jj = B->rowStarts[c]; jj < B->rowStarts[c + 1]; ++jj) {
        e[n].row = i; e[n].col = B->cols[jj]; e[n].val = A->vals[j] * B->vals[jj]; n++;
      }
    }
  orc_csr C = csr_from_coo(A->Nrows, B->Ncols, e, n);
  free(e);
  return C;
}

/* ================================================================ Arnoldi spectral radius of D^{-1}A */

typedef void (*orc_apply_fn)(void *ctx, const double *x, double *y);

static double arnoldi_rho(hlong N, orc_apply_fn apply, void *ctx, const double *invDiag, orc_rand48 *rng) {
  int k = 10;
  if (k > N) k = (int)N;
  double *H = (double *)calloc((size_t)k * k, sizeof(double));
  double **V = (double **)malloc(sizeof(double *) * (k + 1));
  for (int i = 0; i <= k; ++i) V[i] = dalloc(N);
  double *Vx = dalloc(N), *AVx = dalloc(N);
  for (hlong i = 0; i < N; ++i) Vx[i] = orc_drand48(rng);
  double nrm = sqrt(dot(N, Vx, Vx));
  axpy(N, 1. / nrm, Vx, 0.0, V[0]);
  for (int j = 0; j < k; ++j) {
    apply(ctx, V[j], AVx);
    amxpy(N, 1.0, invDiag, AVx, 0.0, V[j + 1]);
    for (int i = 0; i <= j; ++i) {
      double hij = dot(N, V[i], V[j + 1]);
      axpy(N, -hij, V[i], 1.0, V[j + 1]);
      H[i + j * k] = hij;
    }
    if (j + 1 < k) {
      double nj = sqrt(dot(N, V[j + 1], V[j + 1]));
      axpy(N, 0.0, V[j + 1], 1.0 / nj, V[j + 1]);
      H[j + 1 + j * k] = nj;
    }
  }
  double *wr = (double *)malloc(sizeof(double) * k), *wi = (double *)malloc(sizeof(double) * k);
  orc_hessenberg_eigenvalues(k, H, wr, wi);
  double rho = 0;
  for (int i = 0; i < k; ++i) {
    double r = sqrt(wr[i] * wr[i] + wi[i] * wi[i]);
    if (rho < r) rho = r;
  }
  for (int i = 0; i <= k; ++i) free(V[i]);
  free(V); free(Vx); free(AVx); free(H); free(wr); free(wi);
  return rho;
}

/* ================================================================ AMG (parAlmond, one rank) */

typedef struct {
  orc_csr A, P, R;
  double *diagA, *diagInv;
  double rho;
  double lambda0, lambda1, jlambda;
} orc_amg_level;

static void csr_apply_cb(void *ctx, const double *x, double *y) { csr_spmv((const orc_csr *)ctx, 1.0, x, 0.0, y); }

static void amg_diag_setup(orc_amg_level *L, orc_rand48 *rng) {
  const hlong N = L->A.Nrows;
  L->diagA = dalloc(N);
  L->diagInv = dalloc(N);
  for (hlong i = 0; i < N; ++i)
    for (hlong j = L->A.rowStarts[i]; j < L->A.rowStarts[i + 1]; ++j)
      if (L->A.cols[j] == i) L->diagA[i] = L->A.vals[j];
  for (hlong i = 0; i < N; ++i) L->diagInv[i] = (L->diagA[i] != 0.0) ? 1.0 / L->diagA[i] : 0.0;
  /* parCSR::rhoDinvA (parAlmondparCSR.cpp:340-440): same Arnoldi, scaled the same way */
  L->rho = arnoldi_rho(N, csr_apply_cb, &L->A, L->diagInv, rng);
}

static int customLess(int smax, double rmax, hlong imax, int s, double r, hlong i) {
  if (s > smax) return 1;
  if (smax > s) return 0;
  if (r > rmax) return 1;
  if (rmax > r) return 0;
  if (i > imax) return 1;
  return 0;
}

/* strength graph (parAlmondStrongGraph.cpp) -> MIS-2 aggregates (parAlmondFormAggregates.cpp) */
static hlong form_aggregates(const orc_amg_level *L, double theta, int rs, hlong *FineToCoarse, orc_rand48 *rng) {
  const orc_csr *A = &L->A;
  const hlong N = A->Nrows;
  hlong *Crs = (hlong *)calloc(N + 1, sizeof(hlong));
  hlong *Ccols = (hlong *)malloc(sizeof(hlong) * (A->nnz + 1));
  hlong c = 0;
  for (hlong i = 0; i < N; ++i) {
    if (rs) {
      const int sign = (L->diagA[i] >= 0) ? 1 : -1;
      double maxOD = 0;
      for (hlong jj = A->rowStarts[i]; jj < A->rowStarts[i + 1]; ++jj) {
        if (A->cols[jj] == i) continue;
        double OD = -sign * A->vals[jj];
        if (OD > maxOD) maxOD = OD;
      }
      for (hlong jj = A->rowStarts[i]; jj < A->rowStarts[i + 1]; ++jj) {
        const hlong col = A->cols[jj];
        if (col == i) { Ccols[c++] = col; continue; }
        double OD = -sign * A->vals[jj];
        if (OD > theta * maxOD) Ccols[c++] = col;
      }
    } else {
      const double Aii = fabs(L->diagA[i]);
      for (hlong jj = A->rowStarts[i]; jj < A->rowStarts[i + 1]; ++jj) {
        const hlong col = A->cols[jj];
        if (col == i) { Ccols[c++] = col; continue; }
        const double Ajj = fabs(L->diagA[col]);
        if (fabs(A->vals[jj]) > theta * (sqrt(Aii * Ajj))) Ccols[c++] = col;
      }
    }
    Crs[i + 1] = c;
  }
  double *rands = dalloc(N);
  int *states = (int *)calloc(N, sizeof(int));
  double *Tr = dalloc(N);
  int *Ts = (int *)calloc(N, sizeof(int));
  hlong *Ti = (hlong *)malloc(sizeof(hlong) * N), *Tc = (hlong *)malloc(sizeof(hlong) * N);
  for (hlong i = 0; i < N; ++i) rands[i] = orc_drand48(rng);
  int *colCnt = (int *)calloc(N, sizeof(int));
  for (hlong i = 0; i < c; ++i) colCnt[Ccols[i]]++;
  for (hlong i = 0; i < N; ++i) rands[i] += colCnt[i];
  for (;;) {
    for (hlong i = 0; i < N; ++i) {
      int smax = states[i];
      double rmax = rands[i];
      hlong imax = i;
      if (smax != 1)
        for (hlong jj = Crs[i]; jj < Crs[i + 1]; ++jj) {
          const hlong col = Ccols[jj];
          if (col == i) continue;
          if (customLess(smax, rmax, imax, states[col], rands[col], col)) { smax = states[col]; rmax = rands[col]; imax = col; }
        }
      Ts[i] = smax; Tr[i] = rmax; Ti[i] = imax;
    }
    for (hlong i = 0; i < N; ++i) {
      int smax = Ts[i];
      double rmax = Tr[i];
      hlong imax = Ti[i];
      for (hlong jj = Crs[i]; jj < Crs[i + 1]; ++jj) {
        const hlong col = Ccols[jj];
        if (col == i) continue;
        if (customLess(smax, rmax, imax, Ts[col], Tr[col], Ti[col])) { smax = Ts[col]; rmax = Tr[col]; imax = Ti[col]; }
      }
      if (states[i] == 0 && imax == i) states[i] = 1;
      if (states[i] == 0 && smax == 1) states[i] = -1;
    }
    hlong undecided = 0;
    for (hlong n = 0; n < N; ++n) if (states[n] == 0) undecided++;
    if (undecided == 0) break;
  }
  hlong numAggs = 0;
  for (hlong i = 0; i < N; ++i) FineToCoarse[i] = (states[i] == 1) ? numAggs++ : -1;
  for (hlong i = 0; i < N; ++i) {
    int smax = states[i];
    double rmax = rands[i];
    hlong imax = i, cmax = FineToCoarse[i];
    if (smax != 1)
      for (hlong jj = Crs[i]; jj < Crs[i + 1]; ++jj) {
        const hlong col = Ccols[jj];
        if (col == i) continue;
        if (customLess(smax, rmax, imax, states[col], rands[col], col)) {
          smax = states[col]; rmax = rands[col]; imax = col; cmax = FineToCoarse[col];
        }
      }
    Ts[i] = smax; Tr[i] = rmax; Ti[i] = imax; Tc[i] = cmax;
    if (FineToCoarse[i] == -1 && smax == 1 && cmax > -1) FineToCoarse[i] = cmax;
  }
  for (hlong i = 0; i < N; ++i) {
    int smax = Ts[i];
    double rmax = Tr[i];
    hlong imax = Ti[i], cmax = Tc[i];
    for (hlong jj = Crs[i]; jj < Crs[i + 1]; ++jj) {
      const hlong col = Ccols[jj];
      if (col == i) continue;
      if (customLess(smax, rmax, imax, Ts[col], Tr[col], Ti[col])) { smax = Ts[col]; rmax = Tr[col]; imax = Ti[col]; cmax = Tc[col]; }
    }
    if (FineToCoarse[i] == -1 && smax == 1 && cmax > -1) FineToCoarse[i] = cmax;
  }
  free(Crs); free(Ccols); free(rands); free(states); free(Tr); free(Ts); free(Ti); free(Tc); free(colCnt);
  return numAggs;
}

/* coarsenAmgLevel (parAlmondCoarsenLevel.cpp:33-84) */
static void amg_coarsen(orc_amg_level *L, orc_amg_level *Lc, double *nullv, double theta, int rs,
                        int unsmoothed, orc_rand48 *rng) {
  const hlong N = L->A.Nrows;
  hlong *F2C = (hlong *)malloc(sizeof(hlong) * N);
  const hlong Nc = form_aggregates(L, theta, rs, F2C, rng);
  /* tentative prolongator (parAlmondTentativeProlongator.cpp:33-94) */
  orc_nz *e = (orc_nz *)malloc(sizeof(orc_nz) * (N + 1));
  for (hlong i = 0; i < N; ++i) { e[i].row = i; e[i].col = F2C[i]; e[i].val = nullv[i]; }
  orc_csr T = csr_from_coo(N, Nc, e, N);
  free(e);
  double *cn = dalloc(Nc);
  for (hlong i = 0; i < T.nnz; ++i) cn[T.cols[i]] += T.vals[i] * T.vals[i];
  for (hlong i = 0; i < Nc; ++i) cn[i] = sqrt(cn[i]);
  for (hlong i = 0; i < T.nnz; ++i) T.vals[i] /= cn[T.cols[i]];
  for (hlong i = 0; i < Nc; ++i) nullv[i] = cn[i];
  free(cn);
  orc_csr P;
  if (!unsmoothed) {
    /* P = (I - omega D^{-1} A) T, omega = 4/3/rho (parAlmondSmoothPrologator.cpp:33-301) */
    const double omega = (4. / 3.) / L->rho;
    hlong cap = T.nnz;
    for (hlong i = 0; i < N; ++i)
      for (hlong j = L->A.rowStarts[i]; j < L->A.rowStarts[i + 1]; ++j) {
        hlong col = L->A.cols[j];
        cap += T.rowStarts[col + 1] - T.rowStarts[col];
      }
    orc_nz *pe = (orc_nz *)malloc(sizeof(orc_nz) * (cap + 1));
    hlong cnt = 0;
    for (hlong i = 0; i < N; ++i)
      for (hlong j = T.rowStarts[i]; j < T.rowStarts[i + 1]; ++j) { pe[cnt].row = i; pe[cnt].col = T.cols[j]; pe[cnt].val = T.vals[j]; cnt++; }
    for (hlong i = 0; i < N; ++i) {
      const double invDi = 1.0 / L->diagA[i];
      for (hlong j = L->A.rowStarts[i]; j < L->A.rowStarts[i + 1]; ++j) {
        const hlong col = L->A.cols[j];
        const double Aval = -omega * invDi * L->A.vals[j];
        for (hlong jj = T.rowStarts[col]; jj < T.rowStarts[col + 1]; ++jj) {
          pe[cnt].row = i; pe[cnt].col = T.cols[jj]; pe[cnt].val = Aval * T.vals[jj]; cnt++;
        }
      }
    }
    P = csr_from_coo(N, Nc, pe, cnt);
    free(pe);
    csr_free(&T);
  } else {
    P = T;
  }
  orc_csr R = csr_transpose(&P);
  orc_csr AP = csr_spmm(&L->A, &P);
  Lc->A = csr_spmm(&R, &AP);
  csr_free(&AP);
  L->P = P;
  L->R = R;
  amg_diag_setup(Lc, rng);
  free(F2C);
}

/* ================================================================ p-MG level */

typedef struct orc_pmg_level {
  orc_elliptic *el;   /* this level */
  orc_elliptic *elC;  /* next coarser level (owned by the next p-level or the AMG builder) */
  double *invDiag;
  double lambda0, lambda1;
  int smoother;       /* chebyshev / jacobi */
  int chebDegree;
  int Nf, Nc;
  double *P;          /* NqF x NqC, row-major */
} orc_pmg_level;

typedef struct {
  int nP;                       /* p-levels */
  orc_pmg_level plev[16];
  orc_elliptic *owned[17];      /* ellipticals owned by the hierarchy (except level 0) */
  int nowned;
  int nA;                       /* AMG levels (including the base) */
  orc_amg_level alev[64];
  int amg_smoother, amg_cheb;
  double *coarseInv;            /* dense inverse of the base matrix */
  hlong coarseN;
  /* work vectors per level (index over all levels: p then AMG) */
  double *rhs[96], *x[96], *res[96];
  double *s1, *s2, *s3;         /* smoother scratch (largest level) */
  double *xL;                   /* local scratch (largest level) */
} orc_multigrid;

static void op_cb(void *ctx, const double *x, double *y) { orc_operator((const orc_elliptic *)ctx, x, y); }

static void pmg_setup_smoother(orc_pmg_level *L, const orc_settings *s, orc_rand48 *rng) {
  const hlong N = L->el->ogs.Ngather;
  double *diag = dalloc(N);
  orc_build_diagonal(L->el, diag);
  L->invDiag = dalloc(N);
  for (hlong i = 0; i < N; ++i) L->invDiag[i] = 1.0 / diag[i];
  free(diag);
  L->smoother = s->mg_smoother;
  L->chebDegree = s->mg_cheb_degree;
  double rho = arnoldi_rho(N, op_cb, L->el, L->invDiag, rng);
  if (L->smoother == ORC_SMOOTH_CHEBYSHEV) {
    L->lambda1 = rho;
    L->lambda0 = rho / 10.;
  } else {
    L->lambda0 = (4. / 3.) / rho;
    for (hlong i = 0; i < N; ++i) L->invDiag[i] *= L->lambda0;
  }
}

static void pmg_smooth(orc_multigrid *mg, orc_pmg_level *L, const double *r, double *X, int xIsZero) {
  const hlong N = L->el->ogs.Ngather;
  double *RES = mg->s1, *Ad = mg->s2, *d = mg->s3;
  if (L->smoother == ORC_SMOOTH_JACOBI) {
    if (xIsZero) { amxpy(N, 1.0, L->invDiag, r, 0.0, X); return; }
    orc_operator(L->el, X, RES);
    axpy(N, 1.0, r, -1.0, RES);
    amxpy(N, 1.0, L->invDiag, RES, 1.0, X);
    return;
  }
  const double theta = 0.5 * (L->lambda1 + L->lambda0);
  const double delta = 0.5 * (L->lambda1 - L->lambda0);
  const double invTheta = 1.0 / theta;
  const double sigma = theta / delta;
  double rho_n = 1. / sigma, rho_np1;
  if (xIsZero) {
    amxpy(N, 1.0, L->invDiag, r, 0.0, RES);
    axpy(N, invTheta, RES, 0.0, d);
  } else {
    orc_operator(L->el, X, RES);
    axpy(N, 1.0, r, -1.0, RES);
    for (hlong i = 0; i < N; ++i) RES[i] = L->invDiag[i] * RES[i];
    axpy(N, invTheta, RES, 0.0, d);
  }
  for (int k = 0; k < L->chebDegree; k++) {
    if (xIsZero && k == 0) axpy(N, 1.0, d, 0.0, X);
    else axpy(N, 1.0, d, 1.0, X);
    orc_operator(L->el, d, Ad);
    amxpy(N, -1.0, L->invDiag, Ad, 1.0, RES);
    rho_np1 = 1.0 / (2. * sigma - rho_n);
    const double rhoDivDelta = 2.0 * rho_np1 / delta;
    axpy(N, rhoDivDelta, RES, rho_np1 * rho_n, d);
    rho_n = rho_np1;
  }
  axpy(N, 1.0, d, 1.0, X);
}

/* weight, restrict element-wise with P^T, assemble on the coarse level */
static void pmg_coarsen(orc_multigrid *mg, orc_pmg_level *L, const double *X, double *Rx) {
  const orc_elliptic *el = L->el, *elC = L->elC;
  const hlong N = el->ogs.Ngather;
  double *wx = mg->s1;
  amxpy(N, 1.0, el->weightG, X, 0.0, wx);
  const int NqF = L->Nf + 1, NqC = L->Nc + 1, NpF = NqF * NqF * NqF, NpC = NqC * NqC * NqC;
  const hlong E = el->mesh->Nelements;
  double *RxL = mg->xL;
#pragma omp parallel for
  for (hlong e = 0; e < E; ++e) {
    double qf[16][16][16], qcff[16][16][16], qccf[16][16][16];
    for (int k = 0; k < NqF; ++k)
      for (int j = 0; j < NqF; ++j)
        for (int i = 0; i < NqF; ++i) {
          const int g = el->ogs.GlobalToLocal[e * NpF + i + j * NqF + k * NqF * NqF];
          qf[k][j][i] = (g != -1) ? wx[g] : 0.0;
        }
    for (int k = 0; k < NqC; ++k)
      for (int j = 0; j < NqF; ++j)
        for (int i = 0; i < NqF; ++i) {
          double r = 0;
          for (int mm = 0; mm < NqF; ++mm) r += L->P[mm * NqC + k] * qf[mm][j][i];
          qcff[k][j][i] = r;
        }
    for (int k = 0; k < NqC; ++k)
      for (int j = 0; j < NqC; ++j)
        for (int i = 0; i < NqF; ++i) {
          double r = 0;
          for (int mm = 0; mm < NqF; ++mm) r += L->P[mm * NqC + j] * qcff[k][mm][i];
          qccf[k][j][i] = r;
        }
    for (int k = 0; k < NqC; ++k)
      for (int j = 0; j < NqC; ++j)
        for (int i = 0; i < NqC; ++i) {
          double r = 0;
          for (int mm = 0; mm < NqF; ++mm) r += L->P[mm * NqC + i] * qccf[k][j][mm];
          RxL[e * NpC + i + j * NqC + k * NqC * NqC] = r;
        }
  }
  orc_gather_trans(&elC->ogs, RxL, Rx);
}

/* interpolate element-wise with P, pick one copy per dof, add to X */
static void pmg_prolongate(orc_multigrid *mg, orc_pmg_level *L, const double *XC, double *X) {
  const orc_elliptic *el = L->el, *elC = L->elC;
  const int NqF = L->Nf + 1, NqC = L->Nc + 1, NpF = NqF * NqF * NqF, NpC = NqC * NqC * NqC;
  const hlong E = el->mesh->Nelements;
  double *PxL = mg->xL;
#pragma omp parallel for
  for (hlong e = 0; e < E; ++e) {
    double qccc[16][16][16], qccf[16][16][16], qcff[16][16][16];
    for (int k = 0; k < NqC; ++k)
      for (int j = 0; j < NqC; ++j)
        for (int i = 0; i < NqC; ++i) {
          const int g = elC->ogs.GlobalToLocal[e * NpC + i + j * NqC + k * NqC * NqC];
          qccc[k][j][i] = (g != -1) ? XC[g] : 0.0;
        }
    for (int k = 0; k < NqC; ++k)
      for (int j = 0; j < NqC; ++j)
        for (int i = 0; i < NqF; ++i) {
          double r = 0;
          for (int mm = 0; mm < NqC; ++mm) r += L->P[i * NqC + mm] * qccc[k][j][mm];
          qccf[k][j][i] = r;
        }
    for (int k = 0; k < NqC; ++k)
      for (int j = 0; j < NqF; ++j)
        for (int i = 0; i < NqF; ++i) {
          double r = 0;
          for (int mm = 0; mm < NqC; ++mm) r += L->P[j * NqC + mm] * qccf[k][mm][i];
          qcff[k][j][i] = r;
        }
    for (int k = 0; k < NqF; ++k)
      for (int j = 0; j < NqF; ++j)
        for (int i = 0; i < NqF; ++i) {
          double r = 0;
          for (int mm = 0; mm < NqC; ++mm) r += L->P[k * NqC + mm] * qcff[mm][j][i];
          PxL[e * NpF + i + j * NqF + k * NqF * NqF] = r;
        }
  }
  const hlong N = el->ogs.Ngather;
  double *PxG = mg->s1;
  orc_gather_notrans(&el->ogs, PxL, PxG);
  axpy(N, 1.0, PxG, 1.0, X);
}

/* AMG level smoothing (parAlmondAMGSmoother.cpp:35-160, okl/SmoothChebyshev.okl) */
static void amg_smooth(orc_multigrid *mg, orc_amg_level *L, const double *b, double *x, int xIsZero) {
  const hlong N = L->A.Nrows;
  if (mg->amg_smoother == ORC_SMOOTH_JACOBI) {
    if (xIsZero) { amxpy(N, L->jlambda, L->diagInv, b, 0.0, x); return; }
    double *d = mg->s1;
    csr_spmv(&L->A, 1.0, x, 0.0, d);
    for (hlong i = 0; i < N; ++i) d[i] = L->jlambda * L->diagInv[i] * (b[i] - d[i]);
    axpy(N, 1.0, d, 1.0, x);
    return;
  }
  const double theta = 0.5 * (L->lambda1 + L->lambda0);
  const double delta = 0.5 * (L->lambda1 - L->lambda0);
  const double invTheta = 1.0 / theta;
  const double sigma = theta / delta;
  double rho_n = 1. / sigma, rho_np1;
  double *d = mg->s1, *r = mg->s2, *Ad = mg->s3;
  if (xIsZero) {
    for (hlong n = 0; n < N; ++n) { const double rr = L->diagInv[n] * b[n]; r[n] = rr; d[n] = invTheta * rr; x[n] = invTheta * rr; }
  } else {
    csr_spmv(&L->A, 1.0, x, 0.0, Ad);
    for (hlong n = 0; n < N; ++n) r[n] = L->diagInv[n] * (b[n] - Ad[n]);
    for (hlong n = 0; n < N; ++n) { const double dk = invTheta * r[n]; d[n] = dk; x[n] += dk; }
  }
  for (int k = 0; k < mg->amg_cheb; k++) {
    csr_spmv(&L->A, 1.0, d, 0.0, Ad);
    for (hlong n = 0; n < N; ++n) r[n] = r[n] + L->diagInv[n] * (0.0 - Ad[n]);
    rho_np1 = 1.0 / (2. * sigma - rho_n);
    const double a = rho_np1 * rho_n, bb = 2.0 * rho_np1 / delta;
    for (hlong n = 0; n < N; ++n) { const double dk = a * d[n] + bb * r[n]; d[n] = dk; x[n] += dk; }
    rho_n = rho_np1;
  }
}

static void vcycle(orc_multigrid *mg, int k, double *RHS, double *X) {
  const int nlev = mg->nP + mg->nA;
  if (k == nlev - 1) {
    /* exact coarse solve: x = A^{-1} rhs */
    const hlong n = mg->coarseN;
    for (hlong i = 0; i < n; ++i) {
      double s = 0;
      for (hlong j = 0; j < n; ++j) s += mg->coarseInv[i * n + j] * RHS[j];
      X[i] = s;
    }
    return;
  }
  double *RHSC = mg->rhs[k + 1], *XC = mg->x[k + 1], *RES = mg->res[k];
  if (k < mg->nP) {
    orc_pmg_level *L = &mg->plev[k];
    const hlong N = L->el->ogs.Ngather;
    pmg_smooth(mg, L, RHS, X, 1);
    orc_operator(L->el, X, RES);
    axpy(N, 1.0, RHS, -1.0, RES);
    pmg_coarsen(mg, L, RES, RHSC);
    vcycle(mg, k + 1, RHSC, XC);
    pmg_prolongate(mg, L, XC, X);
    pmg_smooth(mg, L, RHS, X, 0);
  } else {
    orc_amg_level *L = &mg->alev[k - mg->nP];
    amg_smooth(mg, L, RHS, X, 1);
    csr_spmv(&L->A, -1.0, X, 0.0, RES);
    axpy(L->A.Nrows, 1.0, RHS, 1.0, RES);
    csr_spmv(&L->R, 1.0, RES, 0.0, RHSC);
    vcycle(mg, k + 1, RHSC, XC);
    csr_spmv(&L->P, 1.0, XC, 1.0, X);
    amg_smooth(mg, L, RHS, X, 0);
  }
}

/* assembled continuous stiffness (+ lambda mass) matrix, element threshold 1e-7 */
static orc_csr build_matrix(const orc_elliptic *el) {
  if (el->ipdg) {
    hlong *R, *C;
    double *V;
    const hlong n = orc_ipdg_matrix(el, &R, &C, &V);
    orc_nz *e = (orc_nz *)malloc(sizeof(orc_nz) * (size_t)(n + 1));
    for (hlong i = 0; i < n; ++i) { e[i].row = R[i]; e[i].col = C[i]; e[i].val = V[i]; }
    free(R); free(C); free(V);
    orc_csr A = csr_from_coo(el->ogs.Ngather, el->ogs.Ngather, e, n);
    free(e);
    return A;
  }
  const orc_mesh *m = el->mesh;
  const int Nq = m->Nq, Np = m->Np;
  const double *D = m->D;
  const hlong E = m->Nelements;
  orc_nz *e = (orc_nz *)malloc(sizeof(orc_nz) * (size_t)(E * Np * Np));
  hlong cnt = 0;
  for (hlong el_ = 0; el_ < E; ++el_) {
    const double *gg = m->ggeo + el_ * Np * 6;
    const double lam = elem_lambda(el, el_);
    for (int nz = 0; nz < Nq; nz++) for (int ny = 0; ny < Nq; ny++) for (int nx = 0; nx < Nq; nx++) {
      const int idn = nx + ny * Nq + nz * Nq * Nq;
      const int gn = el->ogs.GlobalToLocal[el_ * Np + idn];
      if (gn < 0) continue;
      for (int mz = 0; mz < Nq; mz++) for (int my = 0; my < Nq; my++) for (int mx = 0; mx < Nq; mx++) {
        const int idm = mx + my * Nq + mz * Nq * Nq;
        const int gm = el->ogs.GlobalToLocal[el_ * Np + idm];
        if (gm < 0) continue;
        int id;
        double val = 0.;
        if (ny == my && nz == mz)
          for (int k = 0; k < Nq; k++) { id = k + ny * Nq + nz * Nq * Nq; val += gg[id + 0 * Np] * D[nx + k * Nq] * D[mx + k * Nq]; }
        if (nz == mz) {
          id = mx + ny * Nq + nz * Nq * Nq; val += gg[id + 1 * Np] * D[nx + mx * Nq] * D[my + ny * Nq];
          id = nx + my * Nq + nz * Nq * Nq; val += gg[id + 1 * Np] * D[mx + nx * Nq] * D[ny + my * Nq];
        }
        if (ny == my) {
          id = mx + ny * Nq + nz * Nq * Nq; val += gg[id + 2 * Np] * D[nx + mx * Nq] * D[mz + nz * Nq];
          id = nx + ny * Nq + mz * Nq * Nq; val += gg[id + 2 * Np] * D[mx + nx * Nq] * D[nz + mz * Nq];
        }
        if (nx == mx && nz == mz)
          for (int k = 0; k < Nq; k++) { id = nx + k * Nq + nz * Nq * Nq; val += gg[id + 3 * Np] * D[ny + k * Nq] * D[my + k * Nq]; }
        if (nx == mx) {
          id = nx + my * Nq + nz * Nq * Nq; val += gg[id + 4 * Np] * D[ny + my * Nq] * D[mz + nz * Nq];
          id = nx + ny * Nq + mz * Nq * Nq; val += gg[id + 4 * Np] * D[my + ny * Nq] * D[nz + mz * Nq];
        }
        if (nx == mx && ny == my)
          for (int k = 0; k < Nq; k++) { id = nx + ny * Nq + k * Nq * Nq; val += gg[id + 5 * Np] * D[nz + k * Nq] * D[mz + k * Nq]; }
        if (nx == mx && ny == my && nz == mz) val += m->wJ[el_ * Np + idn] * lam;
        if (fabs(val) >= 1e-7) { e[cnt].row = gn; e[cnt].col = gm; e[cnt].val = val; cnt++; }
      }
    }
  }
  orc_csr A = csr_from_coo(el->ogs.Ngather, el->ogs.Ngather, e, cnt);
  free(e);
  return A;
}

/* parAlmond_t::AMGSetup (parAlmondAMGSetup.cpp:35-144) */
static void amg_setup(orc_multigrid *mg, const orc_elliptic *el, const orc_settings *s, orc_rand48 *rng) {
  const int base = 0;
  mg->nA = 0;
  orc_amg_level *L0 = &mg->alev[base];
  memset(L0, 0, sizeof(*L0));
  L0->A = build_matrix(el);
  amg_diag_setup(L0, rng);
  mg->nA = 1;
  hlong Nrows = L0->A.Nrows;
  double *nullv = dalloc(Nrows);
  for (hlong i = 0; i < Nrows; ++i) nullv[i] = 1.0 / sqrt((double)Nrows);
  mg->amg_smoother = s->amg_smoother;
  mg->amg_cheb = s->amg_cheb_degree;
  const hlong target = 1000;
  hlong globalSize = Nrows;
  double theta = s->amg_strength_rs ? 0.5 : 0.08;
  orc_amg_level *Lbase = L0;
  if (globalSize > target) {
    for (;;) {
      orc_amg_level *L = &mg->alev[mg->nA - 1];
      if (s->amg_smoother == ORC_SMOOTH_JACOBI) L->jlambda = (4. / 3.) / L->rho;
      else { L->lambda1 = L->rho; L->lambda0 = L->rho / 10.; }
      orc_amg_level *Lc = &mg->alev[mg->nA];
      memset(Lc, 0, sizeof(*Lc));
      amg_coarsen(L, Lc, nullv, theta, s->amg_strength_rs, s->amg_unsmoothed, rng);
      mg->nA++;
      if (!s->amg_strength_rs) theta = theta / 2;
      const hlong coarseSize = Lc->A.Nrows;
      Lbase = Lc;
      if (coarseSize <= target || globalSize < 2 * coarseSize) break;
      globalSize = coarseSize;
    }
  }
  /* exact coarse solver (parAlmondCoarseExact.cpp:80-227) */
  const hlong n = Lbase->A.Nrows;
  mg->coarseN = n;
  mg->coarseInv = dalloc(n * n);
  for (hlong i = 0; i < n; ++i)
    for (hlong j = Lbase->A.rowStarts[i]; j < Lbase->A.rowStarts[i + 1]; ++j) mg->coarseInv[i * n + Lbase->A.cols[j]] = Lbase->A.vals[j];
  if (el->allNeumann)
    for (hlong i = 0; i < n; ++i)
      for (hlong j = 0; j < n; ++j) mg->coarseInv[i * n + j] += nullv[i] * nullv[j];
  orc_matrix_inverse((int)n, mg->coarseInv);
  free(nullv);
}

/* degree schedule (ellipticPreconMultiGrid.cpp:49-84) plus an explicit list */
static int degree_schedule(const orc_settings *s, int N, int *deg) {
  int n = 0;
  if (s->mg_coarsening == ORC_MG_LIST) {
    for (int i = 0; i < s->mg_ndeg; ++i) deg[n++] = s->mg_degrees[i];
    if (deg[0] != N) { memmove(deg + 1, deg, sizeof(int) * n); deg[0] = N; n++; }
    if (deg[n - 1] != 1) deg[n++] = 1;
    return n;
  }
  int Nf = N, Nc = N, NpFine = (N + 1) * (N + 1) * (N + 1), NpCoarse = NpFine;
  deg[n++] = N;
  while (Nc > 1) {
    if (s->mg_coarsening == ORC_MG_ALLDEGREES) Nc = Nf - 1;
    else if (s->mg_coarsening == ORC_MG_HALFDEGREES) Nc = (1 > (Nf + 1) / 2) ? 1 : (Nf + 1) / 2;
    else {
      while (NpCoarse > NpFine / 2 && Nc > 1) { Nc--; NpCoarse = (Nc + 1) * (Nc + 1) * (Nc + 1); }
    }
    NpCoarse = (Nc + 1) * (Nc + 1) * (Nc + 1);
    deg[n++] = Nc;
    Nf = Nc;
    NpFine = NpCoarse;
  }
  return n;
}

static void mg_alloc_work(orc_multigrid *mg) {
  hlong maxN = 0, maxL = 0;
  const int nlev = mg->nP + mg->nA;
  for (int k = 0; k < nlev; ++k) {
    hlong n = (k < mg->nP) ? mg->plev[k].el->ogs.Ngather : mg->alev[k - mg->nP].A.Nrows;
    if (k < mg->nP) {
      if (mg->plev[k].el->ogs.Nlocal > maxL) maxL = mg->plev[k].el->ogs.Nlocal;
      if (mg->plev[k].elC->ogs.Nlocal > maxL) maxL = mg->plev[k].elC->ogs.Nlocal;
    }
    if (n > maxN) maxN = n;
    mg->rhs[k] = dalloc(n);
    mg->x[k] = dalloc(n);
    mg->res[k] = dalloc(n);
  }
  mg->s1 = dalloc(maxN);
  mg->s2 = dalloc(maxN);
  mg->s3 = dalloc(maxN);
  mg->xL = dalloc(maxL);
}

static void mg_free(orc_multigrid *mg) {
  const int nlev = mg->nP + mg->nA;
  for (int k = 0; k < nlev; ++k) { free(mg->rhs[k]); free(mg->x[k]); free(mg->res[k]); }
  for (int k = 0; k < mg->nP; ++k) { free(mg->plev[k].invDiag); free(mg->plev[k].P); }
  for (int k = 0; k < mg->nA; ++k) {
    csr_free(&mg->alev[k].A); csr_free(&mg->alev[k].P); csr_free(&mg->alev[k].R);
    free(mg->alev[k].diagA); free(mg->alev[k].diagInv);
  }
  for (int k = 0; k < mg->nowned; ++k) orc_elliptic_free(mg->owned[k]);
  free(mg->coarseInv); free(mg->s1); free(mg->s2); free(mg->s3); free(mg->xL);
  free(mg);
}

/* ================================================================ oracle object */

struct orc_solver {
  orc_settings s;
  orc_elliptic *el;
  double *lambdaE;
  double *invDiag;        /* Jacobi */
  orc_multigrid *mg;      /* MULTIGRID, PARALMOND, SEMFEM, or the patch hierarchy of OAS */
  orc_rand48 rng;
  /* OAS: degree-1 problem, its AMG, and the direct transfer N -> 1 */
  orc_elliptic *elC;
  orc_multigrid *mgC;
  orc_pmg_level oasL;
  double *oasRC, *oasZC;
  double last_norm, last_err;
  int last_iters;
};

static orc_multigrid *build_multigrid(orc_solver *S) {
  orc_multigrid *mg = (orc_multigrid *)calloc(1, sizeof(orc_multigrid));
  orc_srand48(&S->rng, 0);
  if (S->s.precon == ORC_PRE_PARALMOND) {
    mg->nP = 0;
    amg_setup(mg, S->el, &S->s, &S->rng);
    mg_alloc_work(mg);
    return mg;
  }
  if (S->s.precon == ORC_PRE_SEMFEM) {
    /* SEMFEMPrecon (ellipticPreconSEMFEM.cpp:30-247, hexahedra): parAlmond AMG of the
     * low-order matrix on the GLL sub-mesh, applied to the degree-N vectors directly */
    mg->nP = 0;
    orc_elliptic *fem = orc_semfem_build(S->el);
    mg->owned[mg->nowned++] = fem;
    amg_setup(mg, fem, &S->s, &S->rng);
    mg_alloc_work(mg);
    return mg;
  }
  int deg[32];
  const int nd = degree_schedule(&S->s, S->s.N, deg);
  orc_elliptic *cur = S->el;
  for (int l = 0; l + 1 < nd; ++l) {
    orc_pmg_level *L = &mg->plev[mg->nP];
    memset(L, 0, sizeof(*L));
    L->el = cur;
    L->Nf = deg[l];
    L->Nc = deg[l + 1];
    pmg_setup_smoother(L, &S->s, &S->rng);
    /* P: interpolation from the coarse GLL nodes to the fine ones (DegreeRaiseMatrix1D) */
    double rc[16], rf[16];
    orc_jacobiGLL(L->Nc, rc, NULL);
    orc_jacobiGLL(L->Nf, rf, NULL);
    L->P = dalloc((L->Nf + 1) * (L->Nc + 1));
    orc_interp1D(L->Nc, rc, L->Nf + 1, rf, L->P);
    orc_elliptic *next = orc_elliptic_build(&S->s, L->Nc, S->lambdaE);
    mg->owned[mg->nowned++] = next;
    L->elC = next;
    cur = next;
    mg->nP++;
  }
  amg_setup(mg, cur, &S->s, &S->rng);
  mg_alloc_work(mg);
  return mg;
}

static void precon_apply(orc_solver *S, const double *r, double *z) {
  const hlong N = S->el->ogs.Ngather;
  if (S->s.precon == ORC_PRE_JACOBI) amxpy(N, 1.0, S->invDiag, r, 0.0, z);
  else if (S->s.precon == ORC_PRE_MULTIGRID || S->s.precon == ORC_PRE_PARALMOND || S->s.precon == ORC_PRE_SEMFEM) {
    /* level 0 rhs/x are the caller's buffers */
    vcycle(S->mg, 0, (double *)r, z);
  } else if (S->s.precon == ORC_PRE_OAS) {
    if (S->s.N > 1) {
      /* patch solve (MultiGridPrecon::Operator, with its zero mean), then the additive
       * degree-1 correction prolongated onto it (ellipticPreconOAS.cpp:33-100) */
      vcycle(S->mg, 0, (double *)r, z);
      if (S->el->allNeumann) zero_mean(S->el, z);
      pmg_coarsen(S->mg, &S->oasL, r, S->oasRC);
      vcycle(S->mgC, 0, S->oasRC, S->oasZC);
      pmg_prolongate(S->mg, &S->oasL, S->oasZC, z);
    } else {
      vcycle(S->mgC, 0, (double *)r, z);
    }
  } else memcpy(z, r, sizeof(double) * N);
  if (S->el->allNeumann && S->s.precon != ORC_PRE_NONE) zero_mean(S->el, z);
}

orc_solver *orc_create(const char *settings_text, int *status) {
  orc_solver *S = (orc_solver *)calloc(1, sizeof(orc_solver));
  int rc = orc_parse_settings(settings_text, &S->s);
  if (status) *status = rc;
  if (rc != 0) { free(S); return NULL; }
  const hlong E = orc_mesh_count(&S->s);
  if (E < 0 || (S->s.mesh_file[0] && S->s.rhs != ORC_RHS_SINE)) {
    if (status) *status = -2;
    free(S);
    return NULL;
  }
  if (S->s.lambda_field == 1) {
    /* lognormal(0,1) per element keyed by element id (no reference counterpart) */
    S->lambdaE = dalloc(E);
    for (hlong e = 0; e < E; ++e) {
      const double u1 = 1.0 - orc_u01(S->s.lambda_seed, 4, (uint64_t)e);
      const double u2 = orc_u01(S->s.lambda_seed, 5, (uint64_t)e);
      const double z = sqrt(-2.0 * log(u1)) * cos(2.0 * ORC_PI * u2);
      S->lambdaE[e] = exp(z);
    }
  }
  S->el = orc_elliptic_build(&S->s, S->s.N, S->lambdaE);
  if (!S->el) {
    if (status) *status = -3;
    free(S->lambdaE);
    free(S);
    return NULL;
  }
  if (S->s.precon == ORC_PRE_JACOBI) {
    const hlong N = S->el->ogs.Ngather;
    double *d = dalloc(N);
    orc_build_diagonal(S->el, d);
    S->invDiag = dalloc(N);
    for (hlong i = 0; i < N; ++i) S->invDiag[i] = 1.0 / d[i];
    free(d);
  } else if (S->s.precon == ORC_PRE_MULTIGRID || S->s.precon == ORC_PRE_PARALMOND || S->s.precon == ORC_PRE_SEMFEM) {
    S->mg = build_multigrid(S);
  } else if (S->s.precon == ORC_PRE_OAS) {
    /* OASPrecon (ellipticPreconOAS.cpp:105-223) on one rank: the one-ring patch is the whole
     * mesh, so the patch preconditioner is the p-multigrid of the problem itself; the coarse
     * problem is the degree-1 problem with its own parAlmond AMG, whose setup continues the
     * random stream after the patch hierarchy (srand48 is seeded once per process). */
    if (S->s.N > 1) S->mg = build_multigrid(S);
    else orc_srand48(&S->rng, 0);
    S->elC = orc_elliptic_build(&S->s, 1, S->lambdaE);
    S->mgC = (orc_multigrid *)calloc(1, sizeof(orc_multigrid));
    amg_setup(S->mgC, S->elC, &S->s, &S->rng);
    mg_alloc_work(S->mgC);
    if (S->s.N > 1) {
      orc_pmg_level *L = &S->oasL;
      L->el = S->el; L->elC = S->elC; L->Nf = S->s.N; L->Nc = 1;
      double rc1[2], rf[16];
      orc_jacobiGLL(1, rc1, NULL);
      orc_jacobiGLL(S->s.N, rf, NULL);
      L->P = dalloc((S->s.N + 1) * 2);
      orc_interp1D(1, rc1, S->s.N + 1, rf, L->P);
      S->oasRC = dalloc(S->elC->ogs.Ngather);
      S->oasZC = dalloc(S->elC->ogs.Ngather);
    }
  }
  return S;
}

void orc_destroy(orc_solver *S) {
  if (!S) return;
  if (S->mg) mg_free(S->mg);
  if (S->mgC) mg_free(S->mgC);
  orc_elliptic_free(S->elC);
  free(S->oasL.P); free(S->oasRC); free(S->oasZC);
  orc_elliptic_free(S->el);
  free(S->invDiag);
  free(S->lambdaE);
  free(S);
}

long long orc_info(const orc_solver *S, int what) {
  const orc_elliptic *el = S->el;
  switch (what) {
    case ORC_INFO_NELEMENTS: return el->mesh->Nelements;
    case ORC_INFO_NP: return el->mesh->Np;
    case ORC_INFO_NGATHER: return el->ogs.Ngather;
    case ORC_INFO_NLOCAL: return el->ogs.Nlocal;
    case ORC_INFO_NQ: return el->mesh->Nq;
    case ORC_INFO_ALLNEUMANN: return el->allNeumann;
    case ORC_INFO_MG_PLEVELS: return S->mg ? S->mg->nP : 0;
    case ORC_INFO_MG_AMGLEVELS: return S->mg ? S->mg->nA : 0;
    case ORC_INFO_COARSE_N: return S->mg ? S->mg->coarseN : 0;
    default: return -1;
  }
}

int orc_get_array(const orc_solver *S, const char *name, void *out) {
  const orc_elliptic *el = S->el;
  const orc_mesh *m = el->mesh;
  const hlong E = m->Nelements, Np = m->Np, Nq = m->Nq, Nl = E * Np;
#define CP(src, n, T) do { memcpy(out, src, sizeof(T) * (size_t)(n)); return 0; } while (0)
  if (!strcmp(name, "ggeo")) CP(m->ggeo, E * 6 * Np, double);
  if (!strcmp(name, "wJ")) CP(m->wJ, Nl, double);
  if (!strcmp(name, "D")) CP(m->D, Nq * Nq, double);
  if (!strcmp(name, "gllz")) CP(m->gllz, Nq, double);
  if (!strcmp(name, "gllw")) CP(m->gllw, Nq, double);
  if (!strcmp(name, "x")) CP(m->x, Nl, double);
  if (!strcmp(name, "y")) CP(m->y, Nl, double);
  if (!strcmp(name, "z")) CP(m->z, Nl, double);
  if (!strcmp(name, "EX")) CP(m->EX, E * 8, double);
  if (!strcmp(name, "EY")) CP(m->EY, E * 8, double);
  if (!strcmp(name, "EZ")) CP(m->EZ, E * 8, double);
  if (!strcmp(name, "GlobalToLocal")) CP(el->ogs.GlobalToLocal, Nl, int);
  if (!strcmp(name, "globalIds")) CP(m->globalIds, Nl, hlong);
  if (!strcmp(name, "mapB")) CP(el->mapB, Nl, int);
  if (!strcmp(name, "weightG")) CP(el->weightG, el->ogs.Ngather, double);
  if (!strcmp(name, "lambdaE")) { if (!el->lambdaE) return -2; CP(el->lambdaE, E, double); }
  if (!strcmp(name, "invDiag")) {
    double *d = dalloc(el->ogs.Ngather);
    orc_build_diagonal(el, d);
    for (hlong i = 0; i < el->ogs.Ngather; ++i) ((double *)out)[i] = 1.0 / d[i];
    free(d);
    return 0;
  }
#undef CP
  return -1;
}

int orc_operator_apply(const orc_solver *S, const double *q, double *Aq) {
  orc_operator(S->el, q, Aq);
  return 0;
}

int orc_partial_ax_apply(const orc_solver *S, const double *q, double *AqL) {
  orc_partial_ax(S->el, q, AqL);
  return 0;
}

int orc_precon_apply(orc_solver *S, const double *r, double *z) {
  precon_apply(S, r, z);
  return 0;
}

/* y = A x with the assembled matrix of the degree-N problem (the matrix the AMG levels start
 * from; small cases only) */
int orc_matrix_apply(orc_solver *S, const double *x, double *y) {
  orc_csr A = build_matrix(S->el);
  csr_spmv(&A, 1.0, x, 0.0, y);
  csr_free(&A);
  return 0;
}

int orc_gather(const orc_solver *S, const double *qL, double *qG, int trans) {
  if (trans) orc_gather_trans(&S->el->ogs, qL, qG);
  else orc_gather_notrans(&S->el->ogs, qL, qG);
  return 0;
}

int orc_scatter_apply(const orc_solver *S, const double *qG, double *qL) {
  orc_scatter(&S->el->ogs, qG, qL);
  return 0;
}

/* forcing f at a node and Dirichlet data g (DATA FILE / RHS FIELD) */
static void rhs_source(const orc_settings *s, double x, double y, double z, double lam, double *f, double *g) {
  if (s->rhs == ORC_RHS_SINE) {
    *f = (3 * ORC_PI * ORC_PI + lam) * sin(ORC_PI * x) * sin(ORC_PI * y) * sin(ORC_PI * z);
    *g = sin(ORC_PI * x) * sin(ORC_PI * y) * sin(ORC_PI * z);
    return;
  }
  /* sum of Gaussian sources with centres U(domain) and widths U[0.05,0.2] */
  double acc = 0;
  for (int k = 0; k < s->nsources; ++k) {
    const double cx = -s->dimx / 2 + s->dimx * orc_u01(s->rhs_seed, 6, (uint64_t)k);
    const double cy = -s->dimy / 2 + s->dimy * orc_u01(s->rhs_seed, 7, (uint64_t)k);
    const double cz = -s->dimz / 2 + s->dimz * orc_u01(s->rhs_seed, 8, (uint64_t)k);
    const double w = 0.05 + 0.15 * orc_u01(s->rhs_seed, 9, (uint64_t)k);
    const double d2 = (x - cx) * (x - cx) + (y - cy) * (y - cy) + (z - cz) * (z - cz);
    acc += exp(-d2 / (2 * w * w));
  }
  *f = acc;
  *g = 0.0;
}

/* right-hand side of elliptic_t::Run: forcing, Dirichlet lifting, gather */
int orc_build_rhs(const orc_solver *S, double *r) {
  const orc_elliptic *el = S->el;
  const orc_mesh *m = el->mesh;
  const hlong Nl = el->ogs.Nlocal;
  const int Np = m->Np;
  double *rL = dalloc(Nl), *gL = dalloc(Nl), *AgL = dalloc(Nl);
  int anyBC = 0;
  for (hlong n = 0; n < Nl; ++n) {
    const hlong e = n / Np;
    double f, g;
    rhs_source(&S->s, m->x[n], m->y[n], m->z[n], elem_lambda(el, e), &f, &g);
    rL[n] = m->wJ[n] * f;
    if (!el->ipdg && el->mapB[n] == 1) { gL[n] = g; anyBC = 1; }
  }
  if (el->ipdg) orc_ipdg_rhs_bc(el, rL);   /* weakly imposed boundary data */
  if (!el->ipdg && S->s.rhs == ORC_RHS_SINE) {
    /* Neumann data of the data file at every face node whose node flag is a Neumann type
     * (ellipticRhsBCHex3D.okl:28-58: rhs -= -WsJ n . grad_B with grad_B = -grad u, as the
     * data file states it); contributions of faces inside the domain cancel in the gather */
    const int Nfp = m->Nfp;
    for (hlong e = 0; e < m->Nelements; ++e)
      for (int f = 0; f < 6; ++f)
        for (int b = 0; b < Nfp; ++b) {
          const hlong id = e * Np + m->faceNodes[f * Nfp + b];
          if (el->mapB[id] < 2) continue;
          double nrm[3], w;
          orc_face_geometry(m, e, f, b, nrm, &w);
          const double x = m->x[id], y = m->y[id], z = m->z[id];
          const double ux = -ORC_PI * cos(ORC_PI * x) * sin(ORC_PI * y) * sin(ORC_PI * z);
          const double uy = -ORC_PI * sin(ORC_PI * x) * cos(ORC_PI * y) * sin(ORC_PI * z);
          const double uz = -ORC_PI * sin(ORC_PI * x) * sin(ORC_PI * y) * cos(ORC_PI * z);
          rL[id] -= -w * (nrm[0] * ux + nrm[1] * uy + nrm[2] * uz);
        }
  }
  if (anyBC) {
    local_ax(el, gL, AgL);
    for (hlong n = 0; n < Nl; ++n) rL[n] -= AgL[n];
  }
  orc_gather_trans(&el->ogs, rL, r);
  free(rL); free(gL); free(AgL);
  return 0;
}

/* NBFPCG, linearSolverNBFPCG.cpp:72-186 (Sanan's notation): one fused update of
 * x, r, u = M r, w = A u-direction with four inner products per iteration, and the
 * recurrences for p, s = A p, q = M s, z = A q; returns iterations */
static int orc_nbfpcg(orc_solver *S, double *x, double *r, double tol, int maxit, double *res_out) {
  const orc_elliptic *el = S->el;
  const hlong N = el->ogs.Ngather;
  double *u = dalloc(N), *p = dalloc(N), *w = dalloc(N), *n = dalloc(N), *m = dalloc(N);
  double *s = dalloc(N), *z = dalloc(N), *q = dalloc(N), *Ax = dalloc(N);
  orc_operator(el, x, Ax);
  axpy(N, -1.0, Ax, 1.0, r);
  precon_apply(S, r, u);
  memcpy(p, u, sizeof(double) * (size_t)N);
  orc_operator(el, p, w);
  double gamma0 = dot(N, u, r), delta0 = dot(N, u, w), rdotr0 = dot(N, r, r);
  precon_apply(S, w, m);
  orc_operator(el, m, n);
  memcpy(s, w, sizeof(double) * (size_t)N);
  memcpy(q, m, sizeof(double) * (size_t)N);
  memcpy(z, n, sizeof(double) * (size_t)N);
  double eta0 = delta0, alpha0 = gamma0 / eta0, beta0 = 0.0;
  const double TOL = fmax(tol * tol * rdotr0, tol * tol);
  int iter;
  for (iter = 0; iter < maxit; ++iter) {
    if (rdotr0 <= TOL) break;
    double ur = 0, us = 0, uw = 0, rr = 0;
#pragma omp parallel for reduction(+ : ur, us, uw, rr)
    for (hlong i = 0; i < N; ++i) {
      x[i] += alpha0 * p[i];
      r[i] -= alpha0 * s[i];
      u[i] -= alpha0 * q[i];
      w[i] -= alpha0 * z[i];
      ur += u[i] * r[i];
      us += u[i] * s[i];
      uw += u[i] * w[i];
      rr += r[i] * r[i];
    }
    for (hlong i = 0; i < N; ++i) n[i] = w[i] - r[i];
    precon_apply(S, n, m);
    axpy(N, 1.0, u, 1.0, m);
    orc_operator(el, m, n);
    gamma0 = ur;
    beta0 = -us / eta0;
    delta0 = uw;
    rdotr0 = rr;
    axpy(N, 1.0, u, beta0, p);
    axpy(N, 1.0, w, beta0, s);
    axpy(N, 1.0, m, beta0, q);
    axpy(N, 1.0, n, beta0, z);
    eta0 = delta0 - beta0 * beta0 * eta0;
    alpha0 = gamma0 / eta0;
  }
  if (res_out) *res_out = sqrt(rdotr0);
  free(u); free(p); free(w); free(n); free(m); free(s); free(z); free(q); free(Ax);
  return iter;
}

/* (F)PCG, linearSolverPCG.cpp:67-171; returns iterations */
int orc_pcg(orc_solver *S, double *x, double *r, double tol, int maxit, double *res_out) {
  if (S->s.solver == ORC_NBFPCG) return orc_nbfpcg(S, x, r, tol, maxit, res_out);
  const orc_elliptic *el = S->el;
  const hlong N = el->ogs.Ngather;
  const int flexible = (S->s.solver == ORC_FPCG);
  double *p = dalloc(N), *z = dalloc(N), *Ax = dalloc(N), *Ap = dalloc(N);
  double rdotz1 = 0, rdotz2 = 0, alpha = 0, beta = 0, pAp = 0, rdotr0 = 0, TOL = 0;
  if (S->s.stop_rhs) {
    const double nb = sqrt(dot(N, r, r));
    TOL = fmax(tol * tol * nb * nb, tol * tol);
  }
  orc_operator(el, x, Ax);
  axpy(N, -1.0, Ax, 1.0, r);
  rdotr0 = dot(N, r, r);
  if (!S->s.stop_rhs) TOL = fmax(tol * tol * rdotr0, tol * tol);
  int iter;
  for (iter = 0; iter < maxit; ++iter) {
    if ((iter == 0 && rdotr0 == 0.0) || (iter > 0 && rdotr0 <= TOL)) break;
    precon_apply(S, r, z);
    rdotz2 = rdotz1;
    rdotz1 = dot(N, r, z);
    if (flexible) {
      const double zdotAp = dot(N, z, Ap);
      beta = (iter == 0) ? 0.0 : -alpha * zdotAp / rdotz2;
    } else {
      beta = (iter == 0) ? 0.0 : rdotz1 / rdotz2;
    }
    axpy(N, 1.0, z, beta, p);
    orc_operator(el, p, Ap);
    pAp = dot(N, p, Ap);
    alpha = rdotz1 / pAp;
    double rr = 0;
#pragma omp parallel for reduction(+ : rr)
    for (hlong i = 0; i < N; ++i) {
      x[i] += alpha * p[i];
      const double rn = r[i] - alpha * Ap[i];
      r[i] = rn;
      rr += rn * rn;
    }
    rdotr0 = rr;
  }
  if (res_out) *res_out = sqrt(rdotr0);
  free(p); free(z); free(Ax); free(Ap);
  return iter;
}

/* elliptic_t::Run: rhs, solve, scatter + AddBC, Solution norm and error vs the
 * manufactured solution (sine data only). xL_out may be NULL. */
int orc_run(orc_solver *S, double *xL_out, int *iters, double *norm, double *err) {
  const orc_elliptic *el = S->el;
  const orc_mesh *m = el->mesh;
  const hlong N = el->ogs.Ngather, Nl = el->ogs.Nlocal;
  double *r = dalloc(N), *x = dalloc(N);
  orc_build_rhs(S, r);
  if (el->allNeumann) zero_mean(el, r);
  const int it = orc_pcg(S, x, r, S->s.tol, S->s.maxit, NULL);
  double *xL = xL_out ? xL_out : dalloc(Nl);
  orc_scatter(&el->ogs, x, xL);
  double nrm = 0, e2 = 0;
  for (hlong n = 0; n < Nl; ++n) {
    double f, g;
    rhs_source(&S->s, m->x[n], m->y[n], m->z[n], 0.0, &f, &g);
    if (!el->ipdg && el->mapB[n] == 1) xL[n] = g;
    nrm += m->wJ[n] * xL[n] * xL[n];
    const double d = xL[n] - g;
    e2 += m->wJ[n] * d * d;
  }
  if (iters) *iters = it;
  if (norm) *norm = sqrt(nrm);
  if (err) *err = (S->s.rhs == ORC_RHS_SINE) ? sqrt(e2) : -1.0;
  if (!xL_out) free(xL);
  free(r); free(x);
  return 0;
}

/* wall-clock seconds for `reps` assembled operator applications with `nthreads`
 * OpenMP threads (CPU baseline of the Ax unit); q is deterministic. */
double orc_time_operator(orc_solver *S, int reps, int nthreads) {
#ifdef _OPENMP
  int old = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const hlong N = S->el->ogs.Ngather;
  double *q = dalloc(N), *Aq = dalloc(N);
  for (hlong i = 0; i < N; ++i) q[i] = 2.0 * orc_u01(1, 3, (uint64_t)i) - 1.0;
  orc_operator(S->el, q, Aq); /* warm-up */
#ifdef _OPENMP
  double t0 = omp_get_wtime();
  for (int r = 0; r < reps; ++r) orc_operator(S->el, q, Aq);
  double t1 = omp_get_wtime();
  omp_set_num_threads(old);
#else
  double t0 = 0, t1 = 0;
#endif
  free(q); free(Aq);
  return t1 - t0;
}

int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
