/*
 * Oracle (test infrastructure only): C API of the CPU restatement of the
 * reference's C0 hex elliptic path. Loaded by tests/ and bench.py's cpu_baseline
 * leg through ctypes (oracle/oracle.py); never linked into the product.
 */
#ifndef ORACLE_H
#define ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_solver orc_solver;

enum {
  ORC_INFO_NELEMENTS = 0,
  ORC_INFO_NP = 1,
  ORC_INFO_NGATHER = 2,
  ORC_INFO_NLOCAL = 3,
  ORC_INFO_NQ = 4,
  ORC_INFO_ALLNEUMANN = 5,
  ORC_INFO_MG_PLEVELS = 6,
  ORC_INFO_MG_AMGLEVELS = 7,
  ORC_INFO_COARSE_N = 8
};

orc_solver *orc_create(const char *settings_text, int *status);
void orc_destroy(orc_solver *S);
long long orc_info(const orc_solver *S, int what);
int orc_get_array(const orc_solver *S, const char *name, void *out);
int orc_operator_apply(const orc_solver *S, const double *q, double *Aq);
int orc_partial_ax_apply(const orc_solver *S, const double *q, double *AqL);
int orc_precon_apply(orc_solver *S, const double *r, double *z);
int orc_matrix_apply(orc_solver *S, const double *x, double *y);
int orc_gather(const orc_solver *S, const double *qL, double *qG, int trans);
int orc_scatter_apply(const orc_solver *S, const double *qG, double *qL);
int orc_build_rhs(const orc_solver *S, double *r);
int orc_pcg(orc_solver *S, double *x, double *r, double tol, int maxit, double *res_out);
int orc_run(orc_solver *S, double *xL_out, int *iters, double *norm, double *err);
double orc_time_operator(orc_solver *S, int reps, int nthreads);
int orc_threads(void);

/* building blocks exposed for unit checks */
double orc_u01(uint64_t seed, uint64_t stream, uint64_t key);
void orc_jacobiGLL(int N, double *x, double *w);
void orc_dmatrix1D(int N, const double *r, double *D);
void orc_hessenberg_eigenvalues(int n, const double *Hcolmajor, double *wr, double *wi);

#ifdef __cplusplus
}
#endif
#endif
