/*
 * Oracle (test infrastructure only): a plain-C CPU restatement of libParanumal's
 * C0 hexahedral elliptic path. It is the checker for the CUDA product path and is
 * used only by tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py.
 * Nothing in the shipped library links or calls it.
 *
 * Parity pins: the reference's own regression tests (test/testElliptic.py:95-98,
 * 199-213, 244-248 through test/test.py:101-161, |norm - golden| < 1e-5) are
 * re-run against this restatement in tests/test_oracle_golden.py.
 *
 * Internal data structures shared by orc_basis.c, orc_mesh.c and orc_solver.c.
 */
#ifndef ORC_INTERNAL_H
#define ORC_INTERNAL_H

#include <stdint.h>
#include <stddef.h>

typedef long long hlong;

#define ORC_PI 3.14159265358979323846

/* ---------------- settings (subset of the reference's .rc keys) ---------------- */
enum { ORC_PCG = 0, ORC_FPCG = 1, ORC_NBFPCG = 2 };
enum { ORC_PRE_NONE = 0, ORC_PRE_JACOBI = 1, ORC_PRE_MULTIGRID = 2, ORC_PRE_PARALMOND = 3, ORC_PRE_SEMFEM = 4,
       ORC_PRE_OAS = 5 };
enum { ORC_MG_HALFDOFS = 0, ORC_MG_HALFDEGREES = 1, ORC_MG_ALLDEGREES = 2, ORC_MG_LIST = 3 };
enum { ORC_SMOOTH_CHEBYSHEV = 0, ORC_SMOOTH_JACOBI = 1 };
enum { ORC_RHS_SINE = 0, ORC_RHS_GAUSSIAN_SOURCES = 1, ORC_RHS_BUMPS = 2 };

typedef struct {
  int nx, ny, nz;
  double dimx, dimy, dimz;
  int bcflag;          /* BOX BOUNDARY FLAG: 1 Dirichlet, 2 Neumann(unsupported), -1 periodic */
  int N;               /* POLYNOMIAL DEGREE */
  double lambda;       /* LAMBDA */
  int lambda_field;    /* LAMBDA FIELD: 0 constant, 1 lognormal(0,1) per element */
  uint64_t lambda_seed;
  double jitter;       /* MESH JITTER: fraction of element width */
  uint64_t jitter_seed;
  int rhs;             /* RHS FIELD */
  uint64_t rhs_seed;
  int nsources;
  int solver;          /* LINEAR SOLVER */
  int stop_rhs;        /* LINEAR SOLVER STOPPING CRITERION == ABS/REL-RHS-2NORM */
  int precon;
  int mg_coarsening;
  int mg_ndeg;
  int mg_degrees[16];
  int mg_smoother;
  int mg_cheb_degree;
  int amg_strength_rs; /* 1: RUGESTUBEN, 0: SYMMETRIC */
  int amg_unsmoothed;  /* 1: UNSMOOTHED aggregation */
  int amg_smoother;
  int amg_cheb_degree;
  double tol;
  int maxit;
  int ipdg;            /* DISCRETIZATION: 0 CONTINUOUS, 1 IPDG */
  char mesh_file[1024]; /* MESH FILE: empty for BOX, else a Gmsh 2.2 ASCII hexahedral mesh */
} orc_settings;

int orc_parse_settings(const char *text, orc_settings *s);

/* ---------------- counter-based RNG shared with the product ---------------- */
uint64_t orc_splitmix64(uint64_t x);
double orc_u01(uint64_t seed, uint64_t stream, uint64_t key);

/* ---------------- drand48 stream (POSIX 48-bit LCG), seeded like srand48(0) ---------------- */
typedef struct { uint64_t x; } orc_rand48;
void orc_srand48(orc_rand48 *r, long seed);
double orc_drand48(orc_rand48 *r);

/* ---------------- 1D basis (libs/mesh/meshBasis1D.cpp) ---------------- */
double orc_jacobiP(double a, double alpha, double beta, int N);
double orc_gradJacobiP(double a, double alpha, double beta, int N);
void orc_jacobiGQ(double alpha, double beta, int N, double *x); /* N+1 nodes */
void orc_jacobiGLL(int N, double *x, double *w);                 /* N+1 nodes/weights */
void orc_dmatrix1D(int N, const double *r, double *D);            /* (N+1)^2, row-major D[i*Nq+j] */
void orc_interp1D(int N, const double *rin, int Nout, const double *rout, double *I); /* Nout x (N+1) */

/* ---------------- dense linear algebra (stand-ins for the reference's LAPACK calls) ---------------- */
int orc_matrix_inverse(int n, double *A);                  /* in place, row-major */
int orc_right_solve(int nrA, int ncA, const double *A, int nB, const double *B, double *C); /* C = A / B, B nB x nB */
void orc_sym_eigenvalues(int n, double *A, double *w);     /* symmetric Jacobi sweeps; A destroyed */
void orc_hessenberg_eigenvalues(int n, const double *Hcolmajor, double *wr, double *wi);

/* ---------------- mesh (one polynomial degree) ---------------- */
typedef struct {
  int N, Nq, Np, Nfp;
  int nx, ny, nz;
  hlong Nelements;
  /* vertices */
  hlong *EToV;       /* E*8 */
  double *EX, *EY, *EZ; /* E*8 */
  int *EToB;         /* E*6: boundary flag per face (0 interior) */
  hlong *EToE;       /* E*6: neighbour element or -1 */
  int *EToF;         /* E*6 */
  /* reference element */
  double *gllz, *gllw, *D;
  double *r, *s, *t;
  int *faceNodes;    /* 6*Nfp */
  /* nodes */
  double *x, *y, *z; /* E*Np */
  double *ggeo;      /* E*6*Np */
  double *wJ;        /* E*Np */
  hlong *globalIds;  /* E*Np */
  int *mapB;         /* E*Np (mesh level: -1 none, >0 flag) */
  hlong *vmapP;      /* E*6*Nfp: volume node on the other side of each face node (self on the boundary) */
} orc_mesh;

orc_mesh *orc_mesh_build(const orc_settings *s, int N);
void orc_mesh_free(orc_mesh *m);

/* ---------------- Gmsh hexahedral meshes (orc_gmsh.c) ---------------- */
typedef struct {
  hlong Nnodes, Nelements, NboundaryFaces;
  double *VX, *VY, *VZ;
  long long *nodeTag;
  hlong *EToV;       /* Nelements*8, 0-based node indices */
  hlong *binfo;      /* NboundaryFaces*5: physical tag, 4 node indices */
} orc_gmsh;
int orc_read_gmsh_hex(const char *path, orc_gmsh *g);  /* 0 ok */
void orc_gmsh_free(orc_gmsh *g);
/* EToE/EToF by sorted face vertices, EToB (0 interior, tag or -1 on the boundary) */
void orc_gmsh_connect(const orc_gmsh *g, hlong *EToE, int *EToF, int *EToB);
/* R[((fM*6 + fP)*4 + rot)*Nfp + nM] = nP, or NULL if a node has no match */
int *orc_face_node_matching(const orc_mesh *m);
/* number of elements of the configured mesh (box or file), -1 on a file error */
hlong orc_mesh_count(const orc_settings *s);

/* ---------------- gather-scatter (libs/ogs, Signed + unique, single rank) ---------------- */
typedef struct {
  hlong Nlocal;     /* E*Np */
  hlong Ngather;    /* assembled unmasked dofs */
  hlong *rowStarts; /* Ngather+1 : all copies (Trans) */
  hlong *colIds;
  hlong *firstCol;  /* Ngather : the copy used by NoTrans gathers */
  int *GlobalToLocal; /* Nlocal: dof index or -1 (masked) */
} orc_ogs;

/* ---------------- elliptic level ---------------- */
typedef struct {
  orc_mesh *mesh;
  orc_ogs ogs;
  int *mapB;         /* elliptic node flags: 0 free, 1 Dirichlet */
  double *weightG;   /* 1/multiplicity, Ngather */
  double lambda;
  double *lambdaE;   /* per-element lambda or NULL */
  int allNeumann;
  double allNeumannScale;
  /* IPDG (DISCRETIZATION = IPDG): unknowns are the E*Np local nodes */
  int ipdg;
  double tau;
  double *vgeo;      /* E*10*Np: rx ry rz sx sy sz tx ty tz JW */
  double *sgeo;      /* E*6*Nfp*5: nx ny nz WsJ hinv */
} orc_elliptic;

orc_elliptic *orc_elliptic_build(const orc_settings *s, int N, const double *lambdaE);
void orc_elliptic_free(orc_elliptic *e);
/* low-order (degree 1) elliptic on the GLL sub-mesh of a degree-N one, sharing its
 * assembled numbering (mesh_t::SetupSEMFEM for hexahedra, meshSetupSEMFEM.cpp:30-214) */
orc_elliptic *orc_semfem_build(const orc_elliptic *sem);

/* IPDG (orc_ipdg.c) */
void orc_ipdg_setup(orc_elliptic *el);
void orc_ipdg_operator(const orc_elliptic *el, const double *q, double *Aq);
void orc_ipdg_diagonal(const orc_elliptic *el, double *diag);
/* rhs -= boundary terms of the Dirichlet / Neumann data of the manufactured solution */
void orc_ipdg_rhs_bc(const orc_elliptic *el, double *rhs);
/* unit outward normal and WsJ at face node b of face f of element e */
void orc_face_geometry(const orc_mesh *m, hlong e, int f, int b, double *nrm, double *wsJ);
/* assembled IPDG matrix as COO (malloc'ed arrays), returns the entry count */
hlong orc_ipdg_matrix(const orc_elliptic *el, hlong **rows, hlong **cols, double **vals);

/* element operators */
void orc_partial_ax(const orc_elliptic *e, const double *q, double *AqL);
void orc_operator(const orc_elliptic *e, const double *q, double *Aq);
void orc_gather_trans(const orc_ogs *o, const double *qL, double *qG);
void orc_gather_notrans(const orc_ogs *o, const double *qL, double *qG);
void orc_scatter(const orc_ogs *o, const double *qG, double *qL);
void orc_build_diagonal(const orc_elliptic *e, double *diagA);

#endif
