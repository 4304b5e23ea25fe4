/* Harness around the reference's own kernels (test infrastructure only).
 *
 * oracle/okl_translate.py turns the reference's OKL kernels into C with OCCA's
 * Serial/OpenMP semantics (oracle/_ref/ref_kernels.c, generated, not committed); this file
 * drives them the way elliptic_t::Operator does on one rank
 * (solvers/elliptic/src/ellipticOperator.cpp:29-106):
 *   partialAxKernel on the first half of the local gather elements, then on the second
 *   half, each writing AqL (E*Np); then ogsMasked.Gather(Aq, AqL, 1, Add, Trans), whose
 *   row blocks (at most gatherNodesPerBlock = 512 entries each) are formed as
 *   ogsOperator_t::setupRowBlocks does (libs/ogs/ogsOperator.cpp:495-560).
 * Built by oracle/build.py into oracle/_ref/libref.so with the reference's release flags
 * (make.top: -O3 -fopenmp -ftree-vectorize). Used by tests as a checker of the oracle and
 * of the CUDA path, and by bench.py as the reference's CPU implementation.
 */
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>

typedef double dfloat;
typedef int dlong;

#define AX_ARGS                                                                                          \
  const dlong Nelements, const dlong *restrict elementList, const dlong *restrict GlobalToLocal,        \
      const dfloat *restrict wJ, const dfloat *restrict ggeo, const dfloat *restrict DT,                 \
      const dfloat *restrict S, const dfloat *restrict MM, const dfloat lambda, const dfloat *restrict q, \
      dfloat *restrict Aq

void ref_partialAxHex3D_N1(AX_ARGS);
void ref_partialAxHex3D_N2(AX_ARGS);
void ref_partialAxHex3D_N3(AX_ARGS);
void ref_partialAxHex3D_N4(AX_ARGS);
void ref_partialAxHex3D_N5(AX_ARGS);
void ref_partialAxHex3D_N6(AX_ARGS);
void ref_partialAxHex3D_N7(AX_ARGS);
void ref_partialAxHex3D_N8(AX_ARGS);
void ref_ogsGatherAdd(const dlong Nblocks, const int K, const dlong *restrict blockStarts,
                      const dlong *restrict gatherStarts, const dlong *restrict gatherIds,
                      const double *restrict q, double *restrict gatherq);

typedef void (*ax_fn)(AX_ARGS);
static ax_fn ax_for(int N) {
  static const ax_fn f[9] = {0,
                             ref_partialAxHex3D_N1,
                             ref_partialAxHex3D_N2,
                             ref_partialAxHex3D_N3,
                             ref_partialAxHex3D_N4,
                             ref_partialAxHex3D_N5,
                             ref_partialAxHex3D_N6,
                             ref_partialAxHex3D_N7,
                             ref_partialAxHex3D_N8};
  return (N >= 1 && N <= 8) ? f[N] : 0;
}

typedef struct {
  int N;
  dlong E, Np, Nlocal, Ngather, Nblocks;
  dlong *elementList, *rowStarts, *colIds, *blockStarts;
  const dlong *g2l;
  const dfloat *wJ, *ggeo, *D;
  dfloat lambda;
  dfloat *AqL;
} ref_op;

/* Gather(Trans) rows: every local copy of each assembled dof, in local-node order; row
 * blocks of at most 512 entries, greedily in row order. Arrays are borrowed, not copied. */
ref_op *ref_op_create(int N, dlong E, const dlong *g2l, dlong Ngather, const dfloat *wJ, const dfloat *ggeo,
                      const dfloat *D, dfloat lambda) {
  if (!ax_for(N) || E < 0 || Ngather < 0) return 0;
  ref_op *o = (ref_op *)calloc(1, sizeof(ref_op));
  o->N = N;
  o->E = E;
  o->Np = (N + 1) * (N + 1) * (N + 1);
  o->Nlocal = E * o->Np;
  o->Ngather = Ngather;
  o->g2l = g2l;
  o->wJ = wJ;
  o->ggeo = ggeo;
  o->D = D;
  o->lambda = lambda;
  o->elementList = (dlong *)malloc(sizeof(dlong) * (E + 1));
  for (dlong e = 0; e < E; ++e) o->elementList[e] = e;
  o->AqL = (dfloat *)malloc(sizeof(dfloat) * (o->Nlocal + 1));
  o->rowStarts = (dlong *)calloc(Ngather + 1, sizeof(dlong));
  for (dlong n = 0; n < o->Nlocal; ++n)
    if (g2l[n] >= 0) o->rowStarts[g2l[n] + 1]++;
  for (dlong r = 0; r < Ngather; ++r) o->rowStarts[r + 1] += o->rowStarts[r];
  o->colIds = (dlong *)malloc(sizeof(dlong) * (o->rowStarts[Ngather] + 1));
  dlong *fill = (dlong *)calloc(Ngather + 1, sizeof(dlong));
  for (dlong n = 0; n < o->Nlocal; ++n)
    if (g2l[n] >= 0) o->colIds[o->rowStarts[g2l[n]] + fill[g2l[n]]++] = n;
  free(fill);
  dlong nb = Ngather ? 1 : 0, sum = 0;
  for (dlong r = 0; r < Ngather; ++r) {
    const dlong sz = o->rowStarts[r + 1] - o->rowStarts[r];
    if (sum + sz > 512) { ++nb; sum = sz; } else sum += sz;
  }
  o->blockStarts = (dlong *)calloc(nb + 1, sizeof(dlong));
  o->Nblocks = nb;
  nb = Ngather ? 1 : 0;
  sum = 0;
  for (dlong r = 0; r < Ngather; ++r) {
    const dlong sz = o->rowStarts[r + 1] - o->rowStarts[r];
    if (sum + sz > 512) { o->blockStarts[nb++] = r; sum = sz; } else sum += sz;
  }
  o->blockStarts[o->Nblocks] = Ngather;
  return o;
}

void ref_op_destroy(ref_op *o) {
  if (!o) return;
  free(o->elementList);
  free(o->AqL);
  free(o->rowStarts);
  free(o->colIds);
  free(o->blockStarts);
  free(o);
}

/* partialAx only: AqL (E*Np) of the listed elements, the kernel's own contract */
void ref_op_partial_ax(const ref_op *o, const dfloat *q, dfloat *AqL) {
  ax_for(o->N)(o->E, o->elementList, o->g2l, o->wJ, o->ggeo, o->D, 0, 0, o->lambda, q, AqL);
}

/* elliptic_t::Operator on one rank: two partialAx launches over the halves of the element
 * list, then the Trans gather of AqL into Aq */
void ref_op_apply(ref_op *o, const dfloat *q, dfloat *Aq) {
  const ax_fn ax = ax_for(o->N);
  const dlong h = o->E / 2;
  if (h) ax(h, o->elementList, o->g2l, o->wJ, o->ggeo, o->D, 0, 0, o->lambda, q, o->AqL);
  if (o->E - h) ax(o->E - h, o->elementList + h, o->g2l, o->wJ, o->ggeo, o->D, 0, 0, o->lambda, q, o->AqL);
  if (o->Nblocks) ref_ogsGatherAdd(o->Nblocks, 1, o->blockStarts, o->rowStarts, o->colIds, o->AqL, Aq);
}

/* wall seconds of `reps` applications after one warm-up, on `nthreads` OpenMP threads
 * (0 = all) */
double ref_op_time(ref_op *o, const dfloat *q, dfloat *Aq, int reps, int nthreads) {
  const int old = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
  ref_op_apply(o, q, Aq);
  const double t0 = omp_get_wtime();
  for (int r = 0; r < reps; ++r) ref_op_apply(o, q, Aq);
  const double t1 = omp_get_wtime();
  omp_set_num_threads(old);
  return t1 - t0;
}

int ref_threads(void) { return omp_get_max_threads(); }
