/*
 * Oracle (test infrastructure only): hexahedral meshes read from Gmsh files and their
 * unstructured connectivity.
 *
 * Follows:
 *   libs/mesh/meshReadGmshHex3D.cpp:33-170     $Nodes, $Elements (type 5 hexahedra, type 3
 *                                              quadrilateral boundary faces with their
 *                                              physical tag), 0-based EToV, EX/EY/EZ
 *   libs/mesh/meshConnect.cpp:51-127           EToE/EToF by sorting faces on their sorted
 *                                              vertex ids
 *   libs/mesh/meshConnectBoundary.cpp:53-143   EToB: element faces without a neighbour matched
 *                                              to the file's boundary faces (largest tag wins)
 *   libs/mesh/meshBasisHex3D.cpp:131-270       face-node permutations R[fM][fP][rot][n]
 *   libs/mesh/meshConnectFaceNodes.cpp:32-101  vmapM/vmapP with the rotation at which the
 *                                              neighbour face's first vertex sits
 * Elements keep the file order (the reference repartitions with parAdogs, which on one
 * rank changes only the element order).
 */
#include "orc_internal.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* vertices of each face, every face listed the same way round (meshSetElementType.cpp:80-81) */
static const int fvH[6][4] = {{0, 1, 2, 3}, {0, 4, 5, 1}, {1, 5, 6, 2}, {2, 6, 7, 3}, {0, 3, 7, 4}, {4, 7, 6, 5}};

void orc_gmsh_free(orc_gmsh *g) {
  if (!g) return;
  free(g->VX); free(g->VY); free(g->VZ); free(g->EToV); free(g->binfo); free(g->nodeTag);
  memset(g, 0, sizeof(*g));
}

static int read_line(FILE *fp, char *buf, int n) { return fgets(buf, n, fp) != NULL; }

static hlong node_index(const orc_gmsh *g, long long tag) {
  /* node tags are normally 1..Nnodes in order; otherwise search */
  if (tag >= 1 && tag <= g->Nnodes && g->nodeTag[tag - 1] == tag) return tag - 1;
  for (hlong i = 0; i < g->Nnodes; ++i)
    if (g->nodeTag[i] == tag) return i;
  return -1;
}

int orc_read_gmsh_hex(const char *path, orc_gmsh *g) {
  memset(g, 0, sizeof(*g));
  FILE *fp = fopen(path, "r");
  if (!fp) return -1;
  char buf[4096];
  do {
    if (!read_line(fp, buf, sizeof(buf))) { fclose(fp); return -2; }
  } while (!strstr(buf, "$Nodes"));
  if (!read_line(fp, buf, sizeof(buf))) { fclose(fp); return -2; }
  g->Nnodes = atoll(buf);
  g->VX = (double *)malloc(sizeof(double) * g->Nnodes);
  g->VY = (double *)malloc(sizeof(double) * g->Nnodes);
  g->VZ = (double *)malloc(sizeof(double) * g->Nnodes);
  g->nodeTag = (long long *)malloc(sizeof(long long) * g->Nnodes);
  for (hlong n = 0; n < g->Nnodes; ++n) {
    if (!read_line(fp, buf, sizeof(buf)) ||
        sscanf(buf, "%lld %lf %lf %lf", g->nodeTag + n, g->VX + n, g->VY + n, g->VZ + n) != 4) {
      fclose(fp); return -2;
    }
  }
  do {
    if (!read_line(fp, buf, sizeof(buf))) { fclose(fp); return -2; }
  } while (!strstr(buf, "$Elements"));
  if (!read_line(fp, buf, sizeof(buf))) { fclose(fp); return -2; }
  const hlong nAll = atoll(buf);
  g->EToV = (hlong *)malloc(sizeof(hlong) * 8 * (nAll > 0 ? nAll : 1));
  g->binfo = (hlong *)malloc(sizeof(hlong) * 5 * (nAll > 0 ? nAll : 1));
  for (hlong i = 0; i < nAll; ++i) {
    if (!read_line(fp, buf, sizeof(buf))) { fclose(fp); return -2; }
    /* elm-number elm-type number-of-tags <tags> node-number-list */
    long long tok[64];
    int nt = 0;
    char *p = buf, *end;
    while (nt < 64) {
      long long v = strtoll(p, &end, 10);
      if (end == p) break;
      tok[nt++] = v;
      p = end;
    }
    if (nt < 3) { fclose(fp); return -2; }
    const int type = (int)tok[1], ntags = (int)tok[2];
    const long long phys = ntags > 0 ? tok[3] : 0;
    const long long *nodes = tok + 3 + ntags;
    const int nn = nt - 3 - ntags;
    if (type == 5) {
      if (nn < 8) { fclose(fp); return -2; }
      for (int v = 0; v < 8; ++v) {
        const hlong id = node_index(g, nodes[v]);
        if (id < 0) { fclose(fp); return -3; }
        g->EToV[g->Nelements * 8 + v] = id;
      }
      ++g->Nelements;
    } else if (type == 3) {
      if (nn < 4) { fclose(fp); return -2; }
      hlong *b = g->binfo + g->NboundaryFaces * 5;
      b[0] = phys;
      for (int v = 0; v < 4; ++v) {
        const hlong id = node_index(g, nodes[v]);
        if (id < 0) { fclose(fp); return -3; }
        b[1 + v] = id;
      }
      ++g->NboundaryFaces;
    }
  }
  fclose(fp);
  return g->Nelements > 0 ? 0 : -4;
}

/* ---------------------------------------------------------------- face sorting */
typedef struct {
  hlong v[4];
  hlong element;
  int face;
  int bctype;
  hlong elementN;
  int faceN;
} face_rec;

static void sort4(hlong *v) {
  for (int i = 1; i < 4; ++i)
    for (int j = i; j > 0 && v[j - 1] > v[j]; --j) { hlong t = v[j]; v[j] = v[j - 1]; v[j - 1] = t; }
}
static int cmp_verts(const void *a, const void *b) {
  const face_rec *x = (const face_rec *)a, *y = (const face_rec *)b;
  for (int i = 0; i < 4; ++i) {
    if (x->v[i] < y->v[i]) return -1;
    if (x->v[i] > y->v[i]) return 1;
  }
  /* stable tie-break so the order of equal keys does not depend on qsort */
  if (x->element != y->element) return x->element < y->element ? -1 : 1;
  return x->face - y->face;
}

void orc_gmsh_connect(const orc_gmsh *g, hlong *EToE, int *EToF, int *EToB) {
  const hlong E = g->Nelements;
  face_rec *F = (face_rec *)malloc(sizeof(face_rec) * E * 6);
  for (hlong e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      face_rec *r = F + e * 6 + f;
      for (int n = 0; n < 4; ++n) r->v[n] = g->EToV[e * 8 + fvH[f][n]];
      sort4(r->v);
      r->element = e; r->face = f; r->elementN = -1; r->faceN = -1;
    }
  qsort(F, E * 6, sizeof(face_rec), cmp_verts);
  for (hlong c = 0; c + 1 < E * 6; ++c)
    if (!memcmp(F[c].v, F[c + 1].v, sizeof(F[c].v))) {
      F[c].elementN = F[c + 1].element; F[c].faceN = F[c + 1].face;
      F[c + 1].elementN = F[c].element; F[c + 1].faceN = F[c].face;
    }
  for (hlong c = 0; c < E * 6; ++c) {
    EToE[F[c].element * 6 + F[c].face] = F[c].elementN;
    EToF[F[c].element * 6 + F[c].face] = F[c].faceN;
  }
  free(F);

  /* boundary faces: element faces without neighbour + the file's tagged faces */
  hlong nb = 0;
  for (hlong i = 0; i < E * 6; ++i) if (EToE[i] < 0) ++nb;
  face_rec *B = (face_rec *)malloc(sizeof(face_rec) * (nb + g->NboundaryFaces + 1));
  hlong c = 0;
  for (hlong e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f)
      if (EToE[e * 6 + f] < 0) {
        for (int n = 0; n < 4; ++n) B[c].v[n] = g->EToV[e * 8 + fvH[f][n]];
        sort4(B[c].v);
        B[c].element = e; B[c].face = f; B[c].bctype = -1;
        ++c;
      }
  for (hlong b = 0; b < g->NboundaryFaces; ++b) {
    for (int n = 0; n < 4; ++n) B[c].v[n] = g->binfo[b * 5 + 1 + n];
    sort4(B[c].v);
    B[c].element = -1; B[c].face = -1; B[c].bctype = (int)g->binfo[b * 5];
    ++c;
  }
  qsort(B, c, sizeof(face_rec), cmp_verts);
  for (hlong i = 0; i < E * 6; ++i) EToB[i] = (EToE[i] < 0) ? -1 : 0;
  for (hlong i = 0; i + 1 < c; ++i)
    if (!memcmp(B[i].v, B[i + 1].v, sizeof(B[i].v))) {
      const hlong e = B[i].element > B[i + 1].element ? B[i].element : B[i + 1].element;
      const int f = B[i].face > B[i + 1].face ? B[i].face : B[i + 1].face;
      const int bc = B[i].bctype > B[i + 1].bctype ? B[i].bctype : B[i + 1].bctype;
      if (e >= 0 && f >= 0) EToB[e * 6 + f] = bc;
    }
  free(B);
}

/* R[((fM*6 + fP)*4 + rot)*Nfp + nM] = nP: face fM of the upper element sits on face fP of
 * the lower one with fP's vertex `rot` under fM's vertex 0; both faces are mapped to the
 * unit square with opposite orientations and nodes matched by position. */
static void trilinear(const double *V, double r, double s, double t, double *out) {
  *out = 0.125 * (1 - r) * (1 - s) * (1 - t) * V[0] + 0.125 * (1 + r) * (1 - s) * (1 - t) * V[1] +
         0.125 * (1 + r) * (1 + s) * (1 - t) * V[2] + 0.125 * (1 - r) * (1 + s) * (1 - t) * V[3] +
         0.125 * (1 - r) * (1 - s) * (1 + t) * V[4] + 0.125 * (1 + r) * (1 - s) * (1 + t) * V[5] +
         0.125 * (1 + r) * (1 + s) * (1 + t) * V[6] + 0.125 * (1 - r) * (1 + s) * (1 + t) * V[7];
}

int *orc_face_node_matching(const orc_mesh *m) {
  static const double V0[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
  static const double V1[4][2] = {{-1, -1}, {-1, 1}, {1, 1}, {1, -1}};
  const int Nfp = m->Nfp;
  int *R = (int *)malloc(sizeof(int) * 6 * 6 * 4 * Nfp);
  double *x0 = (double *)malloc(sizeof(double) * Nfp), *y0 = (double *)malloc(sizeof(double) * Nfp);
  double *x1 = (double *)malloc(sizeof(double) * Nfp), *y1 = (double *)malloc(sizeof(double) * Nfp);
  int ok = 1;
  for (int fM = 0; fM < 6; ++fM) {
    double EX0[8] = {0}, EY0[8] = {0};
    for (int v = 0; v < 4; ++v) { EX0[fvH[fM][v]] = V0[v][0]; EY0[fvH[fM][v]] = V0[v][1]; }
    for (int n = 0; n < Nfp; ++n) {
      const int fn = m->faceNodes[fM * Nfp + n];
      trilinear(EX0, m->r[fn], m->s[fn], m->t[fn], x0 + n);
      trilinear(EY0, m->r[fn], m->s[fn], m->t[fn], y0 + n);
    }
    for (int fP = 0; fP < 6; ++fP)
      for (int rot = 0; rot < 4; ++rot) {
        double EX1[8] = {0}, EY1[8] = {0};
        for (int v = 0; v < 4; ++v) {
          const int fv = fvH[fP][(v + rot) % 4];
          EX1[fv] = V1[v][0]; EY1[fv] = V1[v][1];
        }
        for (int n = 0; n < Nfp; ++n) {
          const int fn = m->faceNodes[fP * Nfp + n];
          trilinear(EX1, m->r[fn], m->s[fn], m->t[fn], x1 + n);
          trilinear(EY1, m->r[fn], m->s[fn], m->t[fn], y1 + n);
        }
        for (int n = 0; n < Nfp; ++n) {
          int hit = -1;
          for (int k = 0; k < Nfp && hit < 0; ++k) {
            const double d = (x0[n] - x1[k]) * (x0[n] - x1[k]) + (y0[n] - y1[k]) * (y0[n] - y1[k]);
            if (d < 1e-5) hit = k;
          }
          if (hit < 0) ok = 0;
          R[((fM * 6 + fP) * 4 + rot) * Nfp + n] = hit < 0 ? 0 : hit;
        }
      }
  }
  free(x0); free(y0); free(x1); free(y1);
  if (!ok) { free(R); return NULL; }
  return R;
}
