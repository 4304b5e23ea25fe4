/*
 * Oracle (test infrastructure only): hexahedral box mesh, node connectivity,
 * geometric factors and the masked gather-scatter of one polynomial degree.
 *
 * Follows:
 *   libs/mesh/meshSetupBoxHex3D.cpp:31-232      box EToV / EX,EY,EZ / boundary faces
 *   libs/mesh/meshBasisHex3D.cpp:34-90          tensor nodes, face node lists
 *   libs/mesh/meshConnectFaceNodes.cpp:32-101   vmapM/vmapP (aligned box faces: rot = 0)
 *   libs/mesh/meshConnectNodes.cpp:32-117       global ids by min propagation, mapB
 *   libs/mesh/meshPhysicalNodesHex3D.cpp:31-112 trilinear vertex map
 *   libs/mesh/meshGeometricFactorsHex3D.cpp:31-193 ggeo (G00..G22) and wJ
 * Meshes read from Gmsh files take their connectivity from orc_gmsh.c.
 *   solvers/elliptic/src/ellipticBoundarySetup.cpp:30-140 Dirichlet mask, weights
 *   libs/ogs/ogsSetup.cpp:44-470,867-886         ordering of gathered dofs and GlobalToLocal
 * Addition with no reference counterpart: interior-vertex jitter keyed by
 * (seed, global vertex id, axis).
 */
#include "orc_internal.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* vertices of each face, every face listed the same way round (meshSetElementType.cpp:80-81) */
static const int faceVertsHex[6][4] = {{0, 1, 2, 3}, {0, 4, 5, 1}, {1, 5, 6, 2},
                                       {2, 6, 7, 3}, {0, 3, 7, 4}, {4, 7, 6, 5}};

hlong orc_mesh_count(const orc_settings *s) {
  if (!s->mesh_file[0]) return (hlong)s->nx * s->ny * s->nz;
  orc_gmsh g;
  const int rc = orc_read_gmsh_hex(s->mesh_file, &g);
  const hlong E = rc ? -1 : g.Nelements;
  orc_gmsh_free(&g);
  return E;
}

static void reference_element(orc_mesh *m);
static void connect_nodes(orc_mesh *m, const hlong *vmapM, const hlong *vmapP);
static void physical_and_geometry(orc_mesh *m);

/* mesh read from a Gmsh file: connectivity by face matching, node pairs on connected
 * faces by the rotation-indexed permutation R */
static orc_mesh *orc_mesh_build_file(const orc_settings *s, int N) {
  orc_gmsh g;
  if (orc_read_gmsh_hex(s->mesh_file, &g)) { orc_gmsh_free(&g); return NULL; }
  orc_mesh *m = (orc_mesh *)calloc(1, sizeof(orc_mesh));
  m->N = N; m->Nq = N + 1; m->Np = m->Nq * m->Nq * m->Nq; m->Nfp = m->Nq * m->Nq;
  const hlong E = g.Nelements;
  const int Np = m->Np, Nfp = m->Nfp;
  m->Nelements = E;
  m->EToV = (hlong *)malloc(sizeof(hlong) * E * 8);
  m->EX = (double *)malloc(sizeof(double) * E * 8);
  m->EY = (double *)malloc(sizeof(double) * E * 8);
  m->EZ = (double *)malloc(sizeof(double) * E * 8);
  for (hlong i = 0; i < E * 8; ++i) {
    const hlong v = g.EToV[i];
    m->EToV[i] = v; m->EX[i] = g.VX[v]; m->EY[i] = g.VY[v]; m->EZ[i] = g.VZ[v];
  }
  m->EToE = (hlong *)malloc(sizeof(hlong) * E * 6);
  m->EToF = (int *)malloc(sizeof(int) * E * 6);
  m->EToB = (int *)malloc(sizeof(int) * E * 6);
  orc_gmsh_connect(&g, m->EToE, m->EToF, m->EToB);
  orc_gmsh_free(&g);
  reference_element(m);
  int *R = orc_face_node_matching(m);
  if (!R) { orc_mesh_free(m); return NULL; }
  hlong *vmapM = (hlong *)malloc(sizeof(hlong) * E * 6 * Nfp);
  hlong *vmapP = (hlong *)malloc(sizeof(hlong) * E * 6 * Nfp);
  for (hlong e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const hlong eP = m->EToE[e * 6 + f];
      const int fP = m->EToF[e * 6 + f];
      int rot = 0;
      if (eP >= 0) {
        const hlong v0P = m->EToV[eP * 8 + faceVertsHex[fP][0]];
        for (; rot < 4; ++rot)
          if (m->EToV[e * 8 + faceVertsHex[f][rot]] == v0P) break;
      }
      for (int n = 0; n < Nfp; ++n) {
        const hlong id = e * 6 * Nfp + f * Nfp + n;
        vmapM[id] = m->faceNodes[f * Nfp + n] + e * Np;
        vmapP[id] = (eP < 0 || rot == 4) ? vmapM[id]
                    : m->faceNodes[fP * Nfp + R[((f * 6 + fP) * 4 + rot) * Nfp + n]] + eP * Np;
      }
    }
  free(R);
  connect_nodes(m, vmapM, vmapP);
  free(vmapM);
  m->vmapP = vmapP;
  physical_and_geometry(m);
  return m;
}

orc_mesh *orc_mesh_build(const orc_settings *s, int N) {
  if (s->mesh_file[0]) return orc_mesh_build_file(s, N);
  orc_mesh *m = (orc_mesh *)calloc(1, sizeof(orc_mesh));
  m->N = N;
  m->Nq = N + 1;
  m->Np = m->Nq * m->Nq * m->Nq;
  m->Nfp = m->Nq * m->Nq;
  m->nx = s->nx; m->ny = s->ny; m->nz = s->nz;
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const int Np = m->Np, Nfp = m->Nfp;
  const hlong E = (hlong)nx * ny * nz;
  m->Nelements = E;
  const int periodic = (s->bcflag == -1);

  /* ---- box (meshSetupBoxHex3D.cpp:76-152) */
  const double dx = s->dimx / nx, dy = s->dimy / ny, dz = s->dimz / nz;
  const double X0 = -s->dimx / 2.0, Y0 = -s->dimy / 2.0, Z0 = -s->dimz / 2.0;
  const hlong NnX = periodic ? nx : nx + 1;
  const hlong NnY = periodic ? ny : ny + 1;
  const hlong NnZ = periodic ? nz : nz + 1;
  m->EToV = (hlong *)malloc(sizeof(hlong) * E * 8);
  m->EX = (double *)malloc(sizeof(double) * E * 8);
  m->EY = (double *)malloc(sizeof(double) * E * 8);
  m->EZ = (double *)malloc(sizeof(double) * E * 8);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const hlong e = i + (hlong)j * nx + (hlong)k * nx * ny;
        const hlong i0 = i, i1 = (i + 1) % NnX, j0 = j, j1 = (j + 1) % NnY, k0 = k, k1 = (k + 1) % NnZ;
        hlong *v = m->EToV + e * 8;
        v[0] = i0 + j0 * NnX + k0 * NnX * NnY; v[1] = i1 + j0 * NnX + k0 * NnX * NnY;
        v[2] = i1 + j1 * NnX + k0 * NnX * NnY; v[3] = i0 + j1 * NnX + k0 * NnX * NnY;
        v[4] = i0 + j0 * NnX + k1 * NnX * NnY; v[5] = i1 + j0 * NnX + k1 * NnX * NnY;
        v[6] = i1 + j1 * NnX + k1 * NnX * NnY; v[7] = i0 + j1 * NnX + k1 * NnX * NnY;
        const double x0 = X0 + dx * i, y0 = Y0 + dy * j, z0 = Z0 + dz * k;
        double *ex = m->EX + e * 8, *ey = m->EY + e * 8, *ez = m->EZ + e * 8;
        ex[0] = x0;      ey[0] = y0;      ez[0] = z0;
        ex[1] = x0 + dx; ey[1] = y0;      ez[1] = z0;
        ex[2] = x0 + dx; ey[2] = y0 + dy; ez[2] = z0;
        ex[3] = x0;      ey[3] = y0 + dy; ez[3] = z0;
        ex[4] = x0;      ey[4] = y0;      ez[4] = z0 + dz;
        ex[5] = x0 + dx; ey[5] = y0;      ez[5] = z0 + dz;
        ex[6] = x0 + dx; ey[6] = y0 + dy; ez[6] = z0 + dz;
        ex[7] = x0;      ey[7] = y0 + dy; ez[7] = z0 + dz;
        /* jitter of interior lattice vertices (no reference counterpart) */
        if (s->jitter != 0.0 && !periodic) {
          for (int vv = 0; vv < 8; ++vv) {
            const hlong vid = v[vv];
            const hlong vi = vid % NnX, vj = (vid / NnX) % NnY, vk = vid / (NnX * NnY);
            if (vi == 0 || vi == nx || vj == 0 || vj == ny || vk == 0 || vk == nz) continue;
            ex[vv] += (2.0 * orc_u01(s->jitter_seed, 0, (uint64_t)vid) - 1.0) * s->jitter * dx;
            ey[vv] += (2.0 * orc_u01(s->jitter_seed, 1, (uint64_t)vid) - 1.0) * s->jitter * dy;
            ez[vv] += (2.0 * orc_u01(s->jitter_seed, 2, (uint64_t)vid) - 1.0) * s->jitter * dz;
          }
        }
      }

  /* ---- element connectivity of the structured box (what meshConnect finds by
   * matching sorted face vertex ids; every box element has the same orientation) */
  m->EToE = (hlong *)malloc(sizeof(hlong) * E * 6);
  m->EToF = (int *)malloc(sizeof(int) * E * 6);
  m->EToB = (int *)calloc(E * 6, sizeof(int));
  static const int opp[6] = {5, 3, 4, 1, 2, 0};
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const hlong e = i + (hlong)j * nx + (hlong)k * nx * ny;
        int nb[6][3] = {{i, j, k - 1}, {i, j - 1, k}, {i + 1, j, k}, {i, j + 1, k}, {i - 1, j, k}, {i, j, k + 1}};
        for (int f = 0; f < 6; ++f) {
          int a = nb[f][0], b = nb[f][1], c = nb[f][2];
          int out = (a < 0 || a >= nx || b < 0 || b >= ny || c < 0 || c >= nz);
          if (out && periodic) { a = (a + nx) % nx; b = (b + ny) % ny; c = (c + nz) % nz; out = 0; }
          if (out) {
            m->EToE[e * 6 + f] = -1; m->EToF[e * 6 + f] = -1;
            m->EToB[e * 6 + f] = s->bcflag;
          } else {
            m->EToE[e * 6 + f] = a + (hlong)b * nx + (hlong)c * nx * ny;
            m->EToF[e * 6 + f] = opp[f];
          }
        }
      }
  reference_element(m);

  /* ---- vmapM / vmapP (aligned faces: face-local node n matches face-local node n) */
  hlong *vmapM = (hlong *)malloc(sizeof(hlong) * E * 6 * Nfp);
  hlong *vmapP = (hlong *)malloc(sizeof(hlong) * E * 6 * Nfp);
  for (hlong e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const hlong eP = m->EToE[e * 6 + f];
      const int fP = m->EToF[e * 6 + f];
      for (int n = 0; n < Nfp; ++n) {
        const hlong id = e * 6 * Nfp + f * Nfp + n;
        vmapM[id] = m->faceNodes[f * Nfp + n] + e * Np;
        vmapP[id] = (eP < 0) ? vmapM[id] : m->faceNodes[fP * Nfp + n] + eP * Np;
      }
    }
  connect_nodes(m, vmapM, vmapP);
  free(vmapM);
  m->vmapP = vmapP;
  physical_and_geometry(m);
  return m;
}

static void reference_element(orc_mesh *m) {
  const int N = m->N, Nq = m->Nq, Np = m->Np, Nfp = m->Nfp;
  m->gllz = (double *)malloc(sizeof(double) * Nq);
  m->gllw = (double *)malloc(sizeof(double) * Nq);
  m->D = (double *)malloc(sizeof(double) * Nq * Nq);
  orc_jacobiGLL(N, m->gllz, m->gllw);
  orc_dmatrix1D(N, m->gllz, m->D);
  m->r = (double *)malloc(sizeof(double) * Np);
  m->s = (double *)malloc(sizeof(double) * Np);
  m->t = (double *)malloc(sizeof(double) * Np);
  for (int k = 0; k < Nq; ++k)
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        int n = i + j * Nq + k * Nq * Nq;
        m->r[n] = m->gllz[i]; m->s[n] = m->gllz[j]; m->t[n] = m->gllz[k];
      }
  m->faceNodes = (int *)malloc(sizeof(int) * 6 * Nfp);
  {
    int cnt[6] = {0, 0, 0, 0, 0, 0};
    const double tol = 1000. * 2.220446049250313e-16;
    for (int n = 0; n < Np; ++n) {
      if (fabs(m->t[n] + 1) < tol) m->faceNodes[0 * Nfp + cnt[0]++] = n;
      if (fabs(m->s[n] + 1) < tol) m->faceNodes[1 * Nfp + cnt[1]++] = n;
      if (fabs(m->r[n] - 1) < tol) m->faceNodes[2 * Nfp + cnt[2]++] = n;
      if (fabs(m->s[n] - 1) < tol) m->faceNodes[3 * Nfp + cnt[3]++] = n;
      if (fabs(m->r[n] + 1) < tol) m->faceNodes[4 * Nfp + cnt[4]++] = n;
      if (fabs(m->t[n] - 1) < tol) m->faceNodes[5 * Nfp + cnt[5]++] = n;
    }
  }

}

/* ConnectNodes: min propagation of 1-based local ids, boundary flags */
static void connect_nodes(orc_mesh *m, const hlong *vmapM, const hlong *vmapP) {
  const hlong E = m->Nelements;
  const int Np = m->Np, Nfp = m->Nfp;
  m->globalIds = (hlong *)malloc(sizeof(hlong) * E * Np);
  m->mapB = (int *)malloc(sizeof(int) * E * Np);
  for (hlong n = 0; n < E * Np; ++n) { m->globalIds[n] = 1 + n; m->mapB[n] = -1; }
  for (hlong e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int bc = m->EToB[e * 6 + f];
      if (bc > 0)
        for (int n = 0; n < Nfp; ++n) {
          const hlong id = m->faceNodes[f * Nfp + n] + e * Np;
          if (m->mapB[id] == -1 || bc < m->mapB[id]) m->mapB[id] = bc;
        }
    }
  for (;;) {
    hlong change = 0;
    for (hlong e = 0; e < E; ++e)
      for (int n = 0; n < 6 * Nfp; ++n) {
        const hlong id = e * 6 * Nfp + n;
        const hlong idM = vmapM[id], idP = vmapP[id];
        if (m->globalIds[idP] < m->globalIds[idM]) { m->globalIds[idM] = m->globalIds[idP]; ++change; }
        const int bcM = m->mapB[idM], bcP = m->mapB[idP];
        if (bcP > 0) {
          if (bcM == -1 || bcP < bcM) { m->mapB[idM] = bcP; ++change; }
        }
      }
    if (!change) break;
  }
}

static void physical_and_geometry(orc_mesh *m) {
  const hlong E = m->Nelements;
  const int Nq = m->Nq, Np = m->Np;
  /* ---- physical nodes */
  m->x = (double *)malloc(sizeof(double) * E * Np);
  m->y = (double *)malloc(sizeof(double) * E * Np);
  m->z = (double *)malloc(sizeof(double) * E * Np);
#pragma omp parallel for
  for (hlong e = 0; e < E; ++e) {
    const double *xe = m->EX + e * 8, *ye = m->EY + e * 8, *ze = m->EZ + e * 8;
    for (int n = 0; n < Np; ++n) {
      const double rn = m->r[n], sn = m->s[n], tn = m->t[n];
      double c[8] = {0.125 * (1 - rn) * (1 - sn) * (1 - tn), 0.125 * (1 + rn) * (1 - sn) * (1 - tn),
                     0.125 * (1 + rn) * (1 + sn) * (1 - tn), 0.125 * (1 - rn) * (1 + sn) * (1 - tn),
                     0.125 * (1 - rn) * (1 - sn) * (1 + tn), 0.125 * (1 + rn) * (1 - sn) * (1 + tn),
                     0.125 * (1 + rn) * (1 + sn) * (1 + tn), 0.125 * (1 - rn) * (1 + sn) * (1 + tn)};
      double xx = 0, yy = 0, zz = 0;
      for (int v = 0; v < 8; ++v) { xx += c[v] * xe[v]; yy += c[v] * ye[v]; zz += c[v] * ze[v]; }
      m->x[e * Np + n] = xx; m->y[e * Np + n] = yy; m->z[e * Np + n] = zz;
    }
  }

  /* ---- geometric factors */
  m->ggeo = (double *)malloc(sizeof(double) * E * 6 * Np);
  m->wJ = (double *)malloc(sizeof(double) * E * Np);
  int bad = 0;
#pragma omp parallel for reduction(+ : bad)
  for (hlong e = 0; e < E; ++e) {
    for (int k = 0; k < Nq; ++k)
      for (int j = 0; j < Nq; ++j)
        for (int i = 0; i < Nq; ++i) {
          const int n = i + j * Nq + k * Nq * Nq;
          double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
          for (int mm = 0; mm < Nq; ++mm) {
            const hlong idr = e * Np + k * Nq * Nq + j * Nq + mm;
            const hlong ids = e * Np + k * Nq * Nq + mm * Nq + i;
            const hlong idt = e * Np + mm * Nq * Nq + j * Nq + i;
            xr += m->D[i * Nq + mm] * m->x[idr]; xs += m->D[j * Nq + mm] * m->x[ids]; xt += m->D[k * Nq + mm] * m->x[idt];
            yr += m->D[i * Nq + mm] * m->y[idr]; ys += m->D[j * Nq + mm] * m->y[ids]; yt += m->D[k * Nq + mm] * m->y[idt];
            zr += m->D[i * Nq + mm] * m->z[idr]; zs += m->D[j * Nq + mm] * m->z[ids]; zt += m->D[k * Nq + mm] * m->z[idt];
          }
          const double J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
          if (J < 1e-12) bad++;
          const double rx = (ys * zt - zs * yt) / J, ry = -(xs * zt - zs * xt) / J, rz = (xs * yt - ys * xt) / J;
          const double sx = -(yr * zt - zr * yt) / J, sy = (xr * zt - zr * xt) / J, sz = -(xr * yt - yr * xt) / J;
          const double tx = (yr * zs - zr * ys) / J, ty = -(xr * zs - zr * xs) / J, tz = (xr * ys - yr * xs) / J;
          const double JW = J * m->gllw[i] * m->gllw[j] * m->gllw[k];
          double *g = m->ggeo + e * 6 * Np + n;
          g[0 * Np] = JW * (rx * rx + ry * ry + rz * rz);
          g[1 * Np] = JW * (rx * sx + ry * sy + rz * sz);
          g[2 * Np] = JW * (rx * tx + ry * ty + rz * tz);
          g[3 * Np] = JW * (sx * sx + sy * sy + sz * sz);
          g[4 * Np] = JW * (sx * tx + sy * ty + sz * tz);
          g[5 * Np] = JW * (tx * tx + ty * ty + tz * tz);
          m->wJ[e * Np + n] = JW;
        }
  }
  if (bad) fprintf(stderr, "oracle: %d nodes with J < 1e-12\n", bad);
}

void orc_mesh_free(orc_mesh *m) {
  if (!m) return;
  free(m->EToV); free(m->EX); free(m->EY); free(m->EZ); free(m->EToB); free(m->EToE); free(m->EToF);
  free(m->gllz); free(m->gllw); free(m->D); free(m->r); free(m->s); free(m->t); free(m->faceNodes);
  free(m->x); free(m->y); free(m->z); free(m->ggeo); free(m->wJ); free(m->globalIds); free(m->mapB); free(m->vmapP);
  free(m);
}

/* ---------------------------------------------------------------- elliptic level */

orc_elliptic *orc_elliptic_build(const orc_settings *s, int N, const double *lambdaE) {
  orc_mesh *m = orc_mesh_build(s, N);
  if (!m) return NULL;
  orc_elliptic *el = (orc_elliptic *)calloc(1, sizeof(orc_elliptic));
  el->mesh = m;
  el->lambda = s->lambda;
  const hlong E = m->Nelements;
  const int Np = m->Np;
  const hlong Nlocal = E * Np;
  if (lambdaE) {
    el->lambdaE = (double *)malloc(sizeof(double) * E);
    memcpy(el->lambdaE, lambdaE, sizeof(double) * E);
  }

  /* BoundarySetup (ellipticBoundarySetup.cpp:30-65): BCType = {0,1,2} */
  el->allNeumann = (s->lambda == 0 && !lambdaE) ? 1 : 0;
  for (hlong f = 0; f < E * 6; ++f)
    if (m->EToB[f] > 0 && m->EToB[f] != 2) el->allNeumann = 0;
  el->mapB = (int *)malloc(sizeof(int) * Nlocal);
  for (hlong n = 0; n < Nlocal; ++n) el->mapB[n] = (m->mapB[n] > 0) ? m->mapB[n] : 0;

  /* masked global ids; gathered dofs numbered in order of first appearance of each
   * id in local node order (ogsSetup.cpp:408-432 with a single rank) */
  hlong *firstDof = (hlong *)malloc(sizeof(hlong) * Nlocal); /* indexed by globalId-1 */
  for (hlong n = 0; n < Nlocal; ++n) firstDof[n] = -1;
  el->ogs.GlobalToLocal = (int *)malloc(sizeof(int) * Nlocal);
  hlong Ng = 0;
  el->ipdg = s->ipdg;
  for (hlong n = 0; n < Nlocal; ++n) {
    if (s->ipdg) { el->ogs.GlobalToLocal[n] = (int)Ng++; continue; }  /* IPDG: every local node is a dof */
    if (el->mapB[n] == 1) { el->ogs.GlobalToLocal[n] = -1; continue; }
    const hlong g = m->globalIds[n] - 1;
    if (firstDof[g] < 0) firstDof[g] = Ng++;
    el->ogs.GlobalToLocal[n] = (int)firstDof[g];
  }
  free(firstDof);
  el->ogs.Nlocal = Nlocal;
  el->ogs.Ngather = Ng;
  el->ogs.rowStarts = (hlong *)calloc(Ng + 1, sizeof(hlong));
  for (hlong n = 0; n < Nlocal; ++n)
    if (el->ogs.GlobalToLocal[n] >= 0) el->ogs.rowStarts[el->ogs.GlobalToLocal[n] + 1]++;
  for (hlong i = 0; i < Ng; ++i) el->ogs.rowStarts[i + 1] += el->ogs.rowStarts[i];
  el->ogs.colIds = (hlong *)malloc(sizeof(hlong) * (el->ogs.rowStarts[Ng] + 1));
  el->ogs.firstCol = (hlong *)malloc(sizeof(hlong) * (Ng + 1));
  hlong *cnt = (hlong *)calloc(Ng + 1, sizeof(hlong));
  for (hlong n = 0; n < Nlocal; ++n) {
    const int g = el->ogs.GlobalToLocal[n];
    if (g < 0) continue;
    if (cnt[g] == 0) el->ogs.firstCol[g] = n;
    el->ogs.colIds[el->ogs.rowStarts[g] + cnt[g]++] = n;
  }
  free(cnt);

  el->allNeumannScale = 1.0 / sqrt((double)Ng);

  /* inverse multiplicity weights */
  el->weightG = (double *)malloc(sizeof(double) * (Ng + 1));
  for (hlong i = 0; i < Ng; ++i) {
    const double c = (double)(el->ogs.rowStarts[i + 1] - el->ogs.rowStarts[i]);
    el->weightG[i] = (c > 0) ? 1.0 / c : 0.0;
  }
  if (el->ipdg) orc_ipdg_setup(el);
  return el;
}

/* SEMFEM sub-mesh (meshSetupSEMFEM.cpp:98-214, ellipticPreconSEMFEM.cpp:56-200 for
 * hexahedra): every degree-N element is cut into N^3 trilinear hexahedra whose vertices
 * are its GLL nodes; their degree-1 nodes keep the assembled dof of the GLL node they sit
 * on (masked nodes stay masked), so the low-order matrix acts on the same vectors. */
orc_elliptic *orc_semfem_build(const orc_elliptic *sem) {
  const orc_mesh *M = sem->mesh;
  const int N = M->N, Nq = M->Nq, Np = M->Np;
  const hlong Es = M->Nelements * N * N * N;
  orc_mesh *m = (orc_mesh *)calloc(1, sizeof(orc_mesh));
  m->N = 1; m->Nq = 2; m->Np = 8; m->Nfp = 4;
  m->Nelements = Es;
  m->EX = (double *)malloc(sizeof(double) * Es * 8);
  m->EY = (double *)malloc(sizeof(double) * Es * 8);
  m->EZ = (double *)malloc(sizeof(double) * Es * 8);
  orc_elliptic *el = (orc_elliptic *)calloc(1, sizeof(orc_elliptic));
  el->mesh = m;
  el->lambda = sem->lambda;
  el->ogs.GlobalToLocal = (int *)malloc(sizeof(int) * Es * 8);
  if (sem->lambdaE) el->lambdaE = (double *)malloc(sizeof(double) * Es);
  static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (hlong e = 0; e < M->Nelements; ++e)
    for (int k = 0; k < N; ++k)
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          const hlong es = ((e * N + k) * N + j) * N + i;
          for (int v = 0; v < 8; ++v) {
            /* vertex v in hexahedron order; degree-1 node a + 2b + 4c in tensor order */
            const hlong id = e * Np + (i + cx[v]) + (j + cy[v]) * Nq + (k + cz[v]) * Nq * Nq;
            m->EX[es * 8 + v] = M->x[id]; m->EY[es * 8 + v] = M->y[id]; m->EZ[es * 8 + v] = M->z[id];
            el->ogs.GlobalToLocal[es * 8 + cx[v] + 2 * cy[v] + 4 * cz[v]] = sem->ogs.GlobalToLocal[id];
          }
          if (el->lambdaE) el->lambdaE[es] = sem->lambdaE[e];
        }
  reference_element(m);
  physical_and_geometry(m);
  el->ogs.Nlocal = Es * 8;
  el->ogs.Ngather = sem->ogs.Ngather;
  el->allNeumann = sem->allNeumann;
  el->allNeumannScale = sem->allNeumannScale;
  return el;
}

void orc_elliptic_free(orc_elliptic *e) {
  if (!e) return;
  orc_mesh_free(e->mesh);
  free(e->ogs.rowStarts); free(e->ogs.colIds); free(e->ogs.firstCol); free(e->ogs.GlobalToLocal);
  free(e->mapB); free(e->weightG); free(e->lambdaE); free(e->vgeo); free(e->sgeo);
  free(e);
}

/* ---------------------------------------------------------------- ogs */

void orc_gather_trans(const orc_ogs *o, const double *qL, double *qG) {
#pragma omp parallel for
  for (hlong r = 0; r < o->Ngather; ++r) {
    double v = 0;
    for (hlong j = o->rowStarts[r]; j < o->rowStarts[r + 1]; ++j) v += qL[o->colIds[j]];
    qG[r] = v;
  }
}

void orc_gather_notrans(const orc_ogs *o, const double *qL, double *qG) {
#pragma omp parallel for
  for (hlong r = 0; r < o->Ngather; ++r) qG[r] = qL[o->firstCol[r]];
}

void orc_scatter(const orc_ogs *o, const double *qG, double *qL) {
#pragma omp parallel for
  for (hlong n = 0; n < o->Nlocal; ++n) {
    const int g = o->GlobalToLocal[n];
    qL[n] = (g >= 0) ? qG[g] : 0.0;
  }
}
