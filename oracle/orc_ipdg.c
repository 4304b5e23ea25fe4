/*
 * Oracle (test infrastructure only): interior-penalty DG discretisation of the screened
 * Poisson operator on hexahedra (DISCRETIZATION = IPDG).
 *
 * Follows:
 *   solvers/elliptic/src/ellipticSetup.cpp:66-81           penalty tau = 2 (N+1)(N+3)
 *   solvers/elliptic/src/ellipticBoundarySetup.cpp:89-93    allNeumannScale = 1/sqrt(Np E)
 *   libs/mesh/meshGeometricFactorsHex3D.cpp                 vgeo: rx..tz and JW at the nodes
 *   libs/mesh/meshSurfaceGeometricFactorsHex3D.cpp:31-175   sgeo: unit normal, WsJ = sJ w_a w_b,
 *                                                           hinv = max(sJ/J on both sides)
 *   solvers/elliptic/okl/ellipticGradientHex3D.okl          physical gradient and value
 *   solvers/elliptic/okl/ellipticAxIpdgHex3D.okl:34-84,363-642  surface terms (homogeneous
 *                                                           Dirichlet / Neumann mirror states)
 *                                                           and the weak divergence
 *   solvers/elliptic/okl/ellipticRhsBCIpdgHex3D.okl         boundary data terms of the rhs
 *   solvers/elliptic/data/ellipticBoundary3D.h, data/ellipticSine3D.h  boundary data
 *   solvers/elliptic/src/ellipticBuildOperatorDiagonal.cpp:874-990  diagonal (Jacobi)
 */
#include "orc_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { RX, RY, RZ, SX, SY, SZ, TX, TY, TZ, JW, NVGEO };
enum { NXs, NYs, NZs, WSJ, IH, NSGEO };

void orc_ipdg_setup(orc_elliptic *el) {
  const orc_mesh *m = el->mesh;
  const int N = m->N, Nq = m->Nq, Np = m->Np, Nfp = m->Nfp;
  const hlong E = m->Nelements;
  const double *D = m->D;
  el->tau = 2.0 * (N + 1) * (N + 3);
  el->vgeo = (double *)malloc(sizeof(double) * E * NVGEO * Np);
  el->sgeo = (double *)malloc(sizeof(double) * E * 6 * Nfp * NSGEO);
  double *hfac = (double *)malloc(sizeof(double) * E * 6 * Nfp);   /* sJ / J per face node */
  for (hlong e = 0; e < E; ++e) {
    const double *x = m->x + e * Np, *y = m->y + e * Np, *z = m->z + e * Np;
    double *vg = el->vgeo + e * NVGEO * Np;
    double Jn[729];
    for (int k = 0; k < Nq; ++k)
      for (int j = 0; j < Nq; ++j)
        for (int i = 0; i < Nq; ++i) {
          const int n = i + j * Nq + k * Nq * Nq;
          double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
          for (int q = 0; q < Nq; ++q) {
            const int ir = q + j * Nq + k * Nq * Nq, is = i + q * Nq + k * Nq * Nq, it = i + j * Nq + q * Nq * Nq;
            xr += D[i * Nq + q] * x[ir]; yr += D[i * Nq + q] * y[ir]; zr += D[i * Nq + q] * z[ir];
            xs += D[j * Nq + q] * x[is]; ys += D[j * Nq + q] * y[is]; zs += D[j * Nq + q] * z[is];
            xt += D[k * Nq + q] * x[it]; yt += D[k * Nq + q] * y[it]; zt += D[k * Nq + q] * z[it];
          }
          const double J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
          vg[RX * Np + n] = (ys * zt - zs * yt) / J; vg[RY * Np + n] = -(xs * zt - zs * xt) / J;
          vg[RZ * Np + n] = (xs * yt - ys * xt) / J;
          vg[SX * Np + n] = -(yr * zt - zr * yt) / J; vg[SY * Np + n] = (xr * zt - zr * xt) / J;
          vg[SZ * Np + n] = -(xr * yt - yr * xt) / J;
          vg[TX * Np + n] = (yr * zs - zr * ys) / J; vg[TY * Np + n] = -(xr * zs - zr * xs) / J;
          vg[TZ * Np + n] = (xr * ys - yr * xs) / J;
          vg[JW * Np + n] = J * m->gllw[i] * m->gllw[j] * m->gllw[k];
          Jn[n] = J;
        }
    for (int f = 0; f < 6; ++f)
      for (int a = 0; a < Nfp; ++a) {
        const int n = m->faceNodes[f * Nfp + a];
        double nx, ny, nz;
        /* outward normal direction: +-(grad r, grad s, grad t) */
        switch (f) {
          case 0: nx = -vg[TX * Np + n]; ny = -vg[TY * Np + n]; nz = -vg[TZ * Np + n]; break;
          case 1: nx = -vg[SX * Np + n]; ny = -vg[SY * Np + n]; nz = -vg[SZ * Np + n]; break;
          case 2: nx = vg[RX * Np + n]; ny = vg[RY * Np + n]; nz = vg[RZ * Np + n]; break;
          case 3: nx = vg[SX * Np + n]; ny = vg[SY * Np + n]; nz = vg[SZ * Np + n]; break;
          case 4: nx = -vg[RX * Np + n]; ny = -vg[RY * Np + n]; nz = -vg[RZ * Np + n]; break;
          default: nx = vg[TX * Np + n]; ny = vg[TY * Np + n]; nz = vg[TZ * Np + n]; break;
        }
        const double J = Jn[n];
        const double len = sqrt(nx * nx + ny * ny + nz * nz);
        const double sJ = len * J;
        double *sg = el->sgeo + ((e * 6 + f) * Nfp + a) * NSGEO;
        sg[NXs] = nx / len; sg[NYs] = ny / len; sg[NZs] = nz / len;
        sg[WSJ] = sJ * m->gllw[a % Nq] * m->gllw[a / Nq];
        hfac[(e * 6 + f) * Nfp + a] = sJ / J;
      }
  }
  /* penalty scale: the larger sJ/J of the two sides (the face node itself on the boundary) */
  for (hlong e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f)
      for (int a = 0; a < Nfp; ++a) {
        const hlong id = (e * 6 + f) * Nfp + a;
        const hlong vP = m->vmapP[id];
        const hlong eP = vP / Np;
        double hP = hfac[id];
        if (m->EToE[e * 6 + f] >= 0) {
          /* the neighbour's face node at the same volume node */
          const int fP = m->EToF[e * 6 + f];
          for (int b = 0; b < Nfp; ++b)
            if (m->faceNodes[fP * Nfp + b] + eP * Np == vP) { hP = hfac[(eP * 6 + fP) * Nfp + b]; break; }
        }
        el->sgeo[id * NSGEO + IH] = hfac[id] > hP ? hfac[id] : hP;
      }
  free(hfac);
}

static inline double elam(const orc_elliptic *el, hlong e) { return el->lambdaE ? el->lambdaE[e] : el->lambda; }

/* gradient (x, y, z) and value of q at every node */
static void gradient(const orc_elliptic *el, const double *q, double *g4) {
  const orc_mesh *m = el->mesh;
  const int Nq = m->Nq, Np = m->Np;
  const double *D = m->D;
#pragma omp parallel for
  for (hlong e = 0; e < m->Nelements; ++e) {
    const double *qe = q + e * Np, *vg = el->vgeo + e * NVGEO * Np;
    for (int k = 0; k < Nq; ++k)
      for (int j = 0; j < Nq; ++j)
        for (int i = 0; i < Nq; ++i) {
          const int n = i + j * Nq + k * Nq * Nq;
          double qr = 0, qs = 0, qt = 0;
          for (int p = 0; p < Nq; ++p) {
            qr += D[i * Nq + p] * qe[p + j * Nq + k * Nq * Nq];
            qs += D[j * Nq + p] * qe[i + p * Nq + k * Nq * Nq];
            qt += D[k * Nq + p] * qe[i + j * Nq + p * Nq * Nq];
          }
          double *o = g4 + (e * Np + n) * 4;
          o[0] = vg[RX * Np + n] * qr + vg[SX * Np + n] * qs + vg[TX * Np + n] * qt;
          o[1] = vg[RY * Np + n] * qr + vg[SY * Np + n] * qs + vg[TY * Np + n] * qt;
          o[2] = vg[RZ * Np + n] * qr + vg[SZ * Np + n] * qs + vg[TZ * Np + n] * qt;
          o[3] = qe[n];
        }
  }
}

/* faces in the order the reference accumulates them: 0, 5, 1, 3, 2, 4 */
static const int face_order[6] = {0, 5, 1, 3, 2, 4};

/* out_e = JW lambda q + D^T-weighted divergence of (JW grad q + lifted jumps) + face terms */
static void weak_divergence(const orc_mesh *m, const double *vg, double *gx, double *gy, double *gz,
                            const double *acc, double *out) {
  const int Nq = m->Nq, Np = m->Np;
  const double *D = m->D;
  double ur[729], us[729], ut[729];
  for (int n = 0; n < Np; ++n) {
    ur[n] = vg[RX * Np + n] * gx[n] + vg[RY * Np + n] * gy[n] + vg[RZ * Np + n] * gz[n];
    us[n] = vg[SX * Np + n] * gx[n] + vg[SY * Np + n] * gy[n] + vg[SZ * Np + n] * gz[n];
    ut[n] = vg[TX * Np + n] * gx[n] + vg[TY * Np + n] * gy[n] + vg[TZ * Np + n] * gz[n];
  }
  for (int k = 0; k < Nq; ++k)
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        const int n = i + j * Nq + k * Nq * Nq;
        double v = acc[n];
        for (int p = 0; p < Nq; ++p) {
          v += D[p * Nq + i] * ur[p + j * Nq + k * Nq * Nq];
          v += D[p * Nq + j] * us[i + p * Nq + k * Nq * Nq];
          v += D[p * Nq + k] * ut[i + j * Nq + p * Nq * Nq];
        }
        out[n] = v;
      }
}

void orc_ipdg_operator(const orc_elliptic *el, const double *q, double *Aq) {
  const orc_mesh *m = el->mesh;
  const int Np = m->Np, Nfp = m->Nfp;
  const hlong E = m->Nelements;
  double *g4 = (double *)malloc(sizeof(double) * E * Np * 4);
  gradient(el, q, g4);
#pragma omp parallel for
  for (hlong e = 0; e < E; ++e) {
    const double *vg = el->vgeo + e * NVGEO * Np;
    double gx[729], gy[729], gz[729], a[729];
    const double lam = elam(el, e);
    for (int n = 0; n < Np; ++n) {
      const double *g = g4 + (e * Np + n) * 4, w = vg[JW * Np + n];
      gx[n] = w * g[0]; gy[n] = w * g[1]; gz[n] = w * g[2];
      a[n] = w * lam * g[3];
    }
    for (int fo = 0; fo < 6; ++fo) {
      const int f = face_order[fo];
      const int bc = m->EToB[e * 6 + f];
      for (int b = 0; b < Nfp; ++b) {
        const hlong id = (e * 6 + f) * Nfp + b;
        const int nM = m->faceNodes[f * Nfp + b];
        const double *sg = el->sgeo + id * NSGEO;
        const double *GM = g4 + (e * Np + nM) * 4;
        const double *GP = g4 + m->vmapP[id] * 4;
        double px = GP[0], py = GP[1], pz = GP[2], pq = GP[3];
        if (bc > 0) {
          /* homogeneous boundary state B, then the mirror 2B - M */
          double bx, by, bz, bq;
          if (bc == 1) { bq = 0; bx = GM[0]; by = GM[1]; bz = GM[2]; }
          else { bq = GM[3]; bx = 0; by = 0; bz = 0; }
          px = 2 * bx - GM[0]; py = 2 * by - GM[1]; pz = 2 * bz - GM[2]; pq = 2 * bq - GM[3];
        }
        const double dq = pq - GM[3];
        const double w = sg[WSJ];
        gx[nM] += 0.5 * w * sg[NXs] * dq;
        gy[nM] += 0.5 * w * sg[NYs] * dq;
        gz[nM] += 0.5 * w * sg[NZs] * dq;
        a[nM] += -0.5 * w * (sg[NXs] * (px + GM[0]) + sg[NYs] * (py + GM[1]) + sg[NZs] * (pz + GM[2]) +
                             el->tau * sg[IH] * dq);
      }
    }
    weak_divergence(m, vg, gx, gy, gz, a, Aq + e * Np);
  }
  free(g4);
}

void orc_ipdg_rhs_bc(const orc_elliptic *el, double *rhs) {
  const orc_mesh *m = el->mesh;
  const int Np = m->Np, Nfp = m->Nfp;
  const hlong E = m->Nelements;
  const double PI = ORC_PI;
#pragma omp parallel for
  for (hlong e = 0; e < E; ++e) {
    int any = 0;
    for (int f = 0; f < 6; ++f) any |= (m->EToB[e * 6 + f] > 0);
    if (!any) continue;
    const double *vg = el->vgeo + e * NVGEO * Np;
    double gx[729], gy[729], gz[729], a[729], out[729];
    for (int n = 0; n < Np; ++n) gx[n] = gy[n] = gz[n] = a[n] = 0;
    for (int fo = 0; fo < 6; ++fo) {
      const int f = face_order[fo];
      const int bc = m->EToB[e * 6 + f];
      if (bc <= 0) continue;
      for (int b = 0; b < Nfp; ++b) {
        const hlong id = (e * 6 + f) * Nfp + b;
        const int nM = m->faceNodes[f * Nfp + b];
        const double x = m->x[e * Np + nM], y = m->y[e * Np + nM], z = m->z[e * Np + nM];
        const double *sg = el->sgeo + id * NSGEO;
        /* boundary state of the manufactured solution u = sin(pi x) sin(pi y) sin(pi z) with
         * zero interior state: Dirichlet value, or the Neumann data of the data file */
        double qP = 0, dx = 0, dy = 0, dz = 0;
        if (bc == 1) qP = sin(PI * x) * sin(PI * y) * sin(PI * z);
        else {
          dx = -PI * cos(PI * x) * sin(PI * y) * sin(PI * z);
          dy = -PI * sin(PI * x) * cos(PI * y) * sin(PI * z);
          dz = -PI * sin(PI * x) * sin(PI * y) * cos(PI * z);
        }
        const double w = sg[WSJ];
        gx[nM] += w * sg[NXs] * qP;
        gy[nM] += w * sg[NYs] * qP;
        gz[nM] += w * sg[NZs] * qP;
        a[nM] += -w * (sg[NXs] * dx + sg[NYs] * dy + sg[NZs] * dz + el->tau * sg[IH] * qP);
      }
    }
    weak_divergence(m, vg, gx, gy, gz, a, out);
    for (int n = 0; n < Np; ++n) rhs[e * Np + n] -= out[n];
  }
}

void orc_ipdg_diagonal(const orc_elliptic *el, double *diag) {
  const orc_mesh *m = el->mesh;
  const int Nq = m->Nq, Np = m->Np, Nfp = m->Nfp;
  const hlong E = m->Nelements;
  const double *D = m->D;
#pragma omp parallel for
  for (hlong e = 0; e < E; ++e) {
    const double *vg = el->vgeo + e * NVGEO * Np;
    const double lam = elam(el, e);
    for (int n = 0; n < Np; ++n) {
      const int ni = n % Nq, nj = (n / Nq) % Nq, nk = n / (Nq * Nq);
      double A = lam * vg[JW * Np + n];   /* lambda (l_n, l_n) */
      /* (grad l_n, grad l_n): only nodes on the three lines through n contribute */
      for (int p = 0; p < Np; ++p) {
        const int pi = p % Nq, pj = (p / Nq) % Nq, pk = p / (Nq * Nq);
        const double br = (pj == nj && pk == nk) ? D[pi * Nq + ni] : 0.0;
        const double bs = (pi == ni && pk == nk) ? D[pj * Nq + nj] : 0.0;
        const double bt = (pi == ni && pj == nj) ? D[pk * Nq + nk] : 0.0;
        if (br == 0.0 && bs == 0.0 && bt == 0.0) continue;
        const double dx = vg[RX * Np + p] * br + vg[SX * Np + p] * bs + vg[TX * Np + p] * bt;
        const double dy = vg[RY * Np + p] * br + vg[SY * Np + p] * bs + vg[TY * Np + p] * bt;
        const double dz = vg[RZ * Np + p] * br + vg[SZ * Np + p] * bs + vg[TZ * Np + p] * bt;
        A += vg[JW * Np + p] * (dx * dx + dy * dy + dz * dz);
      }
      /* face terms where n itself is the face node */
      for (int f = 0; f < 6; ++f) {
        int b = -1;
        for (int c = 0; c < Nfp; ++c)
          if (m->faceNodes[f * Nfp + c] == n) { b = c; break; }
        if (b < 0) continue;
        const double *sg = el->sgeo + ((e * 6 + f) * Nfp + b) * NSGEO;
        const double dx = vg[RX * Np + n] * D[ni * Nq + ni] + vg[SX * Np + n] * D[nj * Nq + nj] + vg[TX * Np + n] * D[nk * Nq + nk];
        const double dy = vg[RY * Np + n] * D[ni * Nq + ni] + vg[SY * Np + n] * D[nj * Nq + nj] + vg[TY * Np + n] * D[nk * Nq + nk];
        const double dz = vg[RZ * Np + n] * D[ni * Nq + ni] + vg[SZ * Np + n] * D[nj * Nq + nj] + vg[TZ * Np + n] * D[nk * Nq + nk];
        const double ndg = sg[NXs] * dx + sg[NYs] * dy + sg[NZs] * dz;
        const int bc = m->EToB[e * 6 + f];
        const int bcD = (bc == 1), bcN = (bc > 0 && bc != 1);
        const double c = 0.5 * (1 + bcD) * (1 - bcN) * sg[WSJ];
        A += -c * ndg - c * ndg + c * el->tau * sg[IH];
      }
      diag[e * Np + n] = A;
    }
  }
}

/* ---------------------------------------------------------------- assembled matrix
 * BuildOperatorMatrixIpdgHex3D (ellipticBuildOperatorMatrixIpdg.cpp:1316-1570): for every
 * element pair (e, e) and (e, face neighbour), the bilinear form of the operator above on
 * the Lagrange basis, entries with |a| <= 1e-8 dropped; rows and columns are local nodes. */
static void basis_grad(const orc_mesh *m, int mm, int p, double *br, double *bs, double *bt) {
  const int Nq = m->Nq;
  const int mi = mm % Nq, mj = (mm / Nq) % Nq, mk = mm / (Nq * Nq);
  const int pi = p % Nq, pj = (p / Nq) % Nq, pk = p / (Nq * Nq);
  *br = (pj == mj && pk == mk) ? m->D[pi * Nq + mi] : 0.0;
  *bs = (pi == mi && pk == mk) ? m->D[pj * Nq + mj] : 0.0;
  *bt = (pi == mi && pj == mj) ? m->D[pk * Nq + mk] : 0.0;
}

/* physical gradient of basis function mm at node p of the element whose vgeo is vg */
static void phys_grad(const orc_mesh *m, const double *vg, int mm, int p, double *g) {
  const int Np = m->Np;
  double br, bs, bt;
  basis_grad(m, mm, p, &br, &bs, &bt);
  g[0] = vg[RX * Np + p] * br + vg[SX * Np + p] * bs + vg[TX * Np + p] * bt;
  g[1] = vg[RY * Np + p] * br + vg[SY * Np + p] * bs + vg[TY * Np + p] * bt;
  g[2] = vg[RZ * Np + p] * br + vg[SZ * Np + p] * bs + vg[TZ * Np + p] * bt;
}

hlong orc_ipdg_matrix(const orc_elliptic *el, hlong **rows, hlong **cols, double **vals) {
  const orc_mesh *m = el->mesh;
  const int Np = m->Np, Nfp = m->Nfp;
  const hlong E = m->Nelements;
  const hlong cap = E * Np * Np * 7;
  hlong *R = (hlong *)malloc(sizeof(hlong) * cap), *C = (hlong *)malloc(sizeof(hlong) * cap);
  double *V = (double *)malloc(sizeof(double) * cap);
  hlong nnz = 0;
  const double tol = 1e-8;
  for (hlong e = 0; e < E; ++e) {
    const double *vg = el->vgeo + e * NVGEO * Np;
    const double lam = elam(el, e);
    for (int n = 0; n < Np; ++n)
      for (int mm = 0; mm < Np; ++mm) {
        double Anm = 0;
        for (int p = 0; p < Np; ++p) {
          double gn[3], gm[3];
          phys_grad(m, vg, n, p, gn);
          phys_grad(m, vg, mm, p, gm);
          Anm += vg[JW * Np + p] * (gn[0] * gm[0] + gn[1] * gm[1] + gn[2] * gm[2]);
          if (n == p && mm == p) Anm += lam * vg[JW * Np + p];
        }
        for (int f = 0; f < 6; ++f) {
          double AnmP = 0;
          const hlong eN = m->EToE[e * 6 + f];
          for (int b = 0; b < Nfp; ++b) {
            const hlong id = (e * 6 + f) * Nfp + b;
            const int vidM = m->faceNodes[f * Nfp + b];
            const hlong vP = m->vmapP[id];
            const int vidP = (int)(vP % Np);
            const double *vgP = el->vgeo + (vP / Np) * NVGEO * Np;
            const double *sg = el->sgeo + id * NSGEO;
            const double w = sg[WSJ], pen = el->tau * sg[IH];
            double gnM[3], gmM[3], gmP[3];
            phys_grad(m, vg, n, vidM, gnM);
            phys_grad(m, vg, mm, vidM, gmM);
            phys_grad(m, vgP, mm, vidP, gmP);
            const double ndnM = sg[NXs] * gnM[0] + sg[NYs] * gnM[1] + sg[NZs] * gnM[2];
            const double ndmM = sg[NXs] * gmM[0] + sg[NYs] * gmM[1] + sg[NZs] * gmM[2];
            const double ndmP = sg[NXs] * gmP[0] + sg[NYs] * gmP[1] + sg[NZs] * gmP[2];
            const double lnM = (n == vidM), lmM = (mm == vidM), lmP = (mm == vidP);
            Anm += -0.5 * w * lnM * ndmM - 0.5 * w * ndnM * lmM + 0.5 * w * pen * lnM * lmM;
            if (eN < 0) {
              const int bc = m->EToB[e * 6 + f];
              const double qSgn = (bc == 1) ? -1.0 : 1.0, gSgn = (bc == 1) ? 1.0 : -1.0;
              Anm += -0.5 * gSgn * w * lnM * ndmM + 0.5 * qSgn * w * ndnM * lmM - 0.5 * qSgn * w * pen * lnM * lmM;
            } else {
              AnmP += -0.5 * w * lnM * ndmP + 0.5 * w * ndnM * lmP - 0.5 * w * pen * lnM * lmP;
            }
          }
          if (fabs(AnmP) > tol) { R[nnz] = e * Np + n; C[nnz] = eN * Np + mm; V[nnz] = AnmP; ++nnz; }
        }
        if (fabs(Anm) > tol) { R[nnz] = e * Np + n; C[nnz] = e * Np + mm; V[nnz] = Anm; ++nnz; }
      }
  }
  *rows = R; *cols = C; *vals = V;
  return nnz;
}

/* unit outward normal and WsJ = sJ w_a w_b at face node b of face f of element e, from the
 * physical nodes (meshSurfaceGeometricFactorsHex3D.cpp:31-150); shared by the C0 Neumann
 * boundary terms */
void orc_face_geometry(const orc_mesh *m, hlong e, int f, int b, double *nrm, double *wsJ) {
  const int Nq = m->Nq, Np = m->Np;
  const int n = m->faceNodes[f * m->Nfp + b];
  const int i = n % Nq, j = (n / Nq) % Nq, k = n / (Nq * Nq);
  const double *x = m->x + e * Np, *y = m->y + e * Np, *z = m->z + e * Np, *D = m->D;
  double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
  for (int q = 0; q < Nq; ++q) {
    const int ir = q + j * Nq + k * Nq * Nq, is = i + q * Nq + k * Nq * Nq, it = i + j * Nq + q * Nq * Nq;
    xr += D[i * Nq + q] * x[ir]; yr += D[i * Nq + q] * y[ir]; zr += D[i * Nq + q] * z[ir];
    xs += D[j * Nq + q] * x[is]; ys += D[j * Nq + q] * y[is]; zs += D[j * Nq + q] * z[is];
    xt += D[k * Nq + q] * x[it]; yt += D[k * Nq + q] * y[it]; zt += D[k * Nq + q] * z[it];
  }
  const double J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
  double g[9] = {(ys * zt - zs * yt) / J,  -(xs * zt - zs * xt) / J, (xs * yt - ys * xt) / J,
                 -(yr * zt - zr * yt) / J, (xr * zt - zr * xt) / J,  -(xr * yt - yr * xt) / J,
                 (yr * zs - zr * ys) / J,  -(xr * zs - zr * xs) / J, (xr * ys - yr * xs) / J};
  const int c0 = (f == 0 || f == 5) ? 6 : (f == 1 || f == 3) ? 3 : 0;
  const double sg = (f == 0 || f == 1 || f == 4) ? -1.0 : 1.0;
  const double nx = sg * g[c0], ny = sg * g[c0 + 1], nz = sg * g[c0 + 2];
  const double len = sqrt(nx * nx + ny * ny + nz * nz);
  nrm[0] = nx / len; nrm[1] = ny / len; nrm[2] = nz / len;
  *wsJ = len * J * m->gllw[b % Nq] * m->gllw[b / Nq];
}
