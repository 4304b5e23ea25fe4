// mesh_t / elliptic_t for structured hexahedral boxes.
//
// Host work is limited to what is O(elements): vertex coordinates (with optional
// interior jitter), per-element dof offsets of the box numbering, the lambda field
// and RHS source parameters. Node-level setup (geometric factors, GlobalToLocal,
// owner copies, multiplicities) runs on the GPU.
//
// Reference counterparts: meshSetupBoxHex3D.cpp:31-232, meshReferenceNodesHex3D.cpp:31-74,
// meshGeometricFactorsHex3D.cpp:31-193, meshConnectNodes.cpp:32-117,
// ellipticBoundarySetup.cpp:30-140, ellipticOperator.cpp:29-106,
// ellipticBuildOperatorDiagonal.cpp:998-1057, ellipticRun.cpp:139-185,
// ellipticBuildOperatorMatrixContinuous.cpp:697-880.
#include "objects.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unistd.h>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace lpg {

// ---------------------------------------------------------------- mesh
int Mesh::setup(const MeshConfig& c, int N_, cudaStream_t s) {
  cfg = c;
  N = N_;
  Nq = N + 1;
  Np = Nq * Nq * Nq;
  if (N < 1 || N > 8) return set_error(LPG_ERR_UNSUPPORTED, "POLYNOMIAL DEGREE must be 1..8");
  if (c.is_box() && (c.nx < 1 || c.ny < 1 || c.nz < 1)) return set_error(LPG_ERR_INVALID, "BOX NX/NY/NZ must be >= 1");
  E = c.is_box() ? (int64_t)c.nx * c.ny * c.nz : c.file->E;
  if (E * Np >= (int64_t)INT32_MAX) return set_error(LPG_ERR_UNSUPPORTED, "more than 2^31 local nodes");
  gll_nodes_weights(N, r1d, w1d);
  gll_derivative(N, r1d, D);
  std::vector<double> ex(E * 8), ey(E * 8), ez(E * 8);
  if (!c.is_box()) {
    // vertex coordinates of the file's hexahedra (meshReadGmshHex3D.cpp:160-170)
    const HexMeshData& f = *c.file;
#pragma omp parallel for
    for (int64_t i = 0; i < E * 8; ++i) {
      const int64_t v = f.EToV[i];
      ex[i] = f.VX[v]; ey[i] = f.VY[v]; ez[i] = f.VZ[v];
    }
  } else {
  // vertex coordinates per element (meshSetupBoxHex3D.cpp:112-152) + interior jitter
  const bool periodic = (c.bcflag == -1);
  const double dx = c.dimx / c.nx, dy = c.dimy / c.ny, dz = c.dimz / c.nz;
  const double X0 = -c.dimx / 2.0, Y0 = -c.dimy / 2.0, Z0 = -c.dimz / 2.0;
  const int64_t NnX = periodic ? c.nx : c.nx + 1, NnY = periodic ? c.ny : c.ny + 1;
  static const int ox[8] = {0, 1, 1, 0, 0, 1, 1, 0}, oy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, oz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
#pragma omp parallel for
  for (int64_t e = 0; e < E; ++e) {
    const int i = (int)(e % c.nx), j = (int)((e / c.nx) % c.ny), k = (int)(e / ((int64_t)c.nx * c.ny));
    for (int v = 0; v < 8; ++v) {
      const int vi = i + ox[v], vj = j + oy[v], vk = k + oz[v];
      double x = X0 + dx * i + (ox[v] ? dx : 0.0);
      double y = Y0 + dy * j + (oy[v] ? dy : 0.0);
      double z = Z0 + dz * k + (oz[v] ? dz : 0.0);
      if (c.jitter != 0.0 && !periodic && vi > 0 && vi < c.nx && vj > 0 && vj < c.ny && vk > 0 && vk < c.nz) {
        const uint64_t vid = (uint64_t)(vi + vj * NnX + (int64_t)vk * NnX * NnY);
        x += (2.0 * hash_u01(c.jitterSeed, 0, vid) - 1.0) * c.jitter * dx;
        y += (2.0 * hash_u01(c.jitterSeed, 1, vid) - 1.0) * c.jitter * dy;
        z += (2.0 * hash_u01(c.jitterSeed, 2, vid) - 1.0) * c.jitter * dz;
      }
      ex[e * 8 + v] = x;
      ey[e * 8 + v] = y;
      ez[e * 8 + v] = z;
    }
  }
  }
  return setup_vertices(ex, ey, ez, s);
}

// device vertex arrays, reference-element data and geometric factors of E elements
int Mesh::setup_vertices(const std::vector<double>& ex, const std::vector<double>& ey, const std::vector<double>& ez,
                         cudaStream_t s) {
  int rc;
  if ((rc = EX.alloc(E * 8)) || (rc = EY.alloc(E * 8)) || (rc = EZ.alloc(E * 8))) return rc;
  if ((rc = EX.upload(ex.data(), E * 8, s)) || (rc = EY.upload(ey.data(), E * 8, s)) ||
      (rc = EZ.upload(ez.data(), E * 8, s)))
    return rc;
  if ((rc = D_d.alloc(Nq * Nq)) || (rc = r1d_d.alloc(Nq)) || (rc = w1d_d.alloc(Nq))) return rc;
  if ((rc = D_d.upload(D.data(), Nq * Nq, s)) || (rc = r1d_d.upload(r1d.data(), Nq, s)) ||
      (rc = w1d_d.upload(w1d.data(), Nq, s)))
    return rc;
  if ((rc = geo.alloc(E * 7 * Np))) return rc;
  DevBuf<int> bad;
  if ((rc = bad.alloc(1))) return rc;
  LPG_CUDA_TRY(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  if ((rc = geometric_factors(N, E, EX.p, EY.p, EZ.p, D_d.p, r1d_d.p, w1d_d.p, geo.p, bad.p, s))) return rc;
  int nbad = 0;
  if ((rc = bad.download(&nbad, 1, s))) return rc;
  if (nbad) return set_error(LPG_ERR_INVALID, "negative or tiny Jacobian at " + std::to_string(nbad) + " nodes");
  return LPG_OK;
}

int Mesh::make_f32(cudaStream_t s) {
  if (geo32.p) return LPG_OK;
  int rc;
  if ((rc = geo32.alloc(E * 7 * Np)) || (rc = D32.alloc(Nq * Nq))) return rc;
  if ((rc = convert<double, float>(E * 7 * Np, geo.p, geo32.p, s))) return rc;
  return convert<double, float>(Nq * Nq, D_d.p, D32.p, s);
}

int Mesh::make_dw(cudaStream_t s) {
  if (geoDW.p) return LPG_OK;
  int rc;
  if ((rc = geoDW.alloc(E * 7 * Np))) return rc;
  return split_to_float2(E * 7 * Np, geo.p, geoDW.p, s);
}

int Mesh::make_bf16(cudaStream_t s) {
  if (geo16.p) return LPG_OK;
  int rc;
  if ((rc = geo16.alloc(E * 7 * Np))) return rc;
  if ((rc = convert<double, __nv_bfloat16>(E * 7 * Np, geo.p, geo16.p, s))) return rc;
  if (!D32.p) {
    if ((rc = D32.alloc(Nq * Nq))) return rc;
    return convert<double, float>(Nq * Nq, D_d.p, D32.p, s);
  }
  return LPG_OK;
}

// ---------------------------------------------------------------- elliptic
int Elliptic::setup(Platform* p, const MeshConfig& c, int N, double lam, const std::vector<double>* lamE,
                    cudaStream_t s) {
  plat = p;
  lambda = lam;
  if (c.ipdg) return setup_ipdg(c, N, lamE, s);
  if (!c.is_box()) return setup_file(c, N, lamE, s);
  if (c.bcflag != 1 && c.bcflag != -1 && c.bcflag != 2)
    return set_error(LPG_ERR_UNSUPPORTED, "BOX BOUNDARY FLAG must be 1 (Dirichlet), 2 (Neumann) or -1 (periodic)");
  if (c.bcflag == -1 && (c.nx < 2 || c.ny < 2 || c.nz < 2))
    return set_error(LPG_ERR_UNSUPPORTED, "periodic boxes need at least 2 elements per direction");
  int rc = mesh.setup(c, N, s);
  if (rc) return rc;
  const int64_t E = mesh.E, Np = mesh.Np;
  Nlocal = E * Np;

  // per-element dof offsets of the box numbering (owned box of nodes per element)
  const bool periodic = (c.bcflag == -1), dirichlet = (c.bcflag == 1);
  auto range = [&](int e, int n, int& lo, int& hi) {
    if (periodic) { lo = (e == 0) ? 0 : 1; hi = (e == n - 1) ? N - 1 : N; }
    else if (dirichlet) { lo = 1; hi = (e == n - 1) ? N - 1 : N; }
    else { lo = (e == 0) ? 0 : 1; hi = N; }
  };
  std::vector<int64_t> base(E + 1, 0);
  for (int64_t e = 0; e < E; ++e) {
    const int i = (int)(e % c.nx), j = (int)((e / c.nx) % c.ny), k = (int)(e / ((int64_t)c.nx * c.ny));
    int lx, hx, ly, hy, lz, hz;
    range(i, c.nx, lx, hx);
    range(j, c.ny, ly, hy);
    range(k, c.nz, lz, hz);
    const int64_t cnt = (int64_t)std::max(0, hx - lx + 1) * std::max(0, hy - ly + 1) * std::max(0, hz - lz + 1);
    base[e + 1] = base[e] + cnt;
  }
  Nglobal = base[E];
  if (Nglobal <= 0) return set_error(LPG_ERR_INVALID, "no unknowns after masking");
  DevBuf<int64_t> base_d;
  DevBuf<int32_t> mult;
  if ((rc = base_d.alloc(E + 1)) || (rc = base_d.upload(base.data(), E + 1, s))) return rc;
  if ((rc = g2l.alloc(Nlocal)) || (rc = owner.alloc(Nglobal)) || (rc = mult.alloc(Nglobal)) ||
      (rc = weightG.alloc(Nglobal)))
    return rc;
  BoxNumbering b{c.nx, c.ny, c.nz, N, periodic ? 1 : 0, dirichlet ? 1 : 0};
  if ((rc = box_numbering(b, base_d.p, g2l.p, owner.p, mult.p, Nglobal, s))) return rc;
  if ((rc = multiplicity_to_weight(Nglobal, mult.p, weightG.p, s))) return rc;

  hasDirichlet = dirichlet;
  if (c.bcflag == 2) {
    // every boundary face node of a Neumann box carries the Neumann data
    const int Nq = N + 1;
    std::vector<int32_t> node, mask;
    for (int64_t e = 0; e < E; ++e) {
      const int i = (int)(e % c.nx), j = (int)((e / c.nx) % c.ny), k = (int)(e / ((int64_t)c.nx * c.ny));
      const int fm = (k == 0 ? 1 : 0) | (j == 0 ? 2 : 0) | (i == c.nx - 1 ? 4 : 0) | (j == c.ny - 1 ? 8 : 0) |
                     (i == 0 ? 16 : 0) | (k == c.nz - 1 ? 32 : 0);
      if (!fm) continue;
      for (int n = 0; n < Np; ++n) {
        const int a = n % Nq, b = (n / Nq) % Nq, d = n / (Nq * Nq);
        const int on = (d == 0 ? 1 : 0) | (b == 0 ? 2 : 0) | (a == N ? 4 : 0) | (b == N ? 8 : 0) | (a == 0 ? 16 : 0) |
                       (d == N ? 32 : 0);
        if (on & fm) { node.push_back((int32_t)(e * Np + n)); mask.push_back(on & fm); }
      }
    }
    if ((rc = set_neumann_nodes(node, mask, s))) return rc;
  }
  return finish_setup(lamE, s);
}

int Elliptic::set_neumann_nodes(const std::vector<int32_t>& node, const std::vector<int32_t>& mask, cudaStream_t s) {
  neuCount = (int64_t)node.size();
  if (!neuCount) return LPG_OK;
  int rc;
  if ((rc = neuNode.alloc(neuCount)) || (rc = neuMask.alloc(neuCount)) ||
      (rc = neuNode.upload(node.data(), neuCount, s)) || (rc = neuMask.upload(mask.data(), neuCount, s)))
    return rc;
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  return LPG_OK;
}

// numbering of a file mesh on the host (union-find over connected face nodes), uploaded
// Element traversal order of the operators on a file mesh whose element order carries no
// locality: Morton (Z-order) keys of the element centroids, quantised to 21 bits per axis
// over the vertices' bounding box. In such a file order concurrently running CTAs gather
// and assemble dofs far apart; in Morton order neighbours run close together and share
// their face dofs through L2 (64^3, N=7, random element order: FP32 operator 1.25 ->
// 1.16 ms, double-word 3.20 -> 3.10 ms; the same mesh in lattice order runs 1.01 ms, and
// Morton order would slow it to 1.14 ms, so files in a local order keep it).
int Elliptic::morton_element_order(const HexMeshData& hm, cudaStream_t s) {
  const int64_t E = hm.E;
  if (E <= 1 || E > INT32_MAX) return LPG_OK;
  // keep the file's order when it already keeps neighbours together (the median distance
  // between consecutive element centroids within twice the median element diagonal): the
  // dofs are numbered by owner element, so that order also matches the dof layout
  {
    std::vector<double> step((size_t)(E - 1)), diag((size_t)E);
    auto centroid = [&](int64_t e, double* c) {
      c[0] = c[1] = c[2] = 0;
      for (int v = 0; v < 8; ++v) {
        const int64_t n = hm.EToV[e * 8 + v];
        c[0] += hm.VX[n] / 8; c[1] += hm.VY[n] / 8; c[2] += hm.VZ[n] / 8;
      }
    };
#pragma omp parallel for
    for (int64_t e = 0; e < E; ++e) {
      const int64_t a = hm.EToV[e * 8 + 0], b = hm.EToV[e * 8 + 6];
      diag[(size_t)e] = std::sqrt((hm.VX[a] - hm.VX[b]) * (hm.VX[a] - hm.VX[b]) +
                                  (hm.VY[a] - hm.VY[b]) * (hm.VY[a] - hm.VY[b]) +
                                  (hm.VZ[a] - hm.VZ[b]) * (hm.VZ[a] - hm.VZ[b]));
      if (e + 1 < E) {
        double c0[3], c1[3];
        centroid(e, c0);
        centroid(e + 1, c1);
        step[(size_t)e] = std::sqrt((c1[0] - c0[0]) * (c1[0] - c0[0]) + (c1[1] - c0[1]) * (c1[1] - c0[1]) +
                                    (c1[2] - c0[2]) * (c1[2] - c0[2]));
      }
    }
    std::nth_element(step.begin(), step.begin() + step.size() / 2, step.end());
    std::nth_element(diag.begin(), diag.begin() + diag.size() / 2, diag.end());
    if (step[step.size() / 2] <= 2.0 * diag[diag.size() / 2]) return LPG_OK;
  }
  auto spread = [](uint64_t v) {   // 21 bits -> every third bit of 63
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x1F00000000FFFFull;
    v = (v | (v << 16)) & 0x1F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
  };
  double span[3];
  for (int d = 0; d < 3; ++d) span[d] = (hm.hi[d] > hm.lo[d]) ? hm.hi[d] - hm.lo[d] : 1.0;
  std::vector<std::pair<uint64_t, int32_t>> key((size_t)E);
#pragma omp parallel for
  for (int64_t e = 0; e < E; ++e) {
    double c[3] = {0, 0, 0};
    for (int v = 0; v < 8; ++v) {
      const int64_t n = hm.EToV[e * 8 + v];
      c[0] += hm.VX[n]; c[1] += hm.VY[n]; c[2] += hm.VZ[n];
    }
    const double lo[3] = {hm.lo[0], hm.lo[1], hm.lo[2]};
    uint64_t q[3];
    for (int d = 0; d < 3; ++d) {
      const double t = (c[d] / 8.0 - lo[d]) / span[d];
      q[d] = (uint64_t)std::min(2097151.0, std::max(0.0, t * 2097152.0));
    }
    key[(size_t)e] = {spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2), (int32_t)e};
  }
  std::sort(key.begin(), key.end());
  std::vector<int32_t> order((size_t)E);
  for (int64_t e = 0; e < E; ++e) order[(size_t)e] = key[(size_t)e].second;
  int rc;
  if ((rc = elemOrder.alloc(E)) || (rc = elemOrder.upload(order.data(), E, s))) return rc;
  return LPG_OK;
}

int Elliptic::setup_file(const MeshConfig& c, int N, const std::vector<double>* lamE, cudaStream_t s) {
  int rc = mesh.setup(c, N, s);
  if (rc) return rc;
  Nlocal = mesh.E * mesh.Np;
  HexNumbering num;
  if ((rc = number_hex_nodes(*c.file, N, mesh.r1d, num))) return rc;
  Nglobal = num.Nglobal;
  if (Nglobal <= 0) return set_error(LPG_ERR_INVALID, "no unknowns after masking");
  DevBuf<int32_t> mult;
  if ((rc = g2l.alloc(Nlocal)) || (rc = owner.alloc(Nglobal)) || (rc = mult.alloc(Nglobal)) ||
      (rc = weightG.alloc(Nglobal)))
    return rc;
  if ((rc = g2l.upload(num.g2l.data(), Nlocal, s)) || (rc = owner.upload(num.owner.data(), Nglobal, s)) ||
      (rc = mult.upload(num.mult.data(), Nglobal, s)))
    return rc;
  if ((rc = multiplicity_to_weight(Nglobal, mult.p, weightG.p, s))) return rc;
  hasDirichlet = num.hasDirichlet;
  if ((rc = morton_element_order(*c.file, s))) return rc;
  {
    // boundary face nodes whose node flag is a Neumann type (tag >= 2)
    const HexMeshData& hm = *c.file;
    const int Np = mesh.Np, Nq = N + 1;
    std::vector<int32_t> node, mask;
    for (int64_t e = 0; e < mesh.E; ++e) {
      int fm = 0;
      for (int f = 0; f < 6; ++f)
        if (hm.EToE[e * 6 + f] < 0) fm |= 1 << f;
      if (!fm) continue;
      for (int n = 0; n < Np; ++n) {
        if (num.flag[e * Np + n] < 2) continue;
        const int a = n % Nq, b = (n / Nq) % Nq, d = n / (Nq * Nq);
        const int on = (d == 0 ? 1 : 0) | (b == 0 ? 2 : 0) | (a == N ? 4 : 0) | (b == N ? 8 : 0) | (a == 0 ? 16 : 0) |
                       (d == N ? 32 : 0);
        if (on & fm) { node.push_back((int32_t)(e * Np + n)); mask.push_back(on & fm); }
      }
    }
    if ((rc = set_neumann_nodes(node, mask, s))) return rc;
  }
  return finish_setup(lamE, s);
}

// SEMFEM low-order problem (mesh_t::SetupSEMFEM meshSetupSEMFEM.cpp:98-214 and
// SEMFEMPrecon ellipticPreconSEMFEM.cpp:56-200, hexahedra): each degree-N element of `sem`
// is cut into N^3 trilinear hexahedra with vertices at its GLL nodes; the degree-1 nodes
// keep the assembled dof of the GLL node they sit on, so the FEM matrix acts on sem's
// vectors. Only what BuildMatrix needs is set up (geometry, GlobalToLocal, lambda).
int Elliptic::setup_semfem(const Elliptic& sem, cudaStream_t s) {
  plat = sem.plat;
  lambda = sem.lambda;
  const int Ns = sem.mesh.N, Nq = Ns + 1, NpS = sem.mesh.Np;
  const int64_t Esem = sem.mesh.E, Es = Esem * Ns * Ns * Ns;
  mesh.cfg = sem.mesh.cfg;
  mesh.N = 1; mesh.Nq = 2; mesh.Np = 8; mesh.E = Es;
  if (Es * 8 >= (int64_t)INT32_MAX) return set_error(LPG_ERR_UNSUPPORTED, "SEMFEM: more than 2^31 local nodes");
  gll_nodes_weights(1, mesh.r1d, mesh.w1d);
  gll_derivative(1, mesh.r1d, mesh.D);
  std::vector<double> vx(Esem * 8), vy(Esem * 8), vz(Esem * 8);
  std::vector<int32_t> semMap(Esem * NpS);
  int rc;
  if ((rc = sem.mesh.EX.download(vx.data(), Esem * 8, s)) || (rc = sem.mesh.EY.download(vy.data(), Esem * 8, s)) ||
      (rc = sem.mesh.EZ.download(vz.data(), Esem * 8, s)) || (rc = sem.g2l.download(semMap.data(), Esem * NpS, s)))
    return rc;
  static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  const std::vector<double>& r = sem.mesh.r1d;
  std::vector<double> ex(Es * 8), ey(Es * 8), ez(Es * 8);
  std::vector<int32_t> map(Es * 8);
  if (sem.hasLambdaE) lambdaE_h.resize(Es);
#pragma omp parallel for
  for (int64_t e = 0; e < Esem; ++e) {
    const double* X = &vx[e * 8];
    const double* Y = &vy[e * 8];
    const double* Z = &vz[e * 8];
    for (int k = 0; k < Ns; ++k)
      for (int j = 0; j < Ns; ++j)
        for (int i = 0; i < Ns; ++i) {
          const int64_t es = ((e * Ns + k) * Ns + j) * Ns + i;
          for (int v = 0; v < 8; ++v) {
            const int a = i + cx[v], b = j + cy[v], c = k + cz[v];
            // GLL node (a,b,c): trilinear image of the element's vertices (meshPhysicalNodesHex3D.cpp)
            const double rr = r[a], ss = r[b], tt = r[c];
            const double w[8] = {(1 - rr) * (1 - ss) * (1 - tt), (1 + rr) * (1 - ss) * (1 - tt),
                                 (1 + rr) * (1 + ss) * (1 - tt), (1 - rr) * (1 + ss) * (1 - tt),
                                 (1 - rr) * (1 - ss) * (1 + tt), (1 + rr) * (1 - ss) * (1 + tt),
                                 (1 + rr) * (1 + ss) * (1 + tt), (1 - rr) * (1 + ss) * (1 + tt)};
            double x = 0, y = 0, z = 0;
            for (int q = 0; q < 8; ++q) { x += 0.125 * w[q] * X[q]; y += 0.125 * w[q] * Y[q]; z += 0.125 * w[q] * Z[q]; }
            ex[es * 8 + v] = x; ey[es * 8 + v] = y; ez[es * 8 + v] = z;
            // degree-1 node cx + 2 cy + 4 cz (tensor order) <- GLL node (a,b,c)
            map[es * 8 + cx[v] + 2 * cy[v] + 4 * cz[v]] = semMap[e * NpS + a + b * Nq + c * Nq * Nq];
          }
          if (sem.hasLambdaE) lambdaE_h[es] = sem.lambdaE_h[e];
        }
  }
  if ((rc = mesh.setup_vertices(ex, ey, ez, s))) return rc;
  Nlocal = Es * 8;
  Nglobal = sem.Nglobal;
  if ((rc = g2l.alloc(Nlocal)) || (rc = g2l.upload(map.data(), Nlocal, s))) return rc;
  hasLambdaE = sem.hasLambdaE;
  hasDirichlet = sem.hasDirichlet;
  allNeumann = sem.allNeumann;
  allNeumannScale = sem.allNeumannScale;
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  return LPG_OK;
}

// IPDG (ellipticSetup.cpp:66-81, ellipticBoundarySetup.cpp:89-93): every local node is an
// unknown; trace maps from the mesh connectivity (box or file), geometric factors on the GPU.
int Elliptic::setup_ipdg(const MeshConfig& c, int N, const std::vector<double>* lamE, cudaStream_t s) {
  ipdg = true;
  if (c.is_box() && c.bcflag != 1 && c.bcflag != -1 && c.bcflag != 2)
    return set_error(LPG_ERR_UNSUPPORTED, "BOX BOUNDARY FLAG must be 1 (Dirichlet), 2 (Neumann) or -1 (periodic)");
  if (c.is_box() && c.bcflag == -1 && (c.nx < 2 || c.ny < 2 || c.nz < 2))
    return set_error(LPG_ERR_UNSUPPORTED, "periodic boxes need at least 2 elements per direction");
  int rc = mesh.setup(c, N, s);
  if (rc) return rc;
  const int Nq = N + 1, Np = mesh.Np, Nfp = Nq * Nq;
  const int64_t E = mesh.E;
  Nlocal = E * Np;
  Nglobal = Nlocal;
  HexMeshData boxMesh;
  const HexMeshData* hm = c.file.get();
  if (!hm) {
    boxMesh = box_hex_mesh(c.nx, c.ny, c.nz, c.bcflag);
    hm = &boxMesh;
  }
  std::vector<int32_t> vP, mP;
  if ((rc = hex_traces(*hm, N, mesh.r1d, vP, mP))) return rc;
  hasDirichlet = false;
  for (int b : hm->EToB) hasDirichlet = hasDirichlet || (b == 1);
  EToE_h = hm->EToE;
  std::vector<int32_t> iota(Nlocal);
  for (int64_t n = 0; n < Nlocal; ++n) iota[n] = (int32_t)n;
  DevBuf<int32_t> mapP;
  DevBuf<double> hfac;
  if ((rc = g2l.alloc(Nlocal)) || (rc = owner.alloc(Nlocal)) || (rc = weightG.alloc(Nlocal)) ||
      (rc = vgeo.alloc(E * 10 * Np)) || (rc = sgeo.alloc(E * 5 * 6 * Nfp)) || (rc = g4.alloc(4 * Nlocal)) ||
      (rc = vmapP.alloc(E * 6 * Nfp)) || (rc = mapP.alloc(E * 6 * Nfp)) || (rc = EToB.alloc(E * 6)) ||
      (rc = hfac.alloc(E * 6 * Nfp)))
    return rc;
  if ((rc = g2l.upload(iota.data(), Nlocal, s)) || (rc = owner.upload(iota.data(), Nlocal, s)) ||
      (rc = vmapP.upload(vP.data(), E * 6 * Nfp, s)) || (rc = mapP.upload(mP.data(), E * 6 * Nfp, s)) ||
      (rc = EToB.upload(hm->EToB.data(), E * 6, s)) || (rc = fill<double>(Nlocal, 1.0, weightG.p, s)))
    return rc;
  tau = 2.0 * (N + 1) * (N + 3);
  IpdgArgs a = ipdg_args();
  a.hfac = hfac.p;
  if ((rc = ipdg_geometry(a, mapP.p, s))) return rc;
  if ((rc = finish_setup(lamE, s))) return rc;   // synchronises before the host vectors go
  return LPG_OK;
}

IpdgArgs Elliptic::ipdg_args() const {
  IpdgArgs a;
  a.N = mesh.N;
  a.E = mesh.E;
  a.EX = mesh.EX.p; a.EY = mesh.EY.p; a.EZ = mesh.EZ.p;
  a.D = mesh.D_d.p; a.r1d = mesh.r1d_d.p; a.w1d = mesh.w1d_d.p;
  a.vgeo = vgeo.p; a.sgeo = sgeo.p;
  a.vmapP = vmapP.p; a.EToB = EToB.p;
  a.lambda = lambda; a.tau = tau;
  a.lambdaE = hasLambdaE ? lambdaE.p : nullptr;
  a.g4 = reinterpret_cast<double4_32a*>(g4.p);
  return a;
}

int Elliptic::finish_setup(const std::vector<double>* lamE, cudaStream_t s) {
  int rc;
  const int64_t E = mesh.E;
  hasLambdaE = (lamE != nullptr);
  allNeumann = (lambda == 0.0 && !hasLambdaE && !hasDirichlet);
  allNeumannScale = 1.0 / std::sqrt((double)Nglobal);
  if (hasLambdaE) {
    lambdaE_h = *lamE;
    std::vector<float> l32(lambdaE_h.begin(), lambdaE_h.end());
    if ((rc = lambdaE.alloc(E)) || (rc = lambdaE.upload(lambdaE_h.data(), E, s))) return rc;
    if ((rc = lambdaE32.alloc(E)) || (rc = lambdaE32.upload(l32.data(), E, s))) return rc;
  }
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  return LPG_OK;
}

int Elliptic::make_f32(bool bf16, cudaStream_t s) {
  int rc;
  if (ipdg) {
    // FP32 copies of the IPDG volume and surface factors (the C0 geometric factors are not used)
    if (bf16) return set_error(LPG_ERR_UNSUPPORTED, "BF16 geometry is defined for CONTINUOUS only");
    const int64_t E = mesh.E, Np = mesh.Np, Nfp = (int64_t)mesh.Nq * mesh.Nq;
    if (!vgeo32.p) {
      if ((rc = vgeo32.alloc(E * 10 * Np)) || (rc = sgeo32.alloc(E * 5 * 6 * Nfp)) || (rc = g4_32.alloc(4 * Nlocal)))
        return rc;
      if ((rc = convert<double, float>(E * 10 * Np, vgeo.p, vgeo32.p, s)) ||
          (rc = convert<double, float>(E * 5 * 6 * Nfp, sgeo.p, sgeo32.p, s)))
        return rc;
    }
    if (!mesh.D32.p) {
      const int Nq = mesh.Nq;
      if ((rc = mesh.D32.alloc(Nq * Nq)) || (rc = convert<double, float>(Nq * Nq, mesh.D_d.p, mesh.D32.p, s))) return rc;
    }
  } else if ((rc = bf16 ? mesh.make_bf16(s) : mesh.make_f32(s))) {
    return rc;
  }
  if (!weightG32.p) {
    if ((rc = weightG32.alloc(Nglobal))) return rc;
    if ((rc = convert<double, float>(Nglobal, weightG.p, weightG32.p, s))) return rc;
  }
  return LPG_OK;
}

int Elliptic::OperatorIpdgDW(const double* q, double* Aq, cudaStream_t s) {
  int rc;
  const int64_t E = mesh.E, Np = mesh.Np, Nfp = (int64_t)mesh.Nq * mesh.Nq;
  if (!vgeoDW.p) {
    if ((rc = vgeoDW.alloc(E * 10 * Np)) || (rc = sgeoDW.alloc(E * 5 * 6 * Nfp)) || (rc = g8.alloc(8 * Nlocal)))
      return rc;
    if ((rc = split_to_float2(E * 10 * Np, vgeo.p, vgeoDW.p, s)) ||
        (rc = split_to_float2(E * 5 * 6 * Nfp, sgeo.p, sgeoDW.p, s)))
      return rc;
  }
  IpdgArgsDW a;
  a.N = mesh.N; a.E = E;
  a.vgeo = vgeoDW.p; a.sgeo = sgeoDW.p; a.D = mesh.D_d.p;
  a.vmapP = vmapP.p; a.EToB = EToB.p;
  a.lambda = lambda; a.tau = tau;
  a.lambdaE = hasLambdaE ? lambdaE.p : nullptr;
  a.q = q; a.out = Aq;
  a.g8 = reinterpret_cast<float4*>(g8.p);
  return ipdg_operator_dw(a, s);
}

int Elliptic::OperatorDW(const double* q, double* Aq, cudaStream_t s) {
  if (ipdg) return OperatorIpdgDW(q, Aq, s);
  int rc;
  if ((rc = mesh.make_dw(s))) return rc;
  AxArgs<double, float2> a;
  const int64_t Np = mesh.Np;
  a.N = mesh.N; a.Nelements = mesh.E; a.elementList = elemOrder.p; a.g2l = g2l.p;
  a.ggeo = mesh.geoDW.p; a.geoStride = 7 * Np; a.wJ = mesh.geoDW.p + 6 * Np; a.wJStride = 7 * Np;
  a.D = mesh.D_d.p; a.lambda = lambda; a.lambdaE = hasLambdaE ? lambdaE.p : nullptr;
  a.q = q; a.out = Aq; a.Nglobal = Nglobal;
  return ax_hex_dw(a, s);
}

int Elliptic::Operator(const double* q, double* Aq, cudaStream_t s) {
  ++nOps;
  if (ipdg && opDW) return OperatorIpdgDW(q, Aq, s);
  if (ipdg) {
    IpdgArgs a = ipdg_args();
    a.q = q;
    a.out = Aq;
    return ipdg_operator(a, s);
  }
  if (opDW) return OperatorDW(q, Aq, s);
  AxArgs<double, double> a;
  const int64_t Np = mesh.Np;
  a.N = mesh.N; a.Nelements = mesh.E; a.elementList = elemOrder.p; a.g2l = g2l.p;
  a.ggeo = mesh.geo.p; a.geoStride = 7 * Np; a.wJ = mesh.geo.p + 6 * Np; a.wJStride = 7 * Np;
  a.D = mesh.D_d.p; a.lambda = lambda; a.lambdaE = hasLambdaE ? lambdaE.p : nullptr;
  a.q = q; a.out = Aq; a.Nglobal = Nglobal;
  return ax_hex<double, double>(a, AxMode::Assemble, s);
}

int Elliptic::OperatorF32(const float* q, float* Aq, Prec prec, cudaStream_t s, float accumulate) {
  ++nOps;
  const int64_t Np = mesh.Np;
  const AxMode mode = accumulate != 0.f ? AxMode::AccumulateAssembled : AxMode::Assemble;
  if (ipdg) {
    if (accumulate != 0.f) return set_error(LPG_ERR_UNSUPPORTED, "IPDG: no accumulating FP32 operator");
    if (prec != Prec::F32 || !vgeo32.p) return set_error(LPG_ERR_UNSUPPORTED, "IPDG: FP32 operator not prepared");
    IpdgArgsF32 a;
    a.N = mesh.N; a.E = mesh.E;
    a.vgeo = vgeo32.p; a.sgeo = sgeo32.p; a.D = mesh.D32.p;
    a.vmapP = vmapP.p; a.EToB = EToB.p;
    a.lambda = (float)lambda; a.tau = (float)tau;
    a.lambdaE = hasLambdaE ? lambdaE32.p : nullptr;
    a.q = q; a.out = Aq;
    a.g4 = reinterpret_cast<float4*>(g4_32.p);
    return ipdg_operator_f32(a, s);
  }
  if (prec == Prec::BF16G) {
    AxArgs<float, __nv_bfloat16> a;
    a.N = mesh.N; a.Nelements = mesh.E; a.elementList = elemOrder.p; a.g2l = g2l.p;
    a.ggeo = mesh.geo16.p; a.geoStride = 7 * Np; a.wJ = mesh.geo16.p + 6 * Np; a.wJStride = 7 * Np;
    a.D = mesh.D32.p; a.lambda = (float)lambda; a.lambdaE = hasLambdaE ? lambdaE32.p : nullptr;
    a.q = q; a.out = Aq; a.Nglobal = Nglobal;
    if (accumulate != 0.f) a.outScale = accumulate;
    return ax_hex<float, __nv_bfloat16>(a, mode, s);
  }
  AxArgs<float, float> a;
  a.N = mesh.N; a.Nelements = mesh.E; a.elementList = elemOrder.p; a.g2l = g2l.p;
  a.ggeo = mesh.geo32.p; a.geoStride = 7 * Np; a.wJ = mesh.geo32.p + 6 * Np; a.wJStride = 7 * Np;
  a.D = mesh.D32.p; a.lambda = (float)lambda; a.lambdaE = hasLambdaE ? lambdaE32.p : nullptr;
  a.q = q; a.out = Aq; a.Nglobal = Nglobal;
  if (accumulate != 0.f) a.outScale = accumulate;
  return ax_hex<float, float>(a, mode, s);
}

// ---------------------------------------------------------------- host-buffer operator
HostPipe::~HostPipe() {
  for (cudaEvent_t ev : inReady) cudaEventDestroy(ev);
  for (cudaEvent_t ev : chunkDone) cudaEventDestroy(ev);
  if (h2d) cudaStreamDestroy(h2d);
  if (d2h) cudaStreamDestroy(d2h);
}

int Elliptic::BuildPipe(cudaStream_t s) {
  if (pipe) return LPG_OK;
  auto p = std::make_unique<HostPipe>();
  const int64_t E = mesh.E;
  // at most 32 chunks of at least 4096 elements (a chunk still fills every SM)
  p->K = (int)std::max<int64_t>(1, std::min<int64_t>(32, E / 4096));
  const int K = p->K;
  std::vector<int32_t> lo(std::max<int64_t>(E, 1)), hi(std::max<int64_t>(E, 1));
  if (E > 0) {
    DevBuf<int32_t> dlo, dhi;
    int rc;
    if ((rc = dlo.alloc(E)) || (rc = dhi.alloc(E))) return rc;
    if ((rc = element_dof_range(mesh.N, E, g2l.p, dlo.p, dhi.p, s))) return rc;
    LPG_CUDA_TRY(cudaMemcpyAsync(lo.data(), dlo.p, sizeof(int32_t) * E, cudaMemcpyDeviceToHost, s));
    LPG_CUDA_TRY(cudaMemcpyAsync(hi.data(), dhi.p, sizeof(int32_t) * E, cudaMemcpyDeviceToHost, s));
    LPG_CUDA_TRY(cudaStreamSynchronize(s));
  }
  // chunk boundaries rounded up to multiples of `wave` elements, and the prefixes of q each
  // chunk reads and of Aq that are final after it
  auto split = [&](PipeSplit& sp, int64_t wave) {
    sp.e0.resize(K + 1);
    for (int c = 0; c <= K; ++c) sp.e0[c] = std::min<int64_t>(E, (E * c / K + wave - 1) / wave * wave);
    sp.e0[K] = E;
    sp.inEnd.assign(K, 0);
    sp.outEnd.assign(K, Nglobal);
    int64_t need = 0;
    for (int c = 0; c < K; ++c) {
      for (int64_t e = sp.e0[c]; e < sp.e0[c + 1]; ++e) need = std::max<int64_t>(need, (int64_t)hi[e] + 1);
      sp.inEnd[c] = std::min<int64_t>(need, Nglobal);
    }
    sp.inEnd[K - 1] = Nglobal;
    int64_t first = Nglobal;   // smallest entry touched by chunks c+1..K-1
    for (int c = K - 1; c >= 0; --c) {
      sp.outEnd[c] = first;
      for (int64_t e = sp.e0[c]; e < sp.e0[c + 1]; ++e) first = std::min<int64_t>(first, (int64_t)lo[e]);
    }
  };
  // The FP64 kernel bounds its pipeline, so its chunks end on whole waves of the kernel
  // instantiation this object launches (64^3, N=7: 12.48 -> 12.05 ms per call); the
  // double-word and FP32 pipelines are bound by the copies and keep even chunks (aligned,
  // the double-word one was 3 % slower).
  const bool mass = !(lambda == 0.0 && !hasLambdaE);
  split(p->native, opDW ? 1 : std::max(1, ax_wave_elements(mesh.N, false, mass)));
  split(p->even, 1);
  LPG_CUDA_TRY(cudaStreamCreateWithFlags(&p->h2d, cudaStreamNonBlocking));
  LPG_CUDA_TRY(cudaStreamCreateWithFlags(&p->d2h, cudaStreamNonBlocking));
  p->inReady.assign(K, nullptr);
  p->chunkDone.assign(K, nullptr);
  for (int c = 0; c < K; ++c) {
    LPG_CUDA_TRY(cudaEventCreateWithFlags(&p->inReady[c], cudaEventDisableTiming));
    LPG_CUDA_TRY(cudaEventCreateWithFlags(&p->chunkDone[c], cudaEventDisableTiming));
  }
  pipe = std::move(p);
  return LPG_OK;
}

// Upload pieces of q on the h2d stream, one operator launch per element chunk on s
// (each waits for the piece it reads), download each final prefix of Aq on d2h.
template <typename T, typename Launch>
static int run_pipe(HostPipe& p, const PipeSplit& sp, const T* qh, T* Aqh, T* dq, T* dAq, int64_t Nglobal,
                    cudaStream_t s, Launch&& launch) {
  auto body = [&]() -> int {
    int64_t up = 0;
    for (int c = 0; c < p.K; ++c) {
      const int64_t end = sp.inEnd[c];
      if (end > up)
        LPG_CUDA_TRY(cudaMemcpyAsync(dq + up, qh + up, sizeof(T) * (end - up), cudaMemcpyHostToDevice, p.h2d));
      up = std::max(up, end);
      LPG_CUDA_TRY(cudaEventRecord(p.inReady[c], p.h2d));
    }
    // chunk c reads and accumulates only into dofs below inEnd[c] (its elements' dofs), so
    // Aq is zeroed piece by piece ahead of each chunk instead of in one pass up front
    int64_t down = 0, zeroed = 0;
    for (int c = 0; c < p.K; ++c) {
      const int64_t zend = std::max<int64_t>(zeroed, sp.inEnd[c]);
      if (zend > zeroed) LPG_CUDA_TRY(cudaMemsetAsync(dAq + zeroed, 0, sizeof(T) * (zend - zeroed), s));
      zeroed = zend;
      LPG_CUDA_TRY(cudaStreamWaitEvent(s, p.inReady[c], 0));
      const int rc = launch(sp.e0[c], sp.e0[c + 1]);
      if (rc) return rc;
      LPG_CUDA_TRY(cudaEventRecord(p.chunkDone[c], s));
      const int64_t end = sp.outEnd[c];
      if (end > down) {
        LPG_CUDA_TRY(cudaStreamWaitEvent(p.d2h, p.chunkDone[c], 0));
        LPG_CUDA_TRY(cudaMemcpyAsync(Aqh + down, dAq + down, sizeof(T) * (end - down), cudaMemcpyDeviceToHost,
                                     p.d2h));
        down = end;
      }
    }
    return LPG_OK;
  };
  const int rc = body();
  // nothing may still be copying into or out of the caller's buffers on return
  const cudaError_t e1 = cudaStreamSynchronize(p.h2d);
  const cudaError_t e2 = cudaStreamSynchronize(s);
  const cudaError_t e3 = cudaStreamSynchronize(p.d2h);
  if (rc) return rc;
  if (e1 != cudaSuccess) return cuda_status(e1, "host operator: upload");
  if (e2 != cudaSuccess) return cuda_status(e2, "host operator: operator");
  if (e3 != cudaSuccess) return cuda_status(e3, "host operator: download");
  return LPG_OK;
}

int Elliptic::OperatorHost(const double* qHost, double* AqHost, cudaStream_t s) {
  int rc;
  if ((rc = BuildPipe(s))) return rc;
  if (!pipe->Aq.p && ((rc = pipe->q.alloc(std::max<int64_t>(Nglobal, 1))) ||
                      (rc = pipe->Aq.alloc(std::max<int64_t>(Nglobal, 1)))))
    return rc;
  const int64_t Np = mesh.Np;
  if (opDW && (rc = mesh.make_dw(s))) return rc;
  auto launch = [&](int64_t a0, int64_t a1) {
    if (opDW) {
      AxArgs<double, float2> a;
      a.N = mesh.N; a.Nelements = a1 - a0; a.g2l = g2l.p + a0 * Np;
      a.ggeo = mesh.geoDW.p + a0 * 7 * Np; a.geoStride = 7 * Np; a.wJ = a.ggeo + 6 * Np; a.wJStride = 7 * Np;
      a.D = mesh.D_d.p; a.lambda = lambda; a.lambdaE = hasLambdaE ? lambdaE.p + a0 : nullptr;
      a.q = pipe->q.p; a.out = pipe->Aq.p; a.Nglobal = 0;   // accumulate: the pipeline zeroed Aq
      return ax_hex_dw(a, s);
    }
    AxArgs<double, double> a;
    a.N = mesh.N; a.Nelements = a1 - a0; a.g2l = g2l.p + a0 * Np;
    a.ggeo = mesh.geo.p + a0 * 7 * Np; a.geoStride = 7 * Np; a.wJ = a.ggeo + 6 * Np; a.wJStride = 7 * Np;
    a.D = mesh.D_d.p; a.lambda = lambda; a.lambdaE = hasLambdaE ? lambdaE.p + a0 : nullptr;
    a.q = pipe->q.p; a.out = pipe->Aq.p; a.Nglobal = Nglobal;
    return ax_hex<double, double>(a, AxMode::AccumulateAssembled, s);
  };
  return run_pipe<double>(*pipe, pipe->native, qHost, AqHost, pipe->q.p, pipe->Aq.p, Nglobal, s, launch);
}

int Elliptic::OperatorHostF32(const float* qHost, float* AqHost, Prec prec, cudaStream_t s) {
  int rc;
  if ((rc = BuildPipe(s))) return rc;
  if (!pipe->Aq32.p && ((rc = pipe->q32.alloc(std::max<int64_t>(Nglobal, 1))) ||
                        (rc = pipe->Aq32.alloc(std::max<int64_t>(Nglobal, 1)))))
    return rc;
  const int64_t Np = mesh.Np;
  auto launch = [&](int64_t a0, int64_t a1) {
    const float* lam = hasLambdaE ? lambdaE32.p + a0 : nullptr;
    if (prec == Prec::BF16G) {
      AxArgs<float, __nv_bfloat16> a;
      a.N = mesh.N; a.Nelements = a1 - a0; a.g2l = g2l.p + a0 * Np;
      a.ggeo = mesh.geo16.p + a0 * 7 * Np; a.geoStride = 7 * Np; a.wJ = a.ggeo + 6 * Np; a.wJStride = 7 * Np;
      a.D = mesh.D32.p; a.lambda = (float)lambda; a.lambdaE = lam;
      a.q = pipe->q32.p; a.out = pipe->Aq32.p; a.Nglobal = Nglobal;
      return ax_hex<float, __nv_bfloat16>(a, AxMode::AccumulateAssembled, s);
    }
    AxArgs<float, float> a;
    a.N = mesh.N; a.Nelements = a1 - a0; a.g2l = g2l.p + a0 * Np;
    a.ggeo = mesh.geo32.p + a0 * 7 * Np; a.geoStride = 7 * Np; a.wJ = a.ggeo + 6 * Np; a.wJStride = 7 * Np;
    a.D = mesh.D32.p; a.lambda = (float)lambda; a.lambdaE = lam;
    a.q = pipe->q32.p; a.out = pipe->Aq32.p; a.Nglobal = Nglobal;
    return ax_hex<float, float>(a, AxMode::AccumulateAssembled, s);
  };
  return run_pipe<float>(*pipe, pipe->even, qHost, AqHost, pipe->q32.p, pipe->Aq32.p, Nglobal, s, launch);
}

int Elliptic::BuildDiagonal(double* diagG, cudaStream_t s) {
  if (ipdg) {   // BuildOperatorDiagonalIpdgHex3D: no rank boost for the hexahedral IPDG diagonal
    IpdgArgs a = ipdg_args();
    a.out = diagG;
    int rc = ipdg_diagonal(a, s);
    if (rc) return rc;
    LPG_CUDA_TRY(cudaStreamSynchronize(s));
    return LPG_OK;
  }
  DevBuf<double> dL;
  int rc = dL.alloc(Nlocal);
  if (rc) return rc;
  const double boost = allNeumann ? allNeumannScale * allNeumannScale : 0.0;
  if ((rc = operator_diagonal_local(mesh.N, mesh.E, mesh.geo.p, mesh.D_d.p, lambda,
                                    hasLambdaE ? lambdaE.p : nullptr, g2l.p, boost, dL.p, s)))
    return rc;
  if ((rc = gather_add<double>(Nlocal, g2l.p, dL.p, diagG, Nglobal, true, s))) return rc;
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  return LPG_OK;
}

int Elliptic::BuildRhs(double* r, cudaStream_t s) {
  DevBuf<double> rL, gL;
  int rc;
  if ((rc = rL.alloc(Nlocal)) || (rc = gL.alloc(Nlocal))) return rc;
  RhsSpec spec{rhsKind, (int)(sources.size() / 4), sources_d.p};
  if ((rc = rhs_local(mesh.N, mesh.E, mesh.EX.p, mesh.EY.p, mesh.EZ.p, mesh.r1d_d.p, mesh.geo.p,
                      hasLambdaE ? lambdaE.p : nullptr, lambda, g2l.p, spec, rL.p, gL.p, s)))
    return rc;
  if (!ipdg && rhsKind == 0 && neuCount > 0 &&
      (rc = neumann_flux(mesh.N, neuCount, neuNode.p, neuMask.p, mesh.EX.p, mesh.EY.p, mesh.EZ.p, mesh.r1d_d.p,
                         mesh.w1d_d.p, rL.p, s)))
    return rc;
  if (ipdg && rhsKind == 0) {
    // weakly imposed boundary data (ellipticRhsBCIpdgHex3D.okl)
    IpdgArgs a = ipdg_args();
    a.out = rL.p;
    if ((rc = ipdg_rhs_bc(a, s))) return rc;
  }
  if (rhsKind == 0 && hasDirichlet && !ipdg) {
    // Dirichlet lifting rhs -= A_e g (ellipticRhsBCHex3D.okl:60-290)
    AxArgs<double, double> a;
    const int64_t Np = mesh.Np;
    a.N = mesh.N; a.Nelements = mesh.E; a.g2l = g2l.p;
    a.ggeo = mesh.geo.p; a.geoStride = 7 * Np; a.wJ = mesh.geo.p + 6 * Np; a.wJStride = 7 * Np;
    a.D = mesh.D_d.p; a.lambda = lambda; a.lambdaE = hasLambdaE ? lambdaE.p : nullptr;
    a.q = gL.p; a.out = rL.p;
    if ((rc = ax_hex<double, double>(a, AxMode::LocalInSubtract, s))) return rc;
  }
  if ((rc = gather_add<double>(Nlocal, g2l.p, rL.p, r, Nglobal, true, s))) return rc;
  LPG_CUDA_TRY(cudaStreamSynchronize(s));
  return LPG_OK;
}

// Assembled stiffness (+ lambda mass) of this degree on the host as CSR with columns
// sorted and duplicates summed in element order; element entries below 1e-7 are dropped
// as in the reference (ellipticBuildOperatorMatrixContinuous.cpp:697-880). Two passes: the
// element loop writes every (row, col, val) straight into its row, at a slot fixed by the
// order of the row's local copies (element order), then each row is stably sorted by
// column and merged; this sums duplicates in the same order as one global stable sort.
// IPDG matrix (the matrix of BuildOperatorMatrixIpdgHex3D, ellipticBuildOperatorMatrixIpdg.cpp:
// 1316-1570) by probing the matrix-free operator: elements get a distance-2 colouring of the
// face-neighbour graph, so for one colour and one local node n the vector with ones at node
// n of every element of that colour returns, in each such element and its neighbours,
// exactly column (e, n) of the matrix. ncolours * Np operator applications; entries with
// |a| <= 1e-8 are dropped as in the reference.
int Elliptic::BuildMatrixIpdg(std::vector<int64_t>& rowStarts, std::vector<int32_t>& cols, std::vector<double>& vals,
                              cudaStream_t s) {
  const int Np = mesh.Np;
  const int64_t E = mesh.E;
  {
    // at most 7 element blocks per row, 12 bytes per entry: refuse beyond a quarter of host memory
    const long pages = sysconf(_SC_PHYS_PAGES), pageSize = sysconf(_SC_PAGE_SIZE);
    const double hostBytes = (pages > 0 && pageSize > 0) ? (double)pages * (double)pageSize : 64e9;
    if ((double)Nlocal * 7.0 * Np * 12.0 > 0.25 * hostBytes)
      return set_error(LPG_ERR_UNSUPPORTED, "IPDG matrix too large for host AMG setup; use MULTIGRID");
  }
  std::vector<int> color(E, -1);
  int ncolor = 0;
  {
    std::vector<int> mark;
    for (int64_t e = 0; e < E; ++e) {
      std::vector<int> used;
      for (int f = 0; f < 6; ++f) {
        const int64_t a = EToE_h[e * 6 + f];
        if (a < 0) continue;
        if (color[a] >= 0) used.push_back(color[a]);
        for (int g = 0; g < 6; ++g) {
          const int64_t b = EToE_h[a * 6 + g];
          if (b >= 0 && color[b] >= 0) used.push_back(color[b]);
        }
      }
      std::sort(used.begin(), used.end());
      int c = 0;
      for (int u : used) { if (u == c) ++c; else if (u > c) break; }
      color[e] = c;
      ncolor = std::max(ncolor, c + 1);
    }
  }
  std::vector<std::vector<int64_t>> byColor(ncolor);
  for (int64_t e = 0; e < E; ++e) byColor[color[e]].push_back(e);
  struct Ent { int32_t col; double val; };
  std::vector<std::vector<Ent>> rowsE(Nlocal);
  DevBuf<double> v, Av;
  int rc;
  if ((rc = v.alloc(Nlocal)) || (rc = Av.alloc(Nlocal))) return rc;
  std::vector<double> hv(Nlocal, 0.0), hA(Nlocal);
  for (int c = 0; c < ncolor; ++c)
    for (int n = 0; n < Np; ++n) {
      for (int64_t e : byColor[c]) hv[e * Np + n] = 1.0;
      if ((rc = v.upload(hv.data(), Nlocal, s)) || (rc = Operator(v.p, Av.p, s)) ||
          (rc = Av.download(hA.data(), Nlocal, s)))
        return rc;
      for (int64_t e : byColor[c]) hv[e * Np + n] = 0.0;
#pragma omp parallel for schedule(dynamic, 64)
      for (size_t q = 0; q < byColor[c].size(); ++q) {
        const int64_t e = byColor[c][q];
        int64_t targets[7];
        int nt = 0;
        targets[nt++] = e;
        for (int f = 0; f < 6; ++f) {
          const int64_t a = EToE_h[e * 6 + f];
          bool seen = (a < 0);
          for (int t = 0; t < nt && !seen; ++t) seen = (targets[t] == a);
          if (!seen) targets[nt++] = a;
        }
        const int32_t col = (int32_t)(e * Np + n);
        for (int t = 0; t < nt; ++t)
          for (int p = 0; p < Np; ++p) {
            const int64_t row = targets[t] * Np + p;
            const double a = hA[row];
            // rows of different elements of this colour never coincide (distance-2 colouring)
            if (std::fabs(a) > 1e-8) rowsE[row].push_back(Ent{col, a});
          }
      }
    }
  rowStarts.assign(Nlocal + 1, 0);
  for (int64_t r = 0; r < Nlocal; ++r) {
    std::sort(rowsE[r].begin(), rowsE[r].end(), [](const Ent& a, const Ent& b) { return a.col < b.col; });
    rowStarts[r + 1] = rowStarts[r] + (int64_t)rowsE[r].size();
  }
  cols.resize(rowStarts[Nlocal]);
  vals.resize(rowStarts[Nlocal]);
  for (int64_t r = 0; r < Nlocal; ++r)
    for (size_t k = 0; k < rowsE[r].size(); ++k) {
      cols[rowStarts[r] + k] = rowsE[r][k].col;
      vals[rowStarts[r] + k] = rowsE[r][k].val;
    }
  return LPG_OK;
}

int Elliptic::BuildMatrix(std::vector<int64_t>& rowStarts, std::vector<int32_t>& cols, std::vector<double>& vals,
                          cudaStream_t s) {
  if (ipdg) return BuildMatrixIpdg(rowStarts, cols, vals, s);
  const int Nq = mesh.Nq, Np = mesh.Np;
  const int64_t E = mesh.E, Ng = Nglobal;
  std::vector<double> geo(E * 7 * Np);
  std::vector<int32_t> map(Nlocal);
  int rc;
  if ((rc = mesh.geo.download(geo.data(), E * 7 * Np, s)) || (rc = g2l.download(map.data(), Nlocal, s))) return rc;
  const double* Dm = mesh.D.data();
  // unmasked nodes per element; slot of each local copy inside its row
  std::vector<int32_t> live(E);
#pragma omp parallel for
  for (int64_t e = 0; e < E; ++e) {
    int c = 0;
    for (int n = 0; n < Np; ++n) c += (map[e * Np + n] >= 0);
    live[e] = c;
  }
  std::vector<int64_t> rowCount(Ng + 1, 0), slot(Nlocal, 0);
  for (int64_t L = 0; L < Nlocal; ++L) {
    const int32_t g = map[L];
    if (g < 0) continue;
    slot[L] = rowCount[g + 1];
    rowCount[g + 1] += live[L / Np];
  }
  for (int64_t g = 0; g < Ng; ++g) rowCount[g + 1] += rowCount[g];
  const int64_t total = rowCount[Ng];
  {
    // the element entries (12 bytes each) and the coarsening that follows must fit in host
    // memory: refuse beyond a quarter of it rather than exhaust it
    const long pages = sysconf(_SC_PHYS_PAGES), pageSize = sysconf(_SC_PAGE_SIZE);
    const double hostBytes = (pages > 0 && pageSize > 0) ? (double)pages * (double)pageSize : 64e9;
    if ((double)total * 12.0 > 0.25 * hostBytes)
      return set_error(LPG_ERR_UNSUPPORTED, "assembled matrix too large for host AMG setup (" + std::to_string(total) +
                                                " element entries); use MULTIGRID with a degree-1 coarse level");
  }
  std::vector<int32_t> ecol(total);
  std::vector<double> eval(total);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < E; ++e) {
    const double* gg = geo.data() + e * 7 * Np;
    const double lam = hasLambdaE ? lambdaE_h[e] : lambda;
    for (int nz = 0; nz < Nq; nz++) for (int ny = 0; ny < Nq; ny++) for (int nx = 0; nx < Nq; nx++) {
      const int idn = nx + ny * Nq + nz * Nq * Nq;
      const int32_t gn = map[e * Np + idn];
      if (gn < 0) continue;
      int64_t pos = rowCount[gn] + slot[e * Np + idn];
      for (int mz = 0; mz < Nq; mz++) for (int my = 0; my < Nq; my++) for (int mx = 0; mx < Nq; mx++) {
        const int idm = mx + my * Nq + mz * Nq * Nq;
        const int32_t gm = map[e * Np + idm];
        if (gm < 0) continue;
        double val = 0;
        int id;
        if (ny == my && nz == mz)
          for (int k = 0; k < Nq; k++) { id = k + ny * Nq + nz * Nq * Nq; val += gg[0 * Np + id] * Dm[nx + k * Nq] * Dm[mx + k * Nq]; }
        if (nz == mz) {
          id = mx + ny * Nq + nz * Nq * Nq; val += gg[1 * Np + id] * Dm[nx + mx * Nq] * Dm[my + ny * Nq];
          id = nx + my * Nq + nz * Nq * Nq; val += gg[1 * Np + id] * Dm[mx + nx * Nq] * Dm[ny + my * Nq];
        }
        if (ny == my) {
          id = mx + ny * Nq + nz * Nq * Nq; val += gg[2 * Np + id] * Dm[nx + mx * Nq] * Dm[mz + nz * Nq];
          id = nx + ny * Nq + mz * Nq * Nq; val += gg[2 * Np + id] * Dm[mx + nx * Nq] * Dm[nz + mz * Nq];
        }
        if (nx == mx && nz == mz)
          for (int k = 0; k < Nq; k++) { id = nx + k * Nq + nz * Nq * Nq; val += gg[3 * Np + id] * Dm[ny + k * Nq] * Dm[my + k * Nq]; }
        if (nx == mx) {
          id = nx + my * Nq + nz * Nq * Nq; val += gg[4 * Np + id] * Dm[ny + my * Nq] * Dm[mz + nz * Nq];
          id = nx + ny * Nq + mz * Nq * Nq; val += gg[4 * Np + id] * Dm[my + ny * Nq] * Dm[nz + mz * Nq];
        }
        if (nx == mx && ny == my)
          for (int k = 0; k < Nq; k++) { id = nx + ny * Nq + k * Nq * Nq; val += gg[5 * Np + id] * Dm[nz + k * Nq] * Dm[mz + k * Nq]; }
        if (nx == mx && ny == my && nz == mz) val += gg[6 * Np + idn] * lam;
        ecol[pos] = (std::fabs(val) >= 1e-7) ? gm : -1;   // dropped entries keep their slot
        eval[pos] = val;
        ++pos;
      }
    }
  }
  std::vector<double>().swap(geo);
  // per row: stable sort by column, merge duplicates, drop marked entries
  std::vector<int64_t> kept(Ng + 1, 0);
#pragma omp parallel
  {
    std::vector<int32_t> idx;
    std::vector<std::pair<int32_t, double>> row;
#pragma omp for schedule(dynamic, 1024)
    for (int64_t g = 0; g < Ng; ++g) {
      const int64_t b = rowCount[g], n = rowCount[g + 1] - b;
      idx.resize(n);
      for (int64_t k = 0; k < n; ++k) idx[k] = (int32_t)k;
      std::stable_sort(idx.begin(), idx.end(), [&](int32_t x, int32_t y) { return ecol[b + x] < ecol[b + y]; });
      // compact in place through a small copy
      row.clear();
      for (int64_t k = 0; k < n; ++k) {
        const int32_t c = ecol[b + idx[k]];
        if (c < 0) continue;
        const double v = eval[b + idx[k]];
        if (!row.empty() && row.back().first == c) row.back().second += v;
        else row.emplace_back(c, v);
      }
      for (size_t k = 0; k < row.size(); ++k) { ecol[b + k] = row[k].first; eval[b + k] = row[k].second; }
      kept[g + 1] = (int64_t)row.size();
    }
  }
  for (int64_t g = 0; g < Ng; ++g) kept[g + 1] += kept[g];
  cols.resize(kept[Ng]);
  vals.resize(kept[Ng]);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t g = 0; g < Ng; ++g) {
    const int64_t n = kept[g + 1] - kept[g];
    std::copy(ecol.begin() + rowCount[g], ecol.begin() + rowCount[g] + n, cols.begin() + kept[g]);
    std::copy(eval.begin() + rowCount[g], eval.begin() + rowCount[g] + n, vals.begin() + kept[g]);
  }
  rowStarts.swap(kept);
  return LPG_OK;
}

}  // namespace lpg
