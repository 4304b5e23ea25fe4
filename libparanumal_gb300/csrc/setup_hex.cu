// Setup kernels for hexahedral box meshes: geometric factors, box numbering
// (GlobalToLocal / owner / multiplicity), right-hand side, operator diagonal and
// the solution/error norms of the run epilogue. All element-parallel; the host
// only builds vertex coordinates and per-element dof offsets.
#include "lpg_common.cuh"
#include "lpg_internal.hpp"

namespace lpg {

// ---------------------------------------------------------------- geometric factors
// One CTA per element. Physical nodes by the trilinear vertex map
// (libs/mesh/meshPhysicalNodesHex3D.cpp:31-112), derivatives by applying D
// (libs/mesh/meshGeometricFactorsHex3D.cpp:95-170), packed output [e][7][Np].
template <int NQ>
__global__ void __launch_bounds__(256)
geo_hex_kernel(const int64_t E, const double* __restrict__ EX, const double* __restrict__ EY,
               const double* __restrict__ EZ, const double* __restrict__ Dg,
               const double* __restrict__ r1d, const double* __restrict__ w1d,
               double* __restrict__ geo, int* __restrict__ badCount) {
  constexpr int NP = NQ * NQ * NQ;
  __shared__ double s_x[NP], s_y[NP], s_z[NP];
  __shared__ double s_D[NQ * NQ], s_r[NQ], s_w[NQ], s_ev[24];
  const int64_t e = blockIdx.x;
  for (int t = threadIdx.x; t < NQ * NQ; t += blockDim.x) s_D[t] = Dg[t];
  for (int t = threadIdx.x; t < NQ; t += blockDim.x) { s_r[t] = r1d[t]; s_w[t] = w1d[t]; }
  if (threadIdx.x < 8) {
    s_ev[threadIdx.x] = EX[e * 8 + threadIdx.x];
    s_ev[8 + threadIdx.x] = EY[e * 8 + threadIdx.x];
    s_ev[16 + threadIdx.x] = EZ[e * 8 + threadIdx.x];
  }
  __syncthreads();
  for (int n = threadIdx.x; n < NP; n += blockDim.x) {
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
    const double rn = s_r[i], sn = s_r[j], tn = s_r[k];
    const double c0 = 0.125 * (1 - rn) * (1 - sn) * (1 - tn), c1 = 0.125 * (1 + rn) * (1 - sn) * (1 - tn);
    const double c2 = 0.125 * (1 + rn) * (1 + sn) * (1 - tn), c3 = 0.125 * (1 - rn) * (1 + sn) * (1 - tn);
    const double c4 = 0.125 * (1 - rn) * (1 - sn) * (1 + tn), c5 = 0.125 * (1 + rn) * (1 - sn) * (1 + tn);
    const double c6 = 0.125 * (1 + rn) * (1 + sn) * (1 + tn), c7 = 0.125 * (1 - rn) * (1 + sn) * (1 + tn);
    const double* v = s_ev;
    s_x[n] = c0 * v[0] + c1 * v[1] + c2 * v[2] + c3 * v[3] + c4 * v[4] + c5 * v[5] + c6 * v[6] + c7 * v[7];
    v += 8;
    s_y[n] = c0 * v[0] + c1 * v[1] + c2 * v[2] + c3 * v[3] + c4 * v[4] + c5 * v[5] + c6 * v[6] + c7 * v[7];
    v += 8;
    s_z[n] = c0 * v[0] + c1 * v[1] + c2 * v[2] + c3 * v[3] + c4 * v[4] + c5 * v[5] + c6 * v[6] + c7 * v[7];
  }
  __syncthreads();
  int bad = 0;
  for (int n = threadIdx.x; n < NP; n += blockDim.x) {
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
    double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      const int idr = k * NQ * NQ + j * NQ + m, ids = k * NQ * NQ + m * NQ + i, idt = m * NQ * NQ + j * NQ + i;
      const double dr = s_D[i * NQ + m], ds = s_D[j * NQ + m], dt = s_D[k * NQ + m];
      xr += dr * s_x[idr]; xs += ds * s_x[ids]; xt += dt * s_x[idt];
      yr += dr * s_y[idr]; ys += ds * s_y[ids]; yt += dt * s_y[idt];
      zr += dr * s_z[idr]; zs += ds * s_z[ids]; zt += dt * s_z[idt];
    }
    const double J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
    if (!(J >= 1e-12)) bad++;
    const double rx = (ys * zt - zs * yt) / J, ry = -(xs * zt - zs * xt) / J, rz = (xs * yt - ys * xt) / J;
    const double sx = -(yr * zt - zr * yt) / J, sy = (xr * zt - zr * xt) / J, sz = -(xr * yt - yr * xt) / J;
    const double tx = (yr * zs - zr * ys) / J, ty = -(xr * zs - zr * xs) / J, tz = (xr * ys - yr * xs) / J;
    const double JW = J * s_w[i] * s_w[j] * s_w[k];
    double* g = geo + e * 7 * NP + n;
    g[0 * NP] = JW * (rx * rx + ry * ry + rz * rz);
    g[1 * NP] = JW * (rx * sx + ry * sy + rz * sz);
    g[2 * NP] = JW * (rx * tx + ry * ty + rz * tz);
    g[3 * NP] = JW * (sx * sx + sy * sy + sz * sz);
    g[4 * NP] = JW * (sx * tx + sy * ty + sz * tz);
    g[5 * NP] = JW * (tx * tx + ty * ty + tz * tz);
    g[6 * NP] = JW;
  }
  if (bad) atomicAdd(badCount, bad);
}

template <int NQ>
static int launch_geo(int64_t E, const double* EX, const double* EY, const double* EZ,
                      const double* D, const double* r1d, const double* w1d, double* geo, int* bad,
                      cudaStream_t s) {
  if (E <= 0) return LPG_OK;
  geo_hex_kernel<NQ><<<(unsigned)E, 256, 0, s>>>(E, EX, EY, EZ, D, r1d, w1d, geo, bad);
  LPG_LAUNCH_CHECK("geo_hex_kernel");
  return LPG_OK;
}

int geometric_factors(int N, int64_t E, const double* EX, const double* EY, const double* EZ,
                      const double* D, const double* r1d, const double* w1d, double* geo,
                      int* badCount, cudaStream_t s) {
  switch (N) {
    case 1: return launch_geo<2>(E, EX, EY, EZ, D, r1d, w1d, geo, badCount, s);
    case 2: return launch_geo<3>(E, EX, EY, EZ, D, r1d, w1d, geo, badCount, s);
    case 3: return launch_geo<4>(E, EX, EY, EZ, D, r1d, w1d, geo, badCount, s);
    case 4: return launch_geo<5>(E, EX, EY, EZ, D, r1d, w1d, geo, badCount, s);
    case 5: return launch_geo<6>(E, EX, EY, EZ, D, r1d, w1d, geo, badCount, s);
    case 6: return launch_geo<7>(E, EX, EY, EZ, D, r1d, w1d, geo, badCount, s);
    case 7: return launch_geo<8>(E, EX, EY, EZ, D, r1d, w1d, geo, badCount, s);
    case 8: return launch_geo<9>(E, EX, EY, EZ, D, r1d, w1d, geo, badCount, s);
    default: return set_error(LPG_ERR_UNSUPPORTED, "geometric factors: N must be 1..8");
  }
}

// ---------------------------------------------------------------- box numbering
// For a structured box the fixed point of the reference's min-propagation
// (libs/mesh/meshConnectNodes.cpp:32-117) is the smallest element index that
// holds the lattice point, and the ogs ordering of gathered dofs
// (libs/ogs/ogsSetup.cpp:408-432) is first appearance in local node order, i.e.
// by (owner element, owner node). Both have a closed form per axis.
__device__ __forceinline__ void owner_axis(int e, int a, int n, int N, int periodic, int& eo, int& ao,
                                           int& boundary) {
  int64_t X = (int64_t)e * N + a;
  const int64_t L = (int64_t)n * N;
  boundary = 0;
  if (periodic) {
    X %= L;
    if (X == 0) { eo = 0; ao = 0; return; }
  } else {
    boundary = (X == 0 || X == L);
  }
  if (X > 0 && X % N == 0) { eo = (int)(X / N) - 1; ao = N; }
  else { eo = (int)(X / N); ao = (int)(X % N); }
}

__device__ __forceinline__ void owned_range(int e, int n, int N, int periodic, int dirichlet, int& lo,
                                            int& hi) {
  if (periodic) { lo = (e == 0) ? 0 : 1; hi = (e == n - 1) ? N - 1 : N; }
  else if (dirichlet) { lo = 1; hi = (e == n - 1) ? N - 1 : N; }
  else { lo = (e == 0) ? 0 : 1; hi = N; }
}

__global__ void box_numbering_kernel(const BoxNumbering b, const int64_t* __restrict__ elemBase,
                                     int32_t* __restrict__ g2l, int32_t* __restrict__ owner,
                                     int32_t* __restrict__ mult, const int64_t Nlocal) {
  const int Nq = b.N + 1, Np = Nq * Nq * Nq;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < Nlocal;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = id / Np;
    const int n = (int)(id % Np);
    const int a = n % Nq, bb = (n / Nq) % Nq, c = n / (Nq * Nq);
    const int ex = (int)(e % b.nx), ey = (int)((e / b.nx) % b.ny), ez = (int)(e / ((int64_t)b.nx * b.ny));
    int ox, ax, bx, oy, ay, by, oz, az, bz;
    owner_axis(ex, a, b.nx, b.N, b.periodic, ox, ax, bx);
    owner_axis(ey, bb, b.ny, b.N, b.periodic, oy, ay, by);
    owner_axis(ez, c, b.nz, b.N, b.periodic, oz, az, bz);
    if (b.dirichlet && (bx || by || bz)) { g2l[id] = -1; continue; }
    int lx, hx, ly, hy, lz, hz;
    owned_range(ox, b.nx, b.N, b.periodic, b.dirichlet, lx, hx);
    owned_range(oy, b.ny, b.N, b.periodic, b.dirichlet, ly, hy);
    owned_range(oz, b.nz, b.N, b.periodic, b.dirichlet, lz, hz);
    const int64_t eo = ox + (int64_t)oy * b.nx + (int64_t)oz * b.nx * b.ny;
    const int64_t rank = ((int64_t)(az - lz) * (hy - ly + 1) + (ay - ly)) * (hx - lx + 1) + (ax - lx);
    const int64_t dof = elemBase[eo] + rank;
    g2l[id] = (int32_t)dof;
    atomicAdd(mult + dof, 1);
    if (eo == e && ax == a && ay == bb && az == c) owner[dof] = (int32_t)id;
  }
}

int box_numbering(const BoxNumbering& b, const int64_t* elemBase, int32_t* g2l, int32_t* owner,
                  int32_t* mult, int64_t Nglobal, cudaStream_t s) {
  const int64_t Nlocal = (int64_t)b.nx * b.ny * b.nz * (b.N + 1) * (b.N + 1) * (b.N + 1);
  LPG_CUDA_TRY(cudaMemsetAsync(mult, 0, sizeof(int32_t) * Nglobal, s));
  const int64_t blocks = std::min<int64_t>((Nlocal + 255) / 256, 152 * 64);
  box_numbering_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(b, elemBase, g2l, owner,
                                                                               mult, Nlocal);
  LPG_LAUNCH_CHECK("box_numbering_kernel");
  return LPG_OK;
}

// ---------------------------------------------------------------- seeded input vectors
__device__ __forceinline__ uint64_t splitmix64_dev(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// q[g] = 2u - 1, u uniform [0,1) keyed by (seed, stream 3, lattice id of dof g's owner node)
__global__ void lattice_random_kernel(const BoxNumbering b, const int64_t Nglobal, const int32_t* __restrict__ owner,
                                      const uint64_t seed, double* __restrict__ q) {
  const int Nq = b.N + 1, Np = Nq * Nq * Nq;
  const int64_t NnX = b.periodic ? (int64_t)b.nx * b.N : (int64_t)b.nx * b.N + 1;
  const int64_t NnY = b.periodic ? (int64_t)b.ny * b.N : (int64_t)b.ny * b.N + 1;
  const uint64_t h0 = splitmix64_dev(seed ^ (3ULL << 56));
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < Nglobal; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t id = owner[g];
    const int64_t e = id / Np;
    const int n = (int)(id % Np);
    const int a = n % Nq, bb = (n / Nq) % Nq, c = n / (Nq * Nq);
    const int64_t ex = e % b.nx, ey = (e / b.nx) % b.ny, ez = e / ((int64_t)b.nx * b.ny);
    const int64_t key = (ex * b.N + a) + (ey * b.N + bb) * NnX + (ez * b.N + c) * NnX * NnY;
    const uint64_t h = splitmix64_dev(h0 + (uint64_t)key);
    q[g] = 2.0 * ((double)(h >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
  }
}

int lattice_random(const BoxNumbering& b, int64_t Nglobal, const int32_t* owner, uint64_t seed, double* q,
                   cudaStream_t s) {
  if (Nglobal <= 0) return LPG_OK;
  const int64_t blocks = std::min<int64_t>((Nglobal + 255) / 256, 152 * 32);
  lattice_random_kernel<<<(unsigned)blocks, 256, 0, s>>>(b, Nglobal, owner, seed, q);
  LPG_LAUNCH_CHECK("lattice_random_kernel");
  return LPG_OK;
}

// ---------------------------------------------------------------- rhs / norms

__device__ __forceinline__ void node_xyz(const double* __restrict__ EX, const double* __restrict__ EY,
                                         const double* __restrict__ EZ, int64_t e, double rn, double sn,
                                         double tn, double& x, double& y, double& z) {
  const double c0 = 0.125 * (1 - rn) * (1 - sn) * (1 - tn), c1 = 0.125 * (1 + rn) * (1 - sn) * (1 - tn);
  const double c2 = 0.125 * (1 + rn) * (1 + sn) * (1 - tn), c3 = 0.125 * (1 - rn) * (1 + sn) * (1 - tn);
  const double c4 = 0.125 * (1 - rn) * (1 - sn) * (1 + tn), c5 = 0.125 * (1 + rn) * (1 - sn) * (1 + tn);
  const double c6 = 0.125 * (1 + rn) * (1 + sn) * (1 + tn), c7 = 0.125 * (1 - rn) * (1 + sn) * (1 + tn);
  const double* v = EX + e * 8;
  x = c0 * v[0] + c1 * v[1] + c2 * v[2] + c3 * v[3] + c4 * v[4] + c5 * v[5] + c6 * v[6] + c7 * v[7];
  v = EY + e * 8;
  y = c0 * v[0] + c1 * v[1] + c2 * v[2] + c3 * v[3] + c4 * v[4] + c5 * v[5] + c6 * v[6] + c7 * v[7];
  v = EZ + e * 8;
  z = c0 * v[0] + c1 * v[1] + c2 * v[2] + c3 * v[3] + c4 * v[4] + c5 * v[5] + c6 * v[6] + c7 * v[7];
}

__device__ __forceinline__ void source_value(int kind, int nsrc, const double* __restrict__ src, double x,
                                             double y, double z, double lam, double& f, double& g) {
  if (kind == 0) {  // solvers/elliptic/data/ellipticSine3D.h:27-51
    const double sxyz = sin(LPG_PI * x) * sin(LPG_PI * y) * sin(LPG_PI * z);
    f = (3 * LPG_PI * LPG_PI + lam) * sxyz;
    g = sxyz;
  } else {  // sum of Gaussian sources exp(-|x-c|^2 / (2 w^2))
    double acc = 0;
    for (int k = 0; k < nsrc; ++k) {
      const double dx = x - src[4 * k], dy = y - src[4 * k + 1], dz = z - src[4 * k + 2], w = src[4 * k + 3];
      acc += exp(-(dx * dx + dy * dy + dz * dz) / (2 * w * w));
    }
    f = acc;
    g = 0.0;
  }
}

__global__ void rhs_kernel(const int Nq, const int64_t Nlocal, const double* __restrict__ EX,
                           const double* __restrict__ EY, const double* __restrict__ EZ,
                           const double* __restrict__ r1d, const double* __restrict__ geo,
                           const double* __restrict__ lambdaE, const double lambda,
                           const int32_t* __restrict__ g2l, const RhsSpec spec,
                           double* __restrict__ rL, double* __restrict__ gL) {
  const int Np = Nq * Nq * Nq;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < Nlocal;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = id / Np;
    const int n = (int)(id % Np);
    double x, y, z;
    node_xyz(EX, EY, EZ, e, r1d[n % Nq], r1d[(n / Nq) % Nq], r1d[n / (Nq * Nq)], x, y, z);
    const double lam = lambdaE ? lambdaE[e] : lambda;
    double f, g;
    source_value(spec.kind, spec.nsources, spec.src, x, y, z, lam, f, g);
    rL[id] = geo[e * 7 * Np + 6 * Np + n] * f;
    gL[id] = (g2l[id] < 0) ? g : 0.0;
  }
}

// Neumann data of the sine data file at boundary face nodes (ellipticRhsBCHex3D.okl:28-58):
// rhs -= -WsJ n . grad_B with grad_B = -grad u as the data file states it. One thread per
// listed local node; faceMask bit f = the node lies on boundary face f of its element.
// Normals and surface Jacobians from the analytic derivatives of the trilinear map.
__global__ void neumann_flux_kernel(const int Nq, const int64_t count, const int32_t* __restrict__ node,
                                    const int32_t* __restrict__ faceMask, const double* __restrict__ EX,
                                    const double* __restrict__ EY, const double* __restrict__ EZ,
                                    const double* __restrict__ r1d, const double* __restrict__ w1d,
                                    double* __restrict__ rL) {
  const int Np = Nq * Nq * Nq;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t id = node[t];
    const int64_t e = id / Np;
    const int n = id % Np;
    const int i = n % Nq, j = (n / Nq) % Nq, k = n / (Nq * Nq);
    const double r = r1d[i], s = r1d[j], q = r1d[k];
    double x, y, z;
    node_xyz(EX, EY, EZ, e, r, s, q, x, y, z);
    // d(x,y,z)/d(r,s,t): vertex v at corner (cx, cy, cz) has weight (1 +- r)(1 +- s)(1 +- t)/8
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};   // J[a][c] = d x_a / d r_c
    const double* V[3] = {EX + e * 8, EY + e * 8, EZ + e * 8};
    for (int v = 0; v < 8; ++v) {
      const int cx = (v == 1 || v == 2 || v == 5 || v == 6), cy = (v == 2 || v == 3 || v == 6 || v == 7), cz = (v >= 4);
      const double fr = cx ? 1 + r : 1 - r, fs = cy ? 1 + s : 1 - s, ft = cz ? 1 + q : 1 - q;
      const double dr = (cx ? 0.125 : -0.125) * fs * ft, ds = (cy ? 0.125 : -0.125) * fr * ft,
                   dt = (cz ? 0.125 : -0.125) * fr * fs;
      for (int a = 0; a < 3; ++a) { J[a][0] += dr * V[a][v]; J[a][1] += ds * V[a][v]; J[a][2] += dt * V[a][v]; }
    }
    const double xr = J[0][0], xs = J[0][1], xt = J[0][2], yr = J[1][0], ys = J[1][1], yt = J[1][2];
    const double zr = J[2][0], zs = J[2][1], zt = J[2][2];
    const double det = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
    const double g[9] = {(ys * zt - zs * yt) / det,  -(xs * zt - zs * xt) / det, (xs * yt - ys * xt) / det,
                         -(yr * zt - zr * yt) / det, (xr * zt - zr * xt) / det,  -(xr * yt - yr * xt) / det,
                         (yr * zs - zr * ys) / det,  -(xr * zs - zr * xs) / det, (xr * ys - yr * xs) / det};
    const double sx = sin(LPG_PI * x), sy = sin(LPG_PI * y), sz = sin(LPG_PI * z);
    const double ux = LPG_PI * cos(LPG_PI * x) * sy * sz, uy = LPG_PI * sx * cos(LPG_PI * y) * sz,
                 uz = LPG_PI * sx * sy * cos(LPG_PI * z);
    double acc = 0;
    const int mask = faceMask[t];
    for (int f = 0; f < 6; ++f) {
      if (!(mask & (1 << f))) continue;
      const int c0 = (f == 0 || f == 5) ? 6 : (f == 1 || f == 3) ? 3 : 0;
      const double sg = (f == 0 || f == 1 || f == 4) ? -1.0 : 1.0;
      const double nx = sg * g[c0], ny = sg * g[c0 + 1], nz = sg * g[c0 + 2];
      const double len = sqrt(nx * nx + ny * ny + nz * nz);
      const int b0 = (f == 0 || f == 5) ? i : (f == 1 || f == 3) ? i : j;
      const int b1 = (f == 0 || f == 5) ? j : k;
      const double wsJ = len * det * w1d[b0] * w1d[b1];
      acc += wsJ * (nx * ux + ny * uy + nz * uz) / len;
    }
    rL[id] -= acc;
  }
}

int neumann_flux(int N, int64_t count, const int32_t* node, const int32_t* faceMask, const double* EX,
                 const double* EY, const double* EZ, const double* r1d, const double* w1d, double* rL,
                 cudaStream_t s) {
  if (count <= 0) return LPG_OK;
  const int64_t blocks = std::min<int64_t>((count + 255) / 256, 152 * 16);
  neumann_flux_kernel<<<(unsigned)blocks, 256, 0, s>>>(N + 1, count, node, faceMask, EX, EY, EZ, r1d, w1d, rL);
  LPG_LAUNCH_CHECK("neumann_flux_kernel");
  return LPG_OK;
}

int rhs_local(int N, int64_t E, const double* EX, const double* EY, const double* EZ,
              const double* r1d, const double* geo, const double* lambdaE, double lambda,
              const int32_t* g2l, RhsSpec spec, double* rL, double* gL, cudaStream_t s) {
  const int Nq = N + 1;
  const int64_t Nlocal = E * Nq * Nq * Nq;
  const int64_t blocks = std::min<int64_t>((Nlocal + 255) / 256, 152 * 32);
  rhs_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(Nq, Nlocal, EX, EY, EZ, r1d, geo,
                                                                    lambdaE, lambda, g2l, spec, rL, gL);
  LPG_LAUNCH_CHECK("rhs_kernel");
  return LPG_OK;
}

__global__ void norms_kernel(const int Nq, const int64_t Nlocal, const double* __restrict__ EX,
                             const double* __restrict__ EY, const double* __restrict__ EZ,
                             const double* __restrict__ r1d, const double* __restrict__ geo,
                             const int32_t* __restrict__ g2l, const int kind, double* __restrict__ xL,
                             double* __restrict__ out) {
  const int Np = Nq * Nq * Nq;
  double a0 = 0, a1 = 0;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < Nlocal;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = id / Np;
    const int n = (int)(id % Np);
    double x, y, z;
    node_xyz(EX, EY, EZ, e, r1d[n % Nq], r1d[(n / Nq) % Nq], r1d[n / (Nq * Nq)], x, y, z);
    const double u = (kind == 0) ? sin(LPG_PI * x) * sin(LPG_PI * y) * sin(LPG_PI * z) : 0.0;
    double v = xL[id];
    if (g2l[id] < 0) { v = u; xL[id] = v; }  // ellipticAddBCHex3D.okl:27-47
    const double w = geo[e * 7 * Np + 6 * Np + n];
    a0 += w * v * v;
    a1 += w * (v - u) * (v - u);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_down_sync(0xffffffffu, a0, o);
    a1 += __shfl_down_sync(0xffffffffu, a1, o);
  }
  __shared__ double s0[32], s1[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { s0[warp] = a0; s1[warp] = a1; }
  __syncthreads();
  if (warp == 0) {
    a0 = (lane < (int)(blockDim.x >> 5)) ? s0[lane] : 0.0;
    a1 = (lane < (int)(blockDim.x >> 5)) ? s1[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_down_sync(0xffffffffu, a0, o);
      a1 += __shfl_down_sync(0xffffffffu, a1, o);
    }
    if (lane == 0) { atomicAdd(out, a0); atomicAdd(out + 1, a1); }
  }
}

int solution_norms(int N, int64_t E, const double* EX, const double* EY, const double* EZ,
                   const double* r1d, const double* geo, const int32_t* g2l, int kind, double* xL,
                   double* out, cudaStream_t s) {
  const int Nq = N + 1;
  const int64_t Nlocal = E * Nq * Nq * Nq;
  LPG_CUDA_TRY(cudaMemsetAsync(out, 0, 2 * sizeof(double), s));
  const int64_t blocks = std::min<int64_t>((Nlocal + 255) / 256, 152 * 16);
  norms_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(Nq, Nlocal, EX, EY, EZ, r1d, geo,
                                                                      g2l, kind, xL, out);
  LPG_LAUNCH_CHECK("norms_kernel");
  return LPG_OK;
}

// ---------------------------------------------------------------- operator diagonal
__global__ void diag_kernel(const int Nq, const int64_t Nlocal, const double* __restrict__ geo,
                            const double* __restrict__ D, const double lambda,
                            const double* __restrict__ lambdaE, const int32_t* __restrict__ g2l,
                            const double rankBoost, double* __restrict__ diagL) {
  const int Np = Nq * Nq * Nq;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < Nlocal;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = id / Np;
    const int idn = (int)(id % Np);
    const int nx = idn % Nq, ny = (idn / Nq) % Nq, nz = idn / (Nq * Nq);
    if (g2l[id] < 0) { diagL[id] = 1.0; continue; }
    const double* gg = geo + e * 7 * Np;
    double a = 0;
    a += 2 * gg[1 * Np + idn] * D[nx + nx * Nq] * D[ny + ny * Nq];
    a += 2 * gg[2 * Np + idn] * D[nx + nx * Nq] * D[nz + nz * Nq];
    a += 2 * gg[4 * Np + idn] * D[ny + ny * Nq] * D[nz + nz * Nq];
    for (int k = 0; k < Nq; k++) a += gg[0 * Np + k + ny * Nq + nz * Nq * Nq] * D[nx + k * Nq] * D[nx + k * Nq];
    for (int k = 0; k < Nq; k++) a += gg[3 * Np + nx + k * Nq + nz * Nq * Nq] * D[ny + k * Nq] * D[ny + k * Nq];
    for (int k = 0; k < Nq; k++) a += gg[5 * Np + nx + ny * Nq + k * Nq * Nq] * D[nz + k * Nq] * D[nz + k * Nq];
    a += gg[6 * Np + idn] * (lambdaE ? lambdaE[e] : lambda);
    diagL[id] = a + rankBoost;
  }
}

int operator_diagonal_local(int N, int64_t E, const double* geo, const double* D, double lambda,
                            const double* lambdaE, const int32_t* g2l, double rankBoost,
                            double* diagL, cudaStream_t s) {
  const int Nq = N + 1;
  const int64_t Nlocal = E * Nq * Nq * Nq;
  const int64_t blocks = std::min<int64_t>((Nlocal + 255) / 256, 152 * 32);
  diag_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(Nq, Nlocal, geo, D, lambda, lambdaE,
                                                                     g2l, rankBoost, diagL);
  LPG_LAUNCH_CHECK("diag_kernel");
  return LPG_OK;
}

// ---------------------------------------------------------------- element dof ranges
// One warp per element: smallest and largest assembled index among its unmasked nodes
// (lo = INT32_MAX, hi = -1 for an element with every node masked).
__global__ void element_dof_range_kernel(const int Np, const int64_t E, const int32_t* __restrict__ g2l,
                                         int32_t* __restrict__ lo, int32_t* __restrict__ hi) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; e < E; e += warps) {
    int mn = INT32_MAX, mx = -1;
    for (int n = lane; n < Np; n += 32) {
      const int32_t id = g2l[e * Np + n];
      if (id >= 0) {
        mn = min(mn, id);
        mx = max(mx, id);
      }
    }
    mn = __reduce_min_sync(0xffffffffu, mn);
    mx = __reduce_max_sync(0xffffffffu, mx);
    if (lane == 0) {
      lo[e] = mn;
      hi[e] = mx;
    }
  }
}

// ---------------------------------------------------------------- assembled mass product
// Mu[g] = sum over local copies n of g of wJ[n] u[g] (the diagonal GLL mass matrix,
// assembled): wJ is row 6 of the packed [e][7][Np] factors. Interior nodes (one copy)
// store, the others add atomically; Mu is zeroed first.
__global__ void mass_apply_kernel(const int Nq, const int64_t Nlocal, const double* __restrict__ geo,
                                  const int32_t* __restrict__ g2l, const double* __restrict__ u,
                                  double* __restrict__ Mu) {
  const int Np = Nq * Nq * Nq;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < Nlocal; n += (int64_t)gridDim.x * blockDim.x) {
    const int32_t g = g2l[n];
    if (g < 0) continue;
    const int64_t e = n / Np;
    const int l = (int)(n % Np);
    const double v = geo[e * 7 * Np + 6 * Np + l] * u[g];
    const int a = l % Nq, b = (l / Nq) % Nq, c = l / (Nq * Nq);
    if (a > 0 && a < Nq - 1 && b > 0 && b < Nq - 1 && c > 0 && c < Nq - 1) Mu[g] = v;
    else atomicAdd(Mu + g, v);
  }
}
int mass_apply(int N, int64_t E, const double* geo, const int32_t* g2l, const double* u, double* Mu, int64_t Nglobal,
               cudaStream_t s) {
  if (Nglobal > 0) LPG_CUDA_TRY(cudaMemsetAsync(Mu, 0, sizeof(double) * Nglobal, s));
  const int Nq = N + 1;
  const int64_t Nlocal = E * Nq * Nq * Nq;
  if (Nlocal <= 0) return LPG_OK;
  const int64_t blocks = std::min<int64_t>((Nlocal + 255) / 256, 152 * 32);
  mass_apply_kernel<<<(unsigned)blocks, 256, 0, s>>>(Nq, Nlocal, geo, g2l, u, Mu);
  LPG_LAUNCH_CHECK("mass_apply_kernel");
  return LPG_OK;
}

int element_dof_range(int N, int64_t E, const int32_t* g2l, int32_t* lo, int32_t* hi, cudaStream_t s) {
  if (E <= 0) return LPG_OK;
  const int Np = (N + 1) * (N + 1) * (N + 1);
  const int64_t blocks = std::min<int64_t>((E + 7) / 8, 152 * 16);
  element_dof_range_kernel<<<(unsigned)blocks, 256, 0, s>>>(Np, E, g2l, lo, hi);
  LPG_LAUNCH_CHECK("element_dof_range_kernel");
  return LPG_OK;
}

}  // namespace lpg
