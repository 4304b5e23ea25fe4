// Interior-penalty DG discretisation of the screened Poisson operator on hexahedra
// (DISCRETIZATION = IPDG): geometry, gradient, operator, boundary data of the rhs and
// the operator diagonal.
//
// Reference: ellipticGradientHex3D.okl, ellipticAxIpdgHex3D.okl:34-84 (surface terms with
// the homogeneous Dirichlet / Neumann mirror states of ellipticBoundary3D.h) and :363-642
// (weak divergence), ellipticRhsBCIpdgHex3D.okl (boundary data), meshSurfaceGeometricFactors
// Hex3D.cpp:31-175 (normals, WsJ, penalty scale), ellipticBuildOperatorDiagonal.cpp:874-990.
//
// Layout (per element, structure of arrays): vgeo [e][10][Np] = rx ry rz sx sy sz tx ty tz JW;
// sgeo [e][5][6 Nfp] = nx ny nz WsJ hinv for the face nodes of faces 0..5 (local index order);
// gradients [E Np] double4_32a = (qx, qy, qz, q). The FP32 preconditioner levels run the same
// gradient and operator kernels on FP32 copies of vgeo and sgeo with float4 gradients.
//
// Kernels run one CTA per element with one thread per node. A node owns its accumulators:
// the face terms of every face it lies on are added by that node's thread, in the face
// order 0, 5, 1, 3, 2, 4, so no two threads write the same value.
#include <type_traits>

#include "df64.cuh"
#include "lpg_common.cuh"
#include "lpg_internal.hpp"

namespace lpg {

namespace {

constexpr int kVgeo = 10;   // rx ry rz sx sy sz tx ty tz JW
constexpr int kSgeo = 5;    // nx ny nz WsJ hinv

__device__ __forceinline__ void node_coords(const double* ev, double r, double s, double t, double& x, double& y,
                                            double& z) {
  const double c[8] = {(1 - r) * (1 - s) * (1 - t), (1 + r) * (1 - s) * (1 - t), (1 + r) * (1 + s) * (1 - t),
                       (1 - r) * (1 + s) * (1 - t), (1 - r) * (1 - s) * (1 + t), (1 + r) * (1 - s) * (1 + t),
                       (1 + r) * (1 + s) * (1 + t), (1 - r) * (1 + s) * (1 + t)};
  x = y = z = 0;
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    x += 0.125 * c[v] * ev[v];
    y += 0.125 * c[v] * ev[8 + v];
    z += 0.125 * c[v] * ev[16 + v];
  }
}

// face index b of node (i,j,k) on face f (faces 0..5 = t-, s-, r+, s+, r-, t+)
template <int NQ>
__device__ __forceinline__ int face_slot(int f, int i, int j, int k) {
  return (f == 0 || f == 5) ? i + j * NQ : (f == 1 || f == 3) ? i + k * NQ : j + k * NQ;
}

// volume node of face slot b on face f (the inverse of face_slot)
template <int NQ>
__device__ __forceinline__ int face_node(int f, int b) {
  constexpr int NFP = NQ * NQ;
  const int a = b % NQ, c = b / NQ;
  switch (f) {
    case 0: return b;
    case 5: return b + (NQ - 1) * NFP;
    case 1: return a + c * NFP;
    case 3: return a + (NQ - 1) * NQ + c * NFP;
    case 2: return (NQ - 1) + a * NQ + c * NFP;
    default: return a * NQ + c * NFP;   // face 4
  }
}

// face of the opposite-face pair handled in phase ph (pairs (0,5), (1,3), (2,4)) by half h
__device__ __forceinline__ int phase_face(int ph, int h) {
  return ph == 0 ? (h ? 5 : 0) : ph == 1 ? (h ? 3 : 1) : (h ? 4 : 2);
}

// Dynamic shared memory of the ax kernels (S = value, S4 = 4-vector): own traces, node
// accumulators, the neighbour traces and surface factors of the 6 Nfp face slots (slot
// t = phase * 2 Nfp + half * Nfp + b, the order the face phases use), and D.
template <int NQ, typename S, typename S4>
struct AxSmem {
  static constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ, NS = 6 * NFP;
  static constexpr size_t oM = 0;
  static constexpr size_t oAcc = oM + sizeof(S4) * NP;
  static constexpr size_t oP = oAcc + sizeof(S4) * NP;
  static constexpr size_t oF = oP + sizeof(S4) * NS;
  static constexpr size_t oD = oF + sizeof(S) * 5 * NS;
  static constexpr size_t bytes = oD + sizeof(S) * NFP;
};

// slot t -> (face, face slot b)
template <int NQ>
__device__ __forceinline__ void slot_face(int t, int& f, int& b) {
  constexpr int NFP = NQ * NQ;
  const int ph = t / (2 * NFP), r = t - ph * 2 * NFP, h = r / NFP;
  f = phase_face(ph, h);
  b = r - h * NFP;
}

// ---------------------------------------------------------------- geometry
template <int NQ>
__global__ void __launch_bounds__(NQ * NQ * NQ)
ipdg_geometry_kernel(const double* __restrict__ EX, const double* __restrict__ EY, const double* __restrict__ EZ,
                     const double* __restrict__ Dg, const double* __restrict__ r1d, const double* __restrict__ w1d,
                     double* __restrict__ vgeo, double* __restrict__ sgeo, double* __restrict__ hfac) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ;
  __shared__ double s_x[NP], s_y[NP], s_z[NP], s_D[NQ * NQ], s_ev[24];
  const int64_t e = blockIdx.x;
  const int n = threadIdx.x;
  if (n < NQ * NQ) s_D[n] = Dg[n];
  if (n < 8) { s_ev[n] = EX[e * 8 + n]; s_ev[8 + n] = EY[e * 8 + n]; s_ev[16 + n] = EZ[e * 8 + n]; }
  __syncthreads();
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / NFP;
  node_coords(s_ev, r1d[i], r1d[j], r1d[k], s_x[n], s_y[n], s_z[n]);
  __syncthreads();
  double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
#pragma unroll
  for (int m = 0; m < NQ; ++m) {
    const int ir = m + j * NQ + k * NFP, is = i + m * NQ + k * NFP, it = i + j * NQ + m * NFP;
    const double dr = s_D[i * NQ + m], ds = s_D[j * NQ + m], dt = s_D[k * NQ + m];
    xr += dr * s_x[ir]; xs += ds * s_x[is]; xt += dt * s_x[it];
    yr += dr * s_y[ir]; ys += ds * s_y[is]; yt += dt * s_y[it];
    zr += dr * s_z[ir]; zs += ds * s_z[is]; zt += dt * s_z[it];
  }
  const double J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
  const double g[9] = {(ys * zt - zs * yt) / J,  -(xs * zt - zs * xt) / J, (xs * yt - ys * xt) / J,
                       -(yr * zt - zr * yt) / J, (xr * zt - zr * xt) / J,  -(xr * yt - yr * xt) / J,
                       (yr * zs - zr * ys) / J,  -(xr * zs - zr * xs) / J, (xr * ys - yr * xs) / J};
  double* vg = vgeo + e * kVgeo * NP;
#pragma unroll
  for (int c = 0; c < 9; ++c) vg[c * NP + n] = g[c];
  vg[9 * NP + n] = J * w1d[i] * w1d[j] * w1d[k];
  // face factors of every face this node lies on
  double* sg = sgeo + e * kSgeo * 6 * NFP;
  const int faces[6] = {k == 0 ? 0 : -1, k == NQ - 1 ? 5 : -1, j == 0 ? 1 : -1,
                        j == NQ - 1 ? 3 : -1, i == NQ - 1 ? 2 : -1, i == 0 ? 4 : -1};
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int f = faces[q];
    if (f < 0) continue;
    // outward normal direction +-(grad r | grad s | grad t)
    const int c0 = (f == 0 || f == 5) ? 6 : (f == 1 || f == 3) ? 3 : 0;
    const double sgn = (f == 0 || f == 1 || f == 4) ? -1.0 : 1.0;
    const double nx = sgn * g[c0], ny = sgn * g[c0 + 1], nz = sgn * g[c0 + 2];
    const double len = sqrt(nx * nx + ny * ny + nz * nz);
    const double sJ = len * J;
    const int b = face_slot<NQ>(f, i, j, k);
    const int col = f * NFP + b;
    const double wa = w1d[b % NQ], wb = w1d[b / NQ];
    sg[0 * 6 * NFP + col] = nx / len;
    sg[1 * 6 * NFP + col] = ny / len;
    sg[2 * 6 * NFP + col] = nz / len;
    sg[3 * 6 * NFP + col] = sJ * wa * wb;
    hfac[e * 6 * NFP + col] = sJ / J;
  }
}

// hinv = max(sJ/J) over the two sides of each face node (meshSurfaceGeometricFactorsHex3D.cpp:160-172)
__global__ void ipdg_hinv_kernel(const int64_t nFaceNodes, const int nfpAll, const double* __restrict__ hfac,
                                 const int32_t* __restrict__ mapP, double* __restrict__ sgeo) {
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < nFaceNodes;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = id / nfpAll;
    const int c = (int)(id % nfpAll);
    sgeo[(e * kSgeo + 4) * nfpAll + c] = fmax(hfac[id], hfac[mapP[id]]);
  }
}

// ---------------------------------------------------------------- gradient
// T = double (the operator) or float (the FP32 preconditioner levels); V4 the matching
// 4-vector (double4_32a, float4)
template <int NQ, typename T, typename V4>
__global__ void __launch_bounds__(NQ * NQ * NQ)
ipdg_gradient_kernel(const T* __restrict__ vgeo, const T* __restrict__ Dg, const T* __restrict__ q,
                     V4* __restrict__ g4) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ;
  __shared__ T s_q[NP], s_D[NQ * NQ];
  const int64_t e = blockIdx.x;
  const int n = threadIdx.x;
  if (n < NQ * NQ) s_D[n] = Dg[n];
  s_q[n] = q[e * NP + n];
  __syncthreads();
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / NFP;
  T qr = 0, qs = 0, qt = 0;
#pragma unroll
  for (int m = 0; m < NQ; ++m) {
    qr += s_D[i * NQ + m] * s_q[m + j * NQ + k * NFP];
    qs += s_D[j * NQ + m] * s_q[i + m * NQ + k * NFP];
    qt += s_D[k * NQ + m] * s_q[i + j * NQ + m * NFP];
  }
  const T* vg = vgeo + e * kVgeo * NP + n;
  V4 o;
  o.x = vg[0 * NP] * qr + vg[3 * NP] * qs + vg[6 * NP] * qt;
  o.y = vg[1 * NP] * qr + vg[4 * NP] * qs + vg[7 * NP] * qt;
  o.z = vg[2 * NP] * qr + vg[5 * NP] * qs + vg[8 * NP] * qt;
  o.w = s_q[n];
  g4[e * NP + n] = o;
}

// FP64 gradient with the even-odd split of D (Nq even; D[N-a][N-m] = -D[a][m] on GLL
// points). Along each direction node i and its mirror N-i form a pair: with e_m = q_m +
// q_{N-m}, o_m = q_m - q_{N-m} (m < Nq/2) and Dp, Dm the even and odd halves of D, the
// lower node of the pair dots row min(i, N-i) of Dp with e, the upper one that row of Dm
// with o, and the partial sums A, B are exchanged through shared memory: d(i) = A + B,
// d(N-i) = B - A. Per node and direction: 1 + Nq/2 + 1 FP64 instructions instead of Nq.
// Every selection between the two halves is an index, so warps do not diverge.
template <int NQ>
__global__ void __launch_bounds__(NQ * NQ * NQ)
ipdg_gradient_eo_kernel(const double* __restrict__ vgeo, const double* __restrict__ Dg,
                        const double* __restrict__ q, double4_32a* __restrict__ g4) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ, H = NQ / 2, N = NQ - 1;
  static_assert(NQ % 2 == 0, "even-odd gradient: Nq even");
  __shared__ double s_q[NP];
  __shared__ double s_eo[3][NP];       // e (lower half of each line) / o (upper half) per direction
  __shared__ double s_x[3][NP];        // partial sums for the pair exchange
  __shared__ double s_DpDm[2 * H * H]; // rows of Dp, then rows of Dm
  const int64_t e = blockIdx.x;
  const int n = threadIdx.x;
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / NFP;
  if (n < H * H) {
    const int a = n / H, m = n % H;
    const double d0 = Dg[a * NQ + m], d1 = Dg[a * NQ + N - m];
    s_DpDm[n] = 0.5 * (d0 + d1);
    s_DpDm[H * H + n] = 0.5 * (d0 - d1);
  }
  const double qn = q[e * NP + n];
  s_q[n] = qn;
  __syncthreads();
  // mirror nodes along r, s, t and the sign that forms e (lower half) or o (upper half)
  const int pi = n + (N - 2 * i), pj = n + (N - 2 * j) * NQ, pk = n + (N - 2 * k) * NFP;
  const double si = i < H ? 1.0 : -1.0, sj = j < H ? 1.0 : -1.0, sk = k < H ? 1.0 : -1.0;
  s_eo[0][n] = fma(si, qn, s_q[pi]);   // i < H: e_i;  i >= H: o_{N-i} = q_{N-i} - q_i
  s_eo[1][n] = fma(sj, qn, s_q[pj]);
  s_eo[2][n] = fma(sk, qn, s_q[pk]);
  __syncthreads();
  const double* ci = s_DpDm + (i < H ? i * H : H * H + (N - i) * H);
  const double* cj = s_DpDm + (j < H ? j * H : H * H + (N - j) * H);
  const double* ck = s_DpDm + (k < H ? k * H : H * H + (N - k) * H);
  double ar = 0, as = 0, at = 0;
#pragma unroll
  for (int m = 0; m < H; ++m) {
    // e_m sits at line position m, o_m at position N - m
    const int mi = i < H ? m : N - m, mj = j < H ? m : N - m, mk = k < H ? m : N - m;
    ar = fma(ci[m], s_eo[0][mi + j * NQ + k * NFP], ar);
    as = fma(cj[m], s_eo[1][i + mj * NQ + k * NFP], as);
    at = fma(ck[m], s_eo[2][i + j * NQ + mk * NFP], at);
  }
  s_x[0][n] = ar;
  s_x[1][n] = as;
  s_x[2][n] = at;
  __syncthreads();
  const double qr = fma(si, s_x[0][pi], ar);   // lower: A + B, upper: B - A
  const double qs = fma(sj, s_x[1][pj], as);
  const double qt = fma(sk, s_x[2][pk], at);
  const double* vg = vgeo + e * kVgeo * NP + n;
  double4_32a o;
  o.x = vg[0 * NP] * qr + vg[3 * NP] * qs + vg[6 * NP] * qt;
  o.y = vg[1 * NP] * qr + vg[4 * NP] * qs + vg[7 * NP] * qt;
  o.z = vg[2 * NP] * qr + vg[5 * NP] * qs + vg[8 * NP] * qt;
  o.w = qn;
  g4[e * NP + n] = o;
}

// ---------------------------------------------------------------- weak divergence (shared by Ax and rhs)
// out_n = acc_n + sum_p D[p][i] ur(p,j,k) + D[p][j] us(i,p,k) + D[p][k] ut(i,j,p), with (ur, us, ut)
// = (grad r, grad s, grad t) . (gx, gy, gz)
template <int NQ, typename T>
__device__ __forceinline__ T weak_divergence(const T* vg, T gx, T gy, T gz, T acc, T* s_ur, T* s_us, T* s_ut,
                                             const T* s_D) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ;
  const int n = threadIdx.x;
  s_ur[n] = vg[0 * NP] * gx + vg[1 * NP] * gy + vg[2 * NP] * gz;
  s_us[n] = vg[3 * NP] * gx + vg[4 * NP] * gy + vg[5 * NP] * gz;
  s_ut[n] = vg[6 * NP] * gx + vg[7 * NP] * gy + vg[8 * NP] * gz;
  __syncthreads();
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / NFP;
  T v = acc;
#pragma unroll
  for (int p = 0; p < NQ; ++p) {
    v += s_D[p * NQ + i] * s_ur[p + j * NQ + k * NFP];
    v += s_D[p * NQ + j] * s_us[i + p * NQ + k * NFP];
    v += s_D[p * NQ + k] * s_ut[i + j * NQ + p * NFP];
  }
  return v;
}

// ---------------------------------------------------------------- operator
// The face terms run in three phases, one per opposite-face pair (0,5), (1,3), (2,4): the
// 2 Nfp face slots of a pair sit on consecutive threads (whole warps), no node lies on both
// faces of a pair, and the node accumulators live in shared memory, so every node receives
// its face terms in the reference's order 0,5,1,3,2,4 without divergent per-node face loops.
template <int NQ, typename T, typename V4>
__global__ void __launch_bounds__(NQ * NQ * NQ)
ipdg_ax_kernel(const T* __restrict__ vgeo, const T* __restrict__ sgeo, const int32_t* __restrict__ vmapP,
               const int* __restrict__ EToB, const T* __restrict__ Dg, const T lambda,
               const T* __restrict__ lambdaE, const T tau, const V4* __restrict__ g4, T* __restrict__ Aq) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ;
  static_assert(2 * NFP <= NP, "a face pair needs 2 Nfp threads");
  using L = AxSmem<NQ, T, V4>;
  extern __shared__ __align__(32) unsigned char smem[];
  V4* s_M = reinterpret_cast<V4*>(smem + L::oM);
  V4* s_acc = reinterpret_cast<V4*>(smem + L::oAcc);
  V4* s_P = reinterpret_cast<V4*>(smem + L::oP);
  T* s_F = reinterpret_cast<T*>(smem + L::oF);
  T* s_D = reinterpret_cast<T*>(smem + L::oD);
  const int64_t e = blockIdx.x;
  const int n = threadIdx.x;
  if (n < NQ * NQ) s_D[n] = Dg[n];
  // stage the surface factors and neighbour traces of all 6 Nfp face slots at once, so the
  // dependent vmapP -> trace loads are in flight together with the volume loads
  const T* sg = sgeo + e * kSgeo * 6 * NFP;
  for (int t = n; t < 6 * NFP; t += NP) {
    int f, b;
    slot_face<NQ>(t, f, b);
    const int col = f * NFP + b;
#pragma unroll
    for (int c = 0; c < kSgeo; ++c) s_F[c * 6 * NFP + t] = sg[c * 6 * NFP + col];
    s_P[t] = g4[vmapP[e * 6 * NFP + col]];
  }
  const T* vg = vgeo + e * kVgeo * NP + n;
  {
    const V4 GM = g4[e * NP + n];
    const T JW = vg[9 * NP];
    const T lam = lambdaE ? lambdaE[e] : lambda;
    V4 acc;
    acc.x = JW * GM.x;
    acc.y = JW * GM.y;
    acc.z = JW * GM.z;
    acc.w = JW * lam * GM.w;
    s_M[n] = GM;
    s_acc[n] = acc;
  }
  __syncthreads();
#pragma unroll
  for (int ph = 0; ph < 3; ++ph) {
    if (n < 2 * NFP) {
      const int t = ph * 2 * NFP + n;
      int f, b;
      slot_face<NQ>(t, f, b);
      const int node = face_node<NQ>(f, b);
      const T nx = s_F[0 * 6 * NFP + t], ny = s_F[1 * 6 * NFP + t], nz = s_F[2 * 6 * NFP + t];
      const T w = s_F[3 * 6 * NFP + t], hinv = s_F[4 * 6 * NFP + t];
      const V4 GM = s_M[node];
      V4 P = s_P[t];
      const int bc = EToB[e * 6 + f];
      if (bc > 0) {
        // homogeneous boundary state B (Dirichlet: q = 0, grad kept; Neumann: q kept, grad = 0),
        // then the mirror state 2B - M
        if (bc == 1) { P.x = GM.x; P.y = GM.y; P.z = GM.z; P.w = -GM.w; }
        else { P.x = -GM.x; P.y = -GM.y; P.z = -GM.z; P.w = GM.w; }
      }
      V4 acc = s_acc[node];
      const T dq = P.w - GM.w;
      acc.x += T(0.5) * w * nx * dq;
      acc.y += T(0.5) * w * ny * dq;
      acc.z += T(0.5) * w * nz * dq;
      acc.w += T(-0.5) * w * (nx * (P.x + GM.x) + ny * (P.y + GM.y) + nz * (P.z + GM.z) + tau * hinv * dq);
      s_acc[node] = acc;
    }
    __syncthreads();
  }
  const V4 acc = s_acc[n];
  T* s_w = reinterpret_cast<T*>(s_M);   // the traces are no longer read: 3 Np values of scratch
  Aq[e * NP + n] = weak_divergence<NQ, T>(vg, acc.x, acc.y, acc.z, acc.w, s_w, s_w + NP, s_w + 2 * NP, s_D);
}

// ---------------------------------------------------------------- double-word operator
// OPERATOR PRECISION = DF64: the gradient and operator kernels in double-FP32 words
// (df64.cuh) on the FP32 pipe, with vgeo and sgeo split once into (hi, lo) pairs and the
// gradients stored as four words per node (two float4: x.h x.l y.h y.l | z.h z.l w.h w.l).
// q is split by integer operations; each result is rebuilt as hi + lo in FP64.
struct dw4 {
  dw x, y, z, w;
};
__device__ __forceinline__ dw4 load_dw4(const float4* __restrict__ g, int64_t node) {
  const float4 a = g[2 * node], b = g[2 * node + 1];
  return {{a.x, a.y}, {a.z, a.w}, {b.x, b.y}, {b.z, b.w}};
}
__device__ __forceinline__ dw ldw(const float2* __restrict__ p) {
  const float2 v = *p;
  return {v.x, v.y};
}
__device__ __forceinline__ dw dw_half(float c, dw x) { return {c * x.h, c * x.l}; }   // c = +-0.5: exact

template <int NQ>
__global__ void __launch_bounds__(NQ * NQ * NQ, (NQ <= 8 ? 4 : 1))
ipdg_gradient_dw_kernel(const float2* __restrict__ vgeo, const double* __restrict__ Dg, const double* __restrict__ q,
                        float4* __restrict__ g8) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ;
  __shared__ dw s_q[NP], s_D[NQ * NQ];
  const int64_t e = blockIdx.x;
  const int n = threadIdx.x;
  if (n < NQ * NQ) s_D[n] = dw_from_double(Dg[n]);
  const dw qn = dw_from_double(q[e * NP + n]);
  s_q[n] = qn;
  __syncthreads();
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / NFP;
  dw_acc ar, as, at;
#pragma unroll
  for (int m = 0; m < NQ; ++m) {
    ar.mac(s_D[i * NQ + m], s_q[m + j * NQ + k * NFP]);
    as.mac(s_D[j * NQ + m], s_q[i + m * NQ + k * NFP]);
    at.mac(s_D[k * NQ + m], s_q[i + j * NQ + m * NFP]);
  }
  const dw qr = ar.get(), qs = as.get(), qt = at.get();
  const float2* vg = vgeo + e * kVgeo * NP + n;
  dw_acc ox, oy, oz;
  ox.mac(ldw(vg + 0 * NP), qr); ox.mac(ldw(vg + 3 * NP), qs); ox.mac(ldw(vg + 6 * NP), qt);
  oy.mac(ldw(vg + 1 * NP), qr); oy.mac(ldw(vg + 4 * NP), qs); oy.mac(ldw(vg + 7 * NP), qt);
  oz.mac(ldw(vg + 2 * NP), qr); oz.mac(ldw(vg + 5 * NP), qs); oz.mac(ldw(vg + 8 * NP), qt);
  const dw gx = ox.get(), gy = oy.get(), gz = oz.get();
  g8[2 * (e * NP + n)] = make_float4(gx.h, gx.l, gy.h, gy.l);
  g8[2 * (e * NP + n) + 1] = make_float4(gz.h, gz.l, qn.h, qn.l);
}

template <int NQ>
__global__ void __launch_bounds__(NQ * NQ * NQ, (NQ <= 8 ? 3 : 1))
ipdg_ax_dw_kernel(const float2* __restrict__ vgeo, const float2* __restrict__ sgeo, const int32_t* __restrict__ vmapP,
                  const int* __restrict__ EToB, const double* __restrict__ Dg, const double lambda,
                  const double* __restrict__ lambdaE, const double tau, const float4* __restrict__ g8,
                  double* __restrict__ Aq) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ;
  static_assert(2 * NFP <= NP, "a face pair needs 2 Nfp threads");
  using L = AxSmem<NQ, dw, dw4>;
  extern __shared__ __align__(32) unsigned char smem[];
  dw4* s_M = reinterpret_cast<dw4*>(smem + L::oM);
  dw4* s_acc = reinterpret_cast<dw4*>(smem + L::oAcc);
  dw4* s_P = reinterpret_cast<dw4*>(smem + L::oP);
  dw* s_F = reinterpret_cast<dw*>(smem + L::oF);
  dw* s_D = reinterpret_cast<dw*>(smem + L::oD);
  const int64_t e = blockIdx.x;
  const int n = threadIdx.x;
  if (n < NQ * NQ) s_D[n] = dw_from_double(Dg[n]);
  // stage surface factors and neighbour traces of all face slots, as in ipdg_ax_kernel
  const float2* sg = sgeo + e * kSgeo * 6 * NFP;
  for (int t = n; t < 6 * NFP; t += NP) {
    int f, b;
    slot_face<NQ>(t, f, b);
    const int col = f * NFP + b;
#pragma unroll
    for (int c = 0; c < kSgeo; ++c) s_F[c * 6 * NFP + t] = ldw(sg + c * 6 * NFP + col);
    s_P[t] = load_dw4(g8, vmapP[e * 6 * NFP + col]);
  }
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / NFP;
  const float2* vg = vgeo + e * kVgeo * NP + n;
  {
    const dw4 GM = load_dw4(g8, e * NP + n);
    const dw JW = ldw(vg + 9 * NP);
    const dw lam = dw_from_double(lambdaE ? lambdaE[e] : lambda);
    s_M[n] = GM;
    s_acc[n] = {dw_mul(JW, GM.x), dw_mul(JW, GM.y), dw_mul(JW, GM.z), dw_mul(dw_mul(JW, lam), GM.w)};
  }
  __syncthreads();
  // face terms by opposite-face pairs, as in ipdg_ax_kernel
  const dw tauw = dw_from_double(tau);
#pragma unroll
  for (int ph = 0; ph < 3; ++ph) {
    if (n < 2 * NFP) {
      const int t = ph * 2 * NFP + n;
      int f, b;
      slot_face<NQ>(t, f, b);
      const int node = face_node<NQ>(f, b);
      const dw nx = s_F[0 * 6 * NFP + t], ny = s_F[1 * 6 * NFP + t], nz = s_F[2 * 6 * NFP + t];
      const dw w = s_F[3 * 6 * NFP + t], hinv = s_F[4 * 6 * NFP + t];
      const dw4 GM = s_M[node];
      dw4 P = s_P[t];
      const int bc = EToB[e * 6 + f];
      if (bc > 0) {
        // mirror state 2B - M of the homogeneous boundary state (Dirichlet / Neumann)
        if (bc == 1) { P.x = GM.x; P.y = GM.y; P.z = GM.z; P.w = dw_neg(GM.w); }
        else { P.x = dw_neg(GM.x); P.y = dw_neg(GM.y); P.z = dw_neg(GM.z); P.w = GM.w; }
      }
      dw4 acc = s_acc[node];
      const dw dq = dw_sub(P.w, GM.w);
      const dw hwdq = dw_half(0.5f, dw_mul(w, dq));
      acc.x = dw_add(acc.x, dw_mul(nx, hwdq));
      acc.y = dw_add(acc.y, dw_mul(ny, hwdq));
      acc.z = dw_add(acc.z, dw_mul(nz, hwdq));
      dw_acc flux;
      flux.mac(nx, dw_add(P.x, GM.x));
      flux.mac(ny, dw_add(P.y, GM.y));
      flux.mac(nz, dw_add(P.z, GM.z));
      flux.mac(dw_mul(tauw, hinv), dq);
      acc.w = dw_add(acc.w, dw_half(-0.5f, dw_mul(w, flux.get())));
      s_acc[node] = acc;
    }
    __syncthreads();
  }
  const dw4 acc = s_acc[n];
  dw* s_ur = reinterpret_cast<dw*>(s_M);   // the traces are no longer read: 3 Np words of scratch
  dw* s_us = s_ur + NP;
  dw* s_ut = s_us + NP;
  // weak divergence
  {
    dw_acc r, s2, t;
    r.mac(ldw(vg + 0 * NP), acc.x); r.mac(ldw(vg + 1 * NP), acc.y); r.mac(ldw(vg + 2 * NP), acc.z);
    s2.mac(ldw(vg + 3 * NP), acc.x); s2.mac(ldw(vg + 4 * NP), acc.y); s2.mac(ldw(vg + 5 * NP), acc.z);
    t.mac(ldw(vg + 6 * NP), acc.x); t.mac(ldw(vg + 7 * NP), acc.y); t.mac(ldw(vg + 8 * NP), acc.z);
    s_ur[n] = r.get();
    s_us[n] = s2.get();
    s_ut[n] = t.get();
  }
  __syncthreads();
  dw_acc v;
  v.h = acc.w.h;
  v.l = acc.w.l;
#pragma unroll
  for (int p = 0; p < NQ; ++p) {
    v.mac(s_D[p * NQ + i], s_ur[p + j * NQ + k * NFP]);
    v.mac(s_D[p * NQ + j], s_us[i + p * NQ + k * NFP]);
    v.mac(s_D[p * NQ + k], s_ut[i + j * NQ + p * NFP]);
  }
  Aq[e * NP + n] = dw_to_double(v.get());
}

// ---------------------------------------------------------------- rhs boundary data
// rhs -= weak form of the boundary state of u = sin(pi x) sin(pi y) sin(pi z) (Dirichlet value,
// or the Neumann data of the sine data file) against a zero interior state
template <int NQ>
__global__ void __launch_bounds__(NQ * NQ * NQ)
ipdg_rhs_bc_kernel(const double* __restrict__ EX, const double* __restrict__ EY, const double* __restrict__ EZ,
                   const double* __restrict__ r1d, const double* __restrict__ vgeo, const double* __restrict__ sgeo,
                   const int* __restrict__ EToB, const double* __restrict__ Dg, const double tau,
                   double* __restrict__ rhs) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ;
  __shared__ double s_ur[NP], s_us[NP], s_ut[NP], s_D[NQ * NQ], s_ev[24];
  __shared__ int s_any;
  const int64_t e = blockIdx.x;
  const int n = threadIdx.x;
  if (n == 0) {
    int any = 0;
    for (int f = 0; f < 6; ++f) any |= (EToB[e * 6 + f] > 0);
    s_any = any;
  }
  if (n < NQ * NQ) s_D[n] = Dg[n];
  if (n < 8) { s_ev[n] = EX[e * 8 + n]; s_ev[8 + n] = EY[e * 8 + n]; s_ev[16 + n] = EZ[e * 8 + n]; }
  __syncthreads();
  if (!s_any) return;   // uniform over the block
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / NFP;
  double x, y, z;
  node_coords(s_ev, r1d[i], r1d[j], r1d[k], x, y, z);
  double gx = 0, gy = 0, gz = 0, a = 0;
  const double* sg = sgeo + e * kSgeo * 6 * NFP;
  const int faces[6] = {k == 0 ? 0 : -1, k == NQ - 1 ? 5 : -1, j == 0 ? 1 : -1,
                        j == NQ - 1 ? 3 : -1, i == NQ - 1 ? 2 : -1, i == 0 ? 4 : -1};
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int f = faces[q];
    if (f < 0) continue;
    const int bc = EToB[e * 6 + f];
    if (bc <= 0) continue;
    const int col = f * NFP + face_slot<NQ>(f, i, j, k);
    const double nx = sg[0 * 6 * NFP + col], ny = sg[1 * 6 * NFP + col], nz = sg[2 * 6 * NFP + col];
    const double w = sg[3 * 6 * NFP + col], hinv = sg[4 * 6 * NFP + col];
    double qP = 0, dx = 0, dy = 0, dz = 0;
    const double sx = sin(LPG_PI * x), sy = sin(LPG_PI * y), sz = sin(LPG_PI * z);
    if (bc == 1) qP = sx * sy * sz;
    else {
      dx = -LPG_PI * cos(LPG_PI * x) * sy * sz;
      dy = -LPG_PI * sx * cos(LPG_PI * y) * sz;
      dz = -LPG_PI * sx * sy * cos(LPG_PI * z);
    }
    gx += w * nx * qP;
    gy += w * ny * qP;
    gz += w * nz * qP;
    a += -w * (nx * dx + ny * dy + nz * dz + tau * hinv * qP);
  }
  const double* vg = vgeo + e * kVgeo * NP + n;
  rhs[e * NP + n] -= weak_divergence<NQ, double>(vg, gx, gy, gz, a, s_ur, s_us, s_ut, s_D);
}

// ---------------------------------------------------------------- diagonal
template <int NQ>
__global__ void __launch_bounds__(NQ * NQ * NQ)
ipdg_diag_kernel(const double* __restrict__ vgeo, const double* __restrict__ sgeo, const int* __restrict__ EToB,
                 const double* __restrict__ Dg, const double lambda, const double* __restrict__ lambdaE,
                 const double tau, double* __restrict__ diag) {
  constexpr int NP = NQ * NQ * NQ, NFP = NQ * NQ;
  __shared__ double s_D[NQ * NQ];
  const int64_t e = blockIdx.x;
  const int n = threadIdx.x;
  if (n < NQ * NQ) s_D[n] = Dg[n];
  __syncthreads();
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / NFP;
  const double* vg = vgeo + e * kVgeo * NP;
  const double lam = lambdaE ? lambdaE[e] : lambda;
  // (grad l_n, grad l_n) over the nodes of the three lines through n, + lambda (l_n, l_n)
  double A = lam * vg[9 * NP + n];
  for (int p = 0; p < NQ; ++p) {
    // r-line (p, j, k), s-line (i, p, k), t-line (i, j, p); node n itself carries all three
    const int pr = p + j * NQ + k * NFP, ps = i + p * NQ + k * NFP, pt = i + j * NQ + p * NFP;
    {
      const double br = s_D[p * NQ + i];
      const double bs = (p == i) ? s_D[j * NQ + j] : 0.0, bt = (p == i) ? s_D[k * NQ + k] : 0.0;
      const double dx = vg[0 * NP + pr] * br + vg[3 * NP + pr] * bs + vg[6 * NP + pr] * bt;
      const double dy = vg[1 * NP + pr] * br + vg[4 * NP + pr] * bs + vg[7 * NP + pr] * bt;
      const double dz = vg[2 * NP + pr] * br + vg[5 * NP + pr] * bs + vg[8 * NP + pr] * bt;
      A += vg[9 * NP + pr] * (dx * dx + dy * dy + dz * dz);
    }
    if (p != j) {
      const double bs = s_D[p * NQ + j];
      const double dx = vg[3 * NP + ps] * bs, dy = vg[4 * NP + ps] * bs, dz = vg[5 * NP + ps] * bs;
      A += vg[9 * NP + ps] * (dx * dx + dy * dy + dz * dz);
    }
    if (p != k) {
      const double bt = s_D[p * NQ + k];
      const double dx = vg[6 * NP + pt] * bt, dy = vg[7 * NP + pt] * bt, dz = vg[8 * NP + pt] * bt;
      A += vg[9 * NP + pt] * (dx * dx + dy * dy + dz * dz);
    }
  }
  // face terms at n itself: -2 c (n . grad l_n) + c tau hinv, c = (1 + D)(1 - N) WsJ / 2
  const double* sg = sgeo + e * kSgeo * 6 * NFP;
  const double dlx = vg[0 * NP + n] * s_D[i * NQ + i] + vg[3 * NP + n] * s_D[j * NQ + j] + vg[6 * NP + n] * s_D[k * NQ + k];
  const double dly = vg[1 * NP + n] * s_D[i * NQ + i] + vg[4 * NP + n] * s_D[j * NQ + j] + vg[7 * NP + n] * s_D[k * NQ + k];
  const double dlz = vg[2 * NP + n] * s_D[i * NQ + i] + vg[5 * NP + n] * s_D[j * NQ + j] + vg[8 * NP + n] * s_D[k * NQ + k];
  const int faces[6] = {k == 0 ? 0 : -1, j == 0 ? 1 : -1, i == NQ - 1 ? 2 : -1,
                        j == NQ - 1 ? 3 : -1, i == 0 ? 4 : -1, k == NQ - 1 ? 5 : -1};
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int f = faces[q];
    if (f < 0) continue;
    const int col = f * NFP + face_slot<NQ>(f, i, j, k);
    const int bc = EToB[e * 6 + f];
    const int bcD = (bc == 1), bcN = (bc > 0 && bc != 1);
    const double c = 0.5 * (1 + bcD) * (1 - bcN) * sg[3 * 6 * NFP + col];
    const double ndg = sg[0 * 6 * NFP + col] * dlx + sg[1 * 6 * NFP + col] * dly + sg[2 * 6 * NFP + col] * dlz;
    A += -c * ndg - c * ndg + c * tau * sg[4 * 6 * NFP + col];
  }
  diag[e * NP + n] = A;
}

template <int NQ, typename T, typename V4>
int launch_operator(int64_t E, const T* vgeo, const T* sgeo, const int32_t* vmapP, const int* EToB, const T* D,
                    T lambda, const T* lambdaE, T tau, const T* q, V4* g4, T* out, cudaStream_t s) {
  constexpr int NP = NQ * NQ * NQ;
  if (E <= 0) return LPG_OK;
  if constexpr (std::is_same<T, double>::value && NQ % 2 == 0) {
    ipdg_gradient_eo_kernel<NQ><<<(unsigned)E, NP, 0, s>>>(vgeo, D, q, g4);
    LPG_LAUNCH_CHECK("ipdg_gradient_eo_kernel");
  } else {
    ipdg_gradient_kernel<NQ, T, V4><<<(unsigned)E, NP, 0, s>>>(vgeo, D, q, g4);
    LPG_LAUNCH_CHECK("ipdg_gradient_kernel");
  }
  constexpr size_t smem = AxSmem<NQ, T, V4>::bytes;
  static PerDeviceConfig perDevice;   // per instantiation: dynamic shared memory opt-in
  KernelConfig cfg;
  const int rc = perDevice.get(
      [&](int, KernelConfig&) {
        LPG_CUDA_TRY(cudaFuncSetAttribute(ipdg_ax_kernel<NQ, T, V4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        return (int)LPG_OK;
      },
      &cfg);
  if (rc) return rc;
  ipdg_ax_kernel<NQ, T, V4><<<(unsigned)E, NP, smem, s>>>(vgeo, sgeo, vmapP, EToB, D, lambda, lambdaE, tau, g4, out);
  LPG_LAUNCH_CHECK("ipdg_ax_kernel");
  return LPG_OK;
}

template <int NQ>
int launch_all(int which, const IpdgArgs& a, cudaStream_t s) {
  constexpr int NP = NQ * NQ * NQ;
  const unsigned E = (unsigned)a.E;
  if (a.E <= 0) return LPG_OK;
  switch (which) {
    case 0:
      ipdg_geometry_kernel<NQ><<<E, NP, 0, s>>>(a.EX, a.EY, a.EZ, a.D, a.r1d, a.w1d, a.vgeo, a.sgeo, a.hfac);
      LPG_LAUNCH_CHECK("ipdg_geometry_kernel");
      return LPG_OK;
    case 1:
      return launch_operator<NQ, double, double4_32a>(a.E, a.vgeo, a.sgeo, a.vmapP, a.EToB, a.D, a.lambda, a.lambdaE,
                                                      a.tau, a.q, a.g4, a.out, s);
    case 2:
      ipdg_rhs_bc_kernel<NQ><<<E, NP, 0, s>>>(a.EX, a.EY, a.EZ, a.r1d, a.vgeo, a.sgeo, a.EToB, a.D, a.tau, a.out);
      LPG_LAUNCH_CHECK("ipdg_rhs_bc_kernel");
      return LPG_OK;
    default:
      ipdg_diag_kernel<NQ><<<E, NP, 0, s>>>(a.vgeo, a.sgeo, a.EToB, a.D, a.lambda, a.lambdaE, a.tau, a.out);
      LPG_LAUNCH_CHECK("ipdg_diag_kernel");
      return LPG_OK;
  }
}

int dispatch(int which, const IpdgArgs& a, cudaStream_t s) {
  switch (a.N) {
    case 1: return launch_all<2>(which, a, s);
    case 2: return launch_all<3>(which, a, s);
    case 3: return launch_all<4>(which, a, s);
    case 4: return launch_all<5>(which, a, s);
    case 5: return launch_all<6>(which, a, s);
    case 6: return launch_all<7>(which, a, s);
    case 7: return launch_all<8>(which, a, s);
    case 8: return launch_all<9>(which, a, s);
    default: return set_error(LPG_ERR_UNSUPPORTED, "IPDG: N must be 1..8");
  }
}

}  // namespace

int ipdg_geometry(const IpdgArgs& a, const int32_t* mapP, cudaStream_t s) {
  int rc = dispatch(0, a, s);
  if (rc) return rc;
  const int nfpAll = 6 * (a.N + 1) * (a.N + 1);
  const int64_t nf = a.E * nfpAll;
  if (nf <= 0) return LPG_OK;
  const int64_t blocks = std::min<int64_t>((nf + 255) / 256, 152 * 16);
  ipdg_hinv_kernel<<<(unsigned)blocks, 256, 0, s>>>(nf, nfpAll, a.hfac, mapP, a.sgeo);
  LPG_LAUNCH_CHECK("ipdg_hinv_kernel");
  return LPG_OK;
}
int ipdg_operator(const IpdgArgs& a, cudaStream_t s) { return dispatch(1, a, s); }
int ipdg_operator_dw(const IpdgArgsDW& a, cudaStream_t s) {
  auto go = [&](auto nq) {
    constexpr int NQ = decltype(nq)::value;
    constexpr int NP = NQ * NQ * NQ;
    if (a.E <= 0) return (int)LPG_OK;
    const unsigned E = (unsigned)a.E;
    ipdg_gradient_dw_kernel<NQ><<<E, NP, 0, s>>>(a.vgeo, a.D, a.q, a.g8);
    LPG_LAUNCH_CHECK("ipdg_gradient_dw_kernel");
    constexpr size_t smem = AxSmem<NQ, dw, dw4>::bytes;
    static PerDeviceConfig perDevice;   // per instantiation: dynamic shared memory opt-in
    KernelConfig cfg;
    const int rc = perDevice.get(
        [&](int, KernelConfig&) {
          LPG_CUDA_TRY(cudaFuncSetAttribute(ipdg_ax_dw_kernel<NQ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
          return (int)LPG_OK;
        },
        &cfg);
    if (rc) return rc;
    ipdg_ax_dw_kernel<NQ><<<E, NP, smem, s>>>(a.vgeo, a.sgeo, a.vmapP, a.EToB, a.D, a.lambda, a.lambdaE, a.tau, a.g8,
                                              a.out);
    LPG_LAUNCH_CHECK("ipdg_ax_dw_kernel");
    return (int)LPG_OK;
  };
  switch (a.N) {
    case 1: return go(std::integral_constant<int, 2>{});
    case 2: return go(std::integral_constant<int, 3>{});
    case 3: return go(std::integral_constant<int, 4>{});
    case 4: return go(std::integral_constant<int, 5>{});
    case 5: return go(std::integral_constant<int, 6>{});
    case 6: return go(std::integral_constant<int, 7>{});
    case 7: return go(std::integral_constant<int, 8>{});
    case 8: return go(std::integral_constant<int, 9>{});
    default: return set_error(LPG_ERR_UNSUPPORTED, "IPDG: N must be 1..8");
  }
}
int ipdg_operator_f32(const IpdgArgsF32& a, cudaStream_t s) {
  auto go = [&](auto nq) {
    constexpr int NQ = decltype(nq)::value;
    return launch_operator<NQ, float, float4>(a.E, a.vgeo, a.sgeo, a.vmapP, a.EToB, a.D, a.lambda, a.lambdaE, a.tau,
                                              a.q, a.g4, a.out, s);
  };
  switch (a.N) {
    case 1: return go(std::integral_constant<int, 2>{});
    case 2: return go(std::integral_constant<int, 3>{});
    case 3: return go(std::integral_constant<int, 4>{});
    case 4: return go(std::integral_constant<int, 5>{});
    case 5: return go(std::integral_constant<int, 6>{});
    case 6: return go(std::integral_constant<int, 7>{});
    case 7: return go(std::integral_constant<int, 8>{});
    case 8: return go(std::integral_constant<int, 9>{});
    default: return set_error(LPG_ERR_UNSUPPORTED, "IPDG: N must be 1..8");
  }
}
int ipdg_rhs_bc(const IpdgArgs& a, cudaStream_t s) { return dispatch(2, a, s); }
int ipdg_diagonal(const IpdgArgs& a, cudaStream_t s) { return dispatch(3, a, s); }

}  // namespace lpg
