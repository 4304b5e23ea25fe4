// Element partition of a box mesh and the halo lists of its assembled dofs, for callers
// that split the operator across ranks (one process per GPU) the way elliptic_t::Operator
// does with MPI (solvers/elliptic/src/ellipticOperator.cpp:29-106: partial Ax on the rank's
// elements, then the ogs gather whose exchange adds the other ranks' contributions to the
// shared dofs; include/ogs.hpp:347-400 halo_t).
//
// Partition: slabs of whole element layers along z. Rank r gets nz_r = NZ/P + (r < NZ%P)
// layers (the reference's per-rank count for a given global size, meshSetupBoxHex3D.cpp:
// 63-69, applied to the z direction alone), i.e. the contiguous element range [e0, e1) of
// the single-rank element order (x fastest, then y, then z).
//
// Local numbering of rank r: the assembled dofs its elements touch, identified by their
// global lattice node (X, Y, Z), X = ex*N + a in [0, nx*N], ... Dofs the rank owns come
// first, then its halo dofs, each group in lattice order (X fastest). The lattice plane
// between slabs r and r+1 is owned by r and is a halo of r+1. Dirichlet boxes mask every
// boundary lattice node (as the single-rank numbering does); Neumann boxes mask none.
// Periodic boxes are not partitioned.
//
// Exchange lists: `above` (rank r < P-1) lists rank r's local indices of the plane it
// shares with r+1, `below` (rank r > 0) rank r's local indices of the plane it shares with
// r-1, both in lattice order of that plane, so rank r's `above` and rank r+1's `below`
// pair entry by entry. After each rank has assembled its own elements' contributions, the
// exchange (pack at one list, send, receive, add at the same list) gives both ranks the
// full sums on the shared plane.
#include <cstring>
#include <new>
#include <vector>

#include "../../../include/lpg.h"
#include "../lpg_errors.hpp"

namespace {

struct Part {
  int64_t e0 = 0, e1 = 0, nowned = 0, nlocal = 0;
  std::vector<int32_t> g2l, below, above;
  std::vector<int64_t> lattice;
};

int build(int nx, int ny, int nz, int N, int bcflag, int nranks, int rank, bool maps, Part& p) {
  using lpg::set_error;
  if (nx < 1 || ny < 1 || nz < 1 || N < 1 || N > 8) return set_error(LPG_ERR_INVALID, "box partition: bad box or degree");
  if (bcflag != 1 && bcflag != 2)
    return set_error(LPG_ERR_UNSUPPORTED, "box partition: boundary flag 1 (Dirichlet) or 2 (Neumann) only");
  if (nranks < 1 || rank < 0 || rank >= nranks || nz < nranks)
    return set_error(LPG_ERR_INVALID, "box partition: need 0 <= rank < nranks <= BOX NZ");
  const int64_t NX = (int64_t)nx * N + 1, NY = (int64_t)ny * N + 1, NZ = (int64_t)nz * N + 1;
  if (NX * NY * NZ > INT32_MAX) return set_error(LPG_ERR_UNSUPPORTED, "box partition: more than 2^31 lattice nodes");
  int z0 = 0;
  for (int q = 0; q < rank; ++q) z0 += nz / nranks + (q < nz % nranks ? 1 : 0);
  const int z1 = z0 + nz / nranks + (rank < nz % nranks ? 1 : 0);
  p.e0 = (int64_t)z0 * nx * ny;
  p.e1 = (int64_t)z1 * nx * ny;
  const bool dir = (bcflag == 1);
  auto masked = [&](int64_t X, int64_t Y, int64_t Z) {
    return dir && (X == 0 || X == NX - 1 || Y == 0 || Y == NY - 1 || Z == 0 || Z == NZ - 1);
  };
  // local lattice planes Z in [Zlo, Zhi]; the halo plane Zlo (rank > 0) comes last
  const int64_t Zlo = (int64_t)z0 * N, Zhi = (int64_t)z1 * N;
  const int64_t Zown0 = rank > 0 ? Zlo + 1 : Zlo;
  const int64_t planes = Zhi - Zlo + 1;
  std::vector<int32_t> idx(maps ? (size_t)(NX * NY * planes) : 0, -1);
  int64_t n = 0;
  auto visit = [&](int64_t Z) {
    for (int64_t Y = 0; Y < NY; ++Y)
      for (int64_t X = 0; X < NX; ++X) {
        if (masked(X, Y, Z)) continue;
        if (maps) {
          idx[(size_t)(((Z - Zlo) * NY + Y) * NX + X)] = (int32_t)n;
          p.lattice.push_back(X + NX * (Y + NY * Z));
        }
        ++n;
      }
  };
  for (int64_t Z = Zown0; Z <= Zhi; ++Z) visit(Z);
  p.nowned = n;
  if (rank > 0) visit(Zlo);
  p.nlocal = n;
  if (!maps) {
    // list lengths: one unmasked plane
    int64_t plane = 0;
    for (int64_t Y = 0; Y < NY; ++Y)
      for (int64_t X = 0; X < NX; ++X) plane += masked(X, Y, 1) ? 0 : 1;
    p.below.resize(rank > 0 ? plane : 0);
    p.above.resize(rank < nranks - 1 ? plane : 0);
    return LPG_OK;
  }
  auto plane_list = [&](int64_t Z, std::vector<int32_t>& out) {
    for (int64_t Y = 0; Y < NY; ++Y)
      for (int64_t X = 0; X < NX; ++X)
        if (!masked(X, Y, Z)) out.push_back(idx[(size_t)(((Z - Zlo) * NY + Y) * NX + X)]);
  };
  if (rank > 0) plane_list(Zlo, p.below);
  if (rank < nranks - 1) plane_list(Zhi, p.above);
  const int Nq = N + 1, Np = Nq * Nq * Nq;
  p.g2l.resize((size_t)((p.e1 - p.e0) * Np));
  for (int64_t e = p.e0; e < p.e1; ++e) {
    const int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / ((int64_t)nx * ny);
    for (int c = 0; c < Nq; ++c)
      for (int b = 0; b < Nq; ++b)
        for (int a = 0; a < Nq; ++a) {
          const int64_t X = ex * N + a, Y = ey * N + b, Z = ez * N + c;
          p.g2l[(size_t)((e - p.e0) * Np + a + Nq * (b + Nq * c))] =
              idx[(size_t)(((Z - Zlo) * NY + Y) * NX + X)];
        }
  }
  return LPG_OK;
}

}  // namespace

extern "C" int lpg_box_partition(int nx, int ny, int nz, int N, int bcflag, int nranks, int rank, int64_t* info,
                                 int32_t* global_to_local, int32_t* below, int32_t* above, int64_t* lattice) {
  if (!info) return lpg::set_error(LPG_ERR_INVALID, "box partition: info is required");
  try {
    Part p;
    const bool maps = global_to_local || below || above || lattice;
    int rc = build(nx, ny, nz, N, bcflag, nranks, rank, maps, p);
    if (rc) return rc;
    info[0] = p.e0;
    info[1] = p.e1;
    info[2] = p.nowned;
    info[3] = p.nlocal;
    info[4] = (int64_t)p.below.size();
    info[5] = (int64_t)p.above.size();
    if (global_to_local) std::memcpy(global_to_local, p.g2l.data(), sizeof(int32_t) * p.g2l.size());
    if (below) std::memcpy(below, p.below.data(), sizeof(int32_t) * p.below.size());
    if (above) std::memcpy(above, p.above.data(), sizeof(int32_t) * p.above.size());
    if (lattice) std::memcpy(lattice, p.lattice.data(), sizeof(int64_t) * p.lattice.size());
    return LPG_OK;
  } catch (const std::bad_alloc&) {
    return lpg::set_error(LPG_ERR_ALLOC, "box partition: host memory");
  }
}
