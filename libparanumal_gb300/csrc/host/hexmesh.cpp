// Gmsh hexahedral meshes: reader, connectivity, per-degree node numbering.
#include "hexmesh.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <unordered_map>

#include "objects.hpp"

namespace lpg {

const int kHexFaceVerts[6][4] = {{0, 1, 2, 3}, {0, 4, 5, 1}, {1, 5, 6, 2}, {2, 6, 7, 3}, {0, 3, 7, 4}, {4, 7, 6, 5}};

namespace {

// whole-file reader with a cursor over lines
struct Text {
  std::vector<char> buf;
  size_t pos = 0;
  bool line(const char*& b, const char*& e) {
    if (pos >= buf.size()) return false;
    b = buf.data() + pos;
    const void* nl = std::memchr(b, '\n', buf.size() - pos);
    e = nl ? (const char*)nl : buf.data() + buf.size();
    pos = (size_t)(e - buf.data()) + 1;
    return true;
  }
  bool seek(const char* tag) {
    const char *b, *e;
    const size_t n = std::strlen(tag);
    while (line(b, e))
      if ((size_t)(e - b) >= n && std::memcmp(b, tag, n) == 0) return true;
    return false;
  }
};

// parses up to `maxn` integers of a line; returns the count
int parse_ints(const char* b, const char* e, long long* out, int maxn) {
  int n = 0;
  const char* p = b;
  while (p < e && n < maxn) {
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    if (p >= e) break;
    char* q = nullptr;
    const long long v = std::strtoll(p, &q, 10);
    if (q == p) break;
    out[n++] = v;
    p = q;
  }
  return n;
}

struct FaceKey {
  std::array<int64_t, 4> v;
  bool operator==(const FaceKey& o) const { return v == o.v; }
};
struct FaceKeyHash {
  size_t operator()(const FaceKey& k) const {
    uint64_t h = 0x9E3779B97F4A7C15ULL;
    for (int64_t x : k.v) h = (h ^ (uint64_t)x) * 0xBF58476D1CE4E5B9ULL + (h >> 29);
    return (size_t)h;
  }
};
FaceKey face_key(const int64_t* v8, int f) {
  FaceKey k;
  for (int a = 0; a < 4; ++a) k.v[a] = v8[kHexFaceVerts[f][a]];
  std::sort(k.v.begin(), k.v.end());
  return k;
}

struct UnionFind {
  std::vector<int32_t> p;
  explicit UnionFind(int64_t n) : p(n) { std::iota(p.begin(), p.end(), 0); }
  int32_t find(int32_t x) {
    while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
    return x;
  }
  void unite(int32_t a, int32_t b) {
    a = find(a); b = find(b);
    if (a == b) return;
    if (a < b) p[b] = a; else p[a] = b;   // the smaller index becomes the root
  }
};

}  // namespace

int read_gmsh_hex(const std::string& path, HexMeshData& m) {
  m = HexMeshData();
  FILE* fp = std::fopen(path.c_str(), "rb");
  if (!fp) return set_error(LPG_ERR_INVALID, "cannot open mesh file: " + path);
  Text t;
  std::fseek(fp, 0, SEEK_END);
  const long sz = std::ftell(fp);
  std::fseek(fp, 0, SEEK_SET);
  t.buf.resize(sz > 0 ? (size_t)sz : 0);
  const size_t got = sz > 0 ? std::fread(t.buf.data(), 1, (size_t)sz, fp) : 0;
  std::fclose(fp);
  if ((long)got != sz) return set_error(LPG_ERR_INVALID, "cannot read mesh file: " + path);
  const std::string bad = "malformed Gmsh file: " + path;
  const char *b, *e;
  if (!t.seek("$Nodes") || !t.line(b, e)) return set_error(LPG_ERR_INVALID, bad + " (no $Nodes)");
  m.Nnodes = std::strtoll(b, nullptr, 10);
  if (m.Nnodes <= 0) return set_error(LPG_ERR_INVALID, bad + " (no nodes)");
  m.VX.resize(m.Nnodes); m.VY.resize(m.Nnodes); m.VZ.resize(m.Nnodes);
  std::vector<long long> tags(m.Nnodes);
  bool contiguous = true;
  for (int64_t n = 0; n < m.Nnodes; ++n) {
    if (!t.line(b, e)) return set_error(LPG_ERR_INVALID, bad + " (short $Nodes)");
    char* q = nullptr;
    tags[n] = std::strtoll(b, &q, 10);
    m.VX[n] = std::strtod(q, &q);
    m.VY[n] = std::strtod(q, &q);
    m.VZ[n] = std::strtod(q, &q);
    if (q > e) return set_error(LPG_ERR_INVALID, bad + " (node record)");
    contiguous = contiguous && (tags[n] == n + 1);
  }
  std::unordered_map<long long, int64_t> tagIndex;
  if (!contiguous)
    for (int64_t n = 0; n < m.Nnodes; ++n) tagIndex[tags[n]] = n;
  auto index_of = [&](long long tag) -> int64_t {
    if (contiguous) return (tag >= 1 && tag <= m.Nnodes) ? tag - 1 : -1;
    auto it = tagIndex.find(tag);
    return it == tagIndex.end() ? -1 : it->second;
  };
  if (!t.seek("$Elements") || !t.line(b, e)) return set_error(LPG_ERR_INVALID, bad + " (no $Elements)");
  const int64_t nAll = std::strtoll(b, nullptr, 10);
  long long tok[64];
  for (int64_t i = 0; i < nAll; ++i) {
    if (!t.line(b, e)) return set_error(LPG_ERR_INVALID, bad + " (short $Elements)");
    // elm-number elm-type number-of-tags <tags> node-number-list
    const int nt = parse_ints(b, e, tok, 64);
    if (nt < 3) return set_error(LPG_ERR_INVALID, bad + " (element record)");
    const int type = (int)tok[1], ntags = (int)tok[2];
    const int nn = nt - 3 - ntags;
    const long long* nodes = tok + 3 + ntags;
    if (type == 5) {
      if (nn < 8) return set_error(LPG_ERR_INVALID, bad + " (hexahedron with fewer than 8 nodes)");
      for (int v = 0; v < 8; ++v) {
        const int64_t id = index_of(nodes[v]);
        if (id < 0) return set_error(LPG_ERR_INVALID, bad + " (unknown node tag)");
        m.EToV.push_back(id);
      }
      ++m.E;
    } else if (type == 3) {
      if (nn < 4) return set_error(LPG_ERR_INVALID, bad + " (quadrilateral with fewer than 4 nodes)");
      m.binfo.push_back(ntags > 0 ? tok[3] : 0);
      for (int v = 0; v < 4; ++v) {
        const int64_t id = index_of(nodes[v]);
        if (id < 0) return set_error(LPG_ERR_INVALID, bad + " (unknown node tag)");
        m.binfo.push_back(id);
      }
    }
  }
  if (m.E <= 0) return set_error(LPG_ERR_INVALID, bad + " (no hexahedra)");
  for (int a = 0; a < 3; ++a) { m.lo[a] = 1e300; m.hi[a] = -1e300; }
  for (int64_t n = 0; n < m.Nnodes; ++n) {
    const double c[3] = {m.VX[n], m.VY[n], m.VZ[n]};
    for (int a = 0; a < 3; ++a) { m.lo[a] = std::min(m.lo[a], c[a]); m.hi[a] = std::max(m.hi[a], c[a]); }
  }
  return connect_hex_mesh(m);
}

int connect_hex_mesh(HexMeshData& m) {
  const int64_t E = m.E;
  m.EToE.assign(E * 6, -1);
  m.EToF.assign(E * 6, -1);
  m.EToB.assign(E * 6, 0);
  std::unordered_map<FaceKey, int64_t, FaceKeyHash> open;   // face key -> e*6+f
  open.reserve((size_t)(E * 3 + 16));
  for (int64_t e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const FaceKey k = face_key(&m.EToV[e * 8], f);
      auto it = open.find(k);
      if (it == open.end()) { open.emplace(k, e * 6 + f); continue; }
      const int64_t o = it->second;
      if (o < 0) return set_error(LPG_ERR_INVALID, "mesh file: a face is shared by more than two hexahedra");
      m.EToE[e * 6 + f] = o / 6; m.EToF[e * 6 + f] = (int)(o % 6);
      m.EToE[o] = e; m.EToF[o] = f;
      it->second = -1;
    }
  // boundary faces: tag from the file's quadrilaterals (largest tag on duplicates), -1 if untagged
  std::unordered_map<FaceKey, int, FaceKeyHash> tagged;
  const int64_t nb = (int64_t)m.binfo.size() / 5;
  for (int64_t b = 0; b < nb; ++b) {
    FaceKey k;
    for (int a = 0; a < 4; ++a) k.v[a] = m.binfo[b * 5 + 1 + a];
    std::sort(k.v.begin(), k.v.end());
    const int tag = (int)m.binfo[b * 5];
    auto it = tagged.find(k);
    if (it == tagged.end()) tagged.emplace(k, tag);
    else it->second = std::max(it->second, tag);
  }
  for (int64_t e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      if (m.EToE[e * 6 + f] >= 0) continue;
      auto it = tagged.find(face_key(&m.EToV[e * 8], f));
      m.EToB[e * 6 + f] = (it == tagged.end()) ? -1 : it->second;
    }
  return LPG_OK;
}

namespace {

// Face nodes of the degree-N hexahedron and the node pairing of two connected faces.
// Nodes of face f are listed in local index order (faces t=-1, s=-1, r=+1, s=+1, r=-1,
// t=+1 as in meshBasisHex3D.cpp); a node of face fM is paired with the node of face fP
// that has the same bilinear weights on the four shared vertices, whatever the relative
// orientation of the two faces. Tables are built on first use per (fM, fP, vertex
// correspondence).
struct FacePairing {
  int Nq = 0, Nfp = 0;
  std::vector<int> faceNodes;   // [6][Nfp]
  std::vector<double> W;        // [6][Nfp][4]
  std::vector<std::vector<int>> tables;
  FacePairing(int N, const std::vector<double>& r1d) : Nq(N + 1), Nfp((N + 1) * (N + 1)) {
    faceNodes.resize(6 * Nfp);
    int cnt[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < Nq; ++k)
      for (int j = 0; j < Nq; ++j)
        for (int i = 0; i < Nq; ++i) {
          const int n = i + j * Nq + k * Nfp;
          if (k == 0) faceNodes[0 * Nfp + cnt[0]++] = n;
          if (j == 0) faceNodes[1 * Nfp + cnt[1]++] = n;
          if (i == N) faceNodes[2 * Nfp + cnt[2]++] = n;
          if (j == N) faceNodes[3 * Nfp + cnt[3]++] = n;
          if (i == 0) faceNodes[4 * Nfp + cnt[4]++] = n;
          if (k == N) faceNodes[5 * Nfp + cnt[5]++] = n;
        }
    static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    W.resize(6 * Nfp * 4);
    for (int f = 0; f < 6; ++f)
      for (int n = 0; n < Nfp; ++n) {
        const int v = faceNodes[f * Nfp + n];
        const double r = r1d[v % Nq], s = r1d[(v / Nq) % Nq], t = r1d[v / Nfp];
        for (int a = 0; a < 4; ++a) {
          const int c = kHexFaceVerts[f][a];
          W[(f * Nfp + n) * 4 + a] = 0.125 * (cx[c] ? 1 + r : 1 - r) * (cy[c] ? 1 + s : 1 - s) * (cz[c] ? 1 + t : 1 - t);
        }
      }
    tables.resize(6 * 6 * 256);
  }
  // T[nM] = nP for face f of element e and its neighbour face; nullptr on a mismatch
  const std::vector<int>* pair(const HexMeshData& m, int64_t e, int f) {
    const int64_t eP = m.EToE[e * 6 + f];
    const int fP = m.EToF[e * 6 + f];
    int sigma[4];
    for (int a = 0; a < 4; ++a) {
      const int64_t g = m.EToV[e * 8 + kHexFaceVerts[f][a]];
      sigma[a] = -1;
      for (int b = 0; b < 4; ++b)
        if (m.EToV[eP * 8 + kHexFaceVerts[fP][b]] == g) sigma[a] = b;
      if (sigma[a] < 0) return nullptr;
    }
    const int code = sigma[0] + 4 * sigma[1] + 16 * sigma[2] + 64 * sigma[3];
    std::vector<int>& T = tables[(f * 6 + fP) * 256 + code];
    if (!T.empty()) return &T;
    T.assign(Nfp, -1);
    for (int n = 0; n < Nfp; ++n)
      for (int q = 0; q < Nfp; ++q) {
        double d = 0;
        for (int a = 0; a < 4; ++a) d += std::fabs(W[(f * Nfp + n) * 4 + a] - W[(fP * Nfp + q) * 4 + sigma[a]]);
        if (d < 1e-10) { T[n] = q; break; }
      }
    for (int n = 0; n < Nfp; ++n)
      if (T[n] < 0) { T.clear(); return nullptr; }
    return &T;
  }
};

}  // namespace

int hex_traces(const HexMeshData& m, int N, const std::vector<double>& r1d, std::vector<int32_t>& vmapP,
               std::vector<int32_t>& mapP) {
  const int Nq = N + 1, Np = Nq * Nq * Nq, Nfp = Nq * Nq;
  const int64_t E = m.E;
  if (E * Np >= (int64_t)INT32_MAX || E * 6 * Nfp >= (int64_t)INT32_MAX)
    return set_error(LPG_ERR_UNSUPPORTED, "more than 2^31 local nodes");
  FacePairing fp(N, r1d);
  vmapP.resize(E * 6 * Nfp);
  mapP.resize(E * 6 * Nfp);
  for (int64_t e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int64_t eP = m.EToE[e * 6 + f];
      const int fP = m.EToF[e * 6 + f];
      const std::vector<int>* T = (eP >= 0) ? fp.pair(m, e, f) : nullptr;
      if (eP >= 0 && !T) return set_error(LPG_ERR_INVALID, "mesh: face nodes of connected faces do not match");
      for (int n = 0; n < Nfp; ++n) {
        const int64_t id = (e * 6 + f) * Nfp + n;
        if (eP < 0) {
          vmapP[id] = (int32_t)(e * Np + fp.faceNodes[f * Nfp + n]);
          mapP[id] = (int32_t)id;
        } else {
          const int q = (*T)[n];
          vmapP[id] = (int32_t)(eP * Np + fp.faceNodes[fP * Nfp + q]);
          mapP[id] = (int32_t)((eP * 6 + fP) * Nfp + q);
        }
      }
    }
  return LPG_OK;
}

HexMeshData box_hex_mesh(int nx, int ny, int nz, int bcflag) {
  HexMeshData m;
  const bool periodic = (bcflag == -1);
  const int64_t NnX = periodic ? nx : nx + 1, NnY = periodic ? ny : ny + 1, NnZ = periodic ? nz : nz + 1;
  m.E = (int64_t)nx * ny * nz;
  m.Nnodes = NnX * NnY * NnZ;
  m.EToV.resize(m.E * 8);
  static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (int64_t e = 0; e < m.E; ++e) {
    const int64_t i = e % nx, j = (e / nx) % ny, k = e / ((int64_t)nx * ny);
    for (int v = 0; v < 8; ++v)
      m.EToV[e * 8 + v] = (i + cx[v]) % NnX + ((j + cy[v]) % NnY) * NnX + ((k + cz[v]) % NnZ) * NnX * NnY;
  }
  connect_hex_mesh(m);
  for (int64_t i = 0; i < m.E * 6; ++i)
    if (m.EToE[i] < 0) m.EToB[i] = bcflag;
  return m;
}

int number_hex_nodes(const HexMeshData& m, int N, const std::vector<double>& r1d, HexNumbering& out) {
  const int Nq = N + 1, Np = Nq * Nq * Nq, Nfp = Nq * Nq;
  const int64_t E = m.E, Nlocal = E * Np;
  if (Nlocal >= (int64_t)INT32_MAX) return set_error(LPG_ERR_UNSUPPORTED, "more than 2^31 local nodes");
  // face nodes in local index order (faces r,s,t = -1/+1 as in meshBasisHex3D.cpp)
  std::vector<int> faceNodes(6 * Nfp);
  {
    int cnt[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < Nq; ++k)
      for (int j = 0; j < Nq; ++j)
        for (int i = 0; i < Nq; ++i) {
          const int n = i + j * Nq + k * Nfp;
          if (k == 0) faceNodes[0 * Nfp + cnt[0]++] = n;
          if (j == 0) faceNodes[1 * Nfp + cnt[1]++] = n;
          if (i == N) faceNodes[2 * Nfp + cnt[2]++] = n;
          if (j == N) faceNodes[3 * Nfp + cnt[3]++] = n;
          if (i == 0) faceNodes[4 * Nfp + cnt[4]++] = n;
          if (k == N) faceNodes[5 * Nfp + cnt[5]++] = n;
        }
  }
  // bilinear weight of face vertex a (kHexFaceVerts order) at each face node
  static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  std::vector<double> W(6 * Nfp * 4);
  for (int f = 0; f < 6; ++f)
    for (int n = 0; n < Nfp; ++n) {
      const int v = faceNodes[f * Nfp + n];
      const double r = r1d[v % Nq], s = r1d[(v / Nq) % Nq], t = r1d[v / Nfp];
      for (int a = 0; a < 4; ++a) {
        const int c = kHexFaceVerts[f][a];
        W[(f * Nfp + n) * 4 + a] = 0.125 * (cx[c] ? 1 + r : 1 - r) * (cy[c] ? 1 + s : 1 - s) * (cz[c] ? 1 + t : 1 - t);
      }
    }
  // node pairing tables per (fM, fP, vertex correspondence), built on first use
  std::vector<std::vector<int>> pairing(6 * 6 * 256);
  auto table = [&](int fM, int fP, const int sigma[4]) -> const std::vector<int>* {
    const int code = sigma[0] + 4 * sigma[1] + 16 * sigma[2] + 64 * sigma[3];
    std::vector<int>& T = pairing[(fM * 6 + fP) * 256 + code];
    if (!T.empty()) return &T;
    T.assign(Nfp, -1);
    for (int n = 0; n < Nfp; ++n)
      for (int q = 0; q < Nfp; ++q) {
        double d = 0;
        for (int a = 0; a < 4; ++a) d += std::fabs(W[(fM * Nfp + n) * 4 + a] - W[(fP * Nfp + q) * 4 + sigma[a]]);
        if (d < 1e-10) { T[n] = q; break; }
      }
    for (int n = 0; n < Nfp; ++n)
      if (T[n] < 0) { T.clear(); return nullptr; }
    return &T;
  };
  UnionFind uf(Nlocal);
  for (int64_t e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int64_t eP = m.EToE[e * 6 + f];
      if (eP < e) continue;   // each connected pair once (and no boundary faces)
      const int fP = m.EToF[e * 6 + f];
      int sigma[4];
      for (int a = 0; a < 4; ++a) {
        const int64_t g = m.EToV[e * 8 + kHexFaceVerts[f][a]];
        sigma[a] = -1;
        for (int b = 0; b < 4; ++b)
          if (m.EToV[eP * 8 + kHexFaceVerts[fP][b]] == g) sigma[a] = b;
        if (sigma[a] < 0) return set_error(LPG_ERR_INVALID, "mesh file: connected faces do not share vertices");
      }
      const std::vector<int>* T = table(f, fP, sigma);
      if (!T) return set_error(LPG_ERR_INVALID, "mesh file: face nodes of connected faces do not match");
      for (int n = 0; n < Nfp; ++n)
        uf.unite((int32_t)(e * Np + faceNodes[f * Nfp + n]), (int32_t)(eP * Np + faceNodes[fP * Nfp + (*T)[n]]));
    }
  // smallest positive boundary tag per component (0 = none)
  std::vector<int> bc(Nlocal, 0);
  for (int64_t e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int tag = m.EToB[e * 6 + f];
      if (tag <= 0) continue;
      for (int n = 0; n < Nfp; ++n) {
        const int32_t root = uf.find((int32_t)(e * Np + faceNodes[f * Nfp + n]));
        if (bc[root] == 0 || tag < bc[root]) bc[root] = tag;
      }
    }
  out.g2l.assign(Nlocal, -1);
  out.flag.assign(Nlocal, 0);
  out.owner.clear();
  out.mult.clear();
  out.hasDirichlet = false;
  std::vector<int32_t> dofOf(Nlocal, -1);
  for (int64_t n = 0; n < Nlocal; ++n) {
    const int32_t root = uf.find((int32_t)n);
    out.flag[n] = (int8_t)std::min(bc[root], 127);
    if (bc[root] == 1) { out.hasDirichlet = true; continue; }
    if (dofOf[root] < 0) {
      dofOf[root] = (int32_t)out.owner.size();
      out.owner.push_back((int32_t)n);
      out.mult.push_back(0);
    }
    out.g2l[n] = dofOf[root];
    out.mult[dofOf[root]]++;
  }
  out.Nglobal = (int64_t)out.owner.size();
  return LPG_OK;
}

}  // namespace lpg
