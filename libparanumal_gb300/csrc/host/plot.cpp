// VTU output of a local nodal field (elliptic_t::PlotFields, ellipticPlotFields.cpp:30-140):
// ASCII UnstructuredGrid with the element fields interpolated to equispaced degree-(N+3)
// plot nodes (meshReferenceNodesHex3D.cpp:53-63), each plot cube split into six
// tetrahedra around its main diagonal. The interpolation runs on the GPU in element
// chunks; formatting runs on host threads, chunk by chunk, in element order.
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "objects.hpp"

namespace lpg {

namespace {

// the six tetrahedra of a cube with corners c = dx + 2 dy + 4 dz, all containing the
// diagonal 0-7, one per order in which the path 0 -> 7 visits the axes; vertices ordered
// for a positive volume
struct TetSplit {
  int t[6][4];
  TetSplit() {
    static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    for (int p = 0; p < 6; ++p) {
      const int a = 1 << perms[p][0], b = 1 << perms[p][1];
      // sign of the axis permutation decides the orientation of (0, a, a+b, 7)
      const int inv = (perms[p][0] > perms[p][1]) + (perms[p][0] > perms[p][2]) + (perms[p][1] > perms[p][2]);
      if (inv % 2 == 0) { t[p][0] = 0; t[p][1] = a; t[p][2] = a + b; t[p][3] = 7; }
      else { t[p][0] = 0; t[p][1] = a + b; t[p][2] = a; t[p][3] = 7; }
    }
  }
};

std::string fmt_chunk(const double* vals, int64_t count, int comps, int64_t stride) {
  std::string s;
  s.reserve((size_t)count * (comps * 14 + 8));
  char buf[96];
  for (int64_t n = 0; n < count; ++n) {
    s += "       ";
    for (int c = 0; c < comps; ++c) {
      const int len = std::snprintf(buf, sizeof(buf), c + 1 < comps ? "%g " : "%g", vals[c * stride + n]);
      s.append(buf, (size_t)len);
    }
    s += '\n';
  }
  return s;
}

}  // namespace

int Elliptic::PlotFields(const double* qL, const std::string& fileName, cudaStream_t s) {
  const int N = mesh.N, Nq = N + 1, pN = N + 3, pNq = pN + 1, pNp = pNq * pNq * pNq;
  const int64_t E = mesh.E;
  if (E * (int64_t)pNp >= (int64_t)INT32_MAX) return set_error(LPG_ERR_UNSUPPORTED, "plot: too many plot points");
  // equispaced plot points and the Lagrange interpolation from the GLL points
  std::vector<double> pr(pNq), I(pNq * Nq);
  for (int i = 0; i < pNq; ++i) pr[i] = -1.0 + 2.0 * i / pN;
  for (int i = 0; i < pNq; ++i)
    for (int m = 0; m < Nq; ++m) {
      double l = 1.0;
      for (int k = 0; k < Nq; ++k)
        if (k != m) l *= (pr[i] - mesh.r1d[k]) / (mesh.r1d[m] - mesh.r1d[k]);
      I[i * Nq + m] = l;
    }
  FILE* fp = std::fopen(fileName.c_str(), "w");
  if (!fp) return set_error(LPG_ERR_INVALID, "cannot open output file: " + fileName);
  DevBuf<double> I_d, pr_d, out_d;
  int rc;
  if ((rc = I_d.alloc(pNq * Nq)) || (rc = pr_d.alloc(pNq)) || (rc = I_d.upload(I.data(), pNq * Nq, s)) ||
      (rc = pr_d.upload(pr.data(), pNq, s))) {
    std::fclose(fp);
    return rc;
  }
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(E, (int64_t)(1 << 27) / (4 * pNp)));
  if ((rc = out_d.alloc(chunk * 4 * pNp))) { std::fclose(fp); return rc; }
  std::vector<double> host(chunk * 4 * pNp);
  const int64_t nCells = E * 6 * (int64_t)pN * pN * pN;
  std::fprintf(fp, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"BigEndian\">\n");
  std::fprintf(fp, "  <UnstructuredGrid>\n");
  std::fprintf(fp, "    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", (long long)(E * pNp),
               (long long)nCells);
  // pass 0: point coordinates, pass 1: the field
  for (int pass = 0; pass < 2 && !rc; ++pass) {
    if (pass == 0) {
      std::fprintf(fp, "      <Points>\n");
      std::fprintf(fp, "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n");
    } else {
      std::fprintf(fp, "      <PointData Scalars=\"scalars\">\n");
      std::fprintf(fp, "        <DataArray type=\"Float32\" Name=\"Fields\" NumberOfComponents=\"1\" Format=\"ascii\">\n");
    }
    for (int64_t e0 = 0; e0 < E && !rc; e0 += chunk) {
      const int64_t ne = std::min(chunk, E - e0);
      if ((rc = plot_interp(N, ne, I_d.p, pr_d.p, qL + e0 * mesh.Np, mesh.EX.p + e0 * 8, mesh.EY.p + e0 * 8,
                            mesh.EZ.p + e0 * 8, out_d.p, s)))
        break;
      if ((rc = out_d.download(host.data(), ne * 4 * pNp, s))) break;
      std::vector<std::string> parts(ne);
#pragma omp parallel for schedule(dynamic, 64)
      for (int64_t e = 0; e < ne; ++e) {
        const double* o = host.data() + e * 4 * pNp;
        parts[e] = (pass == 0) ? fmt_chunk(o, pNp, 3, pNp) : fmt_chunk(o + 3 * pNp, pNp, 1, pNp);
      }
      for (const std::string& p : parts) std::fwrite(p.data(), 1, p.size(), fp);
    }
    if (pass == 0) std::fprintf(fp, "        </DataArray>\n      </Points>\n");
    else std::fprintf(fp, "       </DataArray>\n     </PointData>\n");
  }
  if (rc) { std::fclose(fp); return rc; }
  static const TetSplit split;
  std::fprintf(fp, "    <Cells>\n");
  std::fprintf(fp, "      <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n");
  {
    std::string line;
    char buf[64];
    for (int64_t e = 0; e < E; ++e) {
      line.clear();
      for (int k = 0; k < pN; ++k)
        for (int j = 0; j < pN; ++j)
          for (int i = 0; i < pN; ++i)
            for (int t = 0; t < 6; ++t) {
              line += "       ";
              for (int v = 0; v < 4; ++v) {
                const int c = split.t[t][v];
                const int64_t id = e * pNp + (i + (c & 1)) + (j + ((c >> 1) & 1)) * pNq + (k + ((c >> 2) & 1)) * pNq * pNq;
                const int len = std::snprintf(buf, sizeof(buf), "%lld ", (long long)id);
                line.append(buf, (size_t)len);
              }
              line += '\n';
            }
      std::fwrite(line.data(), 1, line.size(), fp);
    }
  }
  std::fprintf(fp, "        </DataArray>\n");
  std::fprintf(fp, "        <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n");
  for (int64_t c = 1; c <= nCells; ++c) std::fprintf(fp, "       %lld\n", (long long)(4 * c));
  std::fprintf(fp, "       </DataArray>\n");
  std::fprintf(fp, "       <DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n");
  for (int64_t c = 0; c < nCells; ++c) std::fputs("10\n", fp);
  std::fprintf(fp, "        </DataArray>\n");
  std::fprintf(fp, "      </Cells>\n");
  std::fprintf(fp, "    </Piece>\n");
  std::fprintf(fp, "  </UnstructuredGrid>\n");
  std::fprintf(fp, "</VTKFile>\n");
  const bool ok = (std::fclose(fp) == 0);
  if (!ok) return set_error(LPG_ERR_INVALID, "error writing output file: " + fileName);
  return LPG_OK;
}

}  // namespace lpg
