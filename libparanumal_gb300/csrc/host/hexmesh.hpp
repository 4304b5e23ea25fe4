// Unstructured hexahedral meshes read from Gmsh files (mesh_t::ReadGmshHex3D,
// meshReadGmshHex3D.cpp:33-170) and their connectivity and node numbering
// (mesh_t::Connect meshConnect.cpp:51-127, ConnectBoundary meshConnectBoundary.cpp:53-143,
// ConnectFaceNodes meshConnectFaceNodes.cpp:32-101, ConnectNodes meshConnectNodes.cpp:32-117).
//
// Host-side setup, done once per mesh (connectivity) and once per polynomial degree
// (numbering):
//   - faces are matched by hashing their sorted vertex ids;
//   - face nodes of two connected faces are paired by their bilinear weights on the four
//     shared vertices, so no orientation convention is assumed;
//   - nodes are merged with a union-find over those pairs; a component is a Dirichlet node
//     if the smallest positive boundary tag among its copies is 1;
//   - assembled dofs are numbered in order of first appearance in local node order, the
//     single-rank ordering of ogs::Setup (ogsSetup.cpp:408-432).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace lpg {

struct HexMeshData {
  int64_t Nnodes = 0, E = 0;
  std::vector<double> VX, VY, VZ;
  std::vector<int64_t> EToV;   // [E][8], 0-based node indices
  std::vector<int64_t> binfo;  // [NboundaryFaces][5]: physical tag, 4 node indices
  std::vector<int64_t> EToE;   // [E][6] neighbour element or -1
  std::vector<int> EToF;       // [E][6] neighbour face or -1
  std::vector<int> EToB;       // [E][6] 0 interior, boundary tag, or -1 (untagged boundary)
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // bounding box of the vertices
};

// vertices of each hexahedron face, every face listed the same way round
// (meshSetElementType.cpp:80-81)
extern const int kHexFaceVerts[6][4];

// LPG_OK or LPG_ERR_INVALID (message set) on an unreadable or malformed file
int read_gmsh_hex(const std::string& path, HexMeshData& m);
// EToE/EToF/EToB from EToV and the tagged boundary faces
int connect_hex_mesh(HexMeshData& m);

struct HexNumbering {
  std::vector<int32_t> g2l;     // [E*Np] assembled dof or -1 (Dirichlet)
  std::vector<int32_t> owner;   // [Nglobal] first local copy of each dof
  std::vector<int32_t> mult;    // [Nglobal] number of local copies
  int64_t Nglobal = 0;
  bool hasDirichlet = false;
  std::vector<int8_t> flag;     // [E*Np] smallest positive boundary tag of the node (0 none, capped at 127)
};
// numbering of the degree-N nodes (r1d: the N+1 GLL points)
int number_hex_nodes(const HexMeshData& m, int N, const std::vector<double>& r1d, HexNumbering& out);

// Trace maps of the degree-N face nodes ([E][6][Nfp], face nodes in local index order;
// meshConnectFaceNodes.cpp:32-101): vmapP = volume node on the other side (itself on the
// boundary), mapP = index of the paired face node (itself on the boundary).
int hex_traces(const HexMeshData& m, int N, const std::vector<double>& r1d, std::vector<int32_t>& vmapP,
               std::vector<int32_t>& mapP);
// the box mesh's vertex connectivity as a HexMeshData (periodic wrap for bcflag -1; boundary
// faces get EToB = bcflag)
HexMeshData box_hex_mesh(int nx, int ny, int nz, int bcflag);

}  // namespace lpg
