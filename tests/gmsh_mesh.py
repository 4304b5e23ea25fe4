"""Gmsh 2.2 ASCII writer for hexahedral test meshes (test infrastructure).

Writes a structured box of nx*ny*nz hexahedra on [-dimx/2, dimx/2] x ... as an
unstructured mesh, the way a mesh generator would hand it over:
  - node numbering optionally shuffled,
  - each element's vertex list optionally rotated by one of the 24 orientation-preserving
    symmetries of the cube (so neighbouring faces meet at every relative rotation),
  - interior vertices optionally jittered,
  - boundary quadrilaterals (element type 3) with a physical tag per box side
    (-x, +x, -y, +y, -z, +z), hexahedra as element type 5 (physical tag 9).
Record layout follows the format the reference reads (libs/mesh/meshReadGmshHex3D.cpp:33-170):
`elm-number elm-type number-of-tags physical elementary node-list`.
"""
import itertools

import numpy as np

# hex vertex v sits at corner (bits) of the reference cube
_CORNER = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)])
_FACES = [(0, 1, 2, 3), (0, 4, 5, 1), (1, 5, 6, 2), (2, 6, 7, 3), (0, 3, 7, 4), (4, 7, 6, 5)]


def cube_rotations():
    """The 24 proper rotations of the cube as vertex permutations p: new vertex v is old p[v]."""
    out = []
    idx = {tuple(c): v for v, c in enumerate(_CORNER)}
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            Q = np.zeros((3, 3), dtype=int)
            for i in range(3):
                Q[i, perm[i]] = signs[i]
            if round(np.linalg.det(Q)) != 1:
                continue
            p = []
            for v in range(8):
                c = 2 * _CORNER[v] - 1
                q = (Q @ c + 1) // 2
                p.append(idx[tuple(int(x) for x in q)])
            out.append(p)
    return out


def write_box(path, nx, ny, nz, dims=(2.0, 2.0, 2.0), shuffle_seed=None, rotate_seed=None, jitter=0.0,
              jitter_seed=0, tags=(1, 1, 1, 1, 1, 1), element_seed=None):
    """element_seed: the hexahedra are written in a random order (a mesh whose element
    order carries no spatial locality)."""
    nnx, nny, nnz = nx + 1, ny + 1, nz + 1
    X0 = [-d / 2.0 for d in dims]
    h = [dims[0] / nx, dims[1] / ny, dims[2] / nz]
    lid = np.arange(nnx * nny * nnz)          # lattice id = i + j*nnx + k*nnx*nny
    ii, jj, kk = lid % nnx, (lid // nnx) % nny, lid // (nnx * nny)
    xyz = np.stack([X0[0] + h[0] * ii, X0[1] + h[1] * jj, X0[2] + h[2] * kk], axis=1)
    if jitter:
        rng = np.random.default_rng(jitter_seed)
        inner = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)
        xyz[inner] += (2 * rng.random((int(inner.sum()), 3)) - 1) * jitter * np.array(h)
    Nn = nnx * nny * nnz
    tag_of = np.arange(1, Nn + 1)
    if shuffle_seed is not None:
        tag_of = np.random.default_rng(shuffle_seed).permutation(Nn) + 1
    # file position of each node: sorted by tag
    nodes_by_tag = np.empty(Nn, dtype=int)
    nodes_by_tag[tag_of - 1] = np.arange(Nn)

    def vid(i, j, k):
        return i + j * nnx + k * nnx * nny

    rots = cube_rotations()
    rrng = np.random.default_rng(rotate_seed) if rotate_seed is not None else None
    hexes, quads = [], []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                v = [vid(i + c[0], j + c[1], k + c[2]) for c in _CORNER]
                if rrng is not None:
                    p = rots[int(rrng.integers(len(rots)))]
                    v = [v[p[a]] for a in range(8)]
                hexes.append([int(tag_of[x]) for x in v])
    # boundary faces, one quad per element face on a box side
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                base = [vid(i + c[0], j + c[1], k + c[2]) for c in _CORNER]
                sides = []
                if i == 0: sides.append((0, 4))
                if i == nx - 1: sides.append((1, 2))
                if j == 0: sides.append((2, 1))
                if j == ny - 1: sides.append((3, 3))
                if k == 0: sides.append((4, 0))
                if k == nz - 1: sides.append((5, 5))
                for side, f in sides:
                    quads.append((tags[side], [int(tag_of[base[a]]) for a in _FACES[f]]))
    with open(path, "w") as fp:
        fp.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % Nn)
        for t in range(Nn):
            n = nodes_by_tag[t]
            fp.write("%d %.17g %.17g %.17g\n" % (t + 1, xyz[n, 0], xyz[n, 1], xyz[n, 2]))
        fp.write("$EndNodes\n$Elements\n%d\n" % (len(quads) + len(hexes)))
        c = 1
        for tag, q in quads:
            fp.write("%d 3 2 %d %d %s\n" % (c, tag, tag, " ".join(map(str, q))))
            c += 1
        order = range(len(hexes))
        if element_seed is not None:
            order = np.random.default_rng(element_seed).permutation(len(hexes))
        for h_ in order:
            fp.write("%d 5 2 9 1 %s\n" % (c, " ".join(map(str, hexes[h_]))))
            c += 1
        fp.write("$EndElements\n")
    return path
