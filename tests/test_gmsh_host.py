"""Gmsh hexahedral meshes on the host (no GPU): the library's reader, connectivity and
node numbering (lpg_hex_mesh_info / lpg_hex_mesh_numbering) against the oracle's
restatement of mesh_t::ReadGmshHex3D + Connect + ConnectBoundary + ConnectFaceNodes +
ConnectNodes, and the oracle's Gmsh path against its box path (the same mesh written
as a file must give the same discrete solution)."""
import os

import numpy as np
import pytest

import libparanumal_gb300 as lpg
from gmsh_mesh import cube_rotations, write_box
from oracle.oracle import Oracle

BASE = {"BOX NX": 3, "BOX NY": 3, "BOX NZ": 2, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
        "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 4, "LAMBDA": 0.5, "PRECONDITIONER": "JACOBI",
        "LINEAR SOLVER": "PCG"}
MESHES = {
    "plain": dict(),
    "shuffled": dict(shuffle_seed=1),
    "rotated": dict(shuffle_seed=2, rotate_seed=3),
    "mixed_tags": dict(rotate_seed=5, tags=(1, 2, 1, 2, 2, 1)),
    "all_neumann_tags": dict(rotate_seed=7, tags=(2, 2, 2, 2, 2, 2)),
    "jittered": dict(rotate_seed=11, jitter=0.2, jitter_seed=4),
}


def test_cube_rotations_are_the_24_proper_ones():
    rots = cube_rotations()
    assert len({tuple(r) for r in rots}) == 24


@pytest.mark.parametrize("name", sorted(MESHES))
@pytest.mark.parametrize("N", [1, 2, 5, 7])
def test_library_numbering_matches_oracle(tmp_path, name, N):
    f = write_box(str(tmp_path / "m.msh"), 3, 3, 2, **MESHES[name])
    E, Nn, Nb = lpg.hex_mesh_info(f)
    assert (E, Nn, Nb) == (18, 48, 42)
    g2l, ng = lpg.hex_mesh_numbering(f, N)
    o = Oracle(dict(BASE, **{"MESH FILE": f, "POLYNOMIAL DEGREE": N}))
    assert ng == o.Ngather
    assert np.array_equal(g2l, o.array("GlobalToLocal"))


@pytest.mark.parametrize("name", ["plain", "shuffled", "rotated"])
def test_oracle_file_mesh_equals_box(tmp_path, name):
    f = write_box(str(tmp_path / "m.msh"), 3, 3, 2, **MESHES[name])
    rb = Oracle(BASE).run()
    rf = Oracle(dict(BASE, **{"MESH FILE": f})).run()
    assert rf["iterations"] == rb["iterations"]
    assert abs(rf["norm"] - rb["norm"]) < 1e-12
    assert abs(rf["error"] - rb["error"]) < 1e-9 * rb["error"]


# the reference's source tree, when present on this machine (LIBPARANUMAL_DIR=<path>)
CUBE = os.path.join(os.environ.get("LIBPARANUMAL_DIR", ""), "test", "cubeHex.msh")


@pytest.mark.skipif(not os.environ.get("LIBPARANUMAL_DIR") or not os.path.exists(CUBE),
                    reason="reference source tree not given (LIBPARANUMAL_DIR)")
def test_reference_cube_mesh_matches_box():
    """The reference's own 6x6x6 cube mesh (test/cubeHex.msh, used by its mesh tests) solves
    to the same discrete solution as the 6^3 box on [-1,1]^3."""
    s = dict(BASE, **{"BOX NX": 6, "BOX NY": 6, "BOX NZ": 6, "LAMBDA": 1.0})
    assert lpg.hex_mesh_info(CUBE) == (216, 343, 216)
    rb = Oracle(s).run()
    o = Oracle(dict(s, **{"MESH FILE": CUBE}))
    rf = o.run()
    assert rf["iterations"] == rb["iterations"]
    assert abs(rf["norm"] - rb["norm"]) < 1e-12
    g2l, ng = lpg.hex_mesh_numbering(CUBE, 4)
    assert ng == o.Ngather and np.array_equal(g2l, o.array("GlobalToLocal"))


def test_bad_mesh_files_are_rejected(tmp_path):
    p = tmp_path / "bad.msh"
    p.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n1\n1 0 0 0\n$EndNodes\n$Elements\n0\n$EndElements\n")
    with pytest.raises(RuntimeError):
        lpg.hex_mesh_info(str(p))
    with pytest.raises(RuntimeError):
        lpg.hex_mesh_info(str(tmp_path / "missing.msh"))


@pytest.mark.parametrize("disc", ["CONTINUOUS", "IPDG"])
def test_oracle_neumann_box_equals_neumann_tagged_file(tmp_path, disc):
    """BOX BOUNDARY FLAG 2 (every face Neumann) and the same box as a file with every
    boundary face tagged 2 give the same discrete solution, Neumann data included."""
    s = dict(BASE, **{"BOX BOUNDARY FLAG": 2, "LAMBDA": 1.0, "DISCRETIZATION": disc})
    f = write_box(str(tmp_path / "m.msh"), 3, 3, 2, rotate_seed=6, tags=(2, 2, 2, 2, 2, 2))
    rb = Oracle(s).run()
    rf = Oracle(dict(s, **{"MESH FILE": f})).run()
    assert abs(rf["norm"] - rb["norm"]) < 1e-11 * rb["norm"]
    assert abs(rf["iterations"] - rb["iterations"]) <= 1
