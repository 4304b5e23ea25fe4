"""Meshes read from Gmsh files through the CUDA solver path, and VTU output.

Parity: the same file solved by the library and by the oracle (identical iteration
counts for FP64 paths, solution within 1e-7, norms within 1e-9); the file version of a
box equals the library's own box solve; the VTU file's points and field equal the
oracle's plot interpolation (ASCII %g, so 1e-5 relative)."""
import re
import xml.etree.ElementTree as ET

import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from gmsh_mesh import write_box
from gpu_helpers import rel_err
from oracle.oracle import Oracle
from oracle.plot import plot_cells, plot_interp

pytestmark = pytest.mark.gpu

BASE = {"BOX NX": 4, "BOX NY": 3, "BOX NZ": 3, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
        "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 5, "LAMBDA": 0.5, "PRECONDITIONER": "JACOBI",
        "LINEAR SOLVER": "PCG"}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


def mesh(tmp_path, **kw):
    return write_box(str(tmp_path / "m.msh"), 4, 3, 3, **kw)


CASES = {
    "jacobi_rotated": (dict(shuffle_seed=1, rotate_seed=2, jitter=0.15, jitter_seed=3), {}),
    "multigrid_rotated": (dict(rotate_seed=4, jitter=0.1, jitter_seed=5),
                          {"POLYNOMIAL DEGREE": 7, "PRECONDITIONER": "MULTIGRID", "MULTIGRID DEGREES": "7,3,1",
                           "PARALMOND AGGREGATION": "SMOOTHED", "LINEAR SOLVER": "FPCG", "LAMBDA": 0.0}),
    "mixed_dirichlet_neumann": (dict(rotate_seed=6, tags=(1, 2, 2, 1, 2, 1)), {"LAMBDA": 1.0}),
    "all_neumann": (dict(rotate_seed=8, tags=(2, 2, 2, 2, 2, 2)),
                    {"LAMBDA": 0.0, "PRECONDITIONER": "MULTIGRID", "MULTIGRID DEGREES": "5,2,1",
                     "LINEAR SOLVER": "FPCG"}),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_file_mesh_solve_matches_oracle(tmp_path, name):
    kw, over = CASES[name]
    s = dict(BASE, **over, **{"MESH FILE": mesh(tmp_path, **kw)})
    r = lpg.Elliptic(s).Run(want_solution=True)
    ro = Oracle(s).run()
    assert r["converged"]
    assert r["iterations"] == ro["iterations"], (r["iterations"], ro["iterations"])
    assert abs(r["norm"] - ro["norm"]) < 1e-9 * abs(ro["norm"])
    assert rel_err(r["xL"], ro["xL"]) < 1e-7


@pytest.mark.parametrize("over", [{"BOX BOUNDARY FLAG": 2, "LAMBDA": 1.0},
                                  {"BOX BOUNDARY FLAG": 2, "LAMBDA": 0.0, "PRECONDITIONER": "MULTIGRID",
                                   "LINEAR SOLVER": "FPCG"},
                                  {"BOX BOUNDARY FLAG": 2, "LAMBDA": 1.0, "DISCRETIZATION": "IPDG"}],
                         ids=["c0_neumann_box", "c0_all_neumann_pmg", "ipdg_neumann_box"])
def test_neumann_box_matches_oracle(over):
    """BOX BOUNDARY FLAG 2: Neumann faces with the data file's Neumann data in the rhs."""
    s = dict(BASE, **over)
    e = lpg.Elliptic(s)
    o = Oracle(s)
    r = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.rhs(r)
    torch.cuda.synchronize()
    assert rel_err(r.cpu().numpy(), o.rhs()) < 1e-12
    res = e.Run(want_solution=True)
    ro = o.run()
    assert res["converged"]
    assert abs(res["iterations"] - ro["iterations"]) <= 1
    assert rel_err(res["xL"], ro["xL"]) < 1e-7


def test_neumann_tagged_file_rhs_matches_oracle(tmp_path):
    s = dict(BASE, **{"MESH FILE": mesh(tmp_path, rotate_seed=5, jitter=0.1, jitter_seed=2, tags=(1, 2, 2, 1, 3, 2)),
                      "LAMBDA": 1.0})
    e = lpg.Elliptic(s)
    r = torch.zeros(e.Nglobal, dtype=torch.float64, device="cuda")
    e.rhs(r)
    torch.cuda.synchronize()
    assert rel_err(r.cpu().numpy(), Oracle(s).rhs()) < 1e-12


@pytest.mark.parametrize("degree", [7, 3])
def test_random_element_order_file_matches_oracle(tmp_path, degree):
    """A 10^3 file whose hexahedra come in random order: the operators visit the elements
    in Morton order of their centroids (the file's order has no locality), storage keeps the
    file's order. FP64, double-word and FP32 operators against the oracle on the same file,
    and a p-MG solve with the oracle's iteration count and solution."""
    f = write_box(str(tmp_path / "r.msh"), 10, 10, 10, shuffle_seed=2, rotate_seed=3, jitter=0.1, jitter_seed=4,
                  element_seed=5)
    s = dict(BASE, **{"MESH FILE": f, "POLYNOMIAL DEGREE": degree, "LAMBDA": 1.0,
                      "PRECONDITIONER": "MULTIGRID", "LINEAR SOLVER": "FPCG",
                      "MULTIGRID DEGREES": "7,3,1" if degree == 7 else "3,1"})
    e = lpg.Elliptic(s)
    assert e.info("morton_order") == 1
    o = Oracle(s)
    qh = np.random.default_rng(7).uniform(-1, 1, e.Nglobal)
    q = torch.tensor(qh, device="cuda")
    ref = o.operator(qh)
    Aq = torch.full_like(q, np.nan)
    e.Operator(q, Aq)
    torch.cuda.synchronize()
    assert rel_err(Aq.cpu().numpy(), ref) < 1e-12
    e.OperatorDF64(q, Aq)
    torch.cuda.synchronize()
    assert rel_err(Aq.cpu().numpy(), ref) < 1e-12
    q32 = q.float()
    A32 = torch.full_like(q32, np.nan)
    e.OperatorF32(q32, A32)
    torch.cuda.synchronize()
    assert rel_err(A32.double().cpu().numpy(), ref) < 2e-6
    r = e.Run(want_solution=True)
    ro = o.run()
    assert r["converged"]
    assert abs(r["iterations"] - ro["iterations"]) <= 1, (r["iterations"], ro["iterations"])
    assert rel_err(r["xL"], ro["xL"]) < 1e-7


def test_file_mesh_equals_box_on_gpu(tmp_path):
    s = dict(BASE, **{"PRECONDITIONER": "MULTIGRID", "LINEAR SOLVER": "FPCG"})
    rb = lpg.Elliptic(s).Run()
    ef = lpg.Elliptic(dict(s, **{"MESH FILE": mesh(tmp_path, shuffle_seed=3, rotate_seed=9)}))
    assert ef.info("morton_order") == 0   # elements in lattice order: the file's order is kept
    rf = ef.Run()
    assert rf["iterations"] == rb["iterations"]
    assert abs(rf["norm"] - rb["norm"]) < 1e-11
    # both solves stop at a 1e-8 relative residual: their solutions differ at that level,
    # far below the discretisation error
    assert abs(rf["error"] - rb["error"]) < 1e-4 * rb["error"]


def _floats(node):
    return np.array([float(t) for t in node.text.split()])


def test_vtu_output_matches_oracle_plot_interpolation(tmp_path):
    s = dict(BASE, **{"MESH FILE": mesh(tmp_path, rotate_seed=12, jitter=0.1, jitter_seed=1),
                      "POLYNOMIAL DEGREE": 3, "OUTPUT TO FILE": "TRUE",
                      "OUTPUT FILE NAME": str(tmp_path / "sol")})
    e = lpg.Elliptic(s)
    r = e.Run(want_solution=True)
    o = Oracle(s)
    E, N = o.info("nelements"), 3
    root = ET.parse(str(tmp_path / "sol_0000.vtu")).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    pNp = (N + 4) ** 3
    assert int(piece.get("NumberOfPoints")) == E * pNp
    assert int(piece.get("NumberOfCells")) == E * plot_cells(N)
    pts = _floats(piece.find("Points/DataArray")).reshape(-1, 3)
    fld = _floats(piece.find("PointData/DataArray"))
    ref_xyz = np.stack([plot_interp(o.array(c), E, N).ravel() for c in ("x", "y", "z")], axis=1)
    ref_q = plot_interp(r["xL"], E, N).ravel()
    assert np.abs(pts - ref_xyz).max() < 1e-5 * np.abs(ref_xyz).max()
    assert np.abs(fld - ref_q).max() < 1e-5 * np.abs(ref_q).max()
    cells = piece.find("Cells")
    arrays = {a.get("Name"): a for a in cells.findall("DataArray")}
    conn = _floats(arrays["connectivity"]).astype(np.int64).reshape(-1, 4)
    assert conn.min() == 0 and conn.max() == E * pNp - 1
    v = pts[conn]
    vol = np.einsum("ij,ij->i", v[:, 1] - v[:, 0], np.cross(v[:, 2] - v[:, 0], v[:, 3] - v[:, 0]))
    assert (vol > 0).all()
    assert np.array_equal(_floats(arrays["offsets"]).astype(np.int64), 4 * np.arange(1, len(conn) + 1))
    assert (_floats(arrays["types"]) == 10).all()
    # explicit entry on a device field
    xL = torch.tensor(r["xL"], device="cuda")
    e.PlotFields(xL, str(tmp_path / "again.vtu"))
    assert re.sub(r"\s+", " ", open(tmp_path / "again.vtu").read()) == \
        re.sub(r"\s+", " ", open(tmp_path / "sol_0000.vtu").read())


@pytest.mark.parametrize("precision", ["FP64", "FP32"])
def test_host_buffer_operator_on_shuffled_file_mesh(tmp_path, precision):
    """lpg_elliptic_operator_host(_f32) pipelines element chunks with prefix bounds computed
    from the numbering; with a shuffled, rotated file mesh those bounds are loose but the
    result must still equal the device operator (and the oracle)."""
    s = dict(BASE, **{"MESH FILE": mesh(tmp_path, shuffle_seed=4, rotate_seed=5, jitter=0.1, jitter_seed=3),
                      "POLYNOMIAL DEGREE": 7})
    e = lpg.Elliptic(s)
    dt = np.float64 if precision == "FP64" else np.float32
    qh = np.random.default_rng(2).uniform(-1, 1, e.Nglobal).astype(dt)
    Aq = np.zeros(e.Nglobal, dtype=dt)
    e.OperatorHost(qh, Aq, precision)
    ref = Oracle(s).operator(qh.astype(np.float64))
    assert rel_err(Aq.astype(np.float64), ref) < (1e-12 if precision == "FP64" else 2e-6)


def test_vtu_output_ipdg(tmp_path):
    s = dict(BASE, **{"MESH FILE": mesh(tmp_path, rotate_seed=2), "POLYNOMIAL DEGREE": 2,
                      "DISCRETIZATION": "IPDG", "PRECONDITIONER": "JACOBI",
                      "OUTPUT TO FILE": "TRUE", "OUTPUT FILE NAME": str(tmp_path / "dg")})
    r = lpg.Elliptic(s).Run(want_solution=True)
    o = Oracle(s)
    E, N = o.info("nelements"), 2
    piece = ET.parse(str(tmp_path / "dg_0000.vtu")).getroot().find("UnstructuredGrid/Piece")
    fld = _floats(piece.find("PointData/DataArray"))
    ref_q = plot_interp(r["xL"], E, N).ravel()
    assert np.abs(fld - ref_q).max() < 1e-5 * np.abs(ref_q).max()


def test_unsupported_file_mesh_features_fail_loudly(tmp_path):
    f = mesh(tmp_path)
    with pytest.raises(RuntimeError):
        lpg.Elliptic(dict(BASE, **{"MESH FILE": f, "RHS FIELD": "GAUSSIAN SOURCES"}))
    with pytest.raises(RuntimeError):
        lpg.Elliptic(dict(BASE, **{"MESH FILE": str(tmp_path / "none.msh")}))
