"""The partitioned operator path (one process per GPU, as elliptic_t::Operator runs under
MPI: ellipticOperator.cpp:29-106, halo_t include/ogs.hpp:347-400), tested on the CPU.

* lpg_box_partition (host code of the library): z-slab element ranges, rank-local dof
  numbering (owned first, then halo) and the exchange lists, checked for consistency: every
  unmasked lattice node is owned by exactly one rank, the lists of neighbouring ranks pair
  up node by node, and the local GlobalToLocal points at the right lattice nodes.
* two and three gloo ranks (CPU processes): each rank applies the reference's own partial
  Ax and gather kernels (oracle/_ref, translated from its OKL) to its slab's elements with
  its local numbering, packs the shared plane(s), exchanges them over gloo, adds what it
  receives, and must then hold the single-rank operator's values at all its local dofs
  (1e-13 relative). A distributed inner product over owned dofs plus an all-reduce equals
  the single-rank one.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import libparanumal_gb300 as lpg
from gpu_helpers import box, rel_err
from oracle import refimpl
from oracle.oracle import Oracle

CFG = box(**{"BOX NX": 3, "BOX NY": 2, "BOX NZ": 5, "POLYNOMIAL DEGREE": 3, "LAMBDA": 0.7})


def lattice_of_local_nodes(nx, ny, nz, N, e0, e1):
    """global lattice id of every local node of elements [e0, e1), [e][c][b][a] order"""
    Nq = N + 1
    NX, NY = nx * N + 1, ny * N + 1
    e = np.arange(e0, e1)[:, None]
    n = np.arange(Nq ** 3)[None, :]
    a, b, c = n % Nq, (n // Nq) % Nq, n // (Nq * Nq)
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    X, Y, Z = ex * N + a, ey * N + b, ez * N + c
    return (X + NX * (Y + NY * Z)).ravel()


def global_dof_of_lattice(o, nx, ny, nz, N):
    """map lattice id -> the single-rank (oracle) dof index (-1 masked)"""
    E = o.info("nelements")
    lat = lattice_of_local_nodes(nx, ny, nz, N, 0, E)
    g2l = o.array("GlobalToLocal")
    m = np.full((nx * N + 1) * (ny * N + 1) * (nz * N + 1), -1, dtype=np.int64)
    m[lat] = g2l
    return m


@pytest.mark.parametrize("nranks", [1, 2, 3])
@pytest.mark.parametrize("bc", [1, 2])
def test_partition_maps_are_consistent(nranks, bc):
    nx, ny, nz, N = 3, 2, 5, 3
    parts = [lpg.box_partition(nx, ny, nz, N, bc, nranks, r) for r in range(nranks)]
    owned = np.concatenate([p["lattice"][:p["nowned"]] for p in parts])
    o = Oracle(dict(CFG, **{"BOX BOUNDARY FLAG": bc}))
    gmap = global_dof_of_lattice(o, nx, ny, nz, N)
    assert np.array_equal(np.sort(owned), np.sort(np.nonzero(gmap >= 0)[0]))   # each dof owned once
    assert parts[0]["e0"] == 0 and parts[-1]["e1"] == nx * ny * nz
    for r in range(nranks):
        p = parts[r]
        if r > 0:
            assert p["e0"] == parts[r - 1]["e1"]
            # rank r's plane below pairs node by node with rank r-1's plane above
            assert np.array_equal(p["lattice"][p["below"]], parts[r - 1]["lattice"][parts[r - 1]["above"]])
            assert np.all(p["below"] >= p["nowned"])        # halo dofs
        lat = lattice_of_local_nodes(nx, ny, nz, N, p["e0"], p["e1"])
        g = p["global_to_local"]
        assert np.array_equal(g >= 0, gmap[lat] >= 0)       # same masking as one rank
        assert np.array_equal(p["lattice"][g[g >= 0]], lat[g >= 0])
    with pytest.raises(lpg.LPGError):
        lpg.box_partition(nx, ny, nz, N, -1, 2, 0)           # periodic boxes are not partitioned
    with pytest.raises(lpg.LPGError):
        lpg.box_partition(nx, ny, 2, N, 1, 3, 0)             # more ranks than element layers


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    nx, ny, nz, N = CFG["BOX NX"], CFG["BOX NY"], CFG["BOX NZ"], CFG["POLYNOMIAL DEGREE"]
    Np = (N + 1) ** 3
    o = Oracle(CFG)                                  # the single-rank reference result
    p = lpg.box_partition(nx, ny, nz, N, 1, world, rank)
    E0, E1 = p["e0"], p["e1"]
    ggeo = o.array("ggeo").reshape(-1, 6 * Np)[E0:E1].ravel()
    wJ = o.array("wJ").reshape(-1, Np)[E0:E1].ravel()
    ref = refimpl.RefOperator(N, E1 - E0, p["global_to_local"], p["nlocal"], wJ, ggeo, o.array("D"),
                              CFG["LAMBDA"])
    q_of = lambda lat: np.sin(0.37 * lat) + 0.1 * np.cos(1.3 * lat)   # a field keyed by lattice id
    Aq = ref.apply(q_of(p["lattice"]))               # this rank's elements only
    # exchange the shared planes: pack, send/receive, add
    for nb, lst in ((rank - 1, p["below"]), (rank + 1, p["above"])):
        if 0 <= nb < world:
            send = torch.tensor(Aq[lst])
            recv = torch.empty_like(send)
            reqs = [dist.isend(send, nb), dist.irecv(recv, nb)]
            for rq in reqs:
                rq.wait()
            np.add.at(Aq, lst, recv.numpy())
    gmap = global_dof_of_lattice(o, nx, ny, nz, N)
    qg = np.zeros(o.Ngather)
    lat_all = np.nonzero(gmap >= 0)[0]
    qg[gmap[lat_all]] = q_of(lat_all)
    Aqg = o.operator(qg)
    err = rel_err(Aq, Aqg[gmap[p["lattice"]]])
    # inner product over owned dofs, all-reduced
    own = slice(0, p["nowned"])
    d = torch.tensor([float(np.dot(Aq[own], q_of(p["lattice"])[own]))], dtype=torch.float64)
    dist.all_reduce(d)
    out[rank] = (err, float(d), float(np.dot(Aqg, qg)))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.skipif(not refimpl.available(), reason="reference kernels not built here")
@pytest.mark.timeout(240)
@pytest.mark.parametrize("world", [2, 3])
def test_partitioned_operator_with_gloo_ranks(world):
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(200)
        assert pr.exitcode == 0
    for r in range(world):
        err, dot, ref = out[r]
        assert err < 1e-13, (r, err)
        assert abs(dot - ref) <= 1e-12 * abs(ref)
