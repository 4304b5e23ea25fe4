"""The partitioned operator on the GPU: per rank, lpg_ax_hex_f64 on the rank's element slab
(lpg_box_partition's element range and local numbering, the library's own geometric
factors of those elements), then the halo exchange through lpg_halo_pack_f64 /
lpg_halo_unpack_add_f64. The ranks are emulated one after the other on one GPU (the
exchange is a device copy between the ranks' buffers; no kernel waits on another), and
every rank must hold the single-rank operator's values at all its local dofs (1e-12)."""
import numpy as np
import pytest
import torch

import libparanumal_gb300 as lpg
from gpu_helpers import box, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(0)


def lattice_of_local_nodes(nx, ny, N, e0, e1):
    Nq = N + 1
    NX, NY = nx * N + 1, ny * N + 1
    e = np.arange(e0, e1)[:, None]
    n = np.arange(Nq ** 3)[None, :]
    a, b, c = n % Nq, (n // Nq) % Nq, n // (Nq * Nq)
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    return ((ex * N + a) + NX * ((ey * N + b) + NY * (ez * N + c))).ravel()


@pytest.mark.parametrize("nranks", [2, 4])
@pytest.mark.parametrize("bc,N", [(1, 7), (2, 4)])
def test_partitioned_operator_matches_single_rank(nranks, bc, N):
    nx, ny, nz = 3, 4, 6
    cfg = box(**{"BOX NX": nx, "BOX NY": ny, "BOX NZ": nz, "POLYNOMIAL DEGREE": N, "BOX BOUNDARY FLAG": bc,
                 "LAMBDA": 0.5})
    e = lpg.Elliptic(cfg)
    E, Np = e.info("nelements"), e.info("np")
    g2l = e.get("GlobalToLocal")
    gmap = np.full((nx * N + 1) * (ny * N + 1) * (nz * N + 1), -1, dtype=np.int64)
    gmap[lattice_of_local_nodes(nx, ny, N, 0, E)] = g2l
    ggeo, wJ, D = e.get("ggeo").reshape(E, 6 * Np), e.get("wJ").reshape(E, Np), e.get("D")
    q_of = lambda lat: np.sin(0.37 * lat) + 0.1 * np.cos(1.3 * lat)
    lat_all = np.nonzero(gmap >= 0)[0]
    qg = np.zeros(e.Nglobal)
    qg[gmap[lat_all]] = q_of(lat_all)
    dq = torch.tensor(qg, device="cuda")
    dAq = torch.empty_like(dq)
    e.Operator(dq, dAq)
    ref = dAq.cpu().numpy()
    L = lpg.lib()
    parts = [lpg.box_partition(nx, ny, nz, N, bc, nranks, r) for r in range(nranks)]
    dev = []
    for p in parts:
        E0, E1 = p["e0"], p["e1"]
        d = {k: torch.tensor(np.ascontiguousarray(v), device="cuda") for k, v in
             (("g2l", p["global_to_local"]), ("ggeo", ggeo[E0:E1].ravel()), ("wJ", wJ[E0:E1].ravel()),
              ("D", D), ("q", q_of(p["lattice"])), ("below", p["below"]), ("above", p["above"]))}
        d["Aq"] = torch.empty(p["nlocal"], dtype=torch.float64, device="cuda")
        lpg.ax_hex("f64", N, E1 - E0, d["g2l"], d["ggeo"], 6 * Np, d["wJ"], Np, d["D"], 0.5, d["q"], d["Aq"],
                   p["nlocal"])
        for side in ("below", "above"):
            d["buf_" + side] = torch.empty(len(p[side]), dtype=torch.float64, device="cuda")
            lpg.check(L.lpg_halo_pack_f64(len(p[side]), d[side].data_ptr(), d["Aq"].data_ptr(),
                                          d["buf_" + side].data_ptr(), None))
        dev.append(d)
    # exchange: rank r receives rank r+1's "below" at its "above" and rank r-1's "above" at its "below"
    for r, (p, d) in enumerate(zip(parts, dev)):
        if r > 0:
            lpg.check(L.lpg_halo_unpack_add_f64(len(p["below"]), d["below"].data_ptr(),
                                                dev[r - 1]["buf_above"].data_ptr(), d["Aq"].data_ptr(), None))
        if r < nranks - 1:
            lpg.check(L.lpg_halo_unpack_add_f64(len(p["above"]), d["above"].data_ptr(),
                                                dev[r + 1]["buf_below"].data_ptr(), d["Aq"].data_ptr(), None))
    torch.cuda.synchronize()
    for p, d in zip(parts, dev):
        assert rel_err(d["Aq"].cpu().numpy(), ref[gmap[p["lattice"]]]) < 1e-12
