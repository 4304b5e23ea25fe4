"""The allocation-free inner product, lpg_dot_f64_noalloc.

Callers that cannot let a library allocate device memory (host frameworks that own all
device memory through their own pool; latency-sensitive loops where cudaMalloc/cudaFree
would synchronise the device) use this entry point instead of lpg_dot_f64, whose partial
sums live in a buffer allocated on first use. Its partial sums live in a fixed device
array of the library instead.

The test calls it through the C ABI and compares it with the allocating entry point on
two calls in a row (the second smaller than the first, so stale partial sums left in
the shared array would show), using the tolerance of the other reduction tests. It
runs alone in a fresh process as well as after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_dot_noalloc_matches_allocating_dot_on_consecutive_calls():
    import __graft_entry__ as g
    g.build()
    import libparanumal_gb300 as lpg
    L = lpg.lib()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(20)
    for n in (3_000_001, 1_000):
        x = torch.tensor(rng.standard_normal(n), device="cuda")
        y = torch.tensor(rng.standard_normal(n), device="cuda")
        out = torch.zeros(2, dtype=torch.float64, device="cuda")
        lpg.check(L.lpg_dot_f64(n, x.data_ptr(), y.data_ptr(), out.data_ptr(), None))
        lpg.check(L.lpg_dot_f64_noalloc(n, x.data_ptr(), y.data_ptr(), out.data_ptr() + 8, None))
        torch.cuda.synchronize()
        ref, got = out.cpu().numpy()
        assert abs(got - ref) <= 1e-12 * max(1.0, np.sqrt(n)), (n, got, ref)
        assert abs(got - float(np.dot(x.cpu().numpy(), y.cpu().numpy()))) <= 1e-12 * max(1.0, np.sqrt(n))


def test_dot_noalloc_rejects_sizes_beyond_its_maximum():
    import __graft_entry__ as g
    g.build()
    import libparanumal_gb300 as lpg
    L = lpg.lib()
    torch.cuda.set_device(0)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = L.lpg_dot_f64_noalloc((1 << 40) + 1, out.data_ptr(), out.data_ptr(), out.data_ptr(), None)
    assert st == -1
    assert b"2^40" in L.lpg_last_error()
    st = L.lpg_dot_f64_noalloc(-1, out.data_ptr(), out.data_ptr(), out.data_ptr(), None)
    assert st == -1
