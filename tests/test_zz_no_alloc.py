"""The zero-allocation product entry point (dqmc_product_device_noalloc).

Callers that cannot allocate device memory at the point of the call (a host
framework that owns every device buffer through its own pool, or a time loop
that forbids allocation once it runs) pass their own device buffers for A, B and C; the slice scratch is a
fixed array inside the library.  This checks, through the C-ABI, that two
calls in a row give the same products as the allocating entry point
dqmc_product_check, within the product engine's accuracy bound (2^-38 of
|A||B|, as in tests/test_gpu_mixed.py), and that oversize requests are refused.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dq():
    import __graft_entry__ as g

    g.build()
    import dqmc_gb300

    return dqmc_gb300


def _noalloc(dq, a, b):
    import torch

    n = a.shape[0]
    # the caller's device buffers, column-major (Fortran order) as the C-ABI expects
    ta = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    tc = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = dq.load().dqmc_product_device_noalloc(n, ctypes.c_void_p(ta.data_ptr()), ctypes.c_void_p(tb.data_ptr()),
                                               ctypes.c_void_p(tc.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, dq.load().dqmc_last_error().decode()
    torch.cuda.synchronize()
    return tc.cpu().numpy().T


def test_noalloc_matches_allocating_entry_point(dq):
    rng = np.random.default_rng(2024)
    for n in (256, 100):  # two calls in a row share the scratch array
        a = rng.standard_normal((n, n)) * np.exp(rng.uniform(-10, 10, n))[:, None]
        b = rng.standard_normal((n, n)) * np.exp(rng.uniform(-10, 10, n))[None, :]
        c_new = _noalloc(dq, a, b)
        c_old = dq.product_check(a, b)
        bound = np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :] * n
        assert (np.abs(c_new - c_old) <= 2.0 ** -38 * bound).all()
        assert (np.abs(c_new - a @ b) <= 2.0 ** -38 * bound).all()


def test_noalloc_rejects_oversize(dq):
    L = dq.load()
    assert L.dqmc_product_device_noalloc(257, None, None, None, None) == 1
    assert b"256" in L.dqmc_last_error()
