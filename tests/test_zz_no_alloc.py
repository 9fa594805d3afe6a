"""The allocation-free entry point hsdla_zherkx_lower_noalloc, through the C ABI.

It serves callers that cannot allocate device memory: code inside another
framework's memory pool or under a fixed memory budget, plug-ins that may only
touch the buffers they are handed, and processes that must not call cudaMalloc
once running.  Its scratch is one static 128 MiB device array, shared by every
call.  Two calls in a row (different shapes and data) must agree with the
allocating entry point hsdla_zherkx_lower (Ozaki, same slice count) and with the
FP64 product, within the 1e-13 bound the other tests use.  This file is collected
last so that a failure here cannot hide any other test.
"""
import ctypes

import numpy as np
import pytest

import oracle
from hybridhsdla_gb300 import api

pytestmark = pytest.mark.gpu
TOL = 1e-13


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    c = api.Context()
    yield c
    c.close()


def _lower(t):
    return np.tril(t.cpu().numpy().T)      # device buffers are column-major: tensor[col, row]


def test_noalloc_matches_allocating_entry_on_two_calls(ctx):
    import torch
    rng = np.random.default_rng(2024)
    for n, K in ((300, 777), (520, 1500)):
        P = rng.standard_normal((n, K)) + 1j * rng.standard_normal((n, K))
        Q = rng.standard_normal((n, K)) + 1j * rng.standard_normal((n, K))
        w = rng.uniform(0.01, 1.0, K)
        dP, dQ, dw = (torch.from_numpy(x).cuda() for x in (P, Q, w))
        ref = ctx.zherkx_lower(dP, dQ, dw, precision="ozaki", num_slices=11)
        out = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
        got = api.zherkx_lower_noalloc(dP, dQ, dw, num_slices=11, out=out)
        torch.cuda.synchronize()
        g, r = _lower(got), _lower(ref)
        fro, mx = oracle.lower_errors(g, r)
        assert fro <= TOL and mx <= TOL, (n, K, fro, mx)
        exact = np.tril(P.conj() @ (w[:, None] * Q.T))
        fro, mx = oracle.lower_errors(g, exact)
        assert fro <= TOL and mx <= TOL, (n, K, fro, mx)


def test_noalloc_rejects_problems_beyond_the_static_scratch(ctx):
    import torch
    L = api.load()
    small = torch.zeros((4, 4), dtype=torch.complex128, device="cuda")
    p = ctypes.c_void_p(small.data_ptr())
    # n = 4096, k = 8192 needs far more than 128 MiB: rejected before any data is touched
    rc = L.hsdla_zherkx_lower_noalloc(11, 4096, 8192, p, 8192, p, 8192, None, p, 4096, None)
    assert rc == -6
