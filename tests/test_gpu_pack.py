"""GPU tests of the eigensolver hand-off in Fleur's packed form (``hsdla_pack_lower``): the lower
triangle row by row (fleur/src/binmat.f90:194-219; unpacked by flapw_opt/tests/flapw_verify.py:68-82).
Packing is a copy, so results are compared bit for bit; the end-to-end case packs the library's H
and S of the reference's two-atom sample and compares them with Fleur's own packed arrays to 1e-13."""
import numpy as np
import pytest

import oracle
from hybridhsdla_gb300 import api

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    c = api.Context()
    yield c
    c.close()


def _packed_ref(A):
    """Row-by-row lower triangle of a row-major numpy matrix A[r, c]."""
    return A[np.tril_indices(A.shape[0])]


@pytest.mark.parametrize("n", [1, 31, 32, 33, 100, 257])
def test_pack_matches_layout(ctx, n):
    import torch
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    M = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()        # M[col, row] = A[row, col]
    P = ctx.pack_lower(M)
    torch.cuda.synchronize()
    assert np.array_equal(P.cpu().numpy(), _packed_ref(A))


def test_pack_with_leading_dimension(ctx):
    """ld > n: only the n x n block is read."""
    import torch
    n, ld = 70, 96
    rng = np.random.default_rng(5)
    A = rng.standard_normal((ld, ld)) + 1j * rng.standard_normal((ld, ld))
    M = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()        # stride(0) = ld
    out = torch.empty(n * (n + 1) // 2, dtype=torch.complex128, device="cuda")
    ctx.check(ctx.lib.hsdla_pack_lower(ctx.h, n, api.ctypes.c_void_p(M.data_ptr()), ld,
                                       api.ctypes.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), _packed_ref(A[:n, :n]))


def test_pack_rejects_bad_ld(ctx):
    with pytest.raises(api.HsdlaError) as e:
        ctx.check(ctx.lib.hsdla_pack_lower(ctx.h, 10, None, 5, None, None))
    assert e.value.code == -1


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_fleur_packed_handoff(ctx, precision):
    """H and S of the two-atom sample, packed on the GPU, against Fleur's packed dump."""
    import torch
    d = np.load(oracle.GOLDEN_FLEUR)
    gs, gk, _, _ = oracle.fleur_golden()
    pl = ctx.plan(gs, kpoints=[gk], precision=precision)
    outs = pl.alloc_outputs()
    pl.execute(outs)
    for M, ref in ((outs[0][0], d["H_packed"]), (outs[0][1], d["S_packed"])):
        P = ctx.pack_lower(M).cpu().numpy()
        rel = np.linalg.norm(P - ref) / np.linalg.norm(ref)
        assert rel < 1e-13, rel
    pl.close()
