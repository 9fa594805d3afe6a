"""GPU parity of the Ozaki FP8 path (tcgen05) through the C ABI.

* exactness: integer-valued operands whose digits capture every bit must give
  the FP64 product bit for bit (this pins the e4m3 digit encoding, the TMA /
  UMMA descriptors and the exact FP32 accumulation of integer products);
* accuracy: relative Frobenius and max-norm error vs the FP64 oracle <= 1e-13
  (the benchmark spec's bound) for the default slice count;
* the error falls as the slice count grows.
"""
import numpy as np
import pytest

import oracle
from hybridhsdla_gb300 import api, synth

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


def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _exact_limit(s):
    # entries below 2^(5h-1), h = (s+1)//2, have zero digits beyond the h-th, so every
    # nonzero digit product (i, j) has i + j <= s + 1 and is kept by the triangle
    return 2 ** (5 * ((s + 1) // 2) - 2)


@pytest.mark.parametrize("n,K,s", [(128, 128, 3), (200, 300, 5), (300, 1000, 7), (3000, 2000, 5)])
def test_ozaki_exact_on_integer_operands(ctx, n, K, s):
    """Integer operands that the kept digits represent exactly give the exact product, bit for
    bit; n = 3000 spans 78 CTA-pair tiles (more than one wave, a ragged last tile row)."""
    import torch
    rng = np.random.default_rng(n + K)
    lim = _exact_limit(s)
    P = rng.integers(-lim, lim, (n, K)) + 1j * rng.integers(-lim, lim, (n, K))
    Q = rng.integers(-lim, lim, (n, K)) + 1j * rng.integers(-lim, lim, (n, K))
    out = ctx.zherkx_lower(_dev(P), _dev(Q), None, precision="ozaki", num_slices=s)
    torch.cuda.synchronize()
    got = np.tril(out.cpu().numpy().T)
    ref = np.tril(P.conj() @ Q.T)            # exact: integers below 2^53
    assert np.array_equal(got, ref)


def test_ozaki_exact_across_accumulation_chunks(ctx):
    """K large enough that the low diagonals are split into several exact chunks
    (s = 7: diagonal t = 8 has 7 digit pairs, 4608 complex terms per chunk)."""
    import torch
    rng = np.random.default_rng(11)
    n, K, s = 128, 5000, 7
    lim = _exact_limit(s)
    P = rng.integers(-lim, lim, (n, K)) + 1j * rng.integers(-lim, lim, (n, K))
    out = ctx.zherkx_lower(_dev(P), None, None, precision="ozaki", num_slices=s)
    torch.cuda.synchronize()
    got = np.tril(out.cpu().numpy().T)
    ref = np.tril(P.conj() @ P.T)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("s", [6, 8, 10, 12])
def test_ozaki_zherkx_error_vs_fp64(ctx, s):
    import torch
    rng = np.random.default_rng(5)
    n, K = 260, 777
    P = rng.standard_normal((n, K)) + 1j * rng.standard_normal((n, K))
    Q = rng.standard_normal((n, K)) + 1j * rng.standard_normal((n, K))
    w = rng.uniform(0.01, 1.0, K)
    out = ctx.zherkx_lower(_dev(P), _dev(Q), _dev(w), precision="ozaki", num_slices=s)
    torch.cuda.synchronize()
    got = np.tril(out.cpu().numpy().T)
    ref = np.tril(P.conj() @ (w[:, None] * Q.T))
    fro, mx = oracle.lower_errors(got, ref)
    # each digit carries 5 bits: the error bound shrinks by 2^-5 per slice
    bound = 2.0 ** (-5 * s + 10)
    assert fro < bound and mx < bound, (s, fro, mx)


def _hs_parity(res, s, tol=TOL):
    for (H, S), kp in zip(res, s.kpoints):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, R, nm in ((H, Hr, "H"), (S, Sr, "S")):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < tol and mx < tol, (nm, kp.n_g, fro, mx)


@pytest.mark.parametrize("cfg", ["t0", "t1", "c0"])
def test_create_hs_ozaki_matches_oracle(ctx, cfg):
    s = synth.make_system(cfg)
    res, rep = ctx.create_hs(s, precision="ozaki")
    assert rep["num_slices"] >= 2
    _hs_parity(res, s)


def test_create_hs_ozaki_c1(ctx):
    s = synth.make_system("c1")
    res, rep = ctx.create_hs(s, precision="ozaki")
    _hs_parity(res, s)


def test_autotuned_slices_meet_target_c1(ctx):
    """num_slices = 0: the plan samples columns, checks them against FP64 and picks s."""
    import torch
    s = synth.make_system("c1")
    pl = ctx.plan(s, precision="ozaki", num_slices=0)
    outs = pl.alloc_outputs()
    rep = pl.execute(outs)
    torch.cuda.synchronize()
    assert 9 <= rep["num_slices"] <= 12
    assert 0 < rep["est_rel_err"] <= 0.25e-13
    H = np.tril(outs[0][0].cpu().numpy().T)
    S = np.tril(outs[0][1].cpu().numpy().T)
    _hs_parity([(H, S)], s)
    pl.close()


def test_create_hs_ozaki_rotations(ctx):
    s = synth.with_rotations(synth.make_system("t1"))
    res, _ = ctx.create_hs(s, precision="ozaki")
    _hs_parity(res, s)
