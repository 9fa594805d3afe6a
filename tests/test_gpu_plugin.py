"""The BLAS-shaped contraction plugin (hsdla_zherk / hsdla_zher2k / hsdla_zherkx and the
Fortran-style hsdla_dev_* entry points) through the C ABI.

* Semantics: every flag of the reference's dev_zherk_ / dev_zher2k_ / dev_zherkx_
  (flapw_opt/src/include/acc/wrappers.h:19-28) -- uplo 'L' / 'U', trans 'N' / 'C', complex alpha,
  real beta including beta = 1 accumulation -- against the BLAS definitions evaluated by numpy,
  with device and host operands, in FP64 and Ozaki precision.  The other triangle of C stays as it
  was, zherk and zher2k leave a real diagonal, and beta = 0 never reads C.
* Drop-in: create_HS2_stripped_v2's own call sequence (h_and_s_stripped_v2.cpp:100-382) run with
  these entry points as its contraction backend, host buffers as the reference passes them, matches
  the oracle's H and S.
Tolerance 1e-13 relative (Frobenius and max-norm over the triangle written)."""
import zlib

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


def _rand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _op(X, trans):
    return X if trans == "N" else X.conj().T


def _expected(kind, uplo, trans, alpha, A, B, beta, C0):
    oA = _op(A, trans)
    if kind == "herk":
        P = alpha * oA @ oA.conj().T
    elif kind == "her2k":
        oB = _op(B, trans)
        P = alpha * oA @ oB.conj().T + np.conj(alpha) * oB @ oA.conj().T
    else:
        oB = _op(B, trans)
        P = alpha * oA @ oB.conj().T
    out = P + (beta * C0 if beta != 0 else 0)
    if kind != "herkx":
        # BLAS: the diagonal of a Hermitian update is real, the input diagonal's imaginary part ignored
        d = np.arange(C0.shape[0])
        out[d, d] = np.real(np.diag(P)) + (beta * np.real(np.diag(C0)) if beta != 0 else 0)
    return out


def _tri(uplo, n):
    return np.tril_indices(n) if uplo == "L" else np.triu_indices(n)


def _check(kind, uplo, trans, alpha, A, B, beta, C0, got):
    n = C0.shape[0]
    exp = _expected(kind, uplo, trans, alpha, A, B, beta, C0)
    iu = _tri(uplo, n)
    d = got[iu] - exp[iu]
    fro = np.linalg.norm(d) / np.linalg.norm(exp[iu])
    mx = np.abs(d).max() / np.abs(exp[iu]).max()
    assert fro <= TOL and mx <= TOL, (kind, uplo, trans, beta, fro, mx)
    other = _tri("U" if uplo == "L" else "L", n)
    off = other[0] != other[1]
    np.testing.assert_array_equal(got[other[0][off], other[1][off]], C0[other[0][off], other[1][off]])
    if kind != "herkx":
        assert np.all(np.diag(got).imag == 0)


def _call(ctx, kind, where, uplo, trans, n, k, alpha, A, B, beta, C, precision):
    import torch
    lda = A.shape[0]
    if where == "device":
        t = lambda X: torch.from_numpy(np.asfortranarray(X).T.copy()).cuda() if X is not None else None  # noqa: E731
        dA, dB, dC = t(A), t(B), t(C)
        if kind == "herk":
            ctx.zherk(uplo, trans, n, k, alpha.real, dA, lda, beta, dC, n, precision=precision)
        else:
            getattr(ctx, "z" + kind)(uplo, trans, n, k, alpha, dA, lda, dB, lda, beta, dC, n, precision=precision)
        torch.cuda.synchronize()
        return dC.cpu().numpy().T
    hA, hB = np.asfortranarray(A), (np.asfortranarray(B) if B is not None else None)
    hC = np.asfortranarray(C.copy())
    if kind == "herk":
        ctx.zherk(uplo, trans, n, k, alpha.real, hA, lda, beta, hC, n, precision=precision)
    else:
        getattr(ctx, "z" + kind)(uplo, trans, n, k, alpha, hA, lda, hB, lda, beta, hC, n, precision=precision)
    return hC


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("kind", ["herk", "her2k", "herkx"])
@pytest.mark.parametrize("uplo,trans,beta,where", [("L", "C", 0.0, "device"), ("U", "C", 1.0, "device"),
                                                   ("L", "N", 0.5, "host"), ("U", "N", 0.0, "host"),
                                                   ("L", "C", 1.0, "host")])
def test_plugin_semantics(ctx, precision, kind, uplo, trans, beta, where):
    rng = np.random.default_rng(zlib.crc32(repr((precision, kind, uplo, trans, beta, where)).encode()))
    n, k = 203, 345
    shape = (n, k) if trans == "N" else (k, n)
    A = _rand(rng, *shape)
    B = _rand(rng, *shape) if kind != "herk" else None
    alpha = 0.75 if kind == "herk" else 0.6 - 0.8j
    C0 = _rand(rng, n, n)
    if beta == 0.0:
        # beta = 0 must not read C: NaNs in the triangle written do not propagate
        C0[_tri(uplo, n)] = np.nan
    got = _call(ctx, kind, where, uplo, trans, n, k, np.complex128(alpha), A, B, beta, C0, precision)
    ref_C0 = np.where(np.isnan(C0), 0, C0)
    _check(kind, uplo, trans, alpha, A, B, beta, ref_C0, np.where(np.isnan(got), 1e300, got))


def test_plugin_alpha_zero_and_k_zero_scale_c(ctx):
    rng = np.random.default_rng(7)
    n = 70
    C0 = _rand(rng, n, n)
    C = np.asfortranarray(C0.copy())
    A = np.asfortranarray(_rand(rng, 5, n))
    ctx.zherk("L", "C", n, 0, 1.0, A, 5, 0.5, C, n)
    il = np.tril_indices(n)
    exp = 0.5 * C0
    exp[np.arange(n), np.arange(n)] = 0.5 * C0.diagonal().real
    np.testing.assert_allclose(C[il], exp[il], rtol=0, atol=1e-15)
    C = np.asfortranarray(C0.copy())
    ctx.zherkx("U", "C", n, 5, 0.0, A, 5, A, 5, 2.0, C, n)
    iu = np.triu_indices(n)
    np.testing.assert_allclose(C[iu], 2.0 * C0[iu], rtol=0, atol=1e-15)


def test_plugin_rejects_bad_flags(ctx):
    A = np.zeros((4, 4), np.complex128, order="F")
    with pytest.raises(api.HsdlaError) as e:
        ctx.zherk("X", "C", 4, 4, 1.0, A, 4, 0.0, A, 4)
    assert e.value.code == -1 and "uplo" in str(e.value)
    with pytest.raises(api.HsdlaError) as e:
        ctx.zherk("L", "T", 4, 4, 1.0, A, 4, 0.0, A, 4)
    assert e.value.code == -1 and "trans" in str(e.value)
    with pytest.raises(api.HsdlaError) as e:
        ctx.zherk("L", "C", 4, 8, 1.0, A, 4, 0.0, A, 4)       # lda < k
    assert e.value.code == -1


# ------------------------------------------------ create_HS2_stripped_v2 with this backend
def _stripped_v2_on_plugin(L, a, A, B, blocks, lmaxs, sqrt_u_norms):
    """create_HS2_stripped_v2 (h_and_s_stripped_v2.cpp:100-382) call by call, its contraction
    backend calls (dev_zherk_ :158 and :177, dev_zher2k_ :300, dev_zherkx_ :362) going to the
    library's hsdla_dev_* entry points with the reference's arguments and host buffers; the per-atom
    T loops and their row compaction stay on the host, as in the reference."""
    from scipy.linalg import blas
    A = np.array(A, order="F", copy=True)
    B = np.array(B, order="F", copy=True)
    La, G = A.shape
    S = np.zeros((G, G), np.complex128, order="F")
    H = np.zeros((G, G), np.complex128, order="F")
    api.dev_zherk_("L", "C", G, La, 1.0, A, La, 0.0, S, G)
    lin = np.zeros(La)
    for at in range(a):
        for l in range(int(lmaxs[at]) + 1):
            lin[at * L + l * l: at * L + (l + 1) ** 2] = sqrt_u_norms[at][l]
    W = np.asfortranarray(B * lin[:, None])
    api.dev_zherk_("L", "C", G, La, 1.0, W, La, 1.0, S, G)
    X = np.zeros((La, G), np.complex128, order="F")
    xh = 0
    for at in range(a):
        aa, ab, bb = blocks[at]
        nbb, nab = bb.shape[0], ab.shape[0]
        tmp = np.zeros((L, G), np.complex128, order="F")
        if nbb:
            tmp[:nbb] = blas.zhemm(0.5, np.asfortranarray(bb), np.asfortranarray(B[at * L: at * L + nbb]), side=0,
                                   lower=1)
        if nab:
            tmp[:nab] += blas.zgemm(1.0, np.asfortranarray(ab), np.asfortranarray(A[at * L: at * L + nab]),
                                    trans_a=2)
        m = max(nab, nbb)
        X[xh: xh + m] = tmp[:m]
        if xh != at * L:
            B[xh: xh + m] = B[at * L: at * L + m].copy()
        xh += m
    api.dev_zher2k_("L", "C", G, xh, 1.0, B, La, X, La, 0.0, H, G)
    xn = 0
    for at in range(a):
        aa = blocks[at][0]
        m = aa.shape[0]
        if xn != at * L:
            A[xn: xn + m] = A[at * L: at * L + m].copy()
        if m:
            B[xn: xn + m] = blas.zhemm(1.0, np.asfortranarray(aa), np.asfortranarray(A[xn: xn + m]), side=0, lower=1)
        xn += m
    # X' lives in B's storage, as in the reference (X = B, :323)
    api.dev_zherkx_("L", "C", G, xn, 1.0, A, La, B, La, 1.0, H, G)
    return np.tril(H), np.tril(S)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("cfg", ["c0", "c1"])
def test_stripped_v2_sequence_on_the_plugin_matches_oracle(ctx, cfg, precision):
    s = synth.make_system(cfg)
    kp = s.kpoints[0]
    A, B = oracle.construct_ab(s, kp)
    aa, ab, bb = oracle.prepare_tmats(s)
    blocks = [(aa[t], ab[t], bb[t]) for t in s.atom_type]
    un = np.sqrt(oracle.per_atom_unorm(s))
    api.dev_init(0, precision, 0)
    try:
        H, S = _stripped_v2_on_plugin(s.L, s.num_atoms, A, B, blocks, s.type_lmax[s.atom_type], un)
    finally:
        api.dev_finalize()
    Hr, Sr = oracle.reference_hs(s, kp)
    for X, R, nm in ((H, Hr, "H"), (S, Sr, "S")):
        fro, mx = oracle.lower_errors(X, R)
        assert fro <= TOL and mx <= TOL, (cfg, precision, nm, fro, mx)
