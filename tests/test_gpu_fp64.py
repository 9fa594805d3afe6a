"""GPU parity of the plain-FP64 path against the CPU oracle, through the C ABI.

Tolerances: A/B element-wise 1e-13 relative to max|A|, |B| (same FP64
recurrences, different sin/cos implementations and FMA contraction); H and S
1e-13 relative Frobenius and max-norm over the lower triangle (the bound the
north star names for the FP64 path).
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


def _ab_parity(ctx, s):
    import torch
    pl = ctx.plan(s)
    for ik, kp in enumerate(s.kpoints):
        C = pl.construct_ab(ik).cpu().numpy()
        A, B = api.split_ab(C, s.L, s.num_atoms)
        Ar, Br = oracle.construct_ab(s, kp)
        for X, R in ((A, Ar), (B, Br)):
            err = np.abs(X - R).max() / np.abs(R).max()
            assert err < TOL, (ik, err)
    pl.close()


@pytest.mark.parametrize("cfg", ["t0", "t1", "c0"])
def test_construct_ab_matches_oracle(ctx, cfg):
    _ab_parity(ctx, synth.make_system(cfg))


def test_construct_ab_with_rotations_matches_oracle(ctx):
    _ab_parity(ctx, synth.with_rotations(synth.make_system("t1")))


def _hs_parity(res, s, kps, tol=TOL):
    tm = oracle.prepare_tmats(s)
    for (H, S), kp in zip(res, kps):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, R in ((H, Hr), (S, Sr)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < tol and mx < tol, (kp.n_g, fro, mx)
        # the upper triangle is returned as zero
        iu = np.triu_indices(kp.n_g, 1)
        assert np.all(H[iu] == 0) and np.all(S[iu] == 0)


@pytest.mark.parametrize("cfg", ["t0", "t1", "c0"])
def test_create_hs_fp64_matches_oracle(ctx, cfg):
    s = synth.make_system(cfg)
    res, rep = ctx.create_hs(s, precision="fp64")
    assert rep["kernel_launches"] >= 3          # construct, T application, S/H (k-points batched)
    _hs_parity(res, s, s.kpoints)


def test_create_hs_fp64_rotations(ctx):
    s = synth.with_rotations(synth.make_system("t1"))
    res, _ = ctx.create_hs(s, precision="fp64")
    _hs_parity(res, s, s.kpoints)


def test_plan_execute_device_fp64_c1(ctx):
    import torch
    s = synth.make_system("c1")
    pl = ctx.plan(s, precision="fp64")
    outs = pl.alloc_outputs()
    rep = pl.execute(outs)
    torch.cuda.synchronize()
    # device buffers are column-major: tensor[col, row]
    H = outs[0][0].cpu().numpy().T
    S = outs[0][1].cpu().numpy().T
    _hs_parity([(np.tril(H), np.tril(S))], s, s.kpoints)
    assert rep["eff_tflops"] > 0
    pl.close()


def test_zherkx_fp64_standalone(ctx):
    import torch
    rng = np.random.default_rng(3)
    n, K = 300, 517
    P = rng.standard_normal((n, K)) + 1j * rng.standard_normal((n, K))   # row g = column g of the K x n matrix
    Q = rng.standard_normal((n, K)) + 1j * rng.standard_normal((n, K))
    w = rng.uniform(0.1, 1.0, K)
    dP, dQ = torch.from_numpy(P).cuda(), torch.from_numpy(Q).cuda()
    dw = torch.from_numpy(w).cuda()
    out = ctx.zherkx_lower(dP, dQ, dw, precision="fp64")
    torch.cuda.synchronize()
    got = np.tril(out.cpu().numpy().T)
    ref = np.tril(P.conj() @ (w[:, None] * Q.T))
    fro, mx = oracle.lower_errors(got, ref)
    assert fro < 1e-14 and mx < 1e-14


# ------------------------------------------------------------ failure paths
def test_rejects_bad_ld(ctx):
    s = synth.make_system("t0")
    kp = s.kpoints[0]
    small = [(np.zeros((kp.n_g - 1, kp.n_g), np.complex128, order="F"),
              np.zeros((kp.n_g - 1, kp.n_g), np.complex128, order="F"))]
    with pytest.raises(api.HsdlaError) as e:
        ctx.create_hs(s, out=small)
    assert e.value.code == -1


def test_rejects_nan_radial_data(ctx):
    s = synth.make_system("t0")
    s.u[0, 1] = np.nan
    with pytest.raises(api.HsdlaError) as e:
        ctx.create_hs(s)
    assert e.value.code == -4


def test_rejects_zero_wronskian(ctx):
    s = synth.make_system("t0")
    s.u[1, 2], s.u_dr[1, 2], s.dE_u[1, 2], s.dE_u_dr[1, 2] = 1.0, 2.0, 0.5, 1.0   # W = 0.5*2 - 1*1 = 0
    with pytest.raises(api.HsdlaError) as e:
        ctx.create_hs(s)
    assert e.value.code == -4


def test_rejects_non_hermitian_taa(ctx):
    s = synth.make_system("t0")
    tm = list(oracle.prepare_tmats(s))
    tm[0] = tm[0].copy()
    tm[0][0, 1, 0] += 0.5
    with pytest.raises(api.HsdlaError) as e:
        ctx.create_hs(s, tmats=tuple(tm))
    assert e.value.code == -4


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_rejects_non_hermitian_tbb_and_nonfinite_tab(ctx, precision):
    """The T blocks are checked on the device as they are assembled: T_BB not Hermitian, or a
    non-finite value in T_AB, is an input error naming the block, and the context stays usable.
    hsdla_create_hs reads the check after its launches; the non-finite entry is assembled as
    zero, so the Ozaki digit slicing of T and of T M meets finite values only."""
    s = synth.make_system("t0")
    base = oracle.prepare_tmats(s)
    tm = [x.copy() for x in base]
    tm[2][1, 3, 1] += 0.25j
    with pytest.raises(api.HsdlaError) as e:
        ctx.create_hs(s, tmats=tuple(tm), precision=precision)
    assert e.value.code == -4 and "T_BB of type 1 is not Hermitian" in str(e.value)
    tm = [x.copy() for x in base]
    tm[1][0, 2, 3] = np.nan
    with pytest.raises(api.HsdlaError) as e:
        ctx.create_hs(s, tmats=tuple(tm), precision=precision)
    assert e.value.code == -4 and "T block 1 of type 0 not finite" in str(e.value)
    res, _ = ctx.create_hs(s, tmats=base, precision=precision)
    assert np.isfinite(res[0][0]).all()


def test_memory_cap_reports_nomem(ctx):
    s = synth.make_system("c0")
    ctx.set_mem_cap(1 << 16)
    try:
        with pytest.raises(api.HsdlaError) as e:
            ctx.create_hs(s)
        assert e.value.code == -3
    finally:
        ctx.set_mem_cap(0)
    res, _ = ctx.create_hs(s)       # the context stays usable
    assert np.isfinite(res[0][0]).all()


def test_empty_kpoint_is_a_noop(ctx):
    s = synth.make_system("t0")
    kp = synth.KPoint(k=np.zeros(3), g=np.zeros((0, 3), np.int32))
    res, rep = ctx.create_hs(s, kpoints=[kp])
    assert res[0][0].shape == (0, 0)
