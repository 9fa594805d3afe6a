"""Pins of the CPU oracle (test infrastructure) before it is trusted.

The reference's own tests pin no value on this path (``flapw_opt/tests/
FleurWrap_test.cpp:33-67`` only prints Bessel/Ylm values), so the restated
special functions are pinned against independent closed forms (scipy), the
restated BLAS call sequence against the reference's naive formulas
(``h_and_s.cpp:88-162``), and both against the committed golden fixtures.
"""
import math

import numpy as np
import pytest
import scipy.special as sp

import oracle
from hybridhsdla_gb300 import synth


@pytest.mark.parametrize("x", [0.0, 1e-5, 5e-4, 1e-3, 0.37, 3.41, 7.5, 9.9, 10.0, 10.5, 14.2, 25.0])
@pytest.mark.parametrize("lmax", [1, 3, 6, 10, 12])
def test_sphbes_against_closed_form(lmax, x):
    fj = oracle.sphbes(lmax, x)
    ref = sp.spherical_jn(np.arange(lmax + 1), x)
    # downward Miller recursion and the small-x series are accurate to a few ulps of
    # the largest j_l; upward recursion (lmax < x) loses relative accuracy for
    # tiny high-l values, so compare relative to max |j_l|
    scale = max(np.abs(ref).max(), 1e-300)
    assert np.abs(fj - ref).max() / scale < 5e-13
    dfj = oracle.dsphbs(lmax, x, fj)
    dref = sp.spherical_jn(np.arange(lmax + 1), x, derivative=True)
    # dsphbs.f:33-36 uses dj_l = j_{l-1} - (l+1) j_l / x for x >= 1e-4, which cancels
    # catastrophically for small x (relative error ~ eps / x^2): that is the
    # reference's own accuracy, so the bound follows it
    tol = 5e-12 + (1e-15 / x ** 2 if x > 0 else 0.0)
    assert np.abs(dfj - dref).max() / max(np.abs(dref).max(), 1e-300) < tol


def test_sphbes_rejects_bad_arguments():
    with pytest.raises(ValueError):
        oracle.sphbes(0, 1.0)
    with pytest.raises(ValueError):
        oracle.sphbes(3, -1.0)


@pytest.mark.parametrize("v", [(3.12, 4.3, 9.3), (0.0, 0.0, 1.0), (0.0, 0.0, -2.0), (1.0, -2.0, 0.0),
                               (-0.3, 0.1, -0.7), (0.0, 0.0, 0.0), (1e-14, 0.0, 1.0)])
@pytest.mark.parametrize("lmax", [1, 3, 8, 10])
def test_ylm4_against_closed_form(lmax, v):
    y = oracle.ylm4(lmax, v)
    v = np.asarray(v)
    r = np.linalg.norm(v)
    theta = math.acos(v[2] / r) if r > 1e-12 else 0.0
    rxy = math.hypot(v[0], v[1])
    phi = math.atan2(v[1], v[0]) if rxy > 1e-12 else 0.0
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            ref = sp.sph_harm_y(l, m, theta, phi)
            assert abs(y[l * (l + 1) + m] - ref) < 1e-13, (l, m)


def test_kmesh_matches_cartesian_for_diagonal_bmat():
    s = synth.make_system("t0")
    kp = s.kpoints[0]
    rk = oracle.kmesh(kp.k, s.bmat, kp.g)
    cart = np.linalg.norm((kp.g + kp.k[None, :]) @ s.bmat, axis=1)
    np.testing.assert_allclose(rk, cart, rtol=1e-15)


def test_prepare_tmats_semantics():
    s = synth.make_system("t1")
    aa, ab, bb = oracle.prepare_tmats(s)
    L = s.L
    for t in range(s.num_types):
        lm = np.arange(L)
        l_of = np.floor(np.sqrt(lm)).astype(int)
        E = s.energies[t][l_of]
        np.testing.assert_allclose(aa[t] - np.diag(E), s.taa_raw[t], atol=1e-15)
        np.testing.assert_allclose(bb[t] - np.diag(E * s.dE_u_norm[t][l_of]), s.tbb_raw[t], atol=1e-15)
        np.testing.assert_allclose(ab[t] - 0.5 * np.eye(L), s.tab_raw[t], atol=1e-15)
        assert np.allclose(aa[t], aa[t].conj().T) and np.allclose(bb[t], bb[t].conj().T)


def test_prepare_tmats_zero_nonsph():
    s = synth.make_system("t0")
    s.type_lmax_nonsph[:] = 1
    aa, ab, bb = oracle.prepare_tmats(s)
    n0 = 4
    for T in (aa, ab, bb):
        off = T[0].copy()
        off[np.diag_indices(s.L)] = 0
        assert np.all(off[n0:, :] == 0) and np.all(off[:, n0:] == 0)


@pytest.mark.parametrize("cfg", ["t0", "t1"])
def test_blas_sequence_matches_naive(cfg):
    s = synth.make_system(cfg)
    tm = oracle.prepare_tmats(s)
    for kp in s.kpoints:
        A, B = oracle.construct_ab(s, kp)
        Hn, Sn = oracle.hs_naive(s, A, B, tm)
        Hb, Sb = oracle.blas_sequence(s, A.copy(order="F"), B.copy(order="F"), tm)
        assert oracle.lower_errors(Sb, Sn)[0] < 1e-14
        assert oracle.lower_errors(Hb, Hn)[0] < 1e-13
        # H and S are Hermitian by construction
        assert np.abs(Hn - Hn.conj().T).max() <= 1e-13 * np.abs(Hn).max()
        assert np.abs(Sn - Sn.conj().T).max() <= 1e-13 * np.abs(Sn).max()


def test_construct_ab_k_equals_zero_edge():
    # t1's second k-point is Gamma, so G = 0 gives K = 0 (the small-x series branches)
    s = synth.make_system("t1")
    kp = s.kpoints[1]
    assert np.any(np.all(kp.g == 0, axis=1))
    A, B = oracle.construct_ab(s, kp)
    assert np.all(np.isfinite(A)) and np.all(np.isfinite(B))


def test_construct_ab_matches_formula_spot():
    """Spot check of tensor_AB_match.cpp:109-122 with independent scipy special functions."""
    s = synth.make_system("t0")
    kp = s.kpoints[0]
    A, B = oracle.construct_ab(s, kp)
    L = s.L
    for i in (0, 5, kp.n_g - 1):
        K = kp.k + kp.g[i]
        Kc = K @ s.bmat
        kn = np.linalg.norm(Kc)
        theta = math.acos(Kc[2] / kn)
        phi = math.atan2(Kc[1], Kc[0])
        for j in range(s.num_atoms):
            t = s.atom_type[j]
            x = s.type_rmt[t] * kn
            phase = np.exp(2j * math.pi * np.dot(K, s.atom_pos[j]))
            for l in range(s.max_lmax + 1):
                jl = sp.spherical_jn(l, x)
                djl = sp.spherical_jn(l, x, derivative=True)
                w = s.dE_u[t, l] * s.u_dr[t, l] - s.u[t, l] * s.dE_u_dr[t, l]
                common = 4 * math.pi / math.sqrt(s.vol_cell) * phase / w
                au = s.dE_u[t, l] * kn * djl - s.dE_u_dr[t, l] * jl
                bu = -s.u[t, l] * kn * djl + s.u_dr[t, l] * jl
                for m in range(-l, l + 1):
                    y = np.conj(sp.sph_harm_y(l, m, theta, phi))
                    r = l * (l + 1) + m + L * j
                    assert abs(A[r, i] - y * common * au) < 1e-13 * max(1.0, abs(A[r, i]))
                    assert abs(B[r, i] - y * common * bu) < 1e-13 * max(1.0, abs(B[r, i]))
