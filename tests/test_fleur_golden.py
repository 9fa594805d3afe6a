"""Parity pin against the reference's known-answer data: Fleur's own muffin-tin H and S for
the two-atom sample (``flapw_opt/tests/sample_input/two_atoms/fleur_dump.h5``, extracted into
``tests/golden/fleur_two_atoms.npz`` by ``tests/golden/make_fleur_golden.py``).

The oracle rebuilds everything the reference derives from the dump -- radial matching values
(Fleur's radial solver), T-matrix assembly, zero_nonsph and augmentation, A/B, the
create_HS2_stripped_v2 BLAS sequence -- and must land on Fleur's numbers.  Tolerance:
1e-13 relative Frobenius and max-norm on the lower triangles (observed about 3e-15 and 8e-15).
"""
import numpy as np
import pytest

import oracle

TOL = 1e-13


@pytest.fixture(scope="module")
def golden():
    return oracle.fleur_golden()


def test_fixture_shape(golden):
    s, kp, Hf, Sf = golden
    assert s.num_atoms == 2 and s.L == 81 and kp.n_g == 235
    assert list(s.type_lmax_nonsph) == [6, 6]
    # Fleur's H and S are Hermitian with a real diagonal and a positive definite S
    assert np.abs(np.diag(Hf).imag).max() < 1e-15 and np.abs(np.diag(Sf).imag).max() < 1e-15
    Sfull = Sf + np.tril(Sf, -1).conj().T
    assert np.linalg.eigvalsh(Sfull).min() > 0


def test_radial_solver_wronskian(golden):
    """Scalar-relativistic u, udot at R: R^2 (udot u' - u udot') stays close to 2, its value
    for the equations radsra/radsrd integrate (p' = 2M r q + p, Hartree units) in the
    non-relativistic limit; <udot|udot> is positive."""
    s = golden[0]
    R = s.type_rmt[:, None]
    w = R ** 2 * (s.dE_u * s.u_dr - s.u * s.dE_u_dr)
    assert np.all(np.abs(w - 2) < 2e-3), w
    assert np.all(s.dE_u_norm > 0)


def test_oracle_blas_sequence_matches_fleur(golden):
    s, kp, Hf, Sf = golden
    H, S = oracle.reference_hs(s, kp)
    for X, R in ((H, Hf), (S, Sf)):
        fro, mx = oracle.lower_errors(X, R)
        assert fro < TOL and mx < TOL, (fro, mx)


def test_oracle_naive_formulas_match_fleur(golden):
    s, kp, Hf, Sf = golden
    A, B = oracle.construct_ab(s, kp)
    H, S = oracle.hs_naive(s, A, B, oracle.prepare_tmats(s))
    for X, R in ((H, Hf), (S, Sf)):
        fro, mx = oracle.lower_errors(X, R)
        assert fro < TOL and mx < TOL, (fro, mx)


def test_planted_error_is_detected(golden):
    """A radial value off by 1e-9 relative moves H well past the tolerance: the pin is tight."""
    s, kp, Hf, Sf = golden
    s.u = s.u.copy()
    s.u[0, 2] *= 1 + 1e-9
    H, _ = oracle.reference_hs(s, kp)
    assert oracle.lower_errors(H, Hf)[0] > TOL
