"""The reference's contraction-only wire format (data.in / data.out) and the oracle's
general-size restatement of create_HS2_stripped_v2 -- CPU only."""
import numpy as np

import oracle
from hybridhsdla_gb300 import flapw_data, synth


def _data(cfg="t1", shrink=False):
    s = synth.make_system(cfg)
    kp = s.kpoints[0]
    A, B = oracle.construct_ab(s, kp)
    d = flapw_data.from_system(s, kp, A, B, oracle.prepare_tmats(s))
    if shrink:
        # smaller per-atom blocks exercise the reference's row compaction (X_height)
        blocks = []
        for j, (aa, ab, bb) in enumerate(d.blocks):
            n = aa.shape[0] - (j % 3) * 2
            blocks.append((aa[:n, :n].copy(), ab[:n - (j % 2), :n - (j % 2)].copy(), bb[:n, :n].copy()))
        d.blocks = blocks
    return s, kp, d


def test_data_in_round_trip(tmp_path):
    _, _, d = _data()
    p = tmp_path / "data.in"
    flapw_data.write_data_in(str(p), d)
    e = flapw_data.read_data_in(str(p))
    assert (e.L, e.a, e.G, e.max_lmax) == (d.L, d.a, d.G, d.max_lmax)
    assert np.array_equal(e.A, d.A) and np.array_equal(e.B, d.B)
    assert np.array_equal(e.lmaxs, d.lmaxs) and np.array_equal(e.sqrt_u_norms, d.sqrt_u_norms)
    for x, y in zip(e.blocks, d.blocks):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)
    # the byte layout of h_and_s.cpp:763-786
    n = p.stat().st_size
    exp = 12 + 2 * 16 * d.L * d.a * d.G + sum(3 * 4 + 16 * sum(t.shape[0] ** 2 for t in b) for b in d.blocks) \
        + 4 * d.a + 4 + 8 * d.a * (d.max_lmax + 1)
    assert n == exp


def test_data_out_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    H = rng.standard_normal((7, 7)) + 1j * rng.standard_normal((7, 7))
    S = rng.standard_normal((7, 7)) + 1j * rng.standard_normal((7, 7))
    p = tmp_path / "data.out"
    flapw_data.write_data_out(str(p), H, S)
    H2, S2 = flapw_data.read_data_out(str(p))
    assert np.array_equal(H, H2) and np.array_equal(S, S2)
    assert p.stat().st_size == 4 + 2 * 16 * 49


def test_stripped_v2_full_blocks_matches_blas_sequence():
    s, kp, d = _data()
    H1, S1 = oracle.stripped_v2(d.L, d.a, d.A, d.B, d.blocks, d.lmaxs, d.max_lmax, d.sqrt_u_norms)
    H2, S2 = oracle.blas_sequence(s, d.A.copy(order="F"), d.B.copy(order="F"), oracle.prepare_tmats(s))
    assert oracle.lower_errors(H1, H2)[0] < 1e-14 and oracle.lower_errors(S1, S2)[0] < 1e-14


def test_stripped_v2_compaction_equals_zero_padding():
    """Smaller T blocks and the reference's row compaction give the same H as zero-padded
    full-size blocks (the formulation the GPU path uses)."""
    s, kp, d = _data(shrink=True)
    H1, S1 = oracle.stripped_v2(d.L, d.a, d.A, d.B, d.blocks, d.lmaxs, d.max_lmax, d.sqrt_u_norms)
    padded = []
    for aa, ab, bb in d.blocks:
        blk = []
        for T in (aa, ab, bb):
            P = np.zeros((d.L, d.L), np.complex128)
            P[:T.shape[0], :T.shape[0]] = T
            blk.append(P)
        padded.append(tuple(blk))
    H2, S2 = oracle.stripped_v2(d.L, d.a, d.A, d.B, padded, d.lmaxs, d.max_lmax, d.sqrt_u_norms)
    assert oracle.lower_errors(H1, H2)[0] < 1e-14
    assert np.array_equal(S1, S2)
