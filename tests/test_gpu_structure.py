"""The structure-factor form of S and H (atoms sharing their type's rotation): per-type
contractions M_t^H diag(w_t) M_t and M_t^H Z_t combined with SF_t(g' - g) = sum_a e^{i 2pi (g'-g).tau_a}.
It must agree with the per-atom form (HSDLA_SF=0) and with the oracle, in both precisions.
Tolerance 1e-13 relative Frobenius and max-norm on the lower triangles."""
import os

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


def _run(ctx, s, precision, sf):
    old = os.environ.get("HSDLA_SF")
    os.environ["HSDLA_SF"] = "1" if sf else "0"
    try:
        return ctx.create_hs(s, precision=precision, num_slices=11 if precision == "ozaki" else 0)
    finally:
        if old is None:
            os.environ.pop("HSDLA_SF")
        else:
            os.environ["HSDLA_SF"] = old


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("cfg", ["t1", "c0", "c1"])
def test_structure_factor_form_matches_per_atom_and_oracle(ctx, cfg, precision):
    s = synth.make_system(cfg)
    res_sf, rep_sf = _run(ctx, s, precision, True)
    res_pa, _ = _run(ctx, s, precision, False)
    for (H, S), (Hp, Sp), kp in zip(res_sf, res_pa, s.kpoints):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, P, R in ((H, Hp, Hr), (S, Sp, Sr)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (cfg, precision, fro, mx)
            assert oracle.lower_errors(X, P)[0] < TOL
        iu = np.triu_indices(kp.n_g, 1)
        assert np.all(H[iu] == 0) and np.all(S[iu] == 0)


def test_structure_factor_form_is_used(ctx):
    """Without per-atom rotations the S/H work shrinks to one contraction of 2L rows per type."""
    s = synth.make_system("c1")
    _, r_sf = _run(ctx, s, "fp64", True)
    _, r_pa = _run(ctx, s, "fp64", False)
    ratio = r_pa["dominant_flop"] / r_sf["dominant_flop"]
    assert abs(ratio - s.num_atoms / s.num_types) < 1e-9, ratio


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("batch", ["1", "2", "3"])
def test_type_batches_of_the_combine(ctx, precision, batch, monkeypatch):
    """The combine of one type at a time, of two (a full batch and a partial one over c1's four
    types) and of three: every split agrees with the oracle."""
    monkeypatch.setenv("HSDLA_TYPE_BATCH", batch)
    s = synth.make_system("c1")
    res, _ = _run(ctx, s, precision, True)
    for (H, S), kp in zip(res, s.kpoints):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, R in ((H, Hr), (S, Sr)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (batch, precision, fro, mx)


@pytest.mark.parametrize("knob", [("HSDLA_PAIR_HALVES", "1"), ("HSDLA_COMBINE_OVERLAP", "1"), ("HSDLA_MERGE", "0")])
def test_structure_factor_variants(ctx, knob, monkeypatch):
    """Full-width pair tiles, the half of the combine on a side stream, and one accumulation unit
    per digit diagonal: each agrees with the oracle (c1: four types, 3000 columns, so the combine
    of the host-buffer entry point runs in several 512-column blocks)."""
    monkeypatch.setenv(*knob)
    s = synth.make_system("c1")
    res, _ = _run(ctx, s, "ozaki", True)
    for (H, S), kp in zip(res, s.kpoints):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, R in ((H, Hr), (S, Sr)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (knob, fro, mx)
        iu = np.triu_indices(kp.n_g, 1)
        assert np.all(H[iu] == 0) and np.all(S[iu] == 0)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("batch", ["2", "8"])
def test_outputs_written_in_place(ctx, precision, batch, monkeypatch):
    """Page-locked host outputs: the combine writes H and S itself and the lower triangles equal,
    bit for bit, those of the download into pageable buffers; the strict upper triangle is not
    touched at all.  With a batch of 2 types the last batch's combine does it after the earlier
    batches on the device; with every type in one batch (Ozaki) the products run in column blocks
    and each block's combine writes its columns while the next block's products run."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("HSDLA_TYPE_BATCH", batch)
    s = synth.make_system("c1")
    res_ref, rep_ref = _run(ctx, s, precision, True)
    assert rep_ref["outputs_in_place"] == 0
    outs, keep = [], []
    for kp in s.kpoints:
        pair = []
        for _ in range(2):
            t = torch.full((kp.n_g, kp.n_g), complex(7.0, -3.0), dtype=torch.complex128).pin_memory()
            keep.append(t)
            pair.append(t.numpy().T)       # column-major view of the page-locked buffer
        outs.append(tuple(pair))
    monkeypatch.setenv("HSDLA_SF", "1")
    res, rep = ctx.create_hs(s, precision=precision, num_slices=11 if precision == "ozaki" else 0, out=outs)
    assert rep["outputs_in_place"] == 1
    assert (rep["output_blocks"] > 1) == (precision == "ozaki" and batch == "8"), rep["output_blocks"]
    for (H, S), (Hr, Sr), kp in zip(res, res_ref, s.kpoints):
        il = np.tril_indices(kp.n_g)
        iu = np.triu_indices(kp.n_g, 1)
        for X, R in ((H, Hr), (S, Sr)):
            assert np.array_equal(X[il], R[il])
            assert np.all(X[iu] == complex(7.0, -3.0))


def test_streamed_outputs_of_a_kpoint_group(ctx, monkeypatch):
    """Page-locked outputs of a group of three k-points with different basis sizes: the column-block
    launches run over every k-point's tiles, each block's columns go to the host (diagonal square
    in place, the rest by the copy engine) per k-point, and the lower triangles equal, bit for bit,
    the download into pageable buffers; the strict upper triangles stay untouched; the oracle
    agrees on the k-point with the fewest G-vectors."""
    torch = pytest.importorskip("torch")
    cfg = dict(synth.CONFIGS["c1"], kpts=[(0.1, 0.2, 0.3), (0.0, 0.0, 0.0), (0.25, -0.25, 0.5)],
               n_g=(2600, 3000))
    s = synth.make_system(cfg)
    assert len({kp.n_g for kp in s.kpoints}) > 1
    monkeypatch.setenv("HSDLA_TYPE_BATCH", "8")
    res_ref, rep_ref = ctx.create_hs(s, precision="ozaki", num_slices=11)
    assert rep_ref["outputs_in_place"] == 0
    outs, keep = [], []
    for kp in s.kpoints:
        pair = []
        for _ in range(2):
            t = torch.full((kp.n_g, kp.n_g), complex(7.0, -3.0), dtype=torch.complex128).pin_memory()
            keep.append(t)
            pair.append(t.numpy().T)
        outs.append(tuple(pair))
    res, rep = ctx.create_hs(s, precision="ozaki", num_slices=11, out=outs)
    assert rep["outputs_in_place"] == 1 and rep["output_blocks"] > 1, rep
    for (H, S), (Hr, Sr), kp in zip(res, res_ref, s.kpoints):
        il = np.tril_indices(kp.n_g)
        iu = np.triu_indices(kp.n_g, 1)
        for X, R in ((H, Hr), (S, Sr)):
            assert np.array_equal(X[il], R[il])
            assert np.all(X[iu] == complex(7.0, -3.0))
    k = int(np.argmin([kp.n_g for kp in s.kpoints]))
    Ho, So = oracle.reference_hs(s, s.kpoints[k])
    for X, R in ((res[k][0], Ho), (res[k][1], So)):
        fro, mx = oracle.lower_errors(X, R)
        assert fro < TOL and mx < TOL, (fro, mx)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("sf", [True, False])
@pytest.mark.parametrize("cfg,lmaxs", [("t1", (4, 2, 3)), ("c0", (6, 4))])
def test_types_with_different_lmax_match_oracle(ctx, cfg, lmaxs, precision, sf):
    """Types of one system with different lmax (the reference's per-atom lmaxs,
    h_and_s_stripped_v2.cpp:64-86: the rows l > lmax of an atom are zero), in both forms."""
    s = synth.make_system(cfg)
    s.type_lmax = np.asarray(lmaxs, np.int32)
    s.type_lmax_nonsph = np.asarray(lmaxs, np.int32)
    res, rep = _run(ctx, s, precision, sf)
    assert (rep["num_row_sets"] > 0) == sf
    for (H, S), kp in zip(res, s.kpoints):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, R in ((H, Hr), (S, Sr)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (cfg, precision, sf, fro, mx)


EDGE_CONFIGS = {
    # lmax 12 and 14 (2L = 338 and 450 per type: 3 and 4 contraction blocks, other unit plans)
    "lmax12": dict(cell=(10.0, 10.0, 12.0), atoms=4, types=2, rmt=2.0, min_sep=4.2, lmax=12,
                   kpts=[(0.1, 0.2, 0.3)], n_g=300, seed=21),
    "lmax14": dict(cell=(10.0, 10.0, 12.0), atoms=3, types=2, rmt=2.0, min_sep=4.2, lmax=14,
                   kpts=[(0.05, 0.15, 0.25)], n_g=260, seed=22),
    # twelve types of one atom each: every structure factor a single phase
    "types12": dict(cell=(14.0, 14.0, 14.0), atoms=12, types=12, rmt=1.8, min_sep=3.8, lmax=4,
                    kpts=[(0.1, 0.2, 0.3), (0.0, 0.0, 0.0)], n_g=(400, 520), seed=23),
}


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("sf", [True, False])
@pytest.mark.parametrize("name", sorted(EDGE_CONFIGS))
def test_edge_shapes_match_oracle(ctx, name, precision, sf):
    s = synth.make_system(EDGE_CONFIGS[name])
    res, rep = _run(ctx, s, precision, sf)
    assert (rep["num_row_sets"] > 0) == sf
    for (H, S), kp in zip(res, s.kpoints):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, R in ((H, Hr), (S, Sr)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (name, precision, sf, kp.n_g, fro, mx)
