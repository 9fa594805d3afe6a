"""(type, rotation) classes: atoms with their own rotations (as FleurData gives every atom
mrot bmat, FleurData.cpp:52-62, 453-455; the rows use them, tensor_AB_match.cpp:97) keep the
structure-factor form when the atoms of a type share a few rotations.  The library groups them by
itself; the result must match the oracle (which builds every atom's rows with its own rotation)
and the per-atom form, in both precisions.  Tolerance 1e-13 relative Frobenius and max-norm."""
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


def _run(ctx, s, precision, classes=True):
    old = os.environ.get("HSDLA_CLASSES")
    os.environ["HSDLA_CLASSES"] = "1" if classes else "0"
    try:
        return ctx.create_hs(s, precision=precision, num_slices=11 if precision == "ozaki" else 0)
    finally:
        if old is None:
            os.environ.pop("HSDLA_CLASSES")
        else:
            os.environ["HSDLA_CLASSES"] = old


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("cfg", ["t1", "c1"])
def test_two_rotation_classes_per_type_match_oracle(ctx, cfg, precision):
    s = synth.with_class_rotations(synth.make_system(cfg), per_type=2)
    res, rep = _run(ctx, s, precision)
    n_cls = len({(int(t), r.tobytes()) for t, r in zip(s.atom_type, s.atom_rotmat)})
    if 4 * n_cls <= 3 * s.num_atoms:
        assert rep["rotation_classes"] == 1 and rep["num_row_sets"] == n_cls
    else:
        assert rep["num_row_sets"] == 0          # too few atoms per class: the per-atom form
    res_pa, rep_pa = _run(ctx, s, precision, classes=False)
    assert rep_pa["num_row_sets"] == 0
    for (H, S), (Hp, Sp), kp in zip(res, res_pa, s.kpoints):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, P, R, nm in ((H, Hp, Hr, "H"), (S, Sp, Sr, "S")):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (cfg, precision, nm, fro, mx)
            assert oracle.lower_errors(P, R)[0] < TOL


def test_identity_rotations_given_per_atom_take_the_type_form(ctx):
    """A caller that passes every atom's rotation, all mrot = 1 (rotmat = bmat), as the
    reference's AtomData always holds them: the classes are the types."""
    s = synth.make_system("c1")
    s.atom_rotmat = np.repeat(s.bmat[None], s.num_atoms, axis=0)
    res, rep = _run(ctx, s, "ozaki")
    assert rep["rotation_classes"] == 1 and rep["num_row_sets"] == s.num_types
    (H, S), = res
    Hr, Sr = oracle.reference_hs(s, s.kpoints[0])
    for X, R in ((H, Hr), (S, Sr)):
        fro, mx = oracle.lower_errors(X, R)
        assert fro < TOL and mx < TOL, (fro, mx)


def test_every_atom_its_own_rotation_keeps_the_per_atom_form(ctx):
    s = synth.with_rotations(synth.make_system("t1"))
    _, rep = _run(ctx, s, "fp64")
    assert rep["num_row_sets"] == 0 and rep["rotation_classes"] == 0
