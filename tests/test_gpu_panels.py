"""GPU parity of the memory-bounded Ozaki path: the contraction index streamed in atom panels
(each panel sliced with its own exponents, later panels accumulating into H and S), against the
oracle.  Panels are forced with HSDLA_PANELS, or chosen by the library when the workspace budget
(HSDLA_WORKSPACE_BUDGET) cannot hold one k-point's digit planes.  Tolerance 1e-13 relative
Frobenius and max-norm on the lower triangles, as for the resident path."""
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


@pytest.fixture
def env():
    """Panels belong to the per-atom form of the contraction: the structure-factor form (taken when
    no atom carries its own rotation) has small per-type digits and needs none, so it is off here."""
    saved = {k: os.environ.get(k) for k in ("HSDLA_PANELS", "HSDLA_WORKSPACE_BUDGET", "HSDLA_SF")}
    os.environ["HSDLA_SF"] = "0"
    yield os.environ
    for k, v in saved.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = v


def _check(res, s, kps):
    for (H, S), kp in zip(res, kps):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, R in ((H, Hr), (S, Sr)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (kp.n_g, fro, mx)
        iu = np.triu_indices(kp.n_g, 1)
        assert np.all(H[iu] == 0) and np.all(S[iu] == 0)


@pytest.mark.parametrize("cfg,panels,rot", [("t1", 2, False), ("t1", 5, False), ("t1", 3, True),
                                            ("c0", 3, False), ("c0", 4, True)])
def test_forced_panels_match_oracle(ctx, env, cfg, panels, rot):
    s = synth.make_system(cfg)
    if rot:
        s = synth.with_rotations(s)
    env["HSDLA_PANELS"] = str(panels)
    res, rep = ctx.create_hs(s, precision="ozaki")
    pa = -(-s.num_atoms // min(panels, s.num_atoms))
    assert rep["num_panels"] == min(panels, s.num_atoms) and pa >= 1
    _check(res, s, s.kpoints)


def test_panels_match_resident_path(ctx, env):
    """Panels change only the granularity of the exponents: H and S stay within 1e-14 of the
    resident run."""
    s = synth.make_system("c1")
    (r1,), _ = ctx.create_hs(s, precision="ozaki")
    env["HSDLA_PANELS"] = "4"
    (r4,), rep = ctx.create_hs(s, precision="ozaki")
    assert rep["num_panels"] == 4
    for X, R in zip(r4, r1):
        assert oracle.lower_errors(X, R)[0] < 1e-14


def test_budget_chooses_panels(ctx, env):
    """A workspace budget below one k-point's digit planes makes the library stream panels."""
    s = synth.make_system("c0")
    env["HSDLA_WORKSPACE_BUDGET"] = str(16 << 20)     # one k-point's resident digit planes need ~27 MB
    res, rep = ctx.create_hs(s, precision="ozaki", num_slices=11)
    assert rep["num_panels"] > 1, rep
    _check(res, s, s.kpoints)


def test_fleur_golden_with_panels(ctx, env):
    gs, gk, Hf, Sf = oracle.fleur_golden()
    env["HSDLA_PANELS"] = "2"
    (res,), rep = ctx.create_hs(gs, kpoints=[gk], precision="ozaki")
    assert rep["num_panels"] == 2
    for X, R in zip(res, (Hf, Sf)):
        fro, mx = oracle.lower_errors(X, R)
        assert fro < TOL and mx < TOL
