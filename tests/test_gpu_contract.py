"""GPU parity of the contraction-only drop-in (``hsdla_contract_ab``, the counterpart of the
reference's ``create_HS2_stripped_v2``) against the oracle's general-size restatement, and the
data.in -> data.out command-line path.

Tolerance: 1e-13 relative Frobenius and max-norm over the lower triangle, both precisions.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from hybridhsdla_gb300 import api, flapw_data, synth

pytestmark = pytest.mark.gpu
TOL = 1e-13
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    c = api.Context()
    yield c
    c.close()


def _data(cfg, shrink=False):
    s = synth.make_system(cfg)
    kp = s.kpoints[0]
    A, B = oracle.construct_ab(s, kp)
    d = flapw_data.from_system(s, kp, A, B, oracle.prepare_tmats(s))
    if shrink:
        blocks = []
        for j, (aa, ab, bb) in enumerate(d.blocks):
            n = aa.shape[0] - (j % 3) * 2
            blocks.append((aa[:n, :n].copy(), ab[:n - (j % 2), :n - (j % 2)].copy(), bb[:n, :n].copy()))
        d.blocks = blocks
    return d


def _check(H, S, d):
    Hr, Sr = oracle.stripped_v2(d.L, d.a, d.A, d.B, d.blocks, d.lmaxs, d.max_lmax, d.sqrt_u_norms)
    for X, R in ((H, Hr), (S, Sr)):
        fro, mx = oracle.lower_errors(X, R)
        assert fro < TOL and mx < TOL, (fro, mx)
    iu = np.triu_indices(d.G, 1)
    assert np.all(H[iu] == 0) and np.all(S[iu] == 0)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("cfg,shrink", [("t0", False), ("t1", False), ("t1", True), ("c0", True)])
def test_contract_ab_matches_oracle(ctx, cfg, shrink, precision):
    d = _data(cfg, shrink)
    H, S, rep = ctx.contract_ab(d, precision=precision)
    _check(H, S, d)
    assert rep["kernel_launches"] >= 2


def test_contract_ab_equals_create_hs(ctx):
    """Fed the A/B that create_hs builds itself, the contraction-only entry gives the same H, S."""
    s = synth.make_system("t1")
    kp = s.kpoints[1]
    pl = ctx.plan(s, kpoints=[kp])
    A, B = api.split_ab(pl.construct_ab(0).cpu().numpy(), s.L, s.num_atoms)
    pl.close()
    d = flapw_data.from_system(s, kp, A, B, api.prepare_tmats(s))
    H, S, _ = ctx.contract_ab(d, precision="fp64")
    (H2, S2), = ctx.create_hs(s, kpoints=[kp], precision="fp64")[0]
    assert oracle.lower_errors(H, H2)[0] < 1e-14 and oracle.lower_errors(S, S2)[0] < 1e-14


def test_contract_ab_rejects_oversized_block(ctx):
    d = _data("t0")
    aa, ab, bb = d.blocks[0]
    big = np.zeros((d.L + 1, d.L + 1), np.complex128)
    d.blocks[0] = (big, ab, bb)
    with pytest.raises(api.HsdlaError) as e:
        ctx.contract_ab(d)
    assert e.value.code == -1


def test_driver_contract_round_trip(ctx, tmp_path):
    d = _data("t1", shrink=True)
    fin, fout = str(tmp_path / "data.in"), str(tmp_path / "data.out")
    flapw_data.write_data_in(fin, d)
    r = subprocess.run([sys.executable, "-m", "hybridhsdla_gb300.driver", "contract", fin, fout,
                        "--precision", "ozaki"], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    H, S = flapw_data.read_data_out(fout)
    _check(H, S, d)
