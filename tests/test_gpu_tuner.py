"""The autotuner's choices beyond the slice count: the structure-factor form's S/H tile shape
(256 x 256 accumulators, or two 256 x 128 halves in alternating TMEM buffers) and accumulation
split (adjacent digit diagonals merged into one exact FP32 unit, or one unit per diagonal) are
timed on the plan's own data after its first run, cached per shape in the context, and reported.
Every configuration gives H and S within 1e-13 of the oracle, and a CUDA graph captured before the
choice is re-captured with it."""
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


def _lower(t):
    return np.tril(t.cpu().numpy().T)


def test_first_run_tunes_tiles_and_reports_them(ctx):
    import torch
    s = synth.make_system("c1")
    pl = ctx.plan(s, precision="ozaki", num_slices=11)
    outs = pl.alloc_outputs()
    r1 = pl.execute(outs)
    torch.cuda.synchronize()
    assert r1["tile_tuned"] == 1 and r1["tile_halves"] in (1, 2) and r1["merged_units"] in (0, 1)
    r2 = pl.execute(outs)                     # the tuned configuration
    torch.cuda.synchronize()
    assert (r2["tile_halves"], r2["merged_units"]) == (r1["tile_halves"], r1["merged_units"])
    Hr, Sr = oracle.reference_hs(s, s.kpoints[0])
    for X, R in ((_lower(outs[0][0]), Hr), (_lower(outs[0][1]), Sr)):
        fro, mx = oracle.lower_errors(X, R)
        assert fro < TOL and mx < TOL, (fro, mx)
    pl.close()
    # a second plan of the same shape takes the cached choice
    pl2 = ctx.plan(s, precision="ozaki", num_slices=11)
    o2 = pl2.alloc_outputs()
    r3 = pl2.execute(o2)
    assert (r3["tile_halves"], r3["merged_units"], r3["tile_tuned"]) == (r1["tile_halves"], r1["merged_units"], 1)
    pl2.close()


@pytest.mark.parametrize("cfg", ["c0", "t1"])
@pytest.mark.parametrize("halves,merge", [("1", "1"), ("2", "0"), ("1", "0")])
def test_every_tile_configuration_matches_oracle(ctx, cfg, halves, merge):
    """c0 (2L = 98: whole k-blocks) and t1 (2L = 50: the 256 x 256 accumulators stop the
    k-block after two K steps)."""
    env = {"HSDLA_PAIR_HALVES": halves, "HSDLA_MERGE": merge}
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        s = synth.make_system(cfg)
        res, rep = ctx.create_hs(s, precision="ozaki", num_slices=11)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k)
            else:
                os.environ[k] = v
    assert rep["tile_halves"] == int(halves) and rep["merged_units"] == int(merge) and rep["tile_tuned"] == 0
    for (H, S), kp in zip(res, s.kpoints):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, R in ((H, Hr), (S, Sr)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (cfg, halves, merge, fro, mx)


def test_graph_is_recaptured_with_the_tuned_tiles(ctx):
    """A batched plan captured in a CUDA graph on its first run: the replays after the tuner's
    choice match the first run (to rounding) and the oracle."""
    import torch
    s = synth.make_system("t1")
    pl = ctx.plan(s, precision="ozaki", num_slices=11, use_graph=True)
    outs = pl.alloc_outputs()
    pl.execute(outs)
    torch.cuda.synchronize()
    first = [(_lower(H), _lower(S)) for H, S in outs]
    for _ in range(2):
        rep = pl.execute(outs)
    torch.cuda.synchronize()
    assert rep["tile_tuned"] == 1
    for (H, S), (H1, S1), kp in zip(outs, first, s.kpoints):
        Hr, Sr = oracle.reference_hs(s, kp)
        for X, X1, R in ((_lower(H), H1, Hr), (_lower(S), S1, Sr)):
            assert oracle.lower_errors(X, X1)[0] < 1e-15
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (fro, mx)
    pl.close()
