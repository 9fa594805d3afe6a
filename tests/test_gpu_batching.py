"""k-point groups and CUDA-graph execution of a plan (the batched, captured form).

* every k-point of a group goes through one launch per stage; a small workspace
  budget (HSDLA_WORKSPACE_BUDGET) splits a plan into several groups that reuse
  one workspace -- results must not depend on the grouping;
* with use_graph the whole execution is captured once and replayed; outputs move
  through pinned job tables, so new output buffers re-capture and match too.
"""
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


def _host(outs):
    return [(np.tril(h.cpu().numpy().T), np.tril(s.cpu().numpy().T)) for h, s in outs]


def _check(res, sys_, kps):
    for (H, S), kp in zip(res, kps):
        Hr, Sr = oracle.reference_hs(sys_, kp)
        for X, R in ((H, Hr), (S, Sr)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (kp.n_g, fro, mx)


@pytest.mark.parametrize("prec", ["fp64", "ozaki"])
def test_groups_of_one_kpoint_match_one_group(ctx, prec, monkeypatch):
    import torch
    s = synth.make_system("t1")                     # three k-points (one at Gamma)
    # the same type batches in both plans (a budget-chosen batch would differ): types {0, 1}, {2}
    monkeypatch.setenv("HSDLA_TYPE_BATCH", "2")
    one = ctx.plan(s, precision=prec, num_slices=11 if prec == "ozaki" else 0)
    o1 = one.alloc_outputs()
    one.execute(o1)
    torch.cuda.synchronize()
    monkeypatch.setenv("HSDLA_WORKSPACE_BUDGET", "1")   # every k-point its own group
    monkeypatch.setenv("HSDLA_PANELS", "1")             # grouping only: no atom panels
    split = ctx.plan(s, precision=prec, num_slices=11 if prec == "ozaki" else 0)
    o2 = split.alloc_outputs()
    split.execute(o2)
    split.execute(o2)                                  # second run reuses the prepared groups
    torch.cuda.synchronize()
    a, b = _host(o1), _host(o2)
    for (h1, s1), (h2, s2) in zip(a, b):
        assert np.array_equal(h1, h2) and np.array_equal(s1, s2)
    _check(b, s, s.kpoints)
    one.close()
    split.close()


@pytest.mark.parametrize("prec", ["fp64", "ozaki"])
def test_graph_replay_matches_direct_run(ctx, prec):
    import torch
    s = synth.make_system("t1")
    direct = ctx.plan(s, precision=prec, num_slices=11 if prec == "ozaki" else 0)
    od = direct.alloc_outputs()
    direct.execute(od)
    graphed = ctx.plan(s, precision=prec, num_slices=11 if prec == "ozaki" else 0, use_graph=True)
    og = graphed.alloc_outputs()
    for _ in range(3):                                 # capture, then replays
        rep = graphed.execute(og)
    og2 = graphed.alloc_outputs()                      # new outputs: re-capture
    graphed.execute(og2)
    torch.cuda.synchronize()
    ref = _host(od)
    for outs in (og, og2):
        for (h1, s1), (h2, s2) in zip(ref, _host(outs)):
            assert np.array_equal(h1, h2) and np.array_equal(s1, s2)
    assert rep["kernel_launches"] > 0
    assert rep["ms_dominant"] > 0             # the graph keeps external timing nodes
    direct.close()
    graphed.close()


def test_batched_c0_ozaki_multi_kpoint(ctx):
    """Four k-points of c0 (n_G 490..510 after re-targeting) in one group, one S/H launch."""
    import torch
    base = synth.make_system("c0")
    kps = [synth.KPoint(k=np.array(k, dtype=np.float64), g=synth.g_vectors(base.bmat, np.array(k), ng))
           for k, ng in (((0.1, 0.2, 0.3), 500), ((0.0, 0.0, 0.0), 490), ((0.25, 0.25, -0.25), 510),
                         ((-0.3, 0.1, 0.05), 497))]
    pl = ctx.plan(base, kpoints=kps, precision="ozaki", num_slices=11)
    outs = pl.alloc_outputs()
    pl.execute(outs)
    torch.cuda.synchronize()
    _check(_host(outs), base, kps)
    pl.close()


def test_c3_subset_ozaki_graph_vs_fp64(ctx):
    """Batching form (c3: 64 atoms, lmax 8, n_G ~6300): two k-points, graph-captured Ozaki
    against the batched FP64 path on the GPU, and one k-point against the oracle."""
    import torch
    s = synth.make_system("c3")
    kps = s.kpoints[:2]
    oz = ctx.plan(s, kpoints=kps, precision="ozaki", num_slices=0, use_graph=True)
    oo = oz.alloc_outputs()
    oz.execute(oo)
    rep = oz.execute(oo)
    fp = ctx.plan(s, kpoints=kps, precision="fp64")
    of = fp.alloc_outputs()
    fp.execute(of)
    torch.cuda.synchronize()
    for (h1, s1), (h2, s2) in zip(_host(oo), _host(of)):
        for X, R in ((h1, h2), (s1, s2)):
            fro, mx = oracle.lower_errors(X, R)
            assert fro < TOL and mx < TOL, (fro, mx)
    assert rep["num_slices"] >= 9
    _check(_host(of)[:1], s, kps[:1])
    oz.close()
    fp.close()
