"""Failure detection on the GPU without a fault: a bounded wait of the kind the contraction
kernels use (an mbarrier wait, a grid-lockstep wait) runs out on a condition nothing satisfies,
after a short budget.  The kernel records the error word, frees its TMEM and returns; the host
reads HSDLA_ERR_TIMEOUT and the context keeps working."""
import numpy as np
import pytest

import oracle
from hybridhsdla_gb300 import api, synth

pytestmark = pytest.mark.gpu
BUDGET = 20_000_000          # SM cycles: ~10 ms


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    c = api.Context()
    yield c
    c.close()


@pytest.mark.parametrize("which,role", [(0, 7), (1, 5)])
def test_expired_wait_reports_timeout(ctx, which, role):
    rc = ctx.lib.hsdla_selftest_wait_timeout(ctx.h, which, BUDGET)
    assert rc == -5, rc                                      # HSDLA_ERR_TIMEOUT
    msg = ctx.lib.hsdla_last_error(ctx.h).decode()
    assert f"role {role}" in msg, msg


def test_context_usable_after_timeouts(ctx):
    for which in (0, 1, 0):
        assert ctx.lib.hsdla_selftest_wait_timeout(ctx.h, which, BUDGET) == -5
    s = synth.make_system("t0")
    (res,), _ = ctx.create_hs(s, precision="ozaki")
    Hr, Sr = oracle.reference_hs(s, s.kpoints[0])
    for X, R in zip(res, (Hr, Sr)):
        fro, mx = oracle.lower_errors(X, R)
        assert fro < 1e-13 and mx < 1e-13


def test_selftest_rejects_bad_arguments(ctx):
    assert ctx.lib.hsdla_selftest_wait_timeout(ctx.h, 2, BUDGET) == -1
    assert ctx.lib.hsdla_selftest_wait_timeout(ctx.h, 0, 0) == -1
