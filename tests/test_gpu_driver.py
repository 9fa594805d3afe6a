"""The driver's h_and_s run (flapw_opt/src/h_and_s.cpp:897-954) on the GPU: a Fleur dump in, H and
S per k-point through hsdla_create_hs, time.info out.  On the reference's two-atom dump (the
committed fixture, which carries Fleur's own H and S) the whole chain -- the dump reader, the
library's radial solver and T assembly, the GPU path -- must reproduce Fleur's H and S to 1e-13
relative Frobenius and max-norm, in both precisions."""
import io
import json
import os

import numpy as np
import pytest

from hybridhsdla_gb300 import driver

pytestmark = pytest.mark.gpu
FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fleur_two_atoms.npz")
TOL = 1e-13


@pytest.fixture(scope="module", autouse=True)
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


@pytest.mark.parametrize("precision", ["ozaki", "fp64"])
def test_run_on_the_fleur_dump_reproduces_fleur(tmp_path, precision):
    out = io.StringIO()
    ti = str(tmp_path / "time.info")
    times, res = driver.run(FIXTURE, 60, precision, ti, out=out)
    lines = [json.loads(x) for x in out.getvalue().splitlines()]
    err = [x for x in lines if "vs_fleur_k0" in x][0]["vs_fleur_k0"]
    assert max(err.values()) <= TOL, err
    t = driver.read_time_info(ti)
    assert t.size == 1 and t[0] > 0 and np.isclose(t[0], times[0])


def test_run_on_a_synthetic_configuration_caps_the_kpoints(tmp_path):
    ti = str(tmp_path / "time.info")
    times, res = driver.run("t1", 2, "ozaki", ti, out=io.StringIO())
    assert len(times) == 2 and len(res) == 2
    assert driver.read_time_info(ti).size == 2


def test_cli_entry(tmp_path):
    ti = str(tmp_path / "t.info")
    assert driver.main(["run", FIXTURE, "1", "compute", "--precision", "fp64", "--time-info", ti]) == 0
    assert driver.read_time_info(ti).size == 1
