"""Host-side checks of the C-ABI library that need no GPU: it builds, loads,
exports every symbol include/hsdla.h declares, and its host-only helpers
(T-matrix preparation) agree with the oracle."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from hybridhsdla_gb300 import api, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "hsdla.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(hsdla_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    path = api.load().__dict__.get("_name") or api.lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (hsdla_[a-z0-9_]+)", out))
    declared = _declared_symbols()
    assert declared, "no declarations parsed"
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    assert sorted(api.EXPORTS) == declared


def test_struct_layouts_match_header():
    # sizes fixed by include/hsdla.h (LP64)
    assert ctypes.sizeof(api.SystemStruct) == 4 * 4 + 8 + 9 * 8 + 13 * 8
    assert ctypes.sizeof(api.KpointStruct) == 3 * 8 + 8 + 8
    assert ctypes.sizeof(api.OptsStruct) == 48
    assert ctypes.sizeof(api.ReportStruct) == 11 * 8 + 12 * 4


def _header_fields(struct_name):
    txt = open(os.path.join(ROOT, "include", "hsdla.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\}" % struct_name, txt, flags=re.S).group(1)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if decl:
            names += [re.sub(r"\[.*\]", "", v).strip(" *") for v in decl.split(None, 1)[1].split(",")]
    return names


def test_report_fields_match_header():
    """The report's fields in the header's order (the Python mirror reads them by position)."""
    assert [f for f, _ in api.ReportStruct._fields_] == _header_fields("hsdla_report")


@pytest.mark.parametrize("cfg", ["t0", "t1", "c0"])
def test_prepare_tmat_matches_oracle(cfg):
    s = synth.make_system(cfg)
    mine = api.prepare_tmats(s)
    ref = oracle.prepare_tmats(s)
    for a, b in zip(mine, ref):
        np.testing.assert_array_equal(a, b)


def test_prepare_tmat_zero_nonsph_matches_oracle():
    s = synth.make_system("t1")
    s.type_lmax_nonsph[:] = 2
    for a, b in zip(api.prepare_tmats(s), oracle.prepare_tmats(s)):
        np.testing.assert_array_equal(a, b)


def test_prepare_tmat_rejects_mismatched_diagonals():
    s = synth.make_system("t0")
    s.tab_raw[0, 0, 0] += 0.25j      # diag(tab) != diag(tab^H) -> TMat invariant broken
    with pytest.raises(api.HsdlaError):
        api.prepare_tmats(s)


def test_context_without_gpu_reports_device_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(api.HsdlaError) as e:
        api.Context()
    assert e.value.code == -7


def test_noalloc_argument_errors_carry_a_message():
    """The entry point without a context reports through hsdla_last_error(NULL) on the calling
    thread; argument checks run before any device call, so this needs no GPU."""
    L = api.load()
    rc = L.hsdla_zherkx_lower_noalloc(99, 4, 4, None, 4, None, 4, None, None, 4, None)
    assert rc == -1
    assert b"num_slices" in L.hsdla_last_error(None)
    rc = L.hsdla_zherkx_lower_noalloc(11, 4, 8, None, 4, None, 4, None, None, 4, None)
    assert rc == -1
    assert b"leading dimension" in L.hsdla_last_error(None)
