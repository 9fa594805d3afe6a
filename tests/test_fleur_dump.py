"""The library's Fleur-dump side on the CPU: the radial solver behind the matching values
(hsdla_radial_match, Fleur's radfun), the AtomData a dump turns into (FleurData::populate_atomdata,
AtomData::generate_matchdata), the HDF5 reader and the time.info output of the driver.  Checked
against the oracle's own restatement on the reference's two-atom dump (the committed fixture)."""
import os

import numpy as np
import pytest

import oracle
from hybridhsdla_gb300 import api, driver, fleur_dump

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fleur_two_atoms.npz")


def test_radial_match_agrees_with_the_oracle():
    d = fleur_dump.load(FIXTURE)
    worst = 0.0
    for t in range(d.lmax.size):
        vr = d.potential[t][:int(d.mesh_num[t])]
        for l in range(int(d.lmax[t]) + 1):
            a = fleur_dump.radial_match(l, d.energies[t][l], vr, d.mesh_rmt[t], d.mesh_dx[t])
            b = oracle.radfun(l, d.energies[t][l], vr, d.mesh_rmt[t], d.mesh_dx[t])
            worst = max(worst, float(np.max(np.abs(a - b) / np.abs(b))))
    assert worst < 1e-13, worst


def test_radial_match_rejects_bad_meshes():
    L_ = api.load()
    import ctypes
    vr = np.ones(5)
    out = np.zeros(5)
    dp = ctypes.POINTER(ctypes.c_double)
    assert L_.hsdla_radial_match(0, -0.5, vr.ctypes.data_as(dp), 5, 2.0, 0.02, out.ctypes.data_as(dp)) == -1
    vr = np.full(100, np.nan)
    assert L_.hsdla_radial_match(0, -0.5, vr.ctypes.data_as(dp), 100, 2.0, 0.02, out.ctypes.data_as(dp)) == -4


def test_dump_system_matches_the_oracles_reading():
    s = fleur_dump.to_system(fleur_dump.load(FIXTURE))
    g, kp, _, _ = oracle.fleur_golden()
    for f in ("bmat", "atom_pos", "atom_rotmat", "type_rmt", "energies"):
        np.testing.assert_array_equal(getattr(s, f), getattr(g, f), err_msg=f)
    for f in ("atom_type", "type_lmax", "type_lmax_nonsph"):
        np.testing.assert_array_equal(getattr(s, f), getattr(g, f), err_msg=f)
    assert s.vol_cell == g.vol_cell
    for f in ("u", "u_dr", "dE_u", "dE_u_dr", "dE_u_norm"):
        np.testing.assert_allclose(getattr(s, f), getattr(g, f), rtol=1e-13, atol=0, err_msg=f)
    for f in ("taa_raw", "tbb_raw", "tab_raw"):
        np.testing.assert_array_equal(np.tril(getattr(s, f)[0]), np.tril(getattr(g, f)[0]), err_msg=f)
    np.testing.assert_array_equal(s.kpoints[0].g, kp.g)
    np.testing.assert_array_equal(s.kpoints[0].k, kp.k)


def test_time_info_round_trip(tmp_path):
    p = str(tmp_path / "time.info")
    driver.write_time_info(p, [1.5, 2.25, 3.0])
    assert open(p).readline().strip() == "ARMA_MAT_TXT_FN008"
    np.testing.assert_array_equal(driver.read_time_info(p), [1.5, 2.25, 3.0])


@pytest.mark.skipif(not os.environ.get("HSDLA_FLEUR_DUMP"), reason="HSDLA_FLEUR_DUMP names no fleur_dump.h5")
def test_h5_reader_matches_the_fixture():
    """The HDF5 reader on the reference's two-atom dump (where it is available) reads what the
    committed fixture holds."""
    h = fleur_dump.load(os.environ["HSDLA_FLEUR_DUMP"])
    n = fleur_dump.load(FIXTURE)
    for f in ("real_basis", "rec_basis", "atom_type", "atom_pos", "atom_mrot", "mesh_num", "mesh_dx", "mesh_rmt",
              "lmax", "lmax_nonsph", "energies", "potential"):
        np.testing.assert_array_equal(getattr(h, f), getattr(n, f), err_msg=f)
    np.testing.assert_array_equal(h.k_points[0], n.k_points[0])
    np.testing.assert_array_equal(h.g_meshes[0], n.g_meshes[0])
    for th, tn in zip(h.tmats, n.tmats):
        for a, b in zip(th, tn):
            np.testing.assert_array_equal(np.tril(a), np.tril(b))
