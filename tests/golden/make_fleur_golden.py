"""Generate ``fleur_two_atoms.npz``: the reference's only known-answer data for the H/S path.

Source: ``flapw_opt/tests/sample_input/two_atoms/fleur_dump.h5`` in the reference tree, the
dump Fleur writes for the two-atom sample (read by ``flapw_opt/src/FleurData.cpp:175-458``).
It holds the cell, atoms, radial meshes, potentials, energy parameters, Fleur's raw T
matrices and Fleur's own muffin-tin H and S for k-point 1 (packed lower triangles, row-major
packing as ``flapw_opt/tests/flapw_verify.py:68-82`` unpacks them).

There is no HDF5 library in this image; the script reads the dump with the library's minimal
read-only parser (``hybridhsdla_gb300/fleur_dump.py``).  Run it where the reference tree is present, naming the dump (as an argument, or
in the environment variable HSDLA_FLEUR_DUMP):

    python tests/golden/make_fleur_golden.py <reference>/flapw_opt/tests/sample_input/two_atoms/fleur_dump.h5

The fixture keeps the quantities as the dump stores them (Fortran column-major arrays
reinterpreted the way FleurData.cpp reads them); T matrices keep their lower triangles, the
only part the reference reads (``types_helper.cpp:41-61``).
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
from hybridhsdla_gb300.fleur_dump import H5, field  # noqa: E402  (the library's dump reader)

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fleur_two_atoms.npz")


def main(path=None):
    path = path or os.environ.get("HSDLA_FLEUR_DUMP")
    if not path:
        sys.exit("usage: make_fleur_golden.py <fleur_dump.h5> (or set HSDLA_FLEUR_DUMP)")
    f = H5(path)
    f64 = lambda p: f.dataset(p)["raw"].view("<f8")
    i32 = lambda p: f.dataset(p)["raw"].view("<i4")
    na, nt = f.attr_int("/atoms", "num_atoms"), f.attr_int("/atoms", "num_types")
    atoms = f.dataset("/atoms")
    mesh = f.dataset("/mesh")
    km = f.dataset("/k_meshes")
    lmax, lnon = i32("/lmax"), i32("/lmax_nonspherical")
    nl = int(lmax.max()) + 1
    L = nl * nl
    out = dict(
        real_basis=f64("/real_basis").reshape(3, 3, order="F"),
        rec_basis=f64("/rec_basis").reshape(3, 3, order="F"),
        atom_type=field(atoms, "type").copy().view("<i4").reshape(na) - 1,
        atom_pos=field(atoms, "position").copy().view("<f8").reshape(na, 3),
        atom_mrot=field(atoms, "rotation").copy().view("<i4").reshape(na, 3, 3).transpose(0, 2, 1).copy(),
        mesh_num=field(mesh, "num_points").copy().view("<i4").reshape(nt),
        mesh_dx=field(mesh, "dx").copy().view("<f8").reshape(nt),
        mesh_rmt=field(mesh, "rmt").copy().view("<f8").reshape(nt),
        lmax=lmax.copy(), lmax_nonsph=lnon.copy(),
        energies=f64("/energy_params").reshape(nt, -1).copy(),
        potential=f64("/potential").reshape(nt, -1).copy(),
    )
    nk = f.attr_int("/k_meshes", "num_kpts")
    assert nk >= 1
    ng = int(field(km, "num_gpts").copy().view("<i4").reshape(-1)[0])
    out["k_point"] = field(km, "k_point").copy().view("<f8").reshape(nk, 3)[0]
    out["g_mesh"] = field(km, "g_mesh").copy().view("<i4").reshape(nk, -1)[0][:3 * ng].reshape(ng, 3)
    il = np.tril_indices(L)
    for t in range(nt):
        d = f.dataset("/tmat/%d" % (t + 1))
        n = f.attr_int("/tmat/%d" % (t + 1), "n")
        assert n == L
        cube = d["raw"].view("<c16").reshape(4, n, n).transpose(0, 2, 1)   # [slice][row, col]
        for s, nm in enumerate(("aa", "bb", "ab", "ba")):                    # types.h:59 order
            out["t%d_%s_lower" % (t, nm)] = cube[s][il].copy()
    out["H_packed"] = f.dataset("/matrix_hamilton/1")["raw"].view("<c16").copy()
    out["S_packed"] = f.dataset("/matrix_overlap/1")["raw"].view("<c16").copy()
    assert out["H_packed"].size == ng * (ng + 1) // 2
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes; n_g", ng, "L", L, "atoms", na)


if __name__ == "__main__":
    main(*sys.argv[1:])
