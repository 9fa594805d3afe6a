"""Generate ``fleur_two_atoms.npz``: the reference's only known-answer data for the H/S path.

Source: ``flapw_opt/tests/sample_input/two_atoms/fleur_dump.h5`` in the reference tree, the
dump Fleur writes for the two-atom sample (read by ``flapw_opt/src/FleurData.cpp:175-458``).
It holds the cell, atoms, radial meshes, potentials, energy parameters, Fleur's raw T
matrices and Fleur's own muffin-tin H and S for k-point 1 (packed lower triangles, row-major
packing as ``flapw_opt/tests/flapw_verify.py:68-82`` unpacks them).

There is no HDF5 library in this image, so this script carries a minimal read-only parser for
what the file uses: superblock version 0 with 8-byte offsets, version-1 object headers,
symbol-table groups (v1 B-tree + local heap), contiguous layouts, committed (shared) compound
datatypes.  Run it where the reference tree is present, naming the dump (as an argument, or
in the environment variable HSDLA_FLEUR_DUMP):

    python tests/golden/make_fleur_golden.py <reference>/flapw_opt/tests/sample_input/two_atoms/fleur_dump.h5

The fixture keeps the quantities as the dump stores them (Fortran column-major arrays
reinterpreted the way FleurData.cpp reads them); T matrices keep their lower triangles, the
only part the reference reads (``types_helper.cpp:41-61``).
"""
import os
import struct
import sys

import numpy as np

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fleur_two_atoms.npz")


class H5:
    def __init__(self, path):
        self.d = open(path, "rb").read()
        assert self.d[:8] == b"\x89HDF\r\n\x1a\n" and self.d[8] == 0, "superblock v0 expected"
        assert self.d[13] == 8 and self.d[14] == 8, "8-byte offsets/lengths expected"
        self.root = self.u64(64)

    def u8(self, o): return self.d[o]
    def u16(self, o): return struct.unpack_from("<H", self.d, o)[0]
    def u32(self, o): return struct.unpack_from("<I", self.d, o)[0]
    def u64(self, o): return struct.unpack_from("<Q", self.d, o)[0]

    def messages(self, oh):
        assert self.u8(oh) == 1, "object header v1 expected"
        n, size = self.u16(oh + 2), self.u32(oh + 8)
        blocks, out = [(oh + 16, size)], []
        while blocks and len(out) < n:
            p, sz = blocks.pop(0)
            end = p + sz
            while p + 8 <= end and len(out) < n:
                t, s, fl = self.u16(p), self.u16(p + 2), self.u8(p + 4)
                out.append((t, p + 8, s, fl))
                if t == 0x10:                       # continuation
                    blocks.append((self.u64(p + 8), self.u64(p + 16)))
                p += 8 + s
        return out

    def _name(self, heap, off):
        assert self.d[heap:heap + 4] == b"HEAP"
        base = self.u64(heap + 24)
        e = self.d.index(b"\0", base + off)
        return self.d[base + off:e].decode()

    def _entries(self, btree, heap, res):
        assert self.d[btree:btree + 4] == b"TREE"
        level, n = self.u8(btree + 5), self.u16(btree + 6)
        p = btree + 24
        for _ in range(n):
            child = self.u64(p + 8)
            p += 16
            if level > 0:
                self._entries(child, heap, res)
                continue
            assert self.d[child:child + 4] == b"SNOD"
            q = child + 8
            for _ in range(self.u16(child + 6)):
                res[self._name(heap, self.u64(q))] = self.u64(q + 8)
                q += 40
        return res

    def lookup(self, path):
        oh = self.root
        for part in [x for x in path.split("/") if x]:
            st = [m for m in self.messages(oh) if m[0] == 0x11]
            assert st, path
            p = st[0][1]
            oh = self._entries(self.u64(p), self.u64(p + 8), {})[part]
        return oh

    def _dtype(self, p):
        cv = self.u8(p)
        cls, ver = cv & 0xF, cv >> 4
        bf = self.d[p + 1:p + 4]
        size = self.u32(p + 4)
        q = p + 8
        if cls == 0:
            return ("int", size), q + 4
        if cls == 1:
            return ("float", size), q + 12
        if cls == 6:
            mem = []
            for _ in range(bf[0] | (bf[1] << 8)):
                e = self.d.index(b"\0", q)
                name = self.d[q:e].decode()
                q += ((e - q) // 8 + 1) * 8
                off = self.u32(q)
                q += 4
                if ver == 1:
                    q += 28
                t, q = self._dtype(q)
                mem.append((name, off, t))
            return ("compound", size, mem), q
        if cls == 10:
            nd = self.u8(q)
            q += 4 if ver == 2 else 1
            dims = [self.u32(q + 4 * k) for k in range(nd)]
            q += 4 * nd * (2 if ver == 2 else 1)
            t, q = self._dtype(q)
            return ("array", size, dims, t), q
        raise ValueError("datatype class %d not handled" % cls)

    def dataset(self, path):
        info = {"attrs": {}}
        for t, p, s, fl in self.messages(self.lookup(path)):
            if t == 1:
                ver, nd = self.u8(p), self.u8(p + 1)
                off = p + 8 if ver == 1 else p + 4
                info["dims"] = [self.u64(off + 8 * k) for k in range(nd)]
            elif t == 3:
                if fl & 2:                          # committed datatype
                    sh = self.u64(p + 2) if self.u8(p) == 2 else self.u64(p + 8)
                    p = [m for m in self.messages(sh) if m[0] == 3][0][1]
                info["type"] = self._dtype(p)[0]
            elif t == 8:
                assert self.u8(p) == 3 and self.u8(p + 1) == 1, "contiguous layout v3 expected"
                a, n = self.u64(p + 2), self.u64(p + 10)
                info["raw"] = np.frombuffer(self.d[a:a + n], np.uint8)
        return info

    def attr_int(self, path, name):
        for t, p, s, fl in self.messages(self.lookup(path)):
            if t != 0xC:
                continue
            nlen, tlen, slen = self.u16(p + 2), self.u16(p + 4), self.u16(p + 6)
            q = p + 8
            nm = self.d[q:q + nlen - 1].decode()
            q += (nlen + 7) // 8 * 8 + (tlen + 7) // 8 * 8 + (slen + 7) // 8 * 8
            if nm == name:
                return struct.unpack_from("<i", self.d, q)[0]
        raise KeyError(name)


def field(info, name):
    _, size, mem = info["type"]
    n = info["raw"].size // size
    rec = info["raw"].reshape(n, size)
    for nm, off, t in mem:
        if nm == name:
            w = t[1]
            return rec[:, off:off + w]
    raise KeyError(name)


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
