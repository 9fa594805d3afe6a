"""Fleur dump reader: the quantities the reference's FleurData reads from ``fleur_dump.h5``
(``flapw_opt/src/FleurData.cpp:175-458``) and the AtomData it builds from them
(``FleurData::populate_atomdata``, ``FleurData.cpp:40-67``; ``AtomData::generate_matchdata``,
``AtomData.cpp:72-88``), as a :class:`hybridhsdla_gb300.synth.System` for the library.

The image has no HDF5 library, so :class:`H5` is a minimal read-only parser for what the dump
uses: superblock version 0 with 8-byte offsets, version-1 object headers, symbol-table groups
(v1 B-tree + local heap), contiguous layouts, committed (shared) compound datatypes.

:func:`load` takes a dump directory (holding ``fleur_dump.h5``), the ``.h5`` file itself, or an
``.npz`` with the same quantities (the layout of ``tests/golden/fleur_two_atoms.npz``, which also
carries Fleur's own H and S of its first k-point).
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
import struct
from typing import List, Optional

import numpy as np


class H5:
    """Minimal read-only HDF5 parser (superblock v0, v1 object headers, symbol-table groups,
    contiguous layouts, committed compound datatypes): what ``fleur_dump.h5`` uses."""

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
    """The bytes of one member of a compound dataset, one row per record."""
    _, size, mem = info["type"]
    n = info["raw"].size // size
    rec = info["raw"].reshape(n, size)
    for nm, off, t in mem:
        if nm == name:
            w = t[1]
            return rec[:, off:off + w]
    raise KeyError(name)


@dataclasses.dataclass
class FleurDump:
    """The dump's quantities (arrays as FleurData.cpp interprets them)."""
    real_basis: np.ndarray          # (3, 3)
    rec_basis: np.ndarray           # (3, 3), rows b_i (incl. 2 pi)
    atom_type: np.ndarray           # (a,) 0-based
    atom_pos: np.ndarray            # (a, 3) fractional
    atom_mrot: np.ndarray           # (a, 3, 3) integer symmetry rotations
    mesh_num: np.ndarray            # (t,) radial mesh points
    mesh_dx: np.ndarray             # (t,)
    mesh_rmt: np.ndarray            # (t,)
    lmax: np.ndarray                # (t,)
    lmax_nonsph: np.ndarray         # (t,)
    energies: np.ndarray            # (t, >= lmax+1) energy parameters E_l
    potential: np.ndarray           # (t, >= mesh_num) r V(r) on the mesh
    k_points: np.ndarray            # (k, 3) fractional
    g_meshes: List[np.ndarray]      # per k-point (n_g, 3) int32
    tmats: List[tuple]              # per type (aa, bb, ab, ba), L x L complex (lower triangles read)
    H_fleur: Optional[np.ndarray] = None   # Fleur's own H, S of k-point 0 (lower), when present
    S_fleur: Optional[np.ndarray] = None


def _unpack_lower(v: np.ndarray, n: int) -> np.ndarray:
    M = np.zeros((n, n), v.dtype)
    M[np.tril_indices(n)] = v
    return M


def read_h5(path: str) -> FleurDump:
    """``fleur_dump.h5`` as FleurData reads it (``FleurData.cpp:175-458``)."""
    f = H5(path)
    f64 = lambda p: f.dataset(p)["raw"].view("<f8")          # noqa: E731
    i32 = lambda p: f.dataset(p)["raw"].view("<i4")          # noqa: E731
    na, nt = f.attr_int("/atoms", "num_atoms"), f.attr_int("/atoms", "num_types")
    atoms, mesh, km = f.dataset("/atoms"), f.dataset("/mesh"), f.dataset("/k_meshes")
    lmax, lnon = i32("/lmax").copy(), i32("/lmax_nonspherical").copy()
    nl = int(lmax.max()) + 1
    L = nl * nl
    nk = f.attr_int("/k_meshes", "num_kpts")
    ngs = field(km, "num_gpts").copy().view("<i4").reshape(-1)[:nk]
    gm = field(km, "g_mesh").copy().view("<i4").reshape(nk, -1)
    tm = []
    for t in range(nt):
        d = f.dataset("/tmat/%d" % (t + 1))
        n = f.attr_int("/tmat/%d" % (t + 1), "n")
        if n != L:
            raise ValueError("T matrix of type %d has n = %d, expected %d" % (t + 1, n, L))
        cube = d["raw"].view("<c16").reshape(4, n, n).transpose(0, 2, 1)   # [slice][row, col]
        tm.append(tuple(cube[q].copy() for q in range(4)))                  # aa, bb, ab, ba (types.h:59)
    return FleurDump(
        real_basis=f64("/real_basis").reshape(3, 3, order="F").copy(),
        rec_basis=f64("/rec_basis").reshape(3, 3, order="F").copy(),
        atom_type=(field(atoms, "type").copy().view("<i4").reshape(na) - 1).astype(np.int32),
        atom_pos=field(atoms, "position").copy().view("<f8").reshape(na, 3).copy(),
        atom_mrot=field(atoms, "rotation").copy().view("<i4").reshape(na, 3, 3).transpose(0, 2, 1).copy(),
        mesh_num=field(mesh, "num_points").copy().view("<i4").reshape(nt).copy(),
        mesh_dx=field(mesh, "dx").copy().view("<f8").reshape(nt).copy(),
        mesh_rmt=field(mesh, "rmt").copy().view("<f8").reshape(nt).copy(),
        lmax=lmax, lmax_nonsph=lnon,
        energies=f64("/energy_params").reshape(nt, -1).copy(),
        potential=f64("/potential").reshape(nt, -1).copy(),
        k_points=field(km, "k_point").copy().view("<f8").reshape(nk, 3).copy(),
        g_meshes=[gm[k][:3 * int(ngs[k])].reshape(-1, 3).astype(np.int32) for k in range(nk)],
        tmats=tm)


def read_npz(path: str) -> FleurDump:
    """The same quantities from an ``.npz`` in the layout of ``tests/golden/fleur_two_atoms.npz``
    (one k-point; T matrices as lower triangles; Fleur's packed H and S)."""
    d = np.load(path)
    nt = d["lmax"].size
    L = (int(d["lmax"].max()) + 1) ** 2
    tm = [tuple(_unpack_lower(d["t%d_%s_lower" % (t, nm)], L) for nm in ("aa", "bb", "ab", "ba")) for t in range(nt)]
    ng = d["g_mesh"].shape[0]
    return FleurDump(real_basis=d["real_basis"], rec_basis=d["rec_basis"], atom_type=d["atom_type"].astype(np.int32),
                     atom_pos=d["atom_pos"], atom_mrot=d["atom_mrot"], mesh_num=d["mesh_num"], mesh_dx=d["mesh_dx"],
                     mesh_rmt=d["mesh_rmt"], lmax=d["lmax"], lmax_nonsph=d["lmax_nonsph"], energies=d["energies"],
                     potential=d["potential"], k_points=d["k_point"].reshape(1, 3),
                     g_meshes=[d["g_mesh"].astype(np.int32)], tmats=tm,
                     H_fleur=_unpack_lower(d["H_packed"], ng) if "H_packed" in d.files else None,
                     S_fleur=_unpack_lower(d["S_packed"], ng) if "S_packed" in d.files else None)


def load(path: str) -> FleurDump:
    """A dump directory (with ``fleur_dump.h5``), an ``.h5`` file or an ``.npz``."""
    if os.path.isdir(path):
        path = os.path.join(path, "fleur_dump.h5")
    return read_npz(path) if path.endswith(".npz") else read_h5(path)


def radial_match(l: int, e: float, vr: np.ndarray, rmt: float, dx: float) -> np.ndarray:
    """(u, u', udot, udot', ||udot||^2) at R_MT from the library's restatement of Fleur's
    scalar-relativistic radial solver (``hsdla_radial_match``; ``radfun.f``)."""
    from . import api
    L_ = api.load()
    vr = np.ascontiguousarray(vr, np.float64)
    out = np.zeros(5)
    rc = L_.hsdla_radial_match(int(l), float(e), vr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), vr.size,
                               float(rmt), float(dx), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if rc != 0:
        raise api.HsdlaError(rc, "hsdla_radial_match rejected its inputs")
    return out


def to_system(d: FleurDump, kpoints: Optional[int] = None):
    """The AtomData the reference builds (``FleurData::populate_atomdata``, ``FleurData.cpp:40-67``,
    and ``AtomData::generate_matchdata``, ``AtomData.cpp:72-88``), per type with the atom-to-type
    map: rotations ``mrot rec_basis`` (``FleurData.cpp:453-455``), cell volume ``det(real_basis)``,
    matching values from the radial solver per (type, l <= lmax), the raw T blocks with T_AB
    assembled from its lower triangle and T_BA's (``types_helper.cpp:41-61``)."""
    from . import synth
    nt = d.lmax.size
    nl = int(d.lmax.max()) + 1
    u = np.zeros((nt, nl, 5))
    for t in range(nt):
        vr = d.potential[t][:int(d.mesh_num[t])]
        for l in range(int(d.lmax[t]) + 1):
            u[t, l] = radial_match(l, d.energies[t][l], vr, d.mesh_rmt[t], d.mesh_dx[t])
    taa = np.stack([np.tril(x[0]) for x in d.tmats])
    tbb = np.stack([np.tril(x[1]) for x in d.tmats])
    tab = np.stack([np.tril(x[2]) + np.triu(x[3].conj().T, 1) for x in d.tmats])
    bmat = np.asarray(d.rec_basis, np.float64)
    rot = np.einsum("aij,jk->aik", d.atom_mrot.astype(np.float64), bmat)
    nk = len(d.k_points) if kpoints is None else min(kpoints, len(d.k_points))
    kps = [synth.KPoint(k=np.asarray(d.k_points[k], np.float64).copy(), g=d.g_meshes[k]) for k in range(nk)]
    return synth.System(real_basis=np.asarray(d.real_basis, np.float64), bmat=bmat,
                        vol_cell=float(np.linalg.det(d.real_basis)), atom_type=d.atom_type.astype(np.int32),
                        atom_pos=np.asarray(d.atom_pos, np.float64), atom_rotmat=rot,
                        type_rmt=np.asarray(d.mesh_rmt, np.float64).copy(), type_lmax=d.lmax.astype(np.int32),
                        type_lmax_nonsph=d.lmax_nonsph.astype(np.int32), u=u[:, :, 0].copy(), u_dr=u[:, :, 1].copy(),
                        dE_u=u[:, :, 2].copy(), dE_u_dr=u[:, :, 3].copy(), dE_u_norm=u[:, :, 4].copy(),
                        energies=np.asarray(d.energies[:, :nl], np.float64).copy(), taa_raw=taa, tbb_raw=tbb,
                        tab_raw=tab, kpoints=kps, name="fleur_dump")
