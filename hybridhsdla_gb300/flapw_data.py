"""The reference's contraction-only wire format (``DUMP_FLAPW_DATA``).

``data.in`` (``flapw_opt/src/h_and_s.cpp:763-786``), native byte order, int = int32,
cx = two float64:
    L, a, G; A (L*a*G cx, column-major cube); B (same);
    per atom: aa_size, aa (aa_size^2 cx), ab_size, ab (...), bb_size, bb (...);
    lmaxs (a ints); max_lmax; sqrt_u_norms ((max_lmax+1)*a doubles, atom-major).
``data.out`` (``h_and_s.cpp:870-873``): G; H (G*G cx); S (G*G cx), column-major.
"""
from __future__ import annotations

import dataclasses
from typing import List, Tuple

import numpy as np


@dataclasses.dataclass
class DataIn:
    L: int
    a: int
    G: int
    A: np.ndarray                    # (L*a, G) complex, Fortran order
    B: np.ndarray
    blocks: List[Tuple[np.ndarray, np.ndarray, np.ndarray]]   # per atom (aa, ab, bb), column-major squares
    lmaxs: np.ndarray                # (a,) int32
    max_lmax: int
    sqrt_u_norms: np.ndarray         # (a, max_lmax+1)


def write_data_in(path: str, d: DataIn) -> None:
    with open(path, "wb") as f:
        np.array([d.L, d.a, d.G], np.int32).tofile(f)
        np.asfortranarray(d.A, np.complex128).ravel(order="F").tofile(f)
        np.asfortranarray(d.B, np.complex128).ravel(order="F").tofile(f)
        for aa, ab, bb in d.blocks:
            for T in (aa, ab, bb):
                np.array([T.shape[0]], np.int32).tofile(f)
                np.asarray(T, np.complex128).ravel(order="F").tofile(f)
        np.asarray(d.lmaxs, np.int32).tofile(f)
        np.array([d.max_lmax], np.int32).tofile(f)
        np.ascontiguousarray(d.sqrt_u_norms, np.float64).tofile(f)


def read_data_in(path: str) -> DataIn:
    with open(path, "rb") as f:
        L, a, G = (int(x) for x in np.fromfile(f, np.int32, 3))
        n = L * a * G
        A = np.fromfile(f, np.complex128, n).reshape((L * a, G), order="F")
        B = np.fromfile(f, np.complex128, n).reshape((L * a, G), order="F")
        blocks = []
        for _ in range(a):
            t = []
            for _ in range(3):
                s = int(np.fromfile(f, np.int32, 1)[0])
                t.append(np.fromfile(f, np.complex128, s * s).reshape((s, s), order="F"))
            blocks.append(tuple(t))
        lmaxs = np.fromfile(f, np.int32, a)
        max_lmax = int(np.fromfile(f, np.int32, 1)[0])
        un = np.fromfile(f, np.float64, (max_lmax + 1) * a).reshape(a, max_lmax + 1)
    return DataIn(L, a, G, A, B, blocks, lmaxs, max_lmax, un)


def write_data_out(path: str, H: np.ndarray, S: np.ndarray) -> None:
    G = H.shape[0]
    with open(path, "wb") as f:
        np.array([G], np.int32).tofile(f)
        np.asfortranarray(H, np.complex128).ravel(order="F").tofile(f)
        np.asfortranarray(S, np.complex128).ravel(order="F").tofile(f)


def read_data_out(path: str) -> Tuple[np.ndarray, np.ndarray]:
    with open(path, "rb") as f:
        G = int(np.fromfile(f, np.int32, 1)[0])
        H = np.fromfile(f, np.complex128, G * G).reshape((G, G), order="F")
        S = np.fromfile(f, np.complex128, G * G).reshape((G, G), order="F")
    return H, S


def from_system(sys_, kp, A, B, tmats) -> DataIn:
    """data.in of one k-point the way create_HS2 packs it (h_and_s.cpp:700-738): T per atom at
    its full (lmax+1)^2 size, sqrt(||udot_l||^2) per atom and l."""
    aa, ab, bb = tmats
    blocks, lmaxs = [], []
    un = np.zeros((sys_.num_atoms, sys_.max_lmax + 1))
    for j in range(sys_.num_atoms):
        t = int(sys_.atom_type[j])
        lm = int(sys_.type_lmax[t])
        n = (lm + 1) ** 2
        blocks.append((aa[t][:n, :n].copy(), ab[t][:n, :n].copy(), bb[t][:n, :n].copy()))
        lmaxs.append(lm)
        un[j, :lm + 1] = np.sqrt(sys_.dE_u_norm[t, :lm + 1])
    return DataIn(sys_.L, sys_.num_atoms, kp.n_g, np.asfortranarray(A), np.asfortranarray(B), blocks,
                  np.asarray(lmaxs, np.int32), sys_.max_lmax, un)
