"""CPU oracle for the H/S generation path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this package; the GPU library never does.

* ``oracle.cpp`` (built into ``_build/liboracle.so`` by ``Makefile``) restates the
  reference's special functions, ``construct_AB``, T-matrix preparation and the
  naive contraction formulas (citations in that file).
* ``reference_hs`` below restates ``create_HS2_stripped_v2``
  (``flapw_opt/src/h_and_s_stripped_v2.cpp:100-382``) call by call on a host
  BLAS (scipy's bundled OpenBLAS): ``zherk`` (A^H A), the u-norm scaling
  ``apply_u_norm_s`` (``:64-86``), ``zherk`` (W^H W), the per-atom
  ``zhemm``+``zgemm`` loop (``:193-231``), ``zher2k`` (``:300``), the per-atom
  ``zhemm`` loop (``:321-349``) and, in place of MKL's ``zgemmt``, a ``zgemm``
  whose lower triangle is kept (``:362``).

Parity status: PINNED against the reference's own known-answer data.  The reference's
only golden vector for this path is Fleur's muffin-tin H and S for the two-atom sample
(``flapw_opt/tests/sample_input/two_atoms/fleur_dump.h5``; extracted into
``tests/golden/fleur_two_atoms.npz`` by ``tests/golden/make_fleur_golden.py``).
``fleur_golden`` below rebuilds the reference's inputs from that dump (radial solver
``oracle_radfun``, T assembly, rotations) and the oracle reproduces Fleur's H and S to
about 3e-15 relative Frobenius (``tests/test_fleur_golden.py``).  The reference binary itself
cannot be built here (Fortran, HDF5, Armadillo and MKL are absent), so there is no
``_ref`` build; the closed-form checks of the special functions and the agreement of the
BLAS sequence with the naive formulas are pinned as well.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time
from typing import Optional, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile ``liboracle.so`` with the committed Makefile."""
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "oracle.cpp"))):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.oracle_sphbes.argtypes = [ctypes.c_int, ctypes.c_double, dp]
        L.oracle_sphbes.restype = ctypes.c_int
        L.oracle_dsphbs.argtypes = [ctypes.c_int, ctypes.c_double, dp, dp]
        L.oracle_ylm4.argtypes = [ctypes.c_int, dp, dp]
        L.oracle_kmesh.argtypes = [dp, dp, ip, ctypes.c_int64, dp]
        L.oracle_construct_ab.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, ip, dp, dp,
                                          dp, ip, dp, dp, dp, dp, dp, ip, ctypes.c_int64, dp, dp,
                                          ctypes.c_int]
        L.oracle_construct_ab.restype = ctypes.c_int
        L.oracle_prepare_tmat.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.oracle_prepare_tmat.restype = ctypes.c_int
        L.oracle_radfun.argtypes = [ctypes.c_int, ctypes.c_double, dp, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double, dp]
        L.oracle_radfun.restype = ctypes.c_int
        L.oracle_hs_naive.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64, dp, dp,
                                      dp, dp, dp, dp, dp, dp, ctypes.c_int]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    assert a.dtype == np.int32
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def nthreads_default() -> int:
    return max(1, len(os.sched_getaffinity(0)))


# ---------------------------------------------------------------- primitives
def sphbes(lmax: int, x: float) -> np.ndarray:
    out = np.zeros(lmax + 1)
    rc = lib().oracle_sphbes(lmax, float(x), _dp(out))
    if rc != 0:
        raise ValueError("sphbes: lmax < 1 or x < 0")
    return out


def dsphbs(lmax: int, x: float, fj: np.ndarray) -> np.ndarray:
    fj = np.ascontiguousarray(fj, dtype=np.float64)
    out = np.zeros(lmax + 1)
    lib().oracle_dsphbs(lmax, float(x), _dp(fj), _dp(out))
    return out


def ylm4(lmax: int, v) -> np.ndarray:
    v = np.ascontiguousarray(v, dtype=np.float64)
    out = np.zeros(2 * (lmax + 1) ** 2)
    lib().oracle_ylm4(lmax, _dp(v), _dp(out))
    return out[0::2] + 1j * out[1::2]


def kmesh(k, bmat, g) -> np.ndarray:
    k = np.ascontiguousarray(k, dtype=np.float64)
    bmat = np.ascontiguousarray(bmat, dtype=np.float64)
    g = np.ascontiguousarray(g, dtype=np.int32)
    out = np.zeros(g.shape[0])
    lib().oracle_kmesh(_dp(k), _dp(bmat), _ip(g), g.shape[0], _dp(out))
    return out


def prepare_tmats(sys_) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Augmented per-type (aa, ab, bb), each (types, L, L) complex, zero-padded to
    L = (max_lmax+1)^2 (``types_helper.cpp:41-90``, ``AtomData.cpp:95-145``)."""
    nt, L = sys_.num_types, sys_.L
    aa = np.zeros((nt, L, L), np.complex128)
    ab = np.zeros_like(aa)
    bb = np.zeros_like(aa)
    tba = sys_.tba_raw()
    for t in range(nt):
        lm = int(sys_.type_lmax[t])
        n = (lm + 1) ** 2
        ins = [np.asfortranarray(x[t, :n, :n]) for x in (sys_.taa_raw, sys_.tbb_raw, sys_.tab_raw, tba)]
        outs = [np.zeros((n, n), np.complex128, order="F") for _ in range(3)]
        E = np.ascontiguousarray(sys_.energies[t, :lm + 1])
        un = np.ascontiguousarray(sys_.dE_u_norm[t, :lm + 1])
        rc = lib().oracle_prepare_tmat(lm, int(sys_.type_lmax_nonsph[t]), *[_dp(x) for x in ins],
                                       _dp(E), _dp(un), *[_dp(x) for x in outs])
        if rc != 0:
            raise ValueError("prepare_tmat: diagonals of tab and tba differ")
        aa[t, :n, :n], ab[t, :n, :n], bb[t, :n, :n] = outs
    return aa, ab, bb


def construct_ab(sys_, kp, nthreads: Optional[int] = None) -> Tuple[np.ndarray, np.ndarray]:
    """A, B as (La, G) complex Fortran-ordered matrices (the reference cube
    (L, a, G) viewed as its (L*a) x G matrix)."""
    La, G = sys_.La, kp.n_g
    A = np.zeros((La, G), np.complex128, order="F")
    B = np.zeros((La, G), np.complex128, order="F")
    rot = None if sys_.atom_rotmat is None else np.ascontiguousarray(sys_.atom_rotmat, dtype=np.float64)
    args = [sys_.num_atoms, sys_.max_lmax, float(sys_.vol_cell), _dp(np.ascontiguousarray(sys_.bmat)),
            _ip(np.ascontiguousarray(sys_.atom_type)), _dp(np.ascontiguousarray(sys_.atom_pos)),
            _dp(rot) if rot is not None else None,
            _dp(np.ascontiguousarray(sys_.type_rmt)), _ip(np.ascontiguousarray(sys_.type_lmax)),
            _dp(np.ascontiguousarray(sys_.u)), _dp(np.ascontiguousarray(sys_.u_dr)),
            _dp(np.ascontiguousarray(sys_.dE_u)), _dp(np.ascontiguousarray(sys_.dE_u_dr)),
            _dp(np.ascontiguousarray(kp.k, dtype=np.float64)), _ip(np.ascontiguousarray(kp.g)), G,
            _dp(A), _dp(B), nthreads or nthreads_default()]
    rc = lib().oracle_construct_ab(*args)
    if rc != 0:
        raise ValueError("construct_ab failed")
    return A, B


def per_atom_unorm(sys_) -> np.ndarray:
    """(a, max_lmax+1) ||udot_l||^2 replicated per atom (``FleurData.cpp:52-62``)."""
    return np.ascontiguousarray(sys_.dE_u_norm[sys_.atom_type])


def hs_naive(sys_, A, B, tm, nthreads: Optional[int] = None):
    """Direct-formula H and S (``h_and_s.cpp:88-162``), all entries."""
    aa, ab, bb = tm
    at = sys_.atom_type
    paa = np.ascontiguousarray(np.transpose(aa[at], (0, 2, 1)))   # column-major per atom
    pab = np.ascontiguousarray(np.transpose(ab[at], (0, 2, 1)))
    pbb = np.ascontiguousarray(np.transpose(bb[at], (0, 2, 1)))
    un = per_atom_unorm(sys_)
    G = A.shape[1]
    H = np.zeros((G, G), np.complex128, order="F")
    S = np.zeros((G, G), np.complex128, order="F")
    lib().oracle_hs_naive(sys_.L, sys_.num_atoms, sys_.max_lmax, G, _dp(A), _dp(B), _dp(paa), _dp(pab),
                          _dp(pbb), _dp(un), _dp(H), _dp(S), nthreads or nthreads_default())
    return H, S


def blas_sequence(sys_, A, B, tm):
    """``create_HS2_stripped_v2`` (h_and_s_stripped_v2.cpp:100-382) on host BLAS.

    A and B are modified in place exactly as the reference's row compaction
    would (a no-op when every T block has full size L).  Returns (H, S) with only
    the lower triangle defined (upper triangle zero)."""
    from scipy.linalg import blas
    aa, ab, bb = tm
    L, a = sys_.L, sys_.num_atoms
    La = L * a
    G = A.shape[1]
    # S = A^H A                                      (:158)
    S = blas.zherk(1.0, A, trans=2, lower=1)
    # W = diag(sqrt(||udot||^2)) B                   (:167, :64-86)
    un = per_atom_unorm(sys_)
    lin = np.zeros(La)
    for at in range(a):
        for l in range(int(sys_.type_lmax[sys_.atom_type[at]]) + 1):
            lin[at * L + l * l: at * L + (l + 1) ** 2] = np.sqrt(un[at, l])
    W = np.asfortranarray(B * lin[:, None])
    # S += W^H W                                     (:177)
    S = blas.zherk(1.0, W, beta=1.0, c=S, trans=2, lower=1, overwrite_c=1)
    # per-atom loop 1: X_a = 1/2 T_BB B_a + T_AB^H A_a  (:193-231)
    X = np.zeros((La, G), np.complex128, order="F")
    for at in range(a):
        t = sys_.atom_type[at]
        rows = slice(at * L, at * L + L)
        tmp = blas.zhemm(0.5, np.asfortranarray(bb[t]), np.asfortranarray(B[rows]), side=0, lower=1)
        tmp = blas.zgemm(1.0, np.asfortranarray(ab[t]), np.asfortranarray(A[rows]), beta=1.0, c=tmp,
                         trans_a=2, overwrite_c=1)
        X[rows] = tmp
    # H = B^H X + X^H B                              (:300)
    H = blas.zher2k(1.0, B, X, trans=2, lower=1)
    # per-atom loop 2: X'_a = T_AA A_a                (:321-349)
    for at in range(a):
        t = sys_.atom_type[at]
        rows = slice(at * L, at * L + L)
        X[rows] = blas.zhemm(1.0, np.asfortranarray(aa[t]), np.asfortranarray(A[rows]), side=0, lower=1)
    # H += A^H X'  (zgemmt in the reference; zgemm, lower triangle kept)  (:362)
    H2 = blas.zgemm(1.0, A, X, trans_a=2)
    H = H + np.tril(H2)
    return np.tril(H), np.tril(S)


def reference_hs(sys_, kp, nthreads: Optional[int] = None, timings: Optional[dict] = None):
    """The full reference CPU path for one k-point: construct_AB + BLAS sequence."""
    t0 = time.perf_counter()
    A, B = construct_ab(sys_, kp, nthreads)
    t1 = time.perf_counter()
    tm = prepare_tmats(sys_)
    H, S = blas_sequence(sys_, A, B, tm)
    t2 = time.perf_counter()
    if timings is not None:
        timings["construct_ab_s"] = t1 - t0
        timings["contract_s"] = t2 - t1
    return H, S


# ------------------------------------------------------------------ metrics
def lower_errors(X: np.ndarray, X_ref: np.ndarray) -> Tuple[float, float]:
    """(relative Frobenius, relative max-norm) error over the lower triangle."""
    Xl = np.tril(X)
    Rl = np.tril(X_ref)
    d = Xl - Rl
    fro = float(np.linalg.norm(d) / max(np.linalg.norm(Rl), 1e-300))
    mx = float(np.abs(d).max() / max(np.abs(Rl).max(), 1e-300))
    return fro, mx


def stripped_v2(L, a, A, B, blocks, lmaxs, max_lmax, sqrt_u_norms):
    """``create_HS2_stripped_v2`` (h_and_s_stripped_v2.cpp:100-382) call by call for general
    per-atom T block sizes, including its row compaction of X, B and A (``X_height`` at
    :211-230, ``X_nhpd_height`` at :319-347).  A, B: (L*a, G) Fortran-ordered; blocks: per
    atom (aa, ab, bb) square complex arrays; sqrt_u_norms: (a, max_lmax+1).  Returns lower
    triangles (H, S)."""
    from scipy.linalg import blas
    A = np.array(A, order="F", copy=True)
    B = np.array(B, order="F", copy=True)
    La, G = A.shape
    S = blas.zherk(1.0, A, trans=2, lower=1)
    lin = np.zeros(La)
    for at in range(a):
        for l in range(int(lmaxs[at]) + 1):
            lin[at * L + l * l: at * L + (l + 1) ** 2] = sqrt_u_norms[at][l]
    W = np.asfortranarray(B * lin[:, None])
    S = blas.zherk(1.0, W, beta=1.0, c=S, trans=2, lower=1, overwrite_c=1)
    X = np.zeros((La, G), np.complex128, order="F")
    xh = 0
    for at in range(a):
        aa, ab, bb = blocks[at]
        nbb, nab = bb.shape[0], ab.shape[0]
        tmp = np.zeros((L, G), np.complex128, order="F")
        if nbb:
            tmp[:nbb] = blas.zhemm(0.5, np.asfortranarray(bb), np.asfortranarray(B[at * L: at * L + nbb]),
                                   side=0, lower=1)
        if nab:
            tmp[:nab] += blas.zgemm(1.0, np.asfortranarray(ab), np.asfortranarray(A[at * L: at * L + nab]),
                                    trans_a=2)
        n = max(nab, nbb)
        X[xh: xh + n] = tmp[:n]
        if xh != at * L:
            B[xh: xh + n] = B[at * L: at * L + n].copy()
        xh += n
    H = blas.zher2k(1.0, B[:xh], X[:xh], trans=2, lower=1) if xh else np.zeros((G, G), np.complex128)
    xn = 0
    X2 = np.zeros((La, G), np.complex128, order="F")
    for at in range(a):
        aa = blocks[at][0]
        n = aa.shape[0]
        if xn != at * L:
            A[xn: xn + n] = A[at * L: at * L + n].copy()
        if n:
            X2[xn: xn + n] = blas.zhemm(1.0, np.asfortranarray(aa), np.asfortranarray(A[xn: xn + n]), side=0, lower=1)
        xn += n
    if xn:
        H = H + np.tril(blas.zgemm(1.0, A[:xn], X2[:xn], trans_a=2))
    return np.tril(H), np.tril(S)


# --------------------------------------------------------------- Fleur-dump golden
def radfun(l: int, e: float, vr: np.ndarray, rmt: float, dx: float) -> np.ndarray:
    """(u, u', udot, udot', ||udot||^2) at R_MT from Fleur's scalar-relativistic radial
    solver (``radfun.f``/``radsra.f``/``radsrd.F``/``intgr.F``, restated in oracle.cpp)."""
    vr = np.ascontiguousarray(vr, np.float64)
    out = np.zeros(5)
    rc = lib().oracle_radfun(int(l), float(e), _dp(vr), vr.size, float(rmt), float(dx), _dp(out))
    if rc:
        raise ValueError("radfun: bad mesh")
    return out


GOLDEN_FLEUR = os.path.join(os.path.dirname(_HERE), "tests", "golden", "fleur_two_atoms.npz")


def _unpack_lower(v: np.ndarray, n: int) -> np.ndarray:
    M = np.zeros((n, n), v.dtype)
    M[np.tril_indices(n)] = v
    return M


def fleur_golden(path: str = GOLDEN_FLEUR):
    """The two-atom Fleur dump as (System, KPoint, H_fleur, S_fleur).

    Follows ``FleurData::populate_atomdata`` (``flapw_opt/src/FleurData.cpp:41-72``): per-type
    meshes, potentials, cutoffs and energies; rotations ``mrot * rec_basis`` (``:446-456``);
    the cell volume ``det(real_basis)`` (``:46``); matching values from the radial solver
    per (type, l <= lmax) (``AtomData.cpp:73-88``); raw T matrices with the T_AB assembly of
    ``types_helper.cpp:41-61`` (lower T_AB, upper from T_BA^H).  H_fleur and S_fleur are
    Fleur's packed lower triangles unpacked row by row (``tests/flapw_verify.py:68-82``)
    into the lower triangle of a G x G matrix (upper zero).
    """
    from hybridhsdla_gb300 import synth
    d = np.load(path)
    nt = d["lmax"].size
    nl = int(d["lmax"].max()) + 1
    L = nl * nl
    u = np.zeros((nt, nl, 5))
    for t in range(nt):
        vr = d["potential"][t][:int(d["mesh_num"][t])]
        for l in range(int(d["lmax"][t]) + 1):
            u[t, l] = radfun(l, d["energies"][t][l], vr, d["mesh_rmt"][t], d["mesh_dx"][t])
    taa = np.zeros((nt, L, L), np.complex128)
    tbb = np.zeros((nt, L, L), np.complex128)
    tab = np.zeros((nt, L, L), np.complex128)
    for t in range(nt):
        taa[t] = _unpack_lower(d["t%d_aa_lower" % t], L)
        tbb[t] = _unpack_lower(d["t%d_bb_lower" % t], L)
        lo = _unpack_lower(d["t%d_ab_lower" % t], L)
        ba = _unpack_lower(d["t%d_ba_lower" % t], L)
        tab[t] = lo + np.triu(ba.conj().T, 1)
    bmat = d["rec_basis"]
    rot = np.einsum("aij,jk->aik", d["atom_mrot"].astype(np.float64), bmat)
    s = synth.System(real_basis=d["real_basis"], bmat=bmat, vol_cell=float(np.linalg.det(d["real_basis"])),
                     atom_type=d["atom_type"].astype(np.int32), atom_pos=d["atom_pos"],
                     atom_rotmat=rot, type_rmt=d["mesh_rmt"].copy(), type_lmax=d["lmax"].astype(np.int32),
                     type_lmax_nonsph=d["lmax_nonsph"].astype(np.int32),
                     u=u[:, :, 0].copy(), u_dr=u[:, :, 1].copy(), dE_u=u[:, :, 2].copy(),
                     dE_u_dr=u[:, :, 3].copy(), dE_u_norm=u[:, :, 4].copy(),
                     energies=d["energies"][:, :nl].copy(), taa_raw=taa, tbb_raw=tbb, tab_raw=tab,
                     kpoints=[synth.KPoint(k=d["k_point"].copy(), g=d["g_mesh"].astype(np.int32))],
                     name="fleur_two_atoms")
    ng = d["g_mesh"].shape[0]
    return s, s.kpoints[0], _unpack_lower(d["H_packed"], ng), _unpack_lower(d["S_packed"], ng)
