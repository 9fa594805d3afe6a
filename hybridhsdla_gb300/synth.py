"""Seeded synthetic FLAPW inputs for the H/S generation path.

The reference reads these quantities from a Fleur dump (``fleur_dump.h5``,
``flapw_opt/src/FleurData.cpp:175-458``) and a radial solver
(``flapw_opt/src/special_funcs.cpp:21-36``).  Here every quantity that
``create_HS2`` consumes (``flapw_opt/src/h_and_s.cpp:591-893``) is drawn from a
seeded generator instead:

* cell: real basis rows ``a_i``; reciprocal rows ``b_i`` with ``a_i.b_j = 2 pi d_ij``
  (``FleurData.cpp:453-455`` premultiplies rotations by this matrix);
* atoms: uniform fractional positions with a minimum periodic separation;
* radial boundary values ``u, u', udot, udot'`` ~ U[-1,1] per (type, l), rejecting
  ``|W| < 1e-3`` for ``W = udot u' - u udot'`` (``AtomData.cpp:63-66``), and
  ``||udot||^2`` ~ U[0.01, 1];
* raw per-type T blocks in Fleur's lower-triangle convention
  (``types_helper.cpp:41-63``): ``taa``/``tbb`` Hermitian with N(0,1)/sqrt(L)
  complex entries, ``tab`` general with a real diagonal (the reference asserts
  ``diag(tab) == diag(tba)`` with ``tba = tab^H``), energies ``E_l`` ~ U[-1,1];
* G-vectors: all integer ``n`` with ``|bmat^T (k+n)| <= Kmax``, Kmax bisected so
  that exactly the target ``n_G`` vectors fall inside (Fleur ``apws.F``
  semantics); vectors are ordered by ``|k+n|`` then lexicographically.

Everything here is host-side test and benchmark tooling: numpy only.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np


@dataclasses.dataclass
class KPoint:
    k: np.ndarray          # (3,) fractional reciprocal coordinates
    g: np.ndarray          # (n_G, 3) int32 integer G-vectors

    @property
    def n_g(self) -> int:
        return int(self.g.shape[0])


@dataclasses.dataclass
class System:
    """Per-run quantities of one FLAPW cell (what ``AtomData`` holds)."""
    real_basis: np.ndarray     # (3,3) rows a_i, bohr
    bmat: np.ndarray           # (3,3) rows b_i, bohr^-1 (includes 2 pi)
    vol_cell: float
    atom_type: np.ndarray      # (a,) int32, 0-based
    atom_pos: np.ndarray       # (a,3) fractional
    atom_rotmat: Optional[np.ndarray]  # (a,3,3) = mrot @ bmat, or None (identity mrot)
    type_rmt: np.ndarray       # (t,)
    type_lmax: np.ndarray      # (t,) int32, spherical cutoff
    type_lmax_nonsph: np.ndarray  # (t,) int32
    u: np.ndarray              # (t, lmax+1) u(R)
    u_dr: np.ndarray           # (t, lmax+1) u'(R)
    dE_u: np.ndarray           # (t, lmax+1) udot(R)
    dE_u_dr: np.ndarray        # (t, lmax+1) udot'(R)
    dE_u_norm: np.ndarray      # (t, lmax+1) ||udot||^2
    energies: np.ndarray       # (t, lmax+1) E_l
    taa_raw: np.ndarray        # (t, L, L) complex, Hermitian (lower triangle is what Fleur dumps)
    tbb_raw: np.ndarray        # (t, L, L) complex, Hermitian
    tab_raw: np.ndarray        # (t, L, L) complex, general, real diagonal
    kpoints: List[KPoint]
    name: str = ""

    @property
    def num_atoms(self) -> int:
        return int(self.atom_type.shape[0])

    @property
    def num_types(self) -> int:
        return int(self.type_rmt.shape[0])

    @property
    def max_lmax(self) -> int:
        return int(self.type_lmax.max())

    @property
    def L(self) -> int:
        return (self.max_lmax + 1) ** 2

    @property
    def La(self) -> int:
        return self.L * self.num_atoms

    def tba_raw(self) -> np.ndarray:
        """Fleur's ``tdu`` block: the Hermitian transpose of ``tab``."""
        return np.conj(np.transpose(self.tab_raw, (0, 2, 1)))

    def flop_per_kpoint(self, n_g: int) -> float:
        """Canonical work figure of the reference
        (``h_and_s_stripped_v2.cpp:162,181,236,304,354,368``):
        ``20 G^2 La + 24 L^2 a G``."""
        L, a = self.L, self.num_atoms
        return 20.0 * n_g * n_g * L * a + 24.0 * L * L * a * n_g

    def total_flop(self) -> float:
        return sum(self.flop_per_kpoint(kp.n_g) for kp in self.kpoints)


# --------------------------------------------------------------------------
# configurations
# --------------------------------------------------------------------------
# Each entry restates one workload with its sizes.  ``n_g`` is the target basis
# size per k-point (either an int, or a (lo, hi) range drawn per k-point).
CONFIGS: Dict[str, dict] = {
    # 4 atoms / 2 types, lmax 6, n_G 500 -- CPU-runnable reference size
    "c0": dict(cell=(10.0, 10.0, 10.0), atoms=4, types=2, rmt=2.2, min_sep=4.6,
               lmax=6, kpts=[(0.1, 0.2, 0.3)], n_g=500, seed=1000),
    # 32 atoms / 4 types, lmax 8, n_G 3000
    "c1": dict(cell=(14.0, 14.0, 20.0), atoms=32, types=4, rmt=2.0, min_sep=4.0,
               lmax=8, kpts=[(0.1, 0.2, 0.3)], n_g=3000, seed=1001),
    # 128 atoms / 8 types, lmax 10, n_G 8000 -- the precision-form headline size
    "c2": dict(cell=(24.0, 24.0, 24.0), atoms=128, types=8, rmt=2.0, min_sep=4.0,
               lmax=10, kpts=[(0.1, 0.2, 0.3)], n_g=8000, seed=1002),
    # 64 atoms / 4 types, lmax 8, 64 k-points (4x4x4), n_G 6000..6600
    "c3": dict(cell=(14.0 * 2 ** (1 / 3), 14.0 * 2 ** (1 / 3), 20.0 * 2 ** (1 / 3)),
               atoms=64, types=4, rmt=2.0, min_sep=4.0, lmax=8, kpts="mp4",
               n_g=(6000, 6600), seed=1003),
    # 512 atoms / 16 types, lmax 10, 4 k-points, n_G ~20000
    "c4": dict(cell=(40.0, 40.0, 40.0), atoms=512, types=16, rmt=1.9, min_sep=3.8,
               lmax=10, kpts="mp4x1", n_g=(19000, 21000), seed=1004),
    # c2's cell and basis with one type of 16 atoms: one per-type S/H launch of c2's shape on a
    # few GB of device memory (the case profiled in full)
    "c2t1": dict(cell=(24.0, 24.0, 24.0), atoms=16, types=1, rmt=2.0, min_sep=4.0,
                 lmax=10, kpts=[(0.1, 0.2, 0.3)], n_g=8000, seed=1002),
    # c2 with rotations, as a Fleur dump gives them: the atoms of each type in two rotation
    # classes (one the identity), 16 (type, rotation) classes
    "c2r": dict(cell=(24.0, 24.0, 24.0), atoms=128, types=8, rmt=2.0, min_sep=4.0,
                lmax=10, kpts=[(0.1, 0.2, 0.3)], n_g=8000, seed=1002, rot_classes=2),
    # tiny cases for fast parity tests
    "t0": dict(cell=(9.0, 9.5, 10.0), atoms=3, types=2, rmt=2.0, min_sep=4.2,
               lmax=3, kpts=[(0.1, 0.2, 0.3)], n_g=37, seed=7),
    "t1": dict(cell=(9.0, 9.0, 11.0), atoms=5, types=3, rmt=1.8, min_sep=3.8,
               lmax=4, kpts=[(0.1, 0.2, 0.3), (0.0, 0.0, 0.0), (0.25, -0.25, 0.5)],
               n_g=(150, 230), seed=8),
}


def _mp_kpoints(n: int, rng: np.random.Generator, count: Optional[int] = None) -> List[Tuple[float, float, float]]:
    """Monkhorst-Pack-like mesh: (2i-n-1)/(2n) per axis plus a small seeded shift."""
    base = [(2 * i - n - 1) / (2.0 * n) for i in range(1, n + 1)]
    pts = [(x, y, z) for x in base for y in base for z in base]
    shift = rng.uniform(-0.02, 0.02, size=3)
    pts = [tuple(float(p[i] + shift[i]) for i in range(3)) for p in pts]
    if count is not None:
        idx = rng.choice(len(pts), size=count, replace=False)
        pts = [pts[i] for i in sorted(idx)]
    return pts


def g_vectors(bmat: np.ndarray, k: np.ndarray, n_g: int) -> np.ndarray:
    """All integer n with |bmat^T (k+n)| <= Kmax, Kmax chosen so exactly n_g fall inside.

    Returned as (n_g, 3) int32, ordered by |k+n| then lexicographically."""
    # real-space basis lengths bound each index: |n_i + k_i| <= Kmax |a_i| / (2 pi)
    vol_rec = abs(np.linalg.det(bmat))
    # radius estimate from the sphere volume, with margin
    kmax_est = (3.0 * n_g * vol_rec / (4.0 * math.pi)) ** (1.0 / 3.0) * 1.25 + 1e-9
    real = 2.0 * math.pi * np.linalg.inv(bmat).T   # rows a_i
    while True:
        lim = [int(math.ceil(kmax_est * np.linalg.norm(real[i]) / (2 * math.pi))) + 1 for i in range(3)]
        r = [np.arange(-lim[i], lim[i] + 1) for i in range(3)]
        n = np.stack(np.meshgrid(*r, indexing="ij"), axis=-1).reshape(-1, 3)
        kc = (n + k[None, :]) @ bmat          # Cartesian: bmat^T (k+n)
        norms = np.sqrt(np.einsum("ij,ij->i", kc, kc))
        inside = norms <= kmax_est
        if inside.sum() > n_g + 8:
            break
        kmax_est *= 1.2
    order = np.lexsort((n[:, 2], n[:, 1], n[:, 0], norms))
    sel = order[:n_g]
    return np.ascontiguousarray(n[sel].astype(np.int32))


def _positions(rng: np.random.Generator, real_basis: np.ndarray, count: int, min_sep: float) -> np.ndarray:
    pos = np.zeros((0, 3))
    tries = 0
    while pos.shape[0] < count:
        tries += 1
        if tries > 2_000_000:
            raise RuntimeError("could not place atoms with the requested separation")
        cand = rng.uniform(0.0, 1.0, size=(64, 3))
        for c in cand:
            if pos.shape[0] == 0:
                pos = c[None, :]
                continue
            d = pos - c[None, :]
            d -= np.round(d)                   # minimum image (orthogonal cells)
            dist = np.sqrt(((d @ real_basis) ** 2).sum(axis=1))
            if dist.min() >= min_sep:
                pos = np.vstack([pos, c[None, :]])
                if pos.shape[0] == count:
                    break
    return pos


def _herm(rng: np.random.Generator, L: int) -> np.ndarray:
    x = (rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L))) / math.sqrt(L)
    return 0.5 * (x + x.conj().T)


def make_system(cfg: str | dict, *, n_kpoints: Optional[int] = None,
                n_g_override: Optional[int] = None) -> System:
    """Build the seeded system of a named configuration (``CONFIGS``)."""
    name = cfg if isinstance(cfg, str) else "custom"
    c = CONFIGS[cfg] if isinstance(cfg, str) else cfg
    ss = np.random.SeedSequence(c["seed"])
    s_pos, s_rad, s_t, s_k, s_ng = ss.spawn(5)
    rng_pos = np.random.default_rng(s_pos)
    rng_rad = np.random.default_rng(s_rad)
    rng_t = np.random.default_rng(s_t)
    rng_k = np.random.default_rng(s_k)
    rng_ng = np.random.default_rng(s_ng)

    real_basis = np.diag(np.asarray(c["cell"], dtype=np.float64))
    bmat = 2.0 * math.pi * np.linalg.inv(real_basis).T
    vol = float(np.linalg.det(real_basis))

    na, nt, lmax = c["atoms"], c["types"], c["lmax"]
    atom_type = (np.arange(na) % nt).astype(np.int32)
    atom_pos = _positions(rng_pos, real_basis, na, c["min_sep"])

    type_rmt = np.full(nt, c["rmt"], dtype=np.float64)
    type_lmax = np.full(nt, lmax, dtype=np.int32)
    type_lmax_nonsph = np.full(nt, lmax, dtype=np.int32)

    nl = lmax + 1
    u = np.zeros((nt, nl)); u_dr = np.zeros((nt, nl))
    dE_u = np.zeros((nt, nl)); dE_u_dr = np.zeros((nt, nl))
    for t in range(nt):
        for l in range(nl):
            while True:
                v = rng_rad.uniform(-1.0, 1.0, size=4)
                w = v[2] * v[1] - v[0] * v[3]
                if abs(w) >= 1e-3:
                    break
            u[t, l], u_dr[t, l], dE_u[t, l], dE_u_dr[t, l] = v
    dE_u_norm = rng_rad.uniform(0.01, 1.0, size=(nt, nl))
    energies = rng_rad.uniform(-1.0, 1.0, size=(nt, nl))

    L = nl * nl
    taa = np.zeros((nt, L, L), np.complex128)
    tbb = np.zeros((nt, L, L), np.complex128)
    tab = np.zeros((nt, L, L), np.complex128)
    for t in range(nt):
        taa[t] = _herm(rng_t, L)
        tbb[t] = _herm(rng_t, L)
        y = (rng_t.standard_normal((L, L)) + 1j * rng_t.standard_normal((L, L))) / math.sqrt(L)
        y[np.diag_indices(L)] = y[np.diag_indices(L)].real
        tab[t] = y

    kp = c["kpts"]
    if kp == "mp4":
        kpts = _mp_kpoints(4, rng_k)
    elif kp == "mp4x1":
        kpts = _mp_kpoints(4, rng_k, count=4)
    else:
        kpts = [tuple(x) for x in kp]
    if n_kpoints is not None:
        kpts = kpts[:n_kpoints]
    ng = c["n_g"]
    kpoints = []
    for kk in kpts:
        if n_g_override is not None:
            target = n_g_override
        elif isinstance(ng, tuple):
            target = int(rng_ng.integers(ng[0], ng[1] + 1))
        else:
            target = int(ng)
        kvec = np.asarray(kk, dtype=np.float64)
        kpoints.append(KPoint(k=kvec, g=g_vectors(bmat, kvec, target)))

    out = System(real_basis=real_basis, bmat=bmat, vol_cell=vol, atom_type=atom_type,
                 atom_pos=atom_pos, atom_rotmat=None, type_rmt=type_rmt, type_lmax=type_lmax,
                 type_lmax_nonsph=type_lmax_nonsph, u=u, u_dr=u_dr, dE_u=dE_u, dE_u_dr=dE_u_dr,
                 dE_u_norm=dE_u_norm, energies=energies, taa_raw=taa, tbb_raw=tbb, tab_raw=tab,
                 kpoints=kpoints, name=name)
    if c.get("rot_classes"):
        out = with_class_rotations(out, per_type=int(c["rot_classes"]))
    return out


def _rotation(rng: np.random.Generator) -> np.ndarray:
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))[None, :]
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def with_class_rotations(sys_: System, per_type: int = 2, seed: int = 77, identity_first: bool = True) -> System:
    """Copy of ``sys_`` whose atoms carry rotations shared within classes: the atoms of each type
    are dealt round-robin into ``per_type`` classes, each class with one seeded proper rotation
    (the first the identity when ``identity_first``), stored as ``mrot @ bmat`` like
    ``FleurData.cpp:453-455``.  This is the situation of a Fleur dump: one rotation per atom,
    equal for the atoms a symmetry operation maps onto each other."""
    rng = np.random.default_rng(seed)
    rots = np.zeros((sys_.num_atoms, 3, 3))
    for t in range(sys_.num_types):
        atoms = np.flatnonzero(sys_.atom_type == t)
        mats = [np.eye(3) if (identity_first and c == 0) else _rotation(rng) for c in range(per_type)]
        for i, j in enumerate(atoms):
            rots[j] = mats[i % per_type] @ sys_.bmat
    out = dataclasses.replace(sys_)
    out.atom_rotmat = rots
    return out


def with_rotations(sys_: System, seed: int = 99) -> System:
    """Copy of ``sys_`` whose atoms carry seeded proper rotations ``mrot``
    (stored premultiplied, ``rotmat = mrot @ bmat`` as ``FleurData.cpp:453-455``)."""
    rng = np.random.default_rng(seed)
    rots = []
    for _ in range(sys_.num_atoms):
        q, r = np.linalg.qr(rng.standard_normal((3, 3)))
        q = q * np.sign(np.diag(r))[None, :]
        if np.linalg.det(q) < 0:
            q[:, 0] = -q[:, 0]
        rots.append(q @ sys_.bmat)
    out = dataclasses.replace(sys_)
    out.atom_rotmat = np.asarray(rots)
    return out
