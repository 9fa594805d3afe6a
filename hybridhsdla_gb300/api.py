"""Python host mirror of the reference's H/S entry point, over the C ABI.

``create_HS2`` mirrors ``double create_HS2(kpt, kmax, bmat, g_mesh, ad, method,
H, S)`` (``flapw_opt/src/h_and_s.cpp:591-893``): same inputs (k-point, reciprocal
basis, G list, per-atom data), same outputs (lower triangles of H and S,
column-major complex128), and the elapsed milliseconds as return value.  Every
call goes through ``libhsdla_gb300.so``; there is no Python or CPU compute path,
and loading fails loudly when the library or a GPU is missing.

PyTorch is used only to hold device buffers for the device-resident ``Plan``.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import build as _build

PREC_FP64 = 0
PREC_OZAKI_FP8 = 1
_PREC = {"fp64": PREC_FP64, "ozaki": PREC_OZAKI_FP8, "ozaki_fp8": PREC_OZAKI_FP8}

STATUS = {0: "HSDLA_OK", -1: "HSDLA_ERR_ARG", -2: "HSDLA_ERR_CUDA", -3: "HSDLA_ERR_NOMEM",
          -4: "HSDLA_ERR_INPUT", -5: "HSDLA_ERR_TIMEOUT", -6: "HSDLA_ERR_UNSUPPORTED",
          -7: "HSDLA_ERR_DEVICE"}


class HsdlaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)


class Cx(ctypes.Structure):
    _fields_ = [("re", ctypes.c_double), ("im", ctypes.c_double)]


_cxp = ctypes.POINTER(Cx)


class SystemStruct(ctypes.Structure):
    _fields_ = [("num_atoms", ctypes.c_int32), ("num_types", ctypes.c_int32), ("max_lmax", ctypes.c_int32),
                ("reserved0", ctypes.c_int32), ("vol_cell", ctypes.c_double), ("bmat", ctypes.c_double * 9),
                ("atom_type", _ip), ("atom_pos", _dp), ("atom_rotmat", _dp), ("type_rmt", _dp),
                ("type_lmax", _ip), ("type_u", _dp), ("type_u_dr", _dp), ("type_dE_u", _dp),
                ("type_dE_u_dr", _dp), ("type_dE_u_norm", _dp), ("type_t_aa", _cxp), ("type_t_ab", _cxp),
                ("type_t_bb", _cxp)]


class KpointStruct(ctypes.Structure):
    _fields_ = [("k", ctypes.c_double * 3), ("n_g", ctypes.c_int64), ("g", _ip)]


class OptsStruct(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("num_slices", ctypes.c_int32), ("target_rel_err", ctypes.c_double),
                ("use_graph", ctypes.c_int32), ("reserved", ctypes.c_int32 * 7)]


class ReportStruct(ctypes.Structure):
    _fields_ = [("ms_total", ctypes.c_double), ("ms_per_kpoint", ctypes.c_double), ("flop", ctypes.c_double),
                ("eff_tflops", ctypes.c_double), ("ms_construct_ab", ctypes.c_double),
                ("ms_tapply", ctypes.c_double), ("ms_contract", ctypes.c_double),
                ("ms_dominant", ctypes.c_double), ("dominant_flop", ctypes.c_double),
                ("est_rel_err", ctypes.c_double),
                ("num_slices", ctypes.c_int32), ("num_kpoints", ctypes.c_int32),
                ("kernel_launches", ctypes.c_int32), ("num_panels", ctypes.c_int32),
                ("outputs_in_place", ctypes.c_int32), ("num_row_sets", ctypes.c_int32),
                ("rotation_classes", ctypes.c_int32), ("tile_halves", ctypes.c_int32),
                ("merged_units", ctypes.c_int32), ("tile_tuned", ctypes.c_int32), ("output_blocks", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 1), ("ms_host_setup", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


# every symbol include/hsdla.h declares
EXPORTS = ["hsdla_context_create", "hsdla_context_destroy", "hsdla_last_error", "hsdla_set_mem_cap",
           "hsdla_prepare_tmat", "hsdla_create_hs", "hsdla_plan_create", "hsdla_plan_execute",
           "hsdla_plan_workspace_bytes", "hsdla_plan_destroy", "hsdla_plan_construct_ab",
           "hsdla_zherkx_lower", "hsdla_zherkx_lower_noalloc", "hsdla_contract_ab", "hsdla_pack_lower",
           "hsdla_selftest_wait_timeout", "hsdla_zherk", "hsdla_zher2k", "hsdla_zherkx", "hsdla_dev_init",
           "hsdla_dev_finalize", "hsdla_dev_context", "hsdla_dev_status", "hsdla_dev_zherk_", "hsdla_dev_zher2k_",
           "hsdla_dev_zherkx_", "hsdla_radial_match"]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load ``libhsdla_gb300.so`` (building it in-tree if needed); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libhsdla_gb300.so not found at {path}; run hybridhsdla_gb300/build.py")
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    L.hsdla_context_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
    L.hsdla_context_create.restype = ctypes.c_int
    L.hsdla_context_destroy.argtypes = [vp]
    L.hsdla_context_destroy.restype = None
    L.hsdla_last_error.argtypes = [vp]
    L.hsdla_last_error.restype = ctypes.c_char_p
    L.hsdla_set_mem_cap.argtypes = [vp, ctypes.c_int64]
    L.hsdla_prepare_tmat.argtypes = [ctypes.c_int32, ctypes.c_int32, _cxp, _cxp, _cxp, _cxp, _dp, _dp, _cxp,
                                     _cxp, _cxp]
    L.hsdla_create_hs.argtypes = [vp, ctypes.POINTER(SystemStruct), ctypes.POINTER(KpointStruct), ctypes.c_int32,
                                  ctypes.POINTER(_cxp), ctypes.POINTER(_cxp), ctypes.POINTER(ctypes.c_int64),
                                  ctypes.POINTER(OptsStruct), ctypes.POINTER(ReportStruct)]
    L.hsdla_plan_create.argtypes = [vp, ctypes.POINTER(SystemStruct), ctypes.POINTER(KpointStruct),
                                    ctypes.c_int32, ctypes.POINTER(OptsStruct), ctypes.POINTER(vp)]
    L.hsdla_plan_execute.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_int64),
                                     vp, ctypes.POINTER(ReportStruct)]
    L.hsdla_plan_workspace_bytes.argtypes = [vp]
    L.hsdla_plan_workspace_bytes.restype = ctypes.c_int64
    L.hsdla_plan_destroy.argtypes = [vp]
    L.hsdla_plan_destroy.restype = None
    L.hsdla_plan_construct_ab.argtypes = [vp, ctypes.c_int32, vp, vp]
    L.hsdla_zherkx_lower.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, vp,
                                     ctypes.c_int64, vp, ctypes.c_int64, vp, vp, ctypes.c_int64, vp]
    L.hsdla_contract_ab.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, _cxp, _cxp, _ip,
                                    ctypes.POINTER(_cxp), ctypes.POINTER(_cxp), ctypes.POINTER(_cxp), _ip,
                                    ctypes.c_int32, _dp, _cxp, _cxp, ctypes.c_int64, ctypes.POINTER(OptsStruct),
                                    ctypes.POINTER(ReportStruct)]
    L.hsdla_pack_lower.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_int64, vp, vp]
    L.hsdla_selftest_wait_timeout.argtypes = [vp, ctypes.c_int32, ctypes.c_int64]
    L.hsdla_zherkx_lower_noalloc.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, vp, ctypes.c_int64, vp,
                                             ctypes.c_int64, vp, vp, ctypes.c_int64, vp]
    i32, i64, ch, dbl = ctypes.c_int32, ctypes.c_int64, ctypes.c_char, ctypes.c_double
    L.hsdla_zherk.argtypes = [vp, i32, i32, ch, ch, i64, i64, dbl, vp, i64, dbl, vp, i64, vp]
    L.hsdla_zher2k.argtypes = [vp, i32, i32, ch, ch, i64, i64, Cx, vp, i64, vp, i64, dbl, vp, i64, vp]
    L.hsdla_zherkx.argtypes = [vp, i32, i32, ch, ch, i64, i64, Cx, vp, i64, vp, i64, dbl, vp, i64, vp]
    L.hsdla_dev_init.argtypes = [i32, i32, i32]
    L.hsdla_dev_finalize.argtypes = []
    L.hsdla_dev_context.argtypes = []
    L.hsdla_dev_context.restype = vp
    L.hsdla_dev_status.argtypes = []
    ip = ctypes.POINTER(ctypes.c_int)
    cp = ctypes.c_char_p
    L.hsdla_dev_zherk_.argtypes = [cp, cp, ip, ip, _dp, vp, ip, _dp, vp, ip]
    L.hsdla_dev_zherk_.restype = None
    L.hsdla_dev_zher2k_.argtypes = [cp, cp, ip, ip, _cxp, vp, ip, vp, ip, _dp, vp, ip]
    L.hsdla_dev_zher2k_.restype = None
    L.hsdla_dev_zherkx_.argtypes = [cp, cp, ip, ip, _cxp, vp, ip, vp, ip, _dp, vp, ip]
    L.hsdla_dev_zherkx_.restype = None
    L.hsdla_radial_match.argtypes = [i32, dbl, _dp, i32, dbl, dbl, _dp]
    _lib = L
    return L


# ------------------------------------------------------------------ helpers
def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _addr(x):
    """Address of a numpy array or a torch tensor (host or device), or None."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return ctypes.c_void_p(x.data_ptr())
    return ctypes.c_void_p(x.ctypes.data)


def _stream(stream):
    if stream is None:
        return None
    return ctypes.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


def _cx(z) -> Cx:
    z = complex(z)
    return Cx(z.real, z.imag)


def prepare_tmats(sys_) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Augmented (aa, ab, bb) per type, (types, L, L), via ``hsdla_prepare_tmat``
    (TMat + zero_nonsph + augment_tmats, host C++ inside the library)."""
    L_ = load()
    nt, L = sys_.num_types, sys_.L
    outs = [np.zeros((nt, L, L), np.complex128) for _ in range(3)]
    tba = sys_.tba_raw()
    for t in range(nt):
        lm = int(sys_.type_lmax[t])
        n = (lm + 1) ** 2
        ins = [np.asfortranarray(x[t, :n, :n]) for x in (sys_.taa_raw, sys_.tbb_raw, sys_.tab_raw, tba)]
        o = [np.zeros((n, n), np.complex128, order="F") for _ in range(3)]
        E = _c(sys_.energies[t, :lm + 1], np.float64)
        un = _c(sys_.dE_u_norm[t, :lm + 1], np.float64)
        rc = L_.hsdla_prepare_tmat(lm, int(sys_.type_lmax_nonsph[t]),
                                   *[x.ctypes.data_as(_cxp) for x in ins], E.ctypes.data_as(_dp),
                                   un.ctypes.data_as(_dp), *[x.ctypes.data_as(_cxp) for x in o])
        if rc != 0:
            raise HsdlaError(rc, "hsdla_prepare_tmat rejected the T blocks")
        for q in range(3):
            outs[q][t, :n, :n] = o[q]
    return tuple(outs)


class _SysHolder:
    """Keeps the numpy arrays behind an ``hsdla_system`` alive."""

    def __init__(self, sys_, tmats=None):
        aa, ab, bb = tmats if tmats is not None else prepare_tmats(sys_)
        nl = sys_.max_lmax + 1
        pad = lambda x: _c(np.pad(x, ((0, 0), (0, nl - x.shape[1]))), np.float64)
        self.arrays = dict(
            atom_type=_c(sys_.atom_type, np.int32), atom_pos=_c(sys_.atom_pos, np.float64),
            atom_rotmat=None if sys_.atom_rotmat is None else _c(sys_.atom_rotmat, np.float64),
            type_rmt=_c(sys_.type_rmt, np.float64), type_lmax=_c(sys_.type_lmax, np.int32),
            u=pad(sys_.u), u_dr=pad(sys_.u_dr), dE_u=pad(sys_.dE_u), dE_u_dr=pad(sys_.dE_u_dr),
            dE_u_norm=pad(sys_.dE_u_norm),
            # column-major per type: store the transpose contiguously
            aa=_c(np.transpose(aa, (0, 2, 1)), np.complex128), ab=_c(np.transpose(ab, (0, 2, 1)), np.complex128),
            bb=_c(np.transpose(bb, (0, 2, 1)), np.complex128))
        A = self.arrays
        s = SystemStruct()
        s.num_atoms, s.num_types, s.max_lmax = sys_.num_atoms, sys_.num_types, sys_.max_lmax
        s.vol_cell = float(sys_.vol_cell)
        for i, v in enumerate(np.asarray(sys_.bmat, dtype=np.float64).reshape(-1)):
            s.bmat[i] = float(v)
        s.atom_type = A["atom_type"].ctypes.data_as(_ip)
        s.atom_pos = A["atom_pos"].ctypes.data_as(_dp)
        s.atom_rotmat = A["atom_rotmat"].ctypes.data_as(_dp) if A["atom_rotmat"] is not None else None
        s.type_rmt = A["type_rmt"].ctypes.data_as(_dp)
        s.type_lmax = A["type_lmax"].ctypes.data_as(_ip)
        s.type_u, s.type_u_dr = A["u"].ctypes.data_as(_dp), A["u_dr"].ctypes.data_as(_dp)
        s.type_dE_u, s.type_dE_u_dr = A["dE_u"].ctypes.data_as(_dp), A["dE_u_dr"].ctypes.data_as(_dp)
        s.type_dE_u_norm = A["dE_u_norm"].ctypes.data_as(_dp)
        s.type_t_aa = A["aa"].ctypes.data_as(_cxp)
        s.type_t_ab = A["ab"].ctypes.data_as(_cxp)
        s.type_t_bb = A["bb"].ctypes.data_as(_cxp)
        self.struct = s


class _KptHolder:
    def __init__(self, kpoints):
        self.g = [_c(kp.g, np.int32) for kp in kpoints]
        arr = (KpointStruct * max(1, len(kpoints)))()
        for i, kp in enumerate(kpoints):
            for c in range(3):
                arr[i].k[c] = float(kp.k[c])
            arr[i].n_g = int(kp.g.shape[0])
            arr[i].g = self.g[i].ctypes.data_as(_ip)
        self.arr = arr
        self.n = len(kpoints)


def _opts(precision="fp64", num_slices=0, target=0.0, use_graph=0) -> OptsStruct:
    o = OptsStruct()
    o.precision = _PREC[precision] if isinstance(precision, str) else int(precision)
    o.num_slices = int(num_slices)
    o.target_rel_err = float(target)
    o.use_graph = int(use_graph)
    return o


class Context:
    """One device context (``hsdla_context_create``)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.hsdla_context_create(device, ctypes.byref(h))
        if rc != 0:
            raise HsdlaError(rc, "hsdla_context_create failed (no sm_100+ GPU?)")
        self.h = h
        import weakref
        self._plans = weakref.WeakSet()

    def check(self, rc: int):
        if rc != 0:
            raise HsdlaError(rc, self.lib.hsdla_last_error(self.h).decode())

    def set_mem_cap(self, nbytes: int):
        self.check(self.lib.hsdla_set_mem_cap(self.h, int(nbytes)))

    def close(self):
        if self.h:
            # plans hold device memory of this context: destroy them first
            for p in list(self._plans):
                p.close()
            self.lib.hsdla_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --------------------------------------------------------- host-buffer API
    def create_hs(self, sys_, kpoints=None, precision="fp64", num_slices=0, tmats=None,
                  out: Optional[Sequence[Tuple[np.ndarray, np.ndarray]]] = None):
        """H, S (lower triangles, upper zero) for each k-point, host buffers.
        Returns (list of (H, S) Fortran-ordered arrays, report dict)."""
        kpoints = sys_.kpoints if kpoints is None else kpoints
        sh = _SysHolder(sys_, tmats)
        kh = _KptHolder(kpoints)
        nk = len(kpoints)
        if out is None:      # zeroed: the library writes the lower triangles only
            out = [(np.zeros((kp.n_g, kp.n_g), np.complex128, order="F"),
                    np.zeros((kp.n_g, kp.n_g), np.complex128, order="F")) for kp in kpoints]
        Hp = (_cxp * max(nk, 1))(*[o[0].ctypes.data_as(_cxp) for o in out])
        Sp = (_cxp * max(nk, 1))(*[o[1].ctypes.data_as(_cxp) for o in out])
        ld = (ctypes.c_int64 * max(nk, 1))(*[max(1, o[0].shape[0]) for o in out])
        o = _opts(precision, num_slices)
        rep = ReportStruct()
        self.check(self.lib.hsdla_create_hs(self.h, ctypes.byref(sh.struct), kh.arr, nk, Hp, Sp, ld,
                                            ctypes.byref(o), ctypes.byref(rep)))
        return list(out), rep.as_dict()

    def contract_ab(self, d, precision="fp64", num_slices=0):
        """``create_HS2_stripped_v2`` drop-in (``hsdla_contract_ab``): H, S (lower triangles,
        upper zero) from a :class:`hybridhsdla_gb300.flapw_data.DataIn` (caller-built A, B,
        per-atom T blocks).  Returns (H, S, report)."""
        A = np.asfortranarray(d.A, np.complex128)
        B = np.asfortranarray(d.B, np.complex128)
        a, G = d.a, d.G
        sizes = np.ascontiguousarray([[t.shape[0] for t in blk] for blk in d.blocks], np.int32).reshape(-1)
        keep = [[np.asfortranarray(t, np.complex128) for t in blk] for blk in d.blocks]
        paa = (_cxp * a)(*[k[0].ctypes.data_as(_cxp) for k in keep])
        pab = (_cxp * a)(*[k[1].ctypes.data_as(_cxp) for k in keep])
        pbb = (_cxp * a)(*[k[2].ctypes.data_as(_cxp) for k in keep])
        lmaxs = np.ascontiguousarray(d.lmaxs, np.int32)
        un = np.ascontiguousarray(d.sqrt_u_norms, np.float64)
        H = np.zeros((G, G), np.complex128, order="F")     # the library writes the lower triangles
        S = np.zeros((G, G), np.complex128, order="F")
        o = _opts(precision, num_slices)
        rep = ReportStruct()
        self.check(self.lib.hsdla_contract_ab(self.h, d.L, a, G, A.ctypes.data_as(_cxp), B.ctypes.data_as(_cxp),
                                              sizes.ctypes.data_as(_ip), paa, pab, pbb, lmaxs.ctypes.data_as(_ip),
                                              d.max_lmax, un.ctypes.data_as(_dp), H.ctypes.data_as(_cxp),
                                              S.ctypes.data_as(_cxp), max(1, G), ctypes.byref(o), ctypes.byref(rep)))
        return H, S, rep.as_dict()

    def plan(self, sys_, kpoints=None, precision="fp64", num_slices=0, tmats=None, target=0.0, use_graph=False):
        return Plan(self, sys_, sys_.kpoints if kpoints is None else kpoints, precision, num_slices, tmats, target,
                    use_graph)

    def zherkx_lower(self, P, Q=None, w=None, precision="fp64", num_slices=0, out=None, stream=None):
        """Lower triangle of P^H diag(w) Q for device (torch) complex128 K x n matrices
        given as column-major, i.e. torch tensors of shape (n, K) row-major."""
        import torch
        Q = P if Q is None else Q
        n, K = P.shape
        if out is None:
            out = torch.zeros((n, n), dtype=torch.complex128, device=P.device)
        st = ctypes.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        self.check(self.lib.hsdla_zherkx_lower(self.h, _PREC[precision], int(num_slices), n, K,
                                               ctypes.c_void_p(P.data_ptr()), K, ctypes.c_void_p(Q.data_ptr()), K,
                                               ctypes.c_void_p(w.data_ptr()) if w is not None else None,
                                               ctypes.c_void_p(out.data_ptr()), n, st))
        return out

    def pack_lower(self, M, out=None, stream=None):
        """Fleur's packed form (``hsdla_pack_lower``) of a device H or S: the lower triangle
        row by row, element (r, c), c <= r, at r (r + 1) / 2 + c.  ``M`` is the column-major
        n x n matrix as the library returns it (a torch tensor of shape (n, n) holding
        ``M[col, row]``).  Returns a complex128 device tensor of n (n + 1) / 2 elements."""
        import torch
        n = M.shape[0]
        if out is None:
            out = torch.empty(n * (n + 1) // 2, dtype=torch.complex128, device=M.device)
        st = ctypes.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        self.check(self.lib.hsdla_pack_lower(self.h, n, ctypes.c_void_p(M.data_ptr()), M.stride(0),
                                             ctypes.c_void_p(out.data_ptr()), st))
        return out


# ------------------------------------------------- BLAS-shaped contraction plugin
# Argument order and meaning of dev_zherk_ / dev_zher2k_ / dev_zherkx_
# (flapw_opt/src/include/acc/wrappers.h:19-28): column-major matrices given as numpy arrays or torch
# tensors (host or device memory) with explicit leading dimensions.
def _plugin_methods():
    def zherk(self, uplo, trans, n, k, alpha, A, lda, beta, C, ldc, precision="fp64", num_slices=0, stream=None):
        """C = alpha op(A) op(A)^H + beta C on C's uplo triangle (``hsdla_zherk``)."""
        self.check(self.lib.hsdla_zherk(self.h, _PREC[precision], int(num_slices), uplo.encode(), trans.encode(),
                                        int(n), int(k), float(alpha), _addr(A), int(lda), float(beta), _addr(C),
                                        int(ldc), _stream(stream)))

    def zher2k(self, uplo, trans, n, k, alpha, A, lda, B, ldb, beta, C, ldc, precision="fp64", num_slices=0,
               stream=None):
        """C = alpha op(A) op(B)^H + conj(alpha) op(B) op(A)^H + beta C (``hsdla_zher2k``)."""
        self.check(self.lib.hsdla_zher2k(self.h, _PREC[precision], int(num_slices), uplo.encode(), trans.encode(),
                                         int(n), int(k), _cx(alpha), _addr(A), int(lda), _addr(B), int(ldb),
                                         float(beta), _addr(C), int(ldc), _stream(stream)))

    def zherkx(self, uplo, trans, n, k, alpha, A, lda, B, ldb, beta, C, ldc, precision="fp64", num_slices=0,
               stream=None):
        """C = alpha op(A) op(B)^H + beta C, Hermitian result assumed (``hsdla_zherkx``)."""
        self.check(self.lib.hsdla_zherkx(self.h, _PREC[precision], int(num_slices), uplo.encode(), trans.encode(),
                                         int(n), int(k), _cx(alpha), _addr(A), int(lda), _addr(B), int(ldb),
                                         float(beta), _addr(C), int(ldc), _stream(stream)))
    return zherk, zher2k, zherkx


def dev_init(device: int = 0, precision="fp64", num_slices: int = 0):
    """``hsdla_dev_init``: the library-owned context of the Fortran-style entry points."""
    L_ = load()
    rc = L_.hsdla_dev_init(int(device), _PREC[precision] if isinstance(precision, str) else int(precision),
                           int(num_slices))
    if rc != 0:
        raise HsdlaError(rc, "hsdla_dev_init failed")


def dev_finalize():
    load().hsdla_dev_finalize()


def _dev_check():
    L_ = load()
    rc = L_.hsdla_dev_status()
    if rc != 0:
        c = L_.hsdla_dev_context()
        raise HsdlaError(rc, L_.hsdla_last_error(c).decode() if c else "no context")


def _iref(v):
    return ctypes.byref(ctypes.c_int(int(v)))


def dev_zherk_(uplo, trans, n, k, alpha, A, lda, beta, C, ldc):
    """The reference's ``dev_zherk_`` argument list (every argument by reference)."""
    load().hsdla_dev_zherk_(uplo.encode(), trans.encode(), _iref(n), _iref(k), ctypes.byref(ctypes.c_double(alpha)),
                            _addr(A), _iref(lda), ctypes.byref(ctypes.c_double(beta)), _addr(C), _iref(ldc))
    _dev_check()


def dev_zher2k_(uplo, trans, n, k, alpha, A, lda, B, ldb, beta, C, ldc):
    """The reference's ``dev_zher2k_`` argument list."""
    load().hsdla_dev_zher2k_(uplo.encode(), trans.encode(), _iref(n), _iref(k), ctypes.byref(_cx(alpha)), _addr(A),
                             _iref(lda), _addr(B), _iref(ldb), ctypes.byref(ctypes.c_double(beta)), _addr(C),
                             _iref(ldc))
    _dev_check()


def dev_zherkx_(uplo, trans, n, k, alpha, A, lda, B, ldb, beta, C, ldc):
    """The reference's ``dev_zherkx_`` argument list."""
    load().hsdla_dev_zherkx_(uplo.encode(), trans.encode(), _iref(n), _iref(k), ctypes.byref(_cx(alpha)), _addr(A),
                             _iref(lda), _addr(B), _iref(ldb), ctypes.byref(ctypes.c_double(beta)), _addr(C),
                             _iref(ldc))
    _dev_check()


def zherkx_lower_noalloc(P, Q=None, w=None, num_slices=0, out=None, stream=None):
    """Allocation-free Ozaki contraction (``hsdla_zherkx_lower_noalloc``): lower
    triangle of P^H diag(w) Q for device complex128 K x n matrices given as torch
    tensors of shape (n, K).  The library itself allocates no device memory for it;
    its scratch is a static device array of 128 MiB.  ``out`` must be supplied by a
    caller that cannot allocate; otherwise a torch buffer is made here."""
    import torch
    L_ = load()
    Q = P if Q is None else Q
    n, K = P.shape
    if out is None:
        out = torch.zeros((n, n), dtype=torch.complex128, device=P.device)
    st = ctypes.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
    rc = L_.hsdla_zherkx_lower_noalloc(int(num_slices), n, K, ctypes.c_void_p(P.data_ptr()), K,
                                       ctypes.c_void_p(Q.data_ptr()), K,
                                       ctypes.c_void_p(w.data_ptr()) if w is not None else None,
                                       ctypes.c_void_p(out.data_ptr()), n, st)
    if rc != 0:
        raise HsdlaError(rc, L_.hsdla_last_error(None).decode())
    return out


class Plan:
    """Device-resident plan (``hsdla_plan_create``): inputs uploaded once; ``execute``
    writes H/S into device buffers."""

    def __init__(self, ctx: Context, sys_, kpoints, precision, num_slices, tmats, target=0.0, use_graph=False):
        self.ctx = ctx
        self.sys = sys_
        self.kpoints = list(kpoints)
        self._sh = _SysHolder(sys_, tmats)
        self._kh = _KptHolder(self.kpoints)
        o = _opts(precision, num_slices, target, int(bool(use_graph)))
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.hsdla_plan_create(ctx.h, ctypes.byref(self._sh.struct), self._kh.arr, len(self.kpoints),
                                            ctypes.byref(o), ctypes.byref(h)))
        self.h = h
        ctx._plans.add(self)

    def workspace_bytes(self) -> int:
        return int(self.ctx.lib.hsdla_plan_workspace_bytes(self.h))

    def alloc_outputs(self):
        import torch
        outs = []
        for kp in self.kpoints:
            # column-major n x n == row-major tensor whose [col, row] is element (row, col)
            outs.append((torch.zeros((kp.n_g, kp.n_g), dtype=torch.complex128, device="cuda"),
                         torch.zeros((kp.n_g, kp.n_g), dtype=torch.complex128, device="cuda")))
        return outs

    def execute(self, outs, stream=None) -> dict:
        import torch
        nk = len(self.kpoints)
        Hp = (ctypes.c_void_p * max(nk, 1))(*[o[0].data_ptr() for o in outs])
        Sp = (ctypes.c_void_p * max(nk, 1))(*[o[1].data_ptr() for o in outs])
        ld = (ctypes.c_int64 * max(nk, 1))(*[max(1, kp.n_g) for kp in self.kpoints])
        st = ctypes.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        rep = ReportStruct()
        self.ctx.check(self.ctx.lib.hsdla_plan_execute(self.h, Hp, Sp, ld, st, ctypes.byref(rep)))
        return rep.as_dict()

    def construct_ab(self, ik: int, stream=None):
        """Device C = [A_a; B_a] stacked per atom as a torch tensor of shape (n_g, 2 L a)."""
        import torch
        kp = self.kpoints[ik]
        C = torch.empty((kp.n_g, 2 * self.sys.La), dtype=torch.complex128, device="cuda")
        st = ctypes.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        self.ctx.check(self.ctx.lib.hsdla_plan_construct_ab(self.h, ik, ctypes.c_void_p(C.data_ptr()), st))
        return C

    def close(self):
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx.lib.hsdla_plan_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def split_ab(C_rows: np.ndarray, L: int, a: int) -> Tuple[np.ndarray, np.ndarray]:
    """(n_g, 2 L a) row-major device layout -> reference A, B as (L a, n_g) matrices."""
    G = C_rows.shape[0]
    c = C_rows.reshape(G, a, 2, L)
    A = np.asfortranarray(c[:, :, 0, :].reshape(G, a * L).T)
    B = np.asfortranarray(c[:, :, 1, :].reshape(G, a * L).T)
    return A, B


def create_HS2(kpt, kmax, bmat, g_mesh, ad, method="fp64", ctx: Optional[Context] = None):
    """Mirror of ``create_HS2`` (h_and_s.cpp:591-893) for one k-point.

    ``g_mesh`` is the 3 x n_G integer matrix of the reference (columns = G),
    ``ad`` a :class:`hybridhsdla_gb300.synth.System` (the AtomData stand-in);
    ``kmax`` is accepted and unused, as in the reference (types_helper.cpp:28).
    Returns (H, S, elapsed_ms) with lower triangles set."""
    from .synth import KPoint
    del kmax
    ctx = ctx or Context()
    kp = KPoint(k=np.asarray(kpt, dtype=np.float64), g=np.ascontiguousarray(np.asarray(g_mesh).T, dtype=np.int32))
    if bmat is not None and not np.allclose(np.asarray(bmat), ad.bmat):
        raise ValueError("bmat differs from the system's reciprocal basis")
    (res,), rep = ctx.create_hs(ad, [kp], precision=method)
    return res[0], res[1], rep["ms_total"]


Context.zherk, Context.zher2k, Context.zherkx = _plugin_methods()
