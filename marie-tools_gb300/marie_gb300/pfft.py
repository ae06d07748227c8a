"""Coupled coil/body matvec of MARIE's pFFT formulation on the GB300 library.

Mirror of ``Vout = mvp_svie_pfft(Jcb, pfft_PS, pfft_Z_cc, pfft_Z_bc_N,
ext_Mc_inv, func, fN, Multiplier_1, Multiplier_2, emc, N_sie, res,
pfft_dims)`` (src/src_solver/src_mvp/mvp_svie/mvp_svie_pfft.m:1-19): the
extended (pFFT) grid's N operator is a :class:`VieOperator` (grid mode), the
sparse projection and near-zone corrections are scipy.sparse matrices (or
anything with ``tocsr()``), and the products run in the library's kernels
(marie_svie_pfft_*).
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib
from ._lib import C128, C64, check
from .operator import VieOperator


def _csr_arg(M, keep):
    """(scipy.sparse matrix) -> marie_csr with host buffers kept alive in `keep`."""
    A = M.tocsr()
    A.sort_indices()
    rp = np.ascontiguousarray(A.indptr, dtype=np.int64)
    ci = np.ascontiguousarray(A.indices, dtype=np.int64)
    v = np.ascontiguousarray(np.asarray(A.data, dtype=np.complex128)).view(np.float64)
    keep += [rp, ci, v]
    c = _lib.Csr()
    c.rows, c.cols, c.nnz = A.shape[0], A.shape[1], A.nnz
    c.row_ptr = rp.ctypes.data_as(ct.POINTER(ct.c_int64))
    c.col_idx = ci.ctypes.data_as(ct.POINTER(ct.c_int64))
    c.val = v.ctypes.data_as(_lib.c_double_p)
    return c


class SviePfftOperator:
    """Handle of the coupled matvec.  ``grid_op`` holds the extended grid's N
    operator and must outlive this handle; ``PS`` is (grid unknowns) x
    (N_sie + N_b), ``Z_cc`` N_sie x N_sie, ``Z_bc_N`` N_b x N_sie,
    ``ext_Mc_inv`` (pfft_n1, pfft_n2, pfft_n3) (em_assembly.m:35-37);
    M1 / M2 default to ie_solver_svie_pfft.m:25-26."""

    def __init__(self, grid_op: VieOperator, n_sie: int, PS, Z_cc, Z_bc_N, ext_Mc_inv, M1=None, M2=None):
        self._lib = _lib.load()
        self.grid_op = grid_op
        self.n_sie = int(n_sie)
        self.n_b = int(PS.shape[1]) - self.n_sie
        self.n = self.n_sie + self.n_b
        keep = []
        d = _lib.SviePfftDesc()
        d.grid_op = grid_op._h
        d.n_sie, d.n_b = self.n_sie, self.n_b
        d.PS, d.Z_cc, d.Z_bc_N = _csr_arg(PS, keep), _csr_arg(Z_cc, keep), _csr_arg(Z_bc_N, keep)
        mc = np.ascontiguousarray(np.asarray(ext_Mc_inv, dtype=np.complex128).reshape(-1, order="F")).view(np.float64)
        keep.append(mc)
        d.ext_Mc_inv = mc.ctypes.data_as(_lib.c_double_p)
        for name, m in (("M1", M1), ("M2", M2)):
            if m is not None:
                a = np.ascontiguousarray(np.asarray(m, dtype=np.float64).reshape(-1))
                if a.size != self.n:
                    raise ValueError(f"{name} must have N_sie + N_b entries")
                keep.append(a)
                setattr(d, name, a.ctypes.data_as(_lib.c_double_p))
        h = ct.c_void_p()
        check(self._lib.marie_svie_pfft_create(ct.byref(h), ct.byref(d)))
        self._h = h

    def apply(self, x, out=None):
        """Vout = mvp_svie_pfft(x) for x of nrhs*(N_sie + N_b) entries
        (complex64 or complex128 CUDA tensor)."""
        import torch
        if x.device.type != "cuda" or x.dtype not in (torch.complex64, torch.complex128):
            raise ValueError("x must be a complex64 or complex128 CUDA tensor")
        x = x.contiguous()
        if x.numel() % self.n:
            raise ValueError("x length is not a multiple of N_sie + N_b")
        y = torch.empty_like(x) if out is None else out
        prec = C128 if x.dtype == torch.complex128 else C64
        check(self._lib.marie_svie_pfft_apply(self._h, prec, ct.c_void_p(x.data_ptr()), ct.c_void_p(y.data_ptr()),
                                              x.numel() // self.n,
                                              ct.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return y

    def close(self):
        if getattr(self, "_h", None):
            self._lib.marie_svie_pfft_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_OPS: dict = {}


def mvp_svie_pfft(Jcb, pfft_PS, pfft_Z_cc, pfft_Z_bc_N, ext_Mc_inv, func, fN, Multiplier_1, Multiplier_2, emc,
                  N_sie, res, pfft_dims):
    """Signature mirror of mvp_svie_pfft.m:1: builds (once per set of
    operands) and applies a :class:`SviePfftOperator`; ``fN`` is the
    extended grid's :class:`VieOperator`; ``func``, ``emc``, ``res`` and
    ``pfft_dims`` are carried by it and accepted for signature parity."""
    import torch
    key = (id(fN), id(pfft_PS), id(pfft_Z_cc), id(pfft_Z_bc_N), id(ext_Mc_inv))
    op = _OPS.get(key)
    if op is None:
        op = SviePfftOperator(fN, N_sie, pfft_PS, pfft_Z_cc, pfft_Z_bc_N, ext_Mc_inv,
                              None if Multiplier_1 is None else np.real(np.asarray(Multiplier_1)),
                              None if Multiplier_2 is None else np.real(np.asarray(Multiplier_2)))
        for old in _OPS.values():
            old.close()
        _OPS.clear()
        _OPS[key] = op
    was_torch = isinstance(Jcb, torch.Tensor)
    x = Jcb if was_torch else torch.from_numpy(np.ascontiguousarray(np.asarray(Jcb, dtype=np.complex128)))
    y = op.apply(x.to("cuda"))
    return y if was_torch else y.cpu().numpy()
