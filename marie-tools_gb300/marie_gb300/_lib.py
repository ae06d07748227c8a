"""ctypes binding of libmarie_gb300.so (declarations in include/marie_gb300.h).

The library is the product: there is no CPU or PyTorch fallback.  Loading
fails loudly when the shared library is missing.
"""
from __future__ import annotations

import ctypes as ct
import os
import re
from pathlib import Path

from . import _build

c_int32_p = ct.POINTER(ct.c_int32)
c_double_p = ct.POINTER(ct.c_double)

MARIE_OK = 0
STATUS_NAMES = {0: "MARIE_OK", 1: "MARIE_ERR_BAD_ARG", 2: "MARIE_ERR_OOM", 3: "MARIE_ERR_NONFINITE",
                4: "MARIE_ERR_NOT_CONVERGED", 5: "MARIE_ERR_DEVICE_TIMEOUT", 6: "MARIE_ERR_CUDA",
                7: "MARIE_ERR_NOT_SUPPORTED"}
C128, C64 = 0, 1
# marie_vie_desc.precisions bits: native complex128, complex64, complex128 with
# float-float arithmetic (grid edges 16*NB, NB <= 8; exclusive with bit 1)
PREC_C128, PREC_C64, PREC_C128FF = 1, 2, 4
PWC, PWL = 0, 1
SOLVE_FP64, SOLVE_MIXED, SOLVE_MIXED_BLOCK = 0, 1, 2


class MarieError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class TuckerBlock(ct.Structure):
    _fields_ = [("r1", ct.c_int32), ("r2", ct.c_int32), ("r3", ct.c_int32),
                ("G", c_double_p), ("U1", c_double_p), ("U2", c_double_p), ("U3", c_double_p)]


class VieDesc(ct.Structure):
    _fields_ = [("n1", ct.c_int32), ("n2", ct.c_int32), ("n3", ct.c_int32), ("basis", ct.c_int32),
                ("res", ct.c_double), ("freq", ct.c_double), ("n_b", ct.c_int64),
                ("idx_solution", ct.POINTER(ct.c_int64)), ("Mr", c_double_p),
                ("tucker_N", ct.POINTER(TuckerBlock)), ("dense_N", c_double_p),
                ("tucker_K", ct.POINTER(TuckerBlock)), ("dense_K", c_double_p),
                ("precisions", ct.c_int32), ("max_rhs", ct.c_int32), ("mem_cap_bytes", ct.c_int64)]


class GmresOpts(ct.Structure):
    _fields_ = [("restart", ct.c_int32), ("maxit", ct.c_int32), ("tol", ct.c_double), ("mode", ct.c_int32),
                ("x0_present", ct.c_int32), ("inner_tol", ct.c_double), ("max_refine", ct.c_int32),
                ("inner_safety", ct.c_double), ("adjoint", ct.c_int32), ("block_steps", ct.c_int32)]


class GmresReport(ct.Structure):
    _fields_ = [("iters", c_int32_p), ("outer", c_int32_p), ("last_inner", c_int32_p),
                ("true_resid", c_double_p), ("resvec", c_double_p), ("resvec_cap", ct.c_int32),
                ("resvec_len", c_int32_p), ("status", c_int32_p),
                ("matvecs_c128", ct.c_int32), ("matvecs_c64", ct.c_int32)]


class Csr(ct.Structure):
    _fields_ = [("rows", ct.c_int64), ("cols", ct.c_int64), ("nnz", ct.c_int64),
                ("row_ptr", ct.POINTER(ct.c_int64)), ("col_idx", ct.POINTER(ct.c_int64)), ("val", c_double_p)]


class SviePfftDesc(ct.Structure):
    _fields_ = [("grid_op", ct.c_void_p), ("n_sie", ct.c_int64), ("n_b", ct.c_int64), ("PS", Csr),
                ("Z_cc", Csr), ("Z_bc_N", Csr), ("ext_Mc_inv", c_double_p), ("M1", c_double_p),
                ("M2", c_double_p)]


_vp = ct.c_void_p
_PROTOS = {
    "marie_svie_pfft_create": (ct.c_int, [ct.POINTER(_vp), ct.POINTER(SviePfftDesc)]),
    "marie_svie_pfft_apply": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, _vp]),
    "marie_svie_pfft_destroy": (ct.c_int, [_vp]),
    "marie_vie_create": (ct.c_int, [ct.POINTER(_vp), ct.POINTER(VieDesc)]),
    "marie_vie_destroy": (ct.c_int, [_vp]),
    "marie_vie_apply": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, _vp]),
    "marie_vie_apply_adjoint": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, _vp]),
    "marie_vie_apply_N": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, _vp]),
    "marie_vie_apply_N_adj": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, _vp]),
    "marie_vie_apply_K": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, _vp]),
    "marie_vie_apply_K_adj": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, _vp]),
    "marie_gmres_vie": (ct.c_int, [_vp, _vp, _vp, ct.c_int32, ct.POINTER(GmresOpts),
                                   ct.POINTER(GmresReport), _vp]),
    "marie_gmres_vie_host": (ct.c_int, [_vp, _vp, _vp, ct.c_int32, ct.POINTER(GmresOpts),
                                        ct.POINTER(GmresReport), _vp]),
    "marie_assemble_green": (ct.c_int, [ct.c_int32, ct.c_int32, ct.c_int32, ct.c_double, ct.c_double,
                                        ct.c_int32, ct.c_int32, c_double_p]),
    "marie_assemble_green_ex": (ct.c_int, [ct.c_int32, ct.c_int32, ct.c_int32, ct.c_double, ct.c_double,
                                           ct.c_int32, ct.c_int32, ct.c_int32, c_double_p]),
    "marie_incident_loops": (ct.c_int, [_vp, c_double_p, c_double_p, ct.c_int32, ct.c_double,
                                        ct.c_int32, _vp, _vp]),
    "marie_incident_plane_wave": (ct.c_int, [_vp, c_double_p, _vp, _vp]),
    "marie_incident_wire": (ct.c_int, [_vp, ct.c_int32, c_double_p, c_double_p, c_double_p, c_double_p, ct.c_int32,
                                       c_double_p, ct.c_int32, ct.c_int32, ct.c_int32, _vp, _vp]),
    "marie_vie_apply_N_noalloc": (ct.c_int, [ct.c_int32, ct.c_int32, ct.c_int32, ct.c_int32, _vp, _vp, _vp,
                                             _vp]),
    "marie_vie_profile": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, ct.c_int32, c_double_p, _vp]),
    "marie_vie_tiles": (ct.c_int, [_vp, ct.c_int32, c_int32_p]),
    "marie_vie_autotune": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, ct.c_int32, c_int32_p, c_double_p,
                                      ct.c_int32, c_int32_p, _vp]),
    "marie_vie_release_workspace": (ct.c_int, [_vp]),
    "marie_block_gemm_cn": (ct.c_int, [_vp, ct.c_int64, _vp, ct.c_int64, ct.c_int64, ct.c_int32, ct.c_int32, _vp,
                                       ct.c_int64, _vp, ct.c_int64, _vp, _vp]),
    "marie_block_gemm_part_floats": (ct.c_int64, [ct.c_int64, ct.c_int32]),
    "marie_vie_set_materials": (ct.c_int, [_vp, c_double_p]),
    "marie_vie_info": (ct.c_int, [_vp, ct.POINTER(ct.c_int64)]),
    "marie_vie_fields": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, _vp, _vp, _vp, ct.c_int32, _vp]),
    "marie_vie_absorbed_power": (ct.c_int, [_vp, _vp, ct.c_int32, c_double_p, _vp]),
    "marie_vie_b1_plus": (ct.c_int, [_vp, _vp, ct.c_int32, _vp, _vp]),
    "marie_vie_apply_hfield_adjoint": (ct.c_int, [_vp, ct.c_int32, _vp, _vp, ct.c_int32, _vp]),
    "marie_vie_gradient_source": (ct.c_int, [_vp, _vp, _vp, ct.c_double, ct.c_double, _vp, _vp]),
    "marie_vie_gradient": (ct.c_int, [_vp, _vp, _vp, _vp, ct.c_double, ct.c_double, _vp, _vp, _vp]),
    "marie_last_error": (ct.c_char_p, []),
    "marie_version": (ct.c_char_p, []),
    "marie_launch_count": (ct.c_int64, []),
}

_LIB = None


def header_symbols() -> list[str]:
    """Every function declared in include/marie_gb300.h."""
    text = (_build.INCLUDE / "marie_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(marie_[a-zA-Z0-9_]+)\s*\(", text)))


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = False) -> ct.CDLL:
    """Load the library.  Raises if it has not been built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not path.exists():
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(
                f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"`")
    lib = ct.CDLL(str(path))
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int) -> None:
    if status != MARIE_OK:
        msg = load().marie_last_error().decode(errors="replace")
        raise MarieError(status, msg)


def last_error() -> str:
    return load().marie_last_error().decode(errors="replace")


def launch_count() -> int:
    return int(load().marie_launch_count())
