"""The reference's DIRECTFN singular integrals, compiled from its sources
(oracle/Makefile -> oracle/_ref/libdirectfn.so), and the surface-surface
near zone of assembly_N.m:56-81 evaluated with them for the PWC moment.

TEST INFRASTRUCTURE ONLY (pins the oracle's near_zone_relative and, through
it, the library's MARIE_GREEN_NEAR_EXACT cubature to the reference's own
singular quadrature).

For PWC (L = 1) only kernel 1 of surface_surface_kernels_Nop.m contributes
(the moment gradients h of kernels 2-4 vanish), with coefficient
I1_co = (n x p) . (n' x q) (coefficients_Nop.m, case 1) and the plain
Green function e^{-ik0R}/(4 pi R) (kernels_Nop.m, case 1; DIRECTFN kernel
type 1 with l = lp = 0) over every pair of faces of the observation and the
source voxel: coincident faces by DIRECTFN ST, faces sharing an edge by
DIRECTFN EA, the rest by a tensor Gauss rule (non-singular).
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

from . import marie_oracle as O

LIB = Path(__file__).resolve().parent / "_ref" / "libdirectfn.so"
_D = ct.POINTER(ct.c_double)
_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise FileNotFoundError(f"{LIB} not built (make -C oracle REF=<reference checkout>)")
        lib = ct.CDLL(str(LIB))
        lib.oracle_directfn_st.argtypes = [_D] * 4 + [ct.c_int, ct.c_double, ct.c_double] + [_D] * 4 + \
            [ct.c_int] * 3 + [_D]
        lib.oracle_directfn_ea.argtypes = [_D] * 6 + [ct.c_int, ct.c_double, ct.c_double] + [_D] * 4 + \
            [ct.c_int] * 3 + [_D]
        _lib = lib
    return _lib


def _call(fn, pts, k0, dx, N):
    keep = [np.ascontiguousarray(v, dtype=float) for v in pts] + [np.zeros(3)]
    out = np.zeros(2)
    z = keep[-1].ctypes.data_as(_D)
    fn(*[v.ctypes.data_as(_D) for v in keep[:-1]], N, k0, dx, z, z, z, z, 1, 0, 0, out.ctypes.data_as(_D))
    return out[0] + 1j * out[1]


def st(r1, r2, r3, r4, k0, dx, N=16):
    """int int e^{-ik0R}/(4 pi R) over the square r1 r2 r3 r4 with itself."""
    return _call(load().oracle_directfn_st, (r1, r2, r3, r4), k0, dx, N)


def ea(r1, r2, r3, r4, r5, r6, k0, dx, N=16):
    """The same over the squares (r4, r3, r6, r5) and (r3, r4, r1, r2)
    sharing the edge r3-r4."""
    return _call(load().oracle_directfn_ea, (r1, r2, r3, r4, r5, r6), k0, dx, N)


def regular(c1, e1a, e1b, c2, e2a, e2b, k0, q=24):
    """The same over two separated squares c + s e_a + t e_b, s, t in
    [-1/2, 1/2], by a tensor Gauss rule."""
    w, x = O.gauss_1d(q)
    x, w = x / 2, w / 2
    S, T = np.meshgrid(x, x, indexing="ij")
    W = np.outer(w, w).reshape(-1)
    P1 = (c1[None, None, :] + S[..., None] * e1a + T[..., None] * e1b).reshape(-1, 3)
    P2 = (c2[None, None, :] + S[..., None] * e2a + T[..., None] * e2b).reshape(-1, 3)
    A1 = np.linalg.norm(np.cross(e1a, e1b))
    A2 = np.linalg.norm(np.cross(e2a, e2b))
    R = np.linalg.norm(P1[:, None, :] - P2[None, :, :], axis=-1)
    return (W * A1) @ (np.exp(-1j * k0 * R) / (4 * np.pi * R)) @ (W * A2)


def pwc_near_entries(k0, res, N=16):
    """PWC I_V entries of the surface-surface near zone by face pairs:
    self offset xx (= yy = zz) and face neighbour (1,0,0) xx and yy.

    Self: the 4 coincident y/z face pairs (coefficient 1) and the 4 opposite
    y/z pairs (-1); x faces and perpendicular pairs have coefficient 0.
    (1,0,0) xx: the 4 coplanar y/z face pairs sharing an edge (+1) and the
    4 parallel pairs one voxel apart in y or z and shifted by one in x (-1).
    (1,0,0) yy: the shared x face (-1), the two parallel x pairs one voxel
    apart (+1), the x pair two voxels apart (-1), the 2 coplanar z pairs
    (+1) and the 2 shifted parallel z pairs (-1)."""
    X, Y, Z = np.eye(3) * res
    z0 = np.zeros(3)
    S_st = st([0, 0, 0], [res, 0, 0], [res, res, 0], [0, res, 0], k0, res, N)
    S_opp = regular(z0, X, Y, np.array([0, 0, res]), X, Y, k0)
    S_far2 = regular(np.array([0, 0, 2 * res]), X, Y, z0, X, Y, k0)
    S_ea = ea([0, res, 0], [0, 0, 0], [res, 0, 0], [res, res, 0], [2 * res, res, 0], [2 * res, 0, 0], k0, res, N)
    S_par = regular(np.array([res, 0, res]), X, Y, z0, X, Y, k0)
    return {"self_xx": 4 * S_st - 4 * S_opp,
            "face_xx": 4 * S_ea - 4 * S_par,
            "face_yy": -S_st + 2 * S_opp - S_far2 + 2 * S_ea - 2 * S_par}
