"""The reference's wire-to-voxel coupling kernels, compiled from its sources
(oracle/Makefile -> oracle/_ref/libtri_{N,K}_{x,x1,...,z3}.so), for the
checks of the loop and wire right-hand sides.

TEST INFRASTRUCTURE ONLY.

Assemble_tri_coupling_matrix_N_<v>.cpp (called by wvie_mrgf_assembly.m:26-49)
returns, for every voxel and wire triangle basis (positive segment r_p ->
r_2, negative segment r_2 -> r_n), the voxel average of the <v> component of
the field of the basis current (2-point Gauss per voxel axis, 4-point per
segment, Quad_order_vie / Quad_order_wie_coup of load_inputs.m).  Its
get_source_coords_mat weights both halves with a ramp rising from the half's
start point, so unit coefficients on a closed loop carry a sawtooth current
of mean 1 (with line and point charges), where the library's loop kernel
models a uniform current.
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

from . import marie_oracle as O

_D = ct.POINTER(ct.c_double)
_libs = {}


def load(v, kind="N"):
    key = f"{kind}_{v}"
    if key not in _libs:
        path = Path(__file__).resolve().parent / "_ref" / f"libtri_{key}.so"
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (make -C oracle REF=<reference checkout>)")
        lib = ct.CDLL(str(path))
        lib.oracle_tri_coupling.argtypes = [_D] * 7 + [ct.c_double, ct.c_size_t, ct.c_size_t, ct.c_double]
        _libs[key] = lib
    return _libs[key]


def tri_coupling(v, centres, r_p, r_n, r_2, res, k0, q_wire=4, q_vox=2, kind="N"):
    """(N_vox, N_tri) coupling of component v ('x', 'x1', ..., 'z3') of the
    electric (kind "N") or magnetic (kind "K") field; centres and the r_*
    arrays are (N, 3).  Without the res^3 of wvie_mrgf_assembly.m."""
    w, x = O.gauss_1d(q_wire)
    wq = np.ascontiguousarray(np.r_[q_wire, w, x], dtype=float)
    w, x = O.gauss_1d(q_vox)
    vq = np.ascontiguousarray(np.r_[q_vox, w, x], dtype=float)
    arrs = [np.ascontiguousarray(a, dtype=float) for a in (centres, r_p, r_n, r_2)]
    Z = np.zeros(2 * len(arrs[0]) * len(arrs[1]))
    load(v, kind).oracle_tri_coupling(Z.ctypes.data_as(_D), *[a.ctypes.data_as(_D) for a in arrs], wq.ctypes.data_as(_D),
                                vq.ctypes.data_as(_D), res, len(arrs[0]), len(arrs[1]), k0)
    return Z.view(np.complex128).reshape((len(arrs[0]), len(arrs[1])), order="F")


def loop_bases(centre, normal, radius, nseg):
    """Triangle bases of a closed regular nseg-gon (the nodes of
    marie_oracle.loop_points): basis i spans nodes i-1 -> i -> i+1."""
    normal = np.asarray(normal, float) / np.linalg.norm(normal)
    a = np.array([1.0, 0, 0]) if abs(normal[0]) < 0.9 else np.array([0, 1.0, 0])
    e1 = np.cross(normal, a)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(normal, e1)
    t = 2 * np.pi * np.arange(nseg) / nseg
    P = np.asarray(centre, float)[None, :] + radius * (np.cos(t)[:, None] * e1 + np.sin(t)[:, None] * e2)
    return np.roll(P, 1, axis=0), np.roll(P, -1, axis=0), P      # r_p, r_n, r_2


def loop_field_reference(centres, centre, normal, radius, nseg, res, k0):
    """Voxel-averaged field (N_vox, 3) of the loop with unit coefficients on
    every basis, by the reference's kernels."""
    r_p, r_n, r_2 = loop_bases(centre, normal, radius, nseg)
    return np.stack([tri_coupling(v, centres, r_p, r_n, r_2, res, k0).sum(axis=1) for v in "xyz"], axis=1)
