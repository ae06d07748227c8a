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
        lib.oracle_directfn_va.argtypes = [_D] * 7 + [ct.c_int, ct.c_double, ct.c_double] + [_D] * 4 + \
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


# ---------------------------------------------------------------------------
# The whole surface-surface near zone of assembly_N.m:56-81 (any near offset,
# PWC and PWL): surface_surface_coeff_Nop.m + surface_surface_kernels_Nop.m
# with coefficients_Nop.m and kernels_Nop.m, singular face pairs by DIRECTFN.
# The face pairs are classified by their shared vertices (4: ST, 2: EA, 1:
# VA, 0: regular) and the DIRECTFN point orders built from that, instead of
# the hand tables of points_mapping.m.
# ---------------------------------------------------------------------------

_NX = [-1, 1, 0, 0, 0, 0]
_NY = [0, 0, -1, 1, 0, 0]
_NZ = [0, 0, 0, 0, -1, 1]
_P = [1, 1, 1, 2, 2, 3]
_Q = [1, 2, 3, 2, 3, 3]


def _h(l, dx):
    """Gradient of moment l (1-based: 1 const, 2 x/dx, 3 y/dx, 4 z/dx)."""
    h = np.zeros(3)
    if l > 1:
        h[l - 2] = 1.0 / dx
    return h


def coefficients_Nop(dx, n, np_, p, q, l, lp, ker):
    """coefficients_Nop.m:1-89."""
    pp = np.eye(3)[p - 1]
    qq = np.eye(3)[q - 1]
    if ker == 1:
        return float(np.dot(np.cross(n, pp), np.cross(np_, qq)))
    if ker == 2:
        return float(np.dot(np.cross(np.cross(_h(l, dx), pp), qq), n))
    if ker == 3:
        return float(np.dot(np.cross(pp, np.cross(_h(lp, dx), qq)), n))
    a = np.cross(_h(l, dx), pp)
    hp = _h(lp, dx)
    return float(sum(np.dot(np.cross(a, np.eye(3)[j]), n) * np.dot(hp * qq[j], np_) for j in range(3)))


def _face(c, f, dx):
    """Normal and cyclic vertices of face f (0-based, surface_surface_kernels_Nop.m face order) of the voxel
    centred at c."""
    n = np.array([_NX[f], _NY[f], _NZ[f]], dtype=float)
    a = int(np.argmax(np.abs(n)))
    b, e = (a + 1) % 3, (a + 2) % 3
    verts = []
    for sb, se in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
        v = np.array(c, dtype=float)
        v[a] += n[a] * dx / 2
        v[b] += sb * dx / 2
        v[e] += se * dx / 2
        verts.append(v)
    return n, verts


def _rot(verts, first, second=None):
    """Cyclic order of a square's vertices starting at `first` (then `second`
    if given, else either neighbour)."""
    k = next(i for i, v in enumerate(verts) if np.allclose(v, first))
    fwd = [verts[(k + i) % 4] for i in range(4)]
    bwd = [verts[(k - i) % 4] for i in range(4)]
    if second is None or np.allclose(fwd[1], second):
        return fwd
    assert np.allclose(bwd[1], second)
    return bwd


def _kernel_regular(ker, Xo, Xs, k0, dx, rm, rn, l, lp, nsrc):
    """kernels_Nop.m:1-122 at observation points Xo and source points Xs
    (paired rows)."""
    d = Xo - Xs
    R = np.linalg.norm(d, axis=1)
    G = np.exp(-1j * k0 * R) / (4 * np.pi * R)
    G0 = 1 / (4 * np.pi * R)

    def mom(l_, X, c):
        return np.ones(len(X)) if l_ == 1 else (X[:, l_ - 2] - c[l_ - 2]) / dx
    if ker == 1:
        return mom(l, Xo, rm) * mom(lp, Xs, rn) * G
    ff = d / (1j * k0) ** 2 * (-1j * k0 * G / R - G / R ** 2 + G0 / R ** 2)[:, None]
    q2 = ff @ nsrc
    if ker == 2:
        return mom(lp, Xs, rn) * q2
    if ker == 3:
        return mom(l, Xo, rm) * q2
    return (G - G0) / (1j * k0) ** 2


def _pair_integral(Vo, Vs, n, np_, dker, l0, lp0, regular_fn, k0, dx, N, quad):
    """One face-pair integral of the surface form: by the reference's DIRECTFN
    (kernel type dker, 0-based moments l0, lp0) if the two squares share a
    vertex, an edge or everything, else by a tensor Gauss rule of the
    kernel regular_fn(Xo, Xs) (paired observation / source points)."""
    shared = [v for v in Vs if any(np.allclose(v, u) for u in Vo)]
    k = len(shared)
    if k == 0:
        S, T, W2 = quad

        def pts(V):
            e1, e2 = V[1] - V[0], V[3] - V[0]
            return V[0][None, :] + (S + 0.5)[:, None] * e1 + (T + 0.5)[:, None] * e2
        Po, Ps = pts(Vo), pts(Vs)
        Xo = np.repeat(Po, len(Ps), axis=0)
        Xs = np.tile(Ps, (len(Po), 1))
        Wq = np.repeat(W2, len(W2)) * np.tile(W2, len(W2)) * dx ** 4
        return np.sum(Wq * regular_fn(Xo, Xs))
    lib = load()
    if k == 4:                                       # ST: one square
        r = _rot(Vs, Vs[0], Vs[1])
        cq = (r[0] + r[2]) / 2
        args, fn, cs, co = [r[0], r[1], r[2], r[3]], lib.oracle_directfn_st, cq, cq
    elif k == 2:                                     # EA: source (r3, r4, r1, r2), observation (r4, r3, r6, r5)
        e0, e1 = shared
        src = _rot(Vs, e0, e1)
        obs = _rot(Vo, e1, e0)
        r1, r2, r3, r4 = src[2], src[3], src[0], src[1]
        r6, r5 = obs[2], obs[3]
        args, fn = [r1, r2, r3, r4, r5, r6], lib.oracle_directfn_ea
        cs, co = (r1 + r3) / 2, (r4 + r6) / 2        # singular_EA_lin.m
    else:                                            # VA: source (r3, r4, r1, r2), observation (r3, r5, r6, r7)
        src = _rot(Vs, shared[0])
        obs = _rot(Vo, shared[0])
        r3, r4, r1, r2 = src
        r5, r6, r7 = obs[1], obs[2], obs[3]
        args, fn = [r1, r2, r3, r4, r5, r6, r7], lib.oracle_directfn_va
        cs, co = (r1 + r3) / 2, (r3 + r6) / 2        # singular_VA_lin.m
    keep = [np.ascontiguousarray(a, dtype=float) for a in args + [cs, co, np_, n]]
    ptrs = [a.ctypes.data_as(_D) for a in keep]
    out = np.zeros(2)
    fn(*ptrs[:len(args)], N, k0, dx, *ptrs[len(args):], dker, l0, lp0, out.ctypes.data_as(_D))
    return out[0] + 1j * out[1]


def _gauss_squares(qg):
    w, x = O.gauss_1d(qg)
    x, w = x / 2, w / 2
    S, T = np.meshgrid(x, x, indexing="ij")
    return S.ravel(), T.ravel(), np.outer(w, w).ravel()


def surface_near_zone(k0, dx, pwx, m, N=16, qg=16):
    """I_V(m) (pwx, 6) of the N operator by the reference's surface-surface
    formulation (surface_surface_kernels_Nop.m: kernels 1-4, DIRECTFN kernel
    types 1-4 on the singular face pairs); m in {0,1}^3 (observation voxel at
    m dx, source at the origin)."""
    L = 4 if pwx == 10 else 1
    rm, rn = np.array(m, dtype=float) * dx, np.zeros(3)
    quad = _gauss_squares(qg)
    Iss = np.zeros((L, L, 6), dtype=complex)
    for f in range(6):
        n, Vo = _face(rm, f, dx)
        for fp in range(6):
            np_, Vs = _face(rn, fp, dx)
            cache = {}

            def integral(ker, l, lp):
                if (ker, l, lp) not in cache:
                    reg = (lambda Xo, Xs: _kernel_regular(ker, Xo, Xs, k0, dx, rm, rn, l, lp, np_))
                    cache[(ker, l, lp)] = _pair_integral(Vo, Vs, n, np_, ker, l - 1, lp - 1, reg, k0, dx, N, quad)
                return cache[(ker, l, lp)]

            for i in range(6):
                p, q = _P[i], _Q[i]
                for l in range(1, L + 1):
                    for lp in range(1, L + 1):
                        acc = 0.0
                        c = coefficients_Nop(dx, n, np_, p, q, 0, 0, 1)
                        if c:
                            acc += c * integral(1, l, lp)
                        c = coefficients_Nop(dx, n, np_, p, q, l, 0, 2)
                        if c:
                            acc += c * integral(2, 1, lp)
                        c = coefficients_Nop(dx, n, np_, p, q, 0, lp, 3)
                        if c:
                            acc += c * integral(3, l, 1)
                        c = coefficients_Nop(dx, n, np_, p, q, l, lp, 4)
                        if c:
                            acc += c * integral(4, 1, 1)
                        Iss[l - 1, lp - 1, i] += acc
    out = np.zeros((pwx, 6), dtype=complex)
    for llp in range(pwx):
        out[llp] = Iss[O.IND_L[llp], O.IND_LP[llp]]
    return out


# --- the K operator: surface_surface_coeff_Kop.m / surface_surface_kernels_Kop.m
_PK = [3, 1, 2]
_QK = [2, 3, 1]


def coefficients_Kop(dx, ko, n, np_, p, q, l, lp, ker):
    """coefficients_Kop.m:1-89."""
    pp = np.eye(3)[p - 1]
    qq = np.eye(3)[q - 1]
    if ker == 1:
        return complex(np.dot(np.cross(pp, qq), np_))
    if ker == 2:
        return 1 / (1j * ko) ** 2 * np.dot(np_, np.dot(np.cross(qq, pp), _h(lp, dx)) * _h(l, dx))
    if ker == 3:
        return complex(np.dot(n, np_) * np.dot(_h(lp, dx), np.cross(pp, qq)))
    h = _h(l, dx)
    return complex(sum(np.dot(np.cross(qq, np.eye(3)[j]), np_) * np.dot(h * pp[j], n) for j in range(3)))


def _kernel_regular_K(ker, Xo, Xs, k0, dx, rm, rn, l, lp, nobs):
    """kernels_Kop.m:1-114 at paired observation / source points."""
    d = Xo - Xs
    R = np.linalg.norm(d, axis=1)
    G = np.exp(-1j * k0 * R) / (4 * np.pi * R)
    G0 = 1 / (4 * np.pi * R)

    def mom(l_, X, c):
        return np.ones(len(X)) if l_ == 1 else (X[:, l_ - 2] - c[l_ - 2]) / dx
    ff = d / (1j * k0) ** 2 * (-1j * k0 * G / R - G / R ** 2 + G0 / R ** 2)[:, None]
    if ker == 1:
        return mom(l, Xo, rm) * mom(lp, Xs, rn) * (ff @ nobs)
    if ker == 2:
        return (ff - d / 2 * G0[:, None]) @ nobs
    if ker == 3:
        return mom(l, Xo, rm) * (G - G0) / (1j * k0) ** 2
    return mom(lp, Xs, rn) * (G - G0) / (1j * k0) ** 2


def surface_near_zone_K(k0, dx, pwx, m, N=16, qg=16):
    """I_V(m) (pwx, 3) of the K operator by the reference's surface-surface
    formulation (surface_surface_kernels_Kop.m: kernels 1-4 through DIRECTFN
    kernel types 5-8 on singular face pairs), m in {0,1}^3."""
    L = 4 if pwx == 10 else 1
    rm, rn = np.array(m, dtype=float) * dx, np.zeros(3)
    quad = _gauss_squares(qg)
    Iss = np.zeros((L, L, 3), dtype=complex)
    for f in range(6):
        n, Vo = _face(rm, f, dx)
        for fp in range(6):
            np_, Vs = _face(rn, fp, dx)
            cache = {}

            def integral(ker, l, lp):
                if (ker, l, lp) not in cache:
                    reg = (lambda Xo, Xs: _kernel_regular_K(ker, Xo, Xs, k0, dx, rm, rn, l, lp, n))
                    cache[(ker, l, lp)] = _pair_integral(Vo, Vs, n, np_, 4 + ker, l - 1, lp - 1, reg, k0, dx, N,
                                                         quad)
                return cache[(ker, l, lp)]

            for i in range(3):
                p, q = _PK[i], _QK[i]
                for l in range(1, L + 1):
                    for lp in range(1, L + 1):
                        acc = 0.0
                        c = coefficients_Kop(dx, k0, n, np_, p, q, 0, 0, 1)
                        if c:
                            acc += c * integral(1, l, lp)
                        c = coefficients_Kop(dx, k0, n, np_, p, q, l, lp, 2)
                        if c:
                            acc += c * integral(2, 1, 1)
                        c = coefficients_Kop(dx, k0, n, np_, p, q, 0, lp, 3)
                        if c:
                            acc += c * integral(3, l, 1)
                        c = coefficients_Kop(dx, k0, n, np_, p, q, l, 0, 4)
                        if c:
                            acc += c * integral(4, 1, lp)
                        Iss[l - 1, lp - 1, i] += acc
    out = np.zeros((pwx, 3), dtype=complex)
    for llp in range(pwx):
        out[llp] = Iss[O.IND_L[llp], O.IND_LP[llp]]
    return out
