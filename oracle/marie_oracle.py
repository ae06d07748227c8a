"""CPU oracle: an FP64 numpy restatement of MARIE's VIE matvec + GMRES path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, its
C-ABI, or the Python host package) imports, links or executes this module.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, and only as the checker / the timed CPU reference.

Parity status of the hot path: *parity unpinned*.  The reference hot path
is MATLAB (``.m`` files calling ``fftn``/``svd``/``mldivide``); MATLAB and
Octave are not available, and the reference ships no tests, golden vectors
or fixtures for this path.  This restatement follows the reference line by
line (each function cites the file:line it restates, paths relative to the
reference project root) and is pinned instead by algebraic identities
(adjoint and transpose identities, Tucker exactness, an independent
direct-sum convolution) in ``tests/test_oracle.py``, and by known answers
(quasi-static sphere, Mie series) in ``tests/test_green_host.py`` and
``tests/test_physics_sphere.py``.

Operator generation: far and medium zones restate assembly_N.m /
assembly_K.m; the near zone is either the staggered stand-in
(:func:`near_zone_standin`, what the GPU assembly computes by default) or
:func:`near_zone_relative`, an independent cubature of the same integrals
that is pinned to the reference's own surface-surface near zone with its
DIRECTFN C++ compiled from source (``oracle/directfn_ref.py``,
``tests/test_near_zone_directfn.py``).

Conventions are MATLAB's: arrays are indexed (x, y, z, component) and
flattened column-major (``order='F'``); index vectors are 0-based here where
MATLAB's are 1-based.
"""
from __future__ import annotations

import math
import numpy as np

# ---------------------------------------------------------------------------
# Constants and materials
# ---------------------------------------------------------------------------


def em_constants(freq: float) -> dict:
    """Restates src/src_physics/em_constants.m:117-139 for a given frequency.

    The reference derives freq = |gamma| * B0 (em_constants.m:127); the
    frequency is taken directly here.
    """
    mu0 = 4e-7 * math.pi
    c0 = 299792458.0
    e0 = 1.0 / (c0 ** 2 * mu0)
    omega = 2 * math.pi * freq
    lamda = c0 / freq
    k0 = 2 * math.pi / lamda
    return dict(freq=freq, mu0=mu0, c0=c0, e0=e0, omega=omega, lamda=lamda,
                k0=k0, eta0=mu0 * c0, ce=1j * omega * e0, cm=1j * omega * mu0)


def em_assembly(er: np.ndarray, se: np.ndarray, ce: complex) -> dict:
    """Restates src/src_physics/src_electromagnetism/em_assembly.m:14-19."""
    Mr = er + se / ce
    Mc = Mr - 1
    return dict(Mr=Mr, Mc=Mc, Mcr=Mc / Mr, Mr_inv=1.0 / Mr)


def geo_dims(n1, n2, n3, idxS, pwl: bool, res: float) -> dict:
    """Restates src/src_geometry/geo_assembly.m:6-8 and
    src/src_geometry/body_geometry/geo_body_domain.m:14-35.

    ``idxS`` holds 0-based column-major linear voxel indices of the body.
    ``idx_solution`` is component-major: block c holds c*nD + idxS.
    """
    L = 4 if pwl else 1
    ql = 3 * L
    pwx = 10 if pwl else 1
    nD = n1 * n2 * n3
    idxS = np.asarray(idxS, dtype=np.int64)
    idx_solution = np.concatenate([c * nD + idxS for c in range(ql)])
    return dict(n1=n1, n2=n2, n3=n3, l=L, ql=ql, pwx=pwx, res=res, idxS=idxS,
                N_scat=idxS.size, N_b=idxS.size * ql,
                idx_solution=idx_solution)


# ---------------------------------------------------------------------------
# Quadrature and Green's function volume-volume integrals
# ---------------------------------------------------------------------------


def gauss_1d(order: int):
    """Gauss-Legendre rule on [-1, 1]; restates the tabulated values of
    src/src_mathematics/src_quads/gauss_1d.m (ascending abscissas)."""
    x, w = np.polynomial.legendre.leggauss(order)
    return w, x


def weights_points(N: int, dim: int):
    """Restates src/src_integral_equations/src_vie/src_operators_vie/
    cubatures/weights_points.m:3-69 (tensor rule, first variable fastest)."""
    w1, x1 = gauss_1d(N)
    grids = np.meshgrid(*([x1] * dim), indexing="ij")
    wgrid = np.ones([N] * dim)
    for d in range(dim):
        shape = [1] * dim
        shape[d] = N
        wgrid = wgrid * w1.reshape(shape)
    W = wgrid.reshape(-1, order="F")
    pts = [g.reshape(-1, order="F") for g in grids]
    return (W, *pts)


def G_N(x, y, z, xp, yp, zp, k0):
    """Restates cubatures/G_N.m:3-19: the 6 unique entries of the N kernel."""
    dx, dy, dz = x - xp, y - yp, z - zp
    R = np.sqrt(dx ** 2 + dy ** 2 + dz ** 2)
    Gexp = np.exp(-1j * k0 * R) / 4 / np.pi
    R2, R3, R4, R5 = R ** 2, R ** 3, R ** 4, R ** 5
    Gxx = Gexp * (3 * dx ** 2 / R5 + 3j * k0 * dx ** 2 / R4 - (1 + k0 ** 2 * dx ** 2) / R3 - 1j * k0 / R2)
    Gyy = Gexp * (3 * dy ** 2 / R5 + 3j * k0 * dy ** 2 / R4 - (1 + k0 ** 2 * dy ** 2) / R3 - 1j * k0 / R2)
    Gzz = Gexp * (3 * dz ** 2 / R5 + 3j * k0 * dz ** 2 / R4 - (1 + k0 ** 2 * dz ** 2) / R3 - 1j * k0 / R2)
    Gxy = Gexp * (3 * dx * dy / R5 + 3j * k0 * dx * dy / R4 - k0 ** 2 * dx * dy / R3)
    Gxz = Gexp * (3 * dx * dz / R5 + 3j * k0 * dx * dz / R4 - k0 ** 2 * dx * dz / R3)
    Gyz = Gexp * (3 * dy * dz / R5 + 3j * k0 * dy * dz / R4 - k0 ** 2 * dy * dz / R3)
    return np.stack([-Gyy - Gzz, Gxy, Gxz, -Gxx - Gzz, Gyz, -Gxx - Gyy], axis=-1)


def G_K(x, y, z, xp, yp, zp, k0):
    """Restates cubatures/G_K.m:3-13: gradient of the scalar Green function."""
    dx, dy, dz = x - xp, y - yp, z - zp
    R = np.sqrt(dx ** 2 + dy ** 2 + dz ** 2)
    Gexp = np.exp(-1j * k0 * R) / 4 / np.pi
    f = Gexp * (1.0 / R ** 3 + 1j * k0 / R ** 2)
    return np.stack([-dx * f, -dy * f, -dz * f], axis=-1)


# (l, l') pairs of the 10 unique PWL moment products, VV_Nop.m:27-28
IND_L = np.array([1, 2, 3, 4, 1, 1, 1, 2, 2, 3]) - 1
IND_LP = np.array([1, 2, 3, 4, 2, 3, 4, 3, 4, 4]) - 1


def VV_op(W, X, Y, Z, Xp, Yp, Zp, k0, r_m, r_n, dx, pwx, kernel):
    """Restates cubatures/VV_Nop.m:1-48 (kernel='N') and VV_Kop.m:1-50
    (kernel='K'): 6D Gauss volume-volume integral for one offset r_m.

    Returns an array (pwx, 6) for N or (pwx, 3) for K.
    """
    J = (dx / 2) ** 6
    Xg, Yg, Zg = r_m[0] + dx / 2 * X, r_m[1] + dx / 2 * Y, r_m[2] + dx / 2 * Z
    Xpg, Ypg, Zpg = r_n[0] + dx / 2 * Xp, r_n[1] + dx / 2 * Yp, r_n[2] + dx / 2 * Zp
    G = (G_N if kernel == "N" else G_K)(Xg, Yg, Zg, Xpg, Ypg, Zpg, k0)
    T = np.stack([np.ones_like(X), X / 2, Y / 2, Z / 2], axis=-1)      # (dx/2*X)/dx
    B = np.stack([np.ones_like(Xp), Xp / 2, Yp / 2, Zp / 2], axis=-1)
    out = np.zeros((pwx, G.shape[-1]), dtype=complex)
    for llp in range(pwx):
        TB = T[:, IND_L[llp]] * B[:, IND_LP[llp]]
        out[llp] = ((W * TB)[:, None] * G).sum(axis=0) * J
    return out


def near_zone_standin(k0, res, pwx, kernel, offsets):
    """Stand-in for the near-zone (offsets in {0,1}^3) surface-surface
    integrals of assembly_N.m:56-81 / assembly_K.m:56-81.

    The reference evaluates these through DIRECTFN singular integrals.  Until
    that restatement lands, the near offsets are integrated with a staggered
    tensor Gauss rule (observation order 8, source order 7) so that
    quadrature points never coincide.  The same stand-in is used by the GPU
    assembly, so operator parity is unaffected; only the physics of the
    self/adjacent terms is approximate.
    """
    w8, x8 = gauss_1d(8)
    w7, x7 = gauss_1d(7)
    gx, gy, gz = np.meshgrid(x8, x8, x8, indexing="ij")
    gw = (w8[:, None, None] * w8[None, :, None] * w8[None, None, :])
    hx, hy, hz = np.meshgrid(x7, x7, x7, indexing="ij")
    hw = (w7[:, None, None] * w7[None, :, None] * w7[None, None, :])
    X = np.repeat(gx.ravel(), hx.size); Y = np.repeat(gy.ravel(), hx.size)
    Z = np.repeat(gz.ravel(), hx.size)
    Xp = np.tile(hx.ravel(), gx.size); Yp = np.tile(hy.ravel(), gx.size)
    Zp = np.tile(hz.ravel(), gx.size)
    W = np.repeat(gw.ravel(), hw.size) * np.tile(hw.ravel(), gw.size)
    out = {}
    for m in offsets:
        r_m = np.array(m, dtype=float) * res
        out[tuple(m)] = VV_op(W, X, Y, Z, Xp, Yp, Zp, k0, r_m, np.zeros(3), res, pwx, kernel)
    return out


def self_delta_term(res, pwx):
    """The point term of the N kernel at the self offset, (pwx, 6).

    The six N components are those of curl curl (g I) (G_N.m: -Gyy-Gzz, Gxy,
    ...).  As distributions, d_p d_q g = PV(d_p d_q g) - (1/3) delta_pq
    delta(r) and lap g = -k0^2 g - delta(r), so curl curl (g I) = PV[pointwise
    kernel] + (2/3) delta_pq delta(r).  Integrated against T_l(r) B_l'(r') over
    one voxel pair the point term gives (2/3) delta_pq int_V T_l B_l' =
    (2/3) Gram_ll' on the diagonal components (xx, yy, zz: k = 0, 3, 5), with
    Gram = diag(res^3, res^3/12, res^3/12, res^3/12) for the moments
    [1, x/res, y/res, z/res] (the diagonal of mvp_G_pwl.m:5).  The
    reference's surface-surface near zone (assembly_N.m:56-81) contains it;
    a pointwise cubature of the volume kernel does not.
    """
    gram = np.array([res ** 3, res ** 3 / 12, res ** 3 / 12, res ** 3 / 12])
    out = np.zeros((pwx, 6), dtype=complex)
    for llp in range(pwx):
        if IND_L[llp] == IND_LP[llp]:
            out[llp, [0, 3, 5]] = (2.0 / 3.0) * gram[IND_L[llp]]
    return out


def _moment_overlap(u, m_d, res, l_axis, lp_axis):
    """w_d(u) = int T-factor(u + x' - m_d res) B-factor(x') dx' over the
    source-voxel interval x' in [-res/2, res/2] whose image u + x' lies in
    the observation voxel [m_d res - res/2, m_d res + res/2]; the factors are
    s/res on the moment's own axis and 1 otherwise (moments [1, x/res, y/res,
    z/res], VV_Nop.m:18-19).  Exact for the quadratic integrand."""
    lo = np.maximum(-res / 2, m_d * res - res / 2 - u)
    hi = np.minimum(res / 2, m_d * res + res / 2 - u)
    hi = np.maximum(hi, lo)
    a, b = (1.0, 0.0) if not l_axis else ((u - m_d * res) / res, 1.0 / res)     # t(x') = a + b x'
    c, d = (1.0, 0.0) if not lp_axis else (0.0, 1.0 / res)                    # b(x') = c + d x'
    A, B, C = a * c, a * d + b * c, b * d
    return A * (hi - lo) + B * (hi ** 2 - lo ** 2) / 2 + C * (hi ** 3 - lo ** 3) / 3


def _moment_weights(U, m, res, pwx):
    """W_llp(u) = int_{V_0 and V_m - u} T_l(u + r' - c_m) B_l'(r') dr' for the
    pwx moment pairs (IND_L, IND_LP): a product of per-axis overlaps."""
    out = np.ones((U.shape[0], pwx))
    for llp in range(pwx):
        l, lp = IND_L[llp], IND_LP[llp]
        for d in range(3):
            out[:, llp] *= _moment_overlap(U[:, d], m[d], res, l == d + 1, lp == d + 1)
    return out


def near_zone_relative(k0, res, pwx, kernel, offsets, order=16):
    """I_V of the near offsets (the quantity of assembly_N.m:56-81 /
    assembly_K.m:56-81) by an independent cubature, not the reference's
    surface-surface/DIRECTFN route.

    With u = r - r', I(m) = int K(u) W(u) du over the box prod_d [(m_d-1) res,
    (m_d+1) res], W the moment overlap of :func:`_moment_weights` (piecewise
    polynomial, kinks at u_d = m_d res).  The box is split at the kinks and at
    0 so that the kernel's singular point u = 0 is a corner of every piece
    that touches it; pieces away from 0 take a tensor Gauss rule, pieces with
    the corner take three Duffy pyramids (u = t (L_e, L_f v, L_g w), Jacobian
    t^2 L^3), which removes the 1/R^2 singularity of K and the 1/R of the
    dynamic part of N.  The static part K_s of the N kernel (degree -3) is
    integrated as K_s(u~) (W(t u~) - W(0)) / t; the remaining W(0) K_s / t is
    the principal value over the cube around u = 0 (self offset; zero by
    cubic symmetry) or vanishes (W(0) = 0 for the other offsets).  The self
    offset then gets the point term (2/3) delta_pq Gram of
    :func:`self_delta_term`.  Returns {m: (pwx, 6 | 3)}."""
    wq, xq = gauss_1d(order)
    t1, w1 = (xq + 1) / 2, wq / 2                       # Gauss on [0, 1]
    T, V, Wv = np.meshgrid(t1, t1, t1, indexing="ij")
    WT = (w1[:, None, None] * w1[None, :, None] * w1[None, None, :]).ravel()
    T, V, Wv = T.ravel(), V.ravel(), Wv.ravel()
    kfun = G_N if kernel == "N" else G_K
    ncomp = 6 if kernel == "N" else 3
    out = {}
    for m in offsets:
        m = tuple(int(v) for v in m)
        acc = np.zeros((pwx, ncomp), dtype=complex)
        pieces = [[(-res, 0.0), (0.0, res)] if m[d] == 0 else [(0.0, res), (res, 2 * res)] for d in range(3)]
        for px in pieces[0]:
            for py in pieces[1]:
                for pz in pieces[2]:
                    box = (px, py, pz)
                    if all(0.0 in b for b in box):
                        # corner at u = 0: signs and lengths of the box from that corner
                        sg = np.array([1.0 if b[1] > 0 else -1.0 for b in box])
                        L = np.array([b[1] - b[0] for b in box])
                        for e in range(3):
                            f, g = [d for d in range(3) if d != e]
                            Ut = np.zeros((T.size, 3))                   # u~ = u / t
                            Ut[:, e] = sg[e] * L[e]
                            Ut[:, f] = sg[f] * L[f] * V
                            Ut[:, g] = sg[g] * L[g] * Wv
                            U = Ut * T[:, None]
                            jac = L.prod() * T ** 2
                            Wm = _moment_weights(U, m, res, pwx)
                            Kf = kfun(U[:, 0], U[:, 1], U[:, 2], 0, 0, 0, k0)
                            if kernel == "N":
                                Ks = kfun(U[:, 0], U[:, 1], U[:, 2], 0, 0, 0, 0.0)
                                Kst = kfun(Ut[:, 0], Ut[:, 1], Ut[:, 2], 0, 0, 0, 0.0)   # K_s(u~) = t^3 K_s(u)
                                W0 = _moment_weights(np.zeros((1, 3)), m, res, pwx)
                                acc += np.einsum("qc,ql->lc", (Kf - Ks) * (WT * jac)[:, None], Wm)
                                acc += np.einsum("qc,ql->lc", Kst * (WT * L.prod())[:, None],
                                                 (Wm - W0) / T[:, None])
                            else:
                                acc += np.einsum("qc,ql->lc", Kf * (WT * jac)[:, None], Wm)
                    else:
                        lo = np.array([b[0] for b in box])
                        L = np.array([b[1] - b[0] for b in box])
                        U = lo[None, :] + L[None, :] * np.stack([T, V, Wv], axis=1)
                        Wm = _moment_weights(U, m, res, pwx)
                        Kf = kfun(U[:, 0], U[:, 1], U[:, 2], 0, 0, 0, k0)
                        acc += np.einsum("qc,ql->lc", Kf * (WT * L.prod())[:, None], Wm)
        if kernel == "N" and m == (0, 0, 0):
            acc += self_delta_term(res, pwx)
        out[m] = acc
    return out


def assembly_op(n1, n2, n3, res, k0, pwl: bool, kernel: str = "N",
                Np_far=4, Np_medium=8, self_term: str = "pointwise", near: str = "standin"):
    """Restates src/src_integral_equations/src_vie/src_operators_vie/
    assembly_N.m:16-81 and assembly_K.m:16-81 (far, medium, near zones).

    Returns I_V with shape (n1, n2, n3, pwx, 6) for N, (..., 3) for K.
    near="standin": the near zone by :func:`near_zone_standin`, and
    self_term="distributional" adds the point term of the N kernel at the
    self offset (:func:`self_delta_term`; K has none); near="relative": the
    near zone by :func:`near_zone_relative` (point term included).
    """
    near_rule = near
    pwx = 10 if pwl else 1
    ncomp = 6 if kernel == "N" else 3
    I_V = np.zeros((n1, n2, n3, pwx, ncomp), dtype=complex)
    W, X, Y, Z, Xp, Yp, Zp = weights_points(Np_far, 6)
    for mx in range(n1):
        for my in range(n2):
            for mz in range(n3):
                r_m = np.array([mx, my, mz], dtype=float) * res
                if mx == 0 and my == 0 and mz == 0:
                    continue        # singular with coincident points; near zone overwrites
                I_V[mx, my, mz] = VV_op(W, X, Y, Z, Xp, Yp, Zp, k0, r_m, np.zeros(3), res, pwx, kernel)
    thr = 5 if kernel == "N" else 2
    Npm = min(n1, n2, n3) if (n1 <= thr or n2 <= thr or n3 <= thr) else Np_medium
    W, X, Y, Z, Xp, Yp, Zp = weights_points(Npm, 6)
    near = [(a, b, c) for a in range(min(2, n1)) for b in range(min(2, n2)) for c in range(min(2, n3))]
    for mx in range(min(Npm, n1)):
        for my in range(min(Npm, n2)):
            for mz in range(min(Npm, n3)):
                if (mx, my, mz) in near:
                    continue
                r_m = np.array([mx, my, mz], dtype=float) * res
                I_V[mx, my, mz] = VV_op(W, X, Y, Z, Xp, Yp, Zp, k0, r_m, np.zeros(3), res, pwx, kernel)
    if self_term not in ("pointwise", "distributional") or near_rule not in ("standin", "relative"):
        raise ValueError(f"bad self_term {self_term!r} or near {near_rule!r}")
    if near_rule == "relative":
        nz = near_zone_relative(k0, res, pwx, kernel, near)
    else:
        nz = near_zone_standin(k0, res, pwx, kernel, near)
    for m, v in nz.items():
        I_V[m] = v
    if near_rule == "standin" and self_term == "distributional" and kernel == "N":
        I_V[0, 0, 0] += self_delta_term(res, pwx)
    return I_V


# ---------------------------------------------------------------------------
# Tucker compression and circulant embedding
# ---------------------------------------------------------------------------


def nmp(A: np.ndarray, B: np.ndarray, mode: int) -> np.ndarray:
    """Restates src/src_mathematics/src_numerical_linear_algebra/src_tucker/
    nmp.m:1-21: C(.., t, ..) = sum_i A(.., i, ..) * B(i, t) along ``mode``
    (1-based, as in MATLAB)."""
    ax = mode - 1
    C = np.tensordot(A, B, axes=([ax], [0]))
    return np.moveaxis(C, -1, ax)


def _trunc_rank(s, tol):
    """First 1-based index with s <= tol*s1/sqrt(3) and s != 0 (hosvd.m:14-25)."""
    hit = np.nonzero((s <= tol * s[0] / np.sqrt(3)) & (s != 0))[0]
    return int(hit[0]) + 1 if hit.size else s.size


def hosvd(A: np.ndarray, tol: float):
    """Restates src_tucker/hosvd.m:1-36 (truncated HOSVD)."""
    n1, n2, n3 = A.shape
    A1 = A.reshape(n1, -1, order="F")
    A2 = np.transpose(A, (1, 0, 2)).reshape(n2, -1, order="F")
    A3 = np.transpose(A, (2, 0, 1)).reshape(n3, -1, order="F")
    U1, S1, _ = np.linalg.svd(A1, full_matrices=False)
    U2, S2, _ = np.linalg.svd(A2, full_matrices=False)
    U3, S3, _ = np.linalg.svd(A3, full_matrices=False)
    r1 = min(_trunc_rank(S1, tol), U1.shape[1])
    r2 = min(_trunc_rank(S2, tol), U2.shape[1])
    r3 = min(_trunc_rank(S3, tol), U3.shape[1])
    U1, U2, U3 = U1[:, :r1], U2[:, :r2], U3[:, :r3]
    G = nmp(nmp(nmp(A, U1.conj(), 1), U2.conj(), 2), U3.conj(), 3)
    return G, U1, U2, U3


# Circulant-extension signs, assembly_fft_circ_tucker_pwc.m:8-16 and
# assembly_fft_circ_tucker_pwl.m:36-47.
G_N_SIGNS = {6: (np.array([+1, -1, -1, +1, +1, +1]), np.array([+1, -1, +1, +1, -1, +1]),
                 np.array([+1, +1, -1, +1, -1, +1])),
             3: (np.array([-1, +1, +1]), np.array([+1, -1, +1]), np.array([+1, +1, -1]))}
BT_SIGNS = (np.array([+1, +1, +1, +1, -1, +1, +1, -1, -1, +1]),
            np.array([+1, +1, +1, +1, +1, -1, +1, -1, +1, -1]),
            np.array([+1, +1, +1, +1, +1, +1, -1, +1, -1, -1]))


def _circ_factor(U, n, s):
    """fft([U; 0; s*U(n:-1:2,:)], [], 1).'  (assembly_fft_circ_tucker_pwl.m:53)."""
    ext = np.concatenate([U, np.zeros((1, U.shape[1]), dtype=U.dtype), s * U[n - 1:0:-1, :]], axis=0)
    return np.fft.fft(ext, axis=0).T.copy()


def assembly_fft_circ_tucker(A: np.ndarray, tol: float):
    """Restates assembly_fft_circ_tucker_pwc.m:3-26 (A of shape (n1,n2,n3,n4))
    and assembly_fft_circ_tucker_pwl.m:31-58 (A of shape (n1,n2,n3,n4,n5)).

    Returns a dict {(j, k): (G, U1, U2, U3)} with 0-based (j, k); for PWC the
    key is (0, k).  U* are already circulant-extended, FFT'd and transposed
    (shape r x 2n).
    """
    if A.ndim == 4:
        A = A[:, :, :, None, :]
        pwl = False
    else:
        pwl = True
    n1, n2, n3, n4, n5 = A.shape
    g1, g2, g3 = G_N_SIGNS[n5]
    T = {}
    for j in range(n4):
        for k in range(n5):
            G, U1, U2, U3 = hosvd(A[:, :, :, j, k], tol)
            b1, b2, b3 = (BT_SIGNS[0][j], BT_SIGNS[1][j], BT_SIGNS[2][j]) if pwl else (1, 1, 1)
            T[(j, k)] = (G, _circ_factor(U1, n1, g1[k] * b1),
                         _circ_factor(U2, n2, g2[k] * b2), _circ_factor(U3, n3, g3[k] * b3))
    return T


def tucker_block(t) -> np.ndarray:
    """nmp(nmp(nmp(G,U1,1),U2,2),U3,3): the full circulant spectrum of one block."""
    G, U1, U2, U3 = t
    return nmp(nmp(nmp(G, U1, 1), U2, 2), U3, 3)


def circ_spectrum_dense(A3: np.ndarray, s1, s2, s3) -> np.ndarray:
    """FFT of the sign-symmetric circulant embedding of one dense block, i.e.
    the untruncated equivalent of :func:`tucker_block`."""
    n1, n2, n3 = A3.shape
    E = np.zeros((2 * n1, 2 * n2, 2 * n3), dtype=complex)
    ix = np.r_[0:n1, n1 + 1:2 * n1]
    sx = np.r_[np.ones(n1), s1 * np.ones(n1 - 1)]
    jx = np.r_[0:n1, n1 - 1:0:-1]
    iy = np.r_[0:n2, n2 + 1:2 * n2]
    sy = np.r_[np.ones(n2), s2 * np.ones(n2 - 1)]
    jy = np.r_[0:n2, n2 - 1:0:-1]
    iz = np.r_[0:n3, n3 + 1:2 * n3]
    sz = np.r_[np.ones(n3), s3 * np.ones(n3 - 1)]
    jz = np.r_[0:n3, n3 - 1:0:-1]
    E[np.ix_(ix, iy, iz)] = A3[np.ix_(jx, jy, jz)] * sx[:, None, None] * sy[None, :, None] * sz[None, None, :]
    return np.fft.fftn(E)


# ---------------------------------------------------------------------------
# Block tables of the N and K operators
# ---------------------------------------------------------------------------

PQ_N = np.array([[1, 2, 3], [2, 4, 5], [3, 5, 6]])            # mvp_N_pwc_tucker.m:12
PQ_K = np.array([[0, -3, 2], [3, 0, -1], [-2, 1, 0]])         # mvp_K_pwc_tucker.m:12
LLP = np.array([[1, 5, 6, 7], [-5, 2, 8, 9], [-6, 8, 3, 10], [-7, 9, 10, 4]])  # mvp_N_pwl_tucker.m:13
SLP = np.array([[1, -1, -1, -1], [-1, 1, 1, 1], [-1, 1, 1, 1], [-1, 1, 1, 1]])  # mvp_N_herm_adj_pwl_tucker.m:14


def block_table(op: str, pwl: bool, adjoint: bool):
    """Per (out, in) component pair: (sign, (j, k) block key, conj) as used by
    mvp_{N,K}{,_herm_adj}_{pwc,pwl}_tucker.m.  ``None`` where no block."""
    C = 12 if pwl else 3
    tab = [[None] * C for _ in range(C)]
    for p in range(3):
        for q in range(3):
            if op == "N":
                j = PQ_N[p, q] - 1
                sgn_pq = 1
            else:
                if p == q:
                    continue
                j = abs(PQ_K[p, q]) - 1
                sgn_pq = int(np.sign(PQ_K[p, q]))
            if not pwl:
                s = sgn_pq * (-1 if (op == "K" and adjoint) else 1)
                tab[p][q] = (s, (0, j), adjoint)
                continue
            for l in range(4):
                for lp in range(4):
                    i = abs(LLP[l, lp]) - 1
                    s = sgn_pq * int(np.sign(LLP[l, lp]))
                    if adjoint:
                        s *= int(np.sign(SLP[l, lp]))
                        if op == "K":
                            s = -s           # conj(-nmp(...)), mvp_K_herm_adj_pwl_tucker.m:34
                    tab[4 * p + l][4 * q + lp] = (s, (i, j), adjoint)
    return tab


# ---------------------------------------------------------------------------
# Operator applications
# ---------------------------------------------------------------------------


def mvp_op_tucker(Jin: np.ndarray, T: dict, op: str = "N", adjoint: bool = False,
                  cache: dict | None = None) -> np.ndarray:
    """Restates mvp_N_pwc_tucker.m:3-31, mvp_N_pwl_tucker.m:3-41,
    mvp_N_herm_adj_{pwc,pwl}_tucker.m, mvp_K_{pwc,pwl}_tucker.m and
    mvp_K_herm_adj_{pwc,pwl}_tucker.m.

    ``Jin`` has shape (n1, n2, n3, C).  With ``cache=None`` each Tucker block
    is re-expanded for every product, exactly as the reference does
    (reference-faithful); a dict caches the expansions (CPU-best variant).
    """
    n1, n2, n3, C = Jin.shape
    pwl = C == 12
    G0 = next(iter(T.values()))
    m1, m2, m3 = G0[1].shape[1], G0[2].shape[1], G0[3].shape[1]
    fJ = [np.fft.fftn(Jin[..., i], s=(m1, m2, m3), axes=(0, 1, 2)) for i in range(C)]
    tab = block_table(op, pwl, adjoint)
    Jout = np.zeros_like(Jin, dtype=complex)
    for p in range(C):
        acc = np.zeros((m1, m2, m3), dtype=complex)
        for q in range(C):
            e = tab[p][q]
            if e is None:
                continue
            s, key, cj = e
            if cache is not None:
                if key not in cache:
                    cache[key] = tucker_block(T[key])
                blk = cache[key]
            else:
                blk = tucker_block(T[key])
            if cj:
                blk = blk.conj()
            acc += s * blk * fJ[q]
        Jout[..., p] = np.fft.ifftn(acc)[:n1, :n2, :n3]
    return Jout


def _fftn(a, s=None, inverse=False, workers=None):
    """3D FFT on all host cores where scipy is present (numpy otherwise)."""
    try:
        import scipy.fft as sfft
        f = sfft.ifftn if inverse else sfft.fftn
        return f(a, s=s, axes=(0, 1, 2), workers=workers or -1)
    except ImportError:
        f = np.fft.ifftn if inverse else np.fft.fftn
        return f(a, s=s, axes=(0, 1, 2))


def block_spectrum_dense(IV: np.ndarray, key, kernel: str = "N", workers=None) -> np.ndarray:
    """Circulant spectrum of block key = (j, k) of a dense I_V
    (n1, n2, n3, pwx, 6|3): the FFT of the sign-symmetric embedding with the
    signs of assembly_fft_circ_tucker_{pwc,pwl}.m (G_n*, bt_n*), i.e. the
    untruncated equivalent of :func:`tucker_block` of
    :func:`assembly_fft_circ_tucker`."""
    n1, n2, n3, pwx, nc = IV.shape
    j, k = key
    g1, g2, g3 = G_N_SIGNS[nc]
    b = (BT_SIGNS[0][j], BT_SIGNS[1][j], BT_SIGNS[2][j]) if pwx == 10 else (1, 1, 1)
    s1, s2, s3 = g1[k] * b[0], g2[k] * b[1], g3[k] * b[2]
    A3 = IV[:, :, :, j, k]
    E = np.zeros((2 * n1, 2 * n2, 2 * n3), dtype=complex)
    ix, jx = np.r_[0:n1, n1 + 1:2 * n1], np.r_[0:n1, n1 - 1:0:-1]
    iy, jy = np.r_[0:n2, n2 + 1:2 * n2], np.r_[0:n2, n2 - 1:0:-1]
    iz, jz = np.r_[0:n3, n3 + 1:2 * n3], np.r_[0:n3, n3 - 1:0:-1]
    sx = np.r_[np.ones(n1), s1 * np.ones(n1 - 1)]
    sy = np.r_[np.ones(n2), s2 * np.ones(n2 - 1)]
    sz = np.r_[np.ones(n3), s3 * np.ones(n3 - 1)]
    E[np.ix_(ix, iy, iz)] = A3[np.ix_(jx, jy, jz)] * sx[:, None, None] * sy[None, :, None] * sz[None, None, :]
    return _fftn(E, workers=workers)


def _mac(acc, a, b, sgn):
    """acc += sgn * a * b elementwise, split over the host cores (numpy
    releases the interpreter lock inside its loops)."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    fa, fb, fo = a.reshape(-1), b.reshape(-1), acc.reshape(-1)
    n = fo.size
    k = max(1, min(os.cpu_count() or 1, n // (1 << 18)))
    step = (n + k - 1) // k

    def work(lo):
        hi = min(n, lo + step)
        t = fa[lo:hi] * fb[lo:hi]
        if sgn > 0:
            fo[lo:hi] += t
        else:
            fo[lo:hi] -= t

    if k == 1:
        work(0)
        return
    global _POOL
    if _POOL is None:
        _POOL = ThreadPoolExecutor(max_workers=os.cpu_count() or 1)
    list(_POOL.map(work, range(0, n, step)))


_POOL = None


def mvp_op_dense(Jin: np.ndarray, IV: np.ndarray, op: str = "N", adjoint: bool = False,
                 spectra: dict | None = None, workers=None) -> np.ndarray:
    """mvp_{N,K}{,_herm_adj}_{pwc,pwl}_tucker.m (the block products of
    mvp_N_pwl_tucker.m:15-41) with the Green blocks taken untruncated from a
    dense I_V: each block's spectrum is formed once per call and applied to
    every (p, q) pair that uses it, so at most one block spectrum is held
    besides the C input and C output spectra (configuration-size checks:
    ~3 GB at 96^3, ~7 GB at 128^3 PWL).  ``spectra`` (a dict) keeps the block
    spectra across calls instead.  FFTs on all host cores."""
    n1, n2, n3, C = Jin.shape
    pwl = C == 12
    m = (2 * n1, 2 * n2, 2 * n3)
    fJ = [_fftn(Jin[..., q], s=m, workers=workers) for q in range(C)]
    tab = block_table(op, pwl, adjoint)
    uses = {}
    for p in range(C):
        for q in range(C):
            e = tab[p][q]
            if e is not None:
                uses.setdefault(e[1], []).append((p, q, e[0], e[2]))
    acc = [np.zeros(m, dtype=complex) for _ in range(C)]
    for key, lst in uses.items():
        if spectra is not None and key in spectra:
            blk = spectra[key]
        else:
            blk = block_spectrum_dense(IV, key, op, workers)
            if spectra is not None:
                spectra[key] = blk
        bc = blk.conj() if adjoint else blk
        for p, q, sg, _cj in lst:
            _mac(acc[p], bc, fJ[q], sg)
        del blk, bc
    Jout = np.empty(Jin.shape, dtype=complex)
    for p in range(C):
        Jout[..., p] = _fftn(acc[p], inverse=True, workers=workers)[:n1, :n2, :n3]
        acc[p] = None
    return Jout


def mvp_vie_dense(Jb, Mr, Mc, dims, IV, spectra=None, workers=None):
    """mvp_vie.m:1-19 with the N blocks taken from a dense I_V
    (:func:`mvp_op_dense`)."""
    Jp = scatter(Jb, dims)
    pwl = dims["ql"] == 12
    NJ = mvp_op_dense(Jp, IV, "N", False, spectra, workers)
    chi = (1.0 / Mr) * Mc
    Jout = Jp - chi[..., None] * (invG_scale(pwl, dims["res"])[None, None, None, :] * NJ)
    return gather(Jout, dims)


def invG_scale(pwl: bool, res: float) -> np.ndarray:
    """Per-component diagonal of mvp_invG_pwc.m:3 / mvp_invG_pwl.m:3."""
    if not pwl:
        return np.full(3, 1.0 / res ** 3)
    g = np.array([1.0 / res ** 3, 1.0 / (res ** 3 / 12), 1.0 / (res ** 3 / 12), 1.0 / (res ** 3 / 12)])
    return np.tile(g, 3)


def G_scale(pwl: bool, res: float) -> np.ndarray:
    """Per-component diagonal of mvp_G_pwc.m:3 / mvp_G_pwl.m:5."""
    if not pwl:
        return np.full(3, res ** 3)
    return np.tile(np.array([res ** 3, res ** 3 / 12, res ** 3 / 12, res ** 3 / 12]), 3)


def scatter(Jb, dims):
    """Jp = zeros(n1,n2,n3,ql); Jp(idx_solution) = Jb  (mvp_vie.m:12-13)."""
    Jp = np.zeros(dims["n1"] * dims["n2"] * dims["n3"] * dims["ql"], dtype=complex)
    Jp[dims["idx_solution"]] = Jb
    return Jp.reshape(dims["n1"], dims["n2"], dims["n3"], dims["ql"], order="F")


def gather(Jp, dims):
    return Jp.reshape(-1, order="F")[dims["idx_solution"]]


def mvp_vie(Jb, Mr, Mc, dims, T, cache=None):
    """Restates src/src_solver/src_mvp/mvp_vie/mvp_vie.m:1-19:
    Jout = Jp - (Mc./Mr) .* invG(N Jp), restricted to the body."""
    Jp = scatter(Jb, dims)
    pwl = dims["ql"] == 12
    NJ = mvp_op_tucker(Jp, T, "N", False, cache)
    chi = (1.0 / Mr) * Mc
    Jout = Jp - chi[..., None] * (invG_scale(pwl, dims["res"])[None, None, None, :] * NJ)
    return gather(Jout, dims)


def mvp_vie_adjoint(Jb, Mr, Mc, dims, T, cache=None):
    """A^H for A = I - diag(chi) invG N:  y - N^H (invG conj(chi) y), with
    N^H from mvp_N_herm_adj_{pwc,pwl}_tucker.m."""
    Jp = scatter(Jb, dims)
    pwl = dims["ql"] == 12
    chi = (1.0 / Mr) * Mc
    Z = np.conj(chi)[..., None] * invG_scale(pwl, dims["res"])[None, None, None, :] * Jp
    NZ = mvp_op_tucker(Z, T, "N", True, cache)
    return gather(Jp - NZ, dims)


# ---------------------------------------------------------------------------
# Field post-processing
# ---------------------------------------------------------------------------


def em_efield_vie_excitation(Jb, Ue, dims, T_N, ce, cache=None):
    """Restates em_efield_vie_excitation.m:17-23 for one port:
    Ue + mask.*invG((1/ce)(mvp_N(Jb) - mvp_G(Jb))) on the body."""
    Jp = scatter(Jb, dims)
    pwl = dims["ql"] == 12
    NJ = mvp_op_tucker(Jp, T_N, "N", False, cache)
    GJ = G_scale(pwl, dims["res"])[None, None, None, :] * Jp
    e = invG_scale(pwl, dims["res"])[None, None, None, :] * ((NJ - GJ) / ce)
    return Ue + gather(e, dims)


def em_hfield_vie_excitation(Jb, Ub, dims, T_K, cache=None):
    """Restates em_hfield_vie_excitation.m:16-22 for one port:
    Ub + mask.*invG(mvp_K(Jb)) on the body."""
    Jp = scatter(Jb, dims)
    pwl = dims["ql"] == 12
    KJ = mvp_op_tucker(Jp, T_K, "K", False, cache)
    return Ub + gather(invG_scale(pwl, dims["res"])[None, None, None, :] * KJ, dims)


def em_noise_covariance(J, Mc, ce, dims):
    """Restates em_ehfield_vie.m:44-52: Mpow = repmat(Mc_inv(idxS),[ql 1])/ce,
    Gx = mvp_G(J) on the body, phi = conj(J' * (real(Mpow) .* Gx)).
    J: (N_b, N_ports)."""
    pwl = dims["ql"] == 12
    mc = np.asarray(Mc).reshape(-1, order="F")[dims["idxS"]]
    mpow = np.tile(1.0 / mc, dims["ql"]) / ce
    g = np.repeat(G_scale(pwl, dims["res"]), dims["N_scat"])
    Gx = g[:, None] * J
    return np.conj(J.conj().T @ (np.real(mpow)[:, None] * Gx))


def b1_plus(Ub, dims, mu0):
    """B1+ = mu0 (Ub(jj) + 1i Ub(jj + N_scat*l)) per body voxel (em_ehfield_vie.m:68)."""
    ns, l = dims["N_scat"], dims["l"]
    return mu0 * (Ub[:ns] + 1j * Ub[l * ns:l * ns + ns])


def b1_objective(J, Ue, Ub, dims, T_N, T_K, Mc, ce, roi, mu0, cache=None):
    """J_obj = mean_ROI |B1+|^2 / P_abs for one solved current J: E and H by
    em_efield/em_hfield_vie_excitation, B1+ = mu0 (Hx + i Hy)
    (em_ehfield_vie.m:68), P_abs = phi(1,1)/2 (em_ehfield_vie.m:44-52).
    roi: body-voxel indices.  Returns (J_obj, M, P, E, H, b1)."""
    E = em_efield_vie_excitation(J, Ue, dims, T_N, ce, cache)
    H = em_hfield_vie_excitation(J, Ub, dims, T_K, cache)
    b1 = b1_plus(H, dims, mu0)
    M = float(np.mean(np.abs(b1[roi]) ** 2))
    P = 0.5 * float(np.real(em_noise_covariance(J[:, None], Mc, ce, dims)[0, 0]))
    return M / P, M, P, E, H, b1


def hfield_map_adjoint(w, dims, T_K, cache=None):
    """Adjoint of J -> gather(invG K scatter(J)) (the scattered-field part of
    em_hfield_vie_excitation.m:16-22): w -> gather(K^H invG scatter(w)),
    invG being real and diagonal and gather the transpose of scatter."""
    pwl = dims["ql"] == 12
    wp = invG_scale(pwl, dims["res"])[None, None, None, :] * scatter(w, dims)
    return gather(mvp_op_tucker(wp, T_K, "K", True, cache), dims)


def b1_objective_gradient(J, E, b1, M, P, Mr, Mc, ce, dims, T_K, roi, mu0, solve_adjoint, cache=None):
    """dJ_obj/d eps_r and dJ_obj/d sigma per body voxel by one adjoint solve
    (no counterpart in the reference).  With chi = 1 - 1/Mr, A = I - chi
    invG N on the body and b = ce chi Ue, A dJ = dchi (ce E + J) per voxel;
    g = dJ_obj/dconj(J) = gM/P - (M/P^2)(1/2) D J with gM the ROI term
    through the adjoint H map and D = G real(1/(Mc ce)); A^H lam = g
    (solve_adjoint); then
      dJ/dp_s = 2 Re(sum_c conj(lam) (ce E + J) (dMr/dp) / Mr^2)
              + (M/P^2)(1/2) sum_c |J|^2 G_c Re((dMr/dp) / (Mc^2 ce)),
    dMr/d eps_r = 1, dMr/d sigma = 1/ce.  Returns (d_eps, d_sigma, lam)."""
    pwl = dims["ql"] == 12
    ns, ql, l = dims["N_scat"], dims["ql"], dims["l"]
    idx = dims["idxS"]
    mr = np.asarray(Mr).reshape(-1, order="F")[idx]
    mc = np.asarray(Mc).reshape(-1, order="F")[idx]
    w = np.zeros(ns * ql, dtype=complex)
    w[roi] = b1[roi]
    w[l * ns + np.asarray(roi)] = -1j * b1[roi]
    gM = hfield_map_adjoint(w, dims, T_K, cache) * (mu0 / len(roi))
    gc = np.repeat(G_scale(pwl, dims["res"]), ns)
    wpow = np.tile(np.real(1.0 / (mc * ce)), ql)
    g = gM / P - 0.5 * (M / P ** 2) * gc * wpow * J
    lam = solve_adjoint(g)
    q = np.sum((np.conj(lam) * (ce * E + J)).reshape(ql, ns), axis=0)
    jj = np.sum((np.abs(J) ** 2 * gc).reshape(ql, ns), axis=0)
    expl = 0.5 * M / P ** 2
    d_eps = 2 * np.real(q / mr ** 2) + expl * jj * np.real(1.0 / (mc ** 2 * ce))
    d_sig = 2 * np.real(q / mr ** 2 / ce) + expl * jj * np.real(1.0 / (mc ** 2 * ce) / ce)
    return d_eps, d_sig, lam


# ---------------------------------------------------------------------------
# GMRES
# ---------------------------------------------------------------------------


def is_iter_gmres_vie(A, x, r, m, tol):
    """Restates src/src_solver/src_iterative_solvers/is_iter_gmres_vie.m:1-38:
    one restart cycle, classical Gram-Schmidt single pass, LS re-solve per k."""
    N = r.shape[0]
    V = np.zeros((N, m + 1), dtype=complex)
    nr = np.linalg.norm(r)
    V[:, 0] = r / nr
    H = np.zeros((m + 1, m), dtype=complex)
    resvec = np.zeros(m)
    k = 0
    for k in range(1, m + 1):
        w = A(V[:, k - 1])
        H[:k, k - 1] = V[:, :k].conj().T @ w
        w = w - V[:, :k] @ H[:k, k - 1]
        H[k, k - 1] = np.linalg.norm(w)
        V[:, k] = w / H[k, k - 1]
        rhs = np.zeros(k + 1, dtype=complex)
        rhs[0] = nr
        Hc = H[:k + 1, :k]
        y = np.linalg.lstsq(Hc, rhs, rcond=None)[0]
        res = rhs - Hc @ y
        resvec[k - 1] = np.linalg.norm(res)
        if resvec[k - 1] < tol:
            break
    resvec = resvec[:k]
    x = x + V[:, :k] @ y
    r = V[:, :k + 1] @ res
    return x, r, k, resvec


def is_gmres_vie(A, b, restart, tol, maxit, x0):
    """Restates src/src_solver/src_iterative_solvers/is_gmres_vie.m:1-30.
    Returns (x, iter=[p, outit], resvec relative to ||b||)."""
    p = 1
    if np.count_nonzero(x0):
        r = b - A(x0)
    else:
        r = b.copy()
    bnorm = np.linalg.norm(b)
    resvec = [np.linalg.norm(r) / bnorm]
    x = x0.astype(complex).copy()
    outit = 0
    while resvec[-1] > tol and outit < maxit:
        outit += 1
        x, r, p, rin = is_iter_gmres_vie(A, x, r, restart, tol * bnorm)
        resvec.extend(list(rin / bnorm))
    return x, np.array([p, outit]), np.array(resvec)


def vie_rhs(ce, Mr, Mc, idxS, ql, Ue):
    """rhs = ce * repmat((1./Mr(idxS)).*Mc(idxS), ql, 1) .* Ue  (ie_solver_vie.m:18)."""
    chi = ((1.0 / Mr.reshape(-1, order="F")[idxS]) * Mc.reshape(-1, order="F")[idxS])
    return ce * np.tile(chi, ql) * Ue


def ie_solver_vie(Mr, Mc, dims, T, Ue, ce, tol, restart=50, maxit=200, X=None):
    """Restates src/src_solver/src_ie_solver/ie_solver_vie/ie_solver_vie.m:3-32:
    serial loop over ports with warm start x0 = Jb(:, i) = 0 (:16-21); with a
    basis X (MREDM.BASIS.X) also Zbb_hat_inv = X.'*((Ue.'*Jb)*X) and its
    economy SVD (:23-25; plain transposes, no conjugation).  Returns
    (Jb, out, (U, S, V)); the factors are None without X (:27-29)."""
    Nports = Ue.shape[1]
    Jb = np.zeros((dims["N_b"], Nports), dtype=complex)
    cache = {}
    A = lambda J: mvp_vie(J, Mr, Mc, dims, T, cache)
    out = []
    for i in range(Nports):
        rhs = vie_rhs(ce, Mr, Mc, dims["idxS"], dims["ql"], Ue[:, i])
        x, it, rv = is_gmres_vie(A, rhs, restart, tol, maxit, Jb[:, i])
        Jb[:, i] = x
        out.append((it, rv))
    usv = (None, None, None)
    if X is not None:
        Z = X.T @ ((Ue.T @ Jb) @ X)
        U, S, Vh = np.linalg.svd(Z, full_matrices=False)
        usv = (U, np.diag(S), Vh.conj().T)
    return Jb, out, usv


# ---------------------------------------------------------------------------
# Coupled coil/body matvec of the pFFT formulation
# ---------------------------------------------------------------------------


def mvp_svie_pfft(Jcb, PS, Z_cc, Z_bc_N, ext_Mc_inv, T, M1, M2, ce, N_sie, res, pfft_dims, cache=None):
    """Restates src/src_solver/src_mvp/mvp_svie/mvp_svie_pfft.m:1-19 (scipy
    sparse PS / Z_cc / Z_bc_N; ``T`` the extended grid's N operator as
    Tucker blocks, or a dense I_V array; ``.'`` is the plain transpose):
      Jb = PS [0; Jcb(N_sie+1:end)], Jtot = PS Jcb              (:4-5)
      Jout_1 = 1/ce M1 .* (PS.' (mvp_N(Jtot) - mvp_G(Jtot)))    (:8-9)
      Jout_2 = 1/ce M2 .* (PS.' mvp_G(ext_Mc_inv .* Jb))        (:11-12)
      Jout_3 = [Z_cc Jc + Z_bc_N.' Jb; -Z_bc_N Jc]              (:14)"""
    dims = tuple(int(v) for v in pfft_dims)
    pwl = dims[3] == 12
    Jc, Jbv = Jcb[:N_sie], Jcb[N_sie:]
    Jb = (PS @ np.concatenate([np.zeros(N_sie, dtype=complex), Jbv])).reshape(dims, order="F")
    Jtot = (PS @ Jcb).reshape(dims, order="F")
    Gd = G_scale(pwl, res)[None, None, None, :]
    if isinstance(T, dict):
        NJ = mvp_op_tucker(Jtot, T, "N", False, cache)
    else:
        NJ = mvp_op_dense(Jtot, T, "N", False, cache)
    J1 = NJ - Gd * Jtot
    out1 = (1.0 / ce) * M1 * (PS.T @ J1.reshape(-1, order="F"))
    J2 = Gd * (np.asarray(ext_Mc_inv)[..., None] * Jb)
    out2 = (1.0 / ce) * M2 * (PS.T @ J2.reshape(-1, order="F"))
    out3 = np.concatenate([Z_cc @ Jc + Z_bc_N.T @ Jbv, -(Z_bc_N @ Jc)])
    return out1 + out2 + out3


# ---------------------------------------------------------------------------
# Incident fields tested onto the PWC/PWL basis
# ---------------------------------------------------------------------------


def voxel_centres(n1, n2, n3, res, origin=None):
    """Centres of a grid centred on the origin unless ``origin`` (the centre
    of voxel (0,0,0)) is given; shape (n1, n2, n3, 3)."""
    if origin is None:
        origin = -0.5 * res * (np.array([n1, n2, n3]) - 1)
    ax = [origin[d] + res * np.arange(n) for d, n in enumerate((n1, n2, n3))]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    return np.stack([X, Y, Z], axis=-1)


def loop_points(centre, normal, radius, nseg):
    """Mid-points and tangent*length vectors of a regular nseg-gon inscribed
    in a circle (closed loop, uniform unit current)."""
    normal = np.asarray(normal, float) / np.linalg.norm(normal)
    a = np.array([1.0, 0, 0]) if abs(normal[0]) < 0.9 else np.array([0, 1.0, 0])
    e1 = np.cross(normal, a); e1 /= np.linalg.norm(e1)
    e2 = np.cross(normal, e1)
    t = 2 * np.pi * np.arange(nseg + 1) / nseg
    P = centre[None, :] + radius * (np.cos(t)[:, None] * e1 + np.sin(t)[:, None] * e2)
    mid = 0.5 * (P[1:] + P[:-1])
    dl = P[1:] - P[:-1]
    return mid, dl


def incident_moments(centres_body, res, pwl, field_fn, nq=3):
    """Projection coefficients coef_l = int E.f_l / int f_l^2 on each body
    voxel with an nq^3 Gauss rule; f_l in {1, (x-xc)/dx, (y-yc)/dx,
    (z-zc)/dx} (VV_Nop.m:31-32, mvp_G_pwl.m:5).  Returns Ue (N_b,)
    component-major: index (4*p + l)*Ns + s for PWL, p*Ns + s for PWC."""
    w, x = gauss_1d(nq)
    Ns = centres_body.shape[0]
    L = 4 if pwl else 1
    acc = np.zeros((3, L, Ns), dtype=complex)
    for i in range(nq):
        for j in range(nq):
            for k in range(nq):
                wt = w[i] * w[j] * w[k] / 8.0           # cell-normalised weight
                off = np.array([x[i], x[j], x[k]]) * res / 2
                E = field_fn(centres_body + off[None, :])   # (Ns, 3)
                fl = [1.0, x[i] / 2, x[j] / 2, x[k] / 2]
                for l in range(L):
                    acc[:, l, :] += wt * fl[l] * E.T
    norm = np.array([1.0, 1 / 12, 1 / 12, 1 / 12])[:L]
    acc = acc / norm[None, :, None]
    return acc.reshape(3 * L * Ns)


def loop_field(points, mid, dl, k0, omega, mu0, current=1.0):
    """E of a closed thin-wire loop with uniform current (the scalar-potential
    term vanishes): E = -i*omega*mu0*I * sum_seg g(R) dl,
    g = exp(-i k0 R) / (4 pi R) (e^{+jwt}, G_N.m:4)."""
    E = np.zeros((points.shape[0], 3), dtype=complex)
    for s in range(mid.shape[0]):
        R = np.linalg.norm(points - mid[s][None, :], axis=1)
        g = np.exp(-1j * k0 * R) / (4 * np.pi * R)
        E += g[:, None] * dl[s][None, :]
    return -1j * omega * mu0 * current * E


def wire_sources(r_p, r_n, r_2, q_wire=4):
    """Quadrature points of the wire triangle bases as
    Assemble_tri_coupling_matrix_*.cpp (get_source_coords_mat, its :214-238)
    places them: for basis i, the positive half runs r_p -> r_2 and the
    negative half r_2 -> r_n; on each half, Gauss point s = L/2 (x + 1) from
    the half's start carries the current (s/L) * (unit tangent), i.e. both
    halves ramp up from their start point.  Returns (points (N_tri, 2, q, 3),
    current vectors (N_tri, 2, q, 3), weights w_i * L/2 (N_tri, 2, q))."""
    w, x = gauss_1d(q_wire)
    r_p, r_n, r_2 = (np.asarray(a, float).reshape(-1, 3) for a in (r_p, r_n, r_2))
    pts, cur, wts = [], [], []
    for a, b in ((r_p, r_2), (r_2, r_n)):
        d = b - a
        L = np.linalg.norm(d, axis=1)
        frac = 0.5 * (x + 1.0)                                   # s / L
        pts.append(a[:, None, :] + frac[None, :, None] * d[:, None, :])
        cur.append(frac[None, :, None] * (d / L[:, None])[:, None, :])
        wts.append(w[None, :] * (L / 2.0)[:, None])
    return np.stack(pts, 1), np.stack(cur, 1), np.stack(wts, 1)


def wire_coupling(kind, centres, r_p, r_n, r_2, res, k0, pwl, q_wire=4, q_vox=2):
    """Restates Assemble_tri_coupling_matrix_{N,K}_{x,x1,x2,x3,y,...,z3}.cpp
    (src/src_integral_equations/src_wvie/Cpp_Assembly/src, :21-205) times
    res^3 as wvie_mrgf_assembly.m:26-49 applies it: the voxel integral of
    each field component (and, PWL, of its products with the moments
    f = x/2, y/2, z/2 of the voxel's local coordinates in [-1, 1]) of the
    current of each wire basis; kind "N": the electric field by the full
    dyadic kernel, scaled by -1/(4 pi ce), ce = i k0 c0 e0; kind "K": the
    magnetic field G (R x t), G = e^{-i k0 R} (1 + i k0 R) / R^3 * (-1/4pi).
    Gauss rules q_vox^3 per voxel, q_wire per half (Quad_order_vie = 2,
    Quad_order_wie_coup = 4, load_inputs.m:81-83).  Returns (ql, N_vox,
    N_tri) in the reference's component order (x, x1, x2, x3, y, ... for
    PWL)."""
    wv, xv = gauss_1d(q_vox)
    spts, scur, swts = wire_sources(r_p, r_n, r_2, q_wire)
    ntri = spts.shape[0]
    c = np.asarray(centres, float).reshape(-1, 3)
    nv = c.shape[0]
    L = 4 if pwl else 1
    mu0, c0 = 4e-7 * math.pi, 299792458.0
    e0 = 1.0 / (c0 * c0 * mu0)
    ce = 1j * k0 * c0 * e0
    out = np.zeros((3, L, nv, ntri), dtype=complex)
    S = spts.reshape(ntri, -1, 3)
    Tc = scur.reshape(ntri, -1, 3)
    W = swts.reshape(ntri, -1)
    for a in range(q_vox):
        for b in range(q_vox):
            for cc in range(q_vox):
                loc = np.array([xv[a], xv[b], xv[cc]])
                wt = wv[a] * wv[b] * wv[cc] / 8.0
                obs = c + 0.5 * res * loc[None, :]
                R = obs[:, None, None, :] - S[None, :, :, :]          # (nv, ntri, nsrc, 3)
                Rd = np.linalg.norm(R, axis=-1)
                kR = k0 * Rd
                kappa = np.exp(-1j * kR) / Rd ** 3
                if kind == "N":
                    P = (kR ** 2 - 3j * kR - 3.0) / Rd ** 2
                    Q = (kR ** 2 - 1j * kR - 1.0) / P
                    Rt = np.sum(R * Tc[None], axis=-1)
                    F = (kappa * P)[..., None] * (R * Rt[..., None] - Q[..., None] * Tc[None])
                    F = F * (-1.0 / ce / (4 * math.pi))
                else:
                    G = kappa * (1j * kR + 1.0) * (-1.0 / (4 * math.pi))
                    F = G[..., None] * np.cross(R, np.broadcast_to(Tc[None], R.shape))
                fld = np.sum(F * W[None, :, :, None], axis=2)          # (nv, ntri, 3)
                fl = [1.0, 0.5 * loc[0], 0.5 * loc[1], 0.5 * loc[2]]
                for p in range(3):
                    for l in range(L):
                        out[p, l] += wt * fl[l] * fld[:, :, p]
    return out.reshape(3 * L, nv, ntri) * res ** 3


def wire_incident(kind, centres, r_p, r_n, r_2, coef, res, k0, pwl, q_wire=4, q_vox=2):
    """Incident field coefficients on the body of wire currents ``coef``
    (N_tri,): invG(Zbw coef) (the tested field of em_efield_wvie.m:43-47 /
    em_hfield_wvie.m:38, restricted to the body), component-major (N_b,)."""
    Z = wire_coupling(kind, centres, r_p, r_n, r_2, res, k0, pwl, q_wire, q_vox)
    t = Z @ np.asarray(coef, dtype=complex)
    g = invG_scale(pwl, res)
    return (t * g[:, None]).reshape(-1)


def plane_wave_field(points, k0):
    """E = x_hat * exp(-i k0 z): unit x-polarised plane wave along +z."""
    E = np.zeros((points.shape[0], 3), dtype=complex)
    E[:, 0] = np.exp(-1j * k0 * points[:, 2])
    return E
