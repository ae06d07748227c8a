"""Tucker compression of a dense Green's tensor I_V into the reference's
operator format (the input of marie_vie_create's tucker_N / tucker_K).

The reference stores each block I_V(:,:,:,j,k) as a truncated HOSVD
(hosvd.m:1-36: factors from the SVD of each mode unfolding, rank cut where
the singular values fall below tol * s_1 / sqrt(3), core = I_V x1 U1^H x2
U2^H x3 U3^H) whose factors are circulant-extended with the block's mirror
sign and transformed (assembly_fft_circ_tucker_pwl.m:31-58): the format
returned here, {(j, k): (G, U1, U2, U3)} with U* of shape (r, 2n).  numpy
(LAPACK) on the host; an operator set-up step, not part of the hot path.
"""
from __future__ import annotations

import numpy as np

# mirror signs of the circulant extension: per N (6) or K (3) component and
# per PWL moment pair (assembly_fft_circ_tucker_pwl.m:36-47)
_G_SIGNS = {6: ((+1, -1, -1, +1, +1, +1), (+1, -1, +1, +1, -1, +1), (+1, +1, -1, +1, -1, +1)),
            3: ((-1, +1, +1), (+1, -1, +1), (+1, +1, -1))}
_BT_SIGNS = ((+1, +1, +1, +1, -1, +1, +1, -1, -1, +1),
             (+1, +1, +1, +1, +1, -1, +1, -1, +1, -1),
             (+1, +1, +1, +1, +1, +1, -1, +1, -1, -1))


def _rank(s, tol):
    cut = tol * s[0] / np.sqrt(3.0)
    small = np.nonzero((s <= cut) & (s != 0))[0]
    return int(small[0]) + 1 if small.size else s.size


def _factor(A, mode, tol):
    """Left singular vectors of the mode-`mode` unfolding, truncated."""
    M = np.moveaxis(A, mode, 0).reshape(A.shape[mode], -1)
    U, s, _ = np.linalg.svd(M, full_matrices=False)
    return U[:, : min(_rank(s, tol), U.shape[1])]


def _extend(U, sign):
    """FFT over the circulant extension [U; 0; sign * U(n-1:-1:1)], transposed (r x 2n)."""
    n = U.shape[0]
    ext = np.concatenate([U, np.zeros((1, U.shape[1]), U.dtype), sign * U[n - 1:0:-1]], axis=0)
    return np.ascontiguousarray(np.fft.fft(ext, axis=0).T)


def compress(IV: np.ndarray, tol: float = 1e-7) -> dict:
    """{(j, k): (G, U1, U2, U3)} of a dense I_V (n1, n2, n3, pwx, 6 | 3)."""
    IV = np.asarray(IV)
    if IV.ndim == 4:
        IV = IV[:, :, :, None, :]
    n1, n2, n3, pwx, nc = IV.shape
    gs = _G_SIGNS[nc]
    out = {}
    for j in range(pwx):
        bt = (_BT_SIGNS[0][j], _BT_SIGNS[1][j], _BT_SIGNS[2][j]) if pwx == 10 else (1, 1, 1)
        for k in range(nc):
            A = np.asarray(IV[:, :, :, j, k], dtype=np.complex128)
            U = [_factor(A, d, tol) for d in range(3)]
            G = np.einsum("abc,ai,bj,ck->ijk", A, U[0].conj(), U[1].conj(), U[2].conj(), optimize=True)
            out[(j, k)] = (G,) + tuple(_extend(U[d], gs[d][k] * bt[d]) for d in range(3))
    return out


def ranks(T: dict) -> np.ndarray:
    """(r1, r2, r3) of every block, in key order."""
    return np.array([T[key][0].shape for key in sorted(T)])
