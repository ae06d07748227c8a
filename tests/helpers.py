"""Seeded small problems for the parity tests (built with the CPU oracle)."""
from __future__ import annotations

import numpy as np

from oracle import marie_oracle as O


def random_body(n, seed, density=0.6, box=None):
    """Random voxel body; box = ((x0, x1), (y0, y1), (z0, z1)) keeps it inside
    that sub-box (grid rows and slices outside it hold no body voxel)."""
    rng = np.random.default_rng(seed)
    n1, n2, n3 = n
    mask = rng.uniform(size=(n1, n2, n3)) < density
    if box is None:
        mask[0, 0, 0] = True
    else:
        keep = np.zeros_like(mask)
        keep[box[0][0]:box[0][1], box[1][0]:box[1][1], box[2][0]:box[2][1]] = True
        mask &= keep
        mask[box[0][0], box[1][0], box[2][0]] = True
    idxS = np.nonzero(mask.reshape(-1, order="F"))[0].astype(np.int64)
    er = np.where(mask, rng.uniform(5, 80, size=(n1, n2, n3)), 1.0)
    se = np.where(mask, rng.uniform(0.02, 2.0, size=(n1, n2, n3)), 0.0)
    return idxS, er, se


def synthetic_IV(n, pwl, kernel, seed):
    """Random dense I_V with a decaying magnitude: any block content exercises
    the operator algebra identically; physics is not needed for parity."""
    rng = np.random.default_rng(seed)
    n1, n2, n3 = n
    pwx = 10 if pwl else 1
    nc = 6 if kernel == "N" else 3
    x, y, z = np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3), indexing="ij")
    decay = 1.0 / (1.0 + x ** 2 + y ** 2 + z ** 2)
    A = rng.normal(size=(n1, n2, n3, pwx, nc)) + 1j * rng.normal(size=(n1, n2, n3, pwx, nc))
    A = A * decay[..., None, None]
    # circulant parity of the physical kernel: a block that is odd along an
    # axis vanishes on that axis' zero-offset plane
    g1, g2, g3 = O.G_N_SIGNS[nc]
    for j in range(pwx):
        for k in range(nc):
            b = (O.BT_SIGNS[0][j], O.BT_SIGNS[1][j], O.BT_SIGNS[2][j]) if pwl else (1, 1, 1)
            if g1[k] * b[0] < 0:
                A[0, :, :, j, k] = 0
            if g2[k] * b[1] < 0:
                A[:, 0, :, j, k] = 0
            if g3[k] * b[2] < 0:
                A[:, :, 0, j, k] = 0
    return A


class Problem:
    """Operator data of one small case, in the reference's formats."""

    def __init__(self, n, pwl, seed=0, res=5e-3, freq=128e6, tucker_tol=1e-14, physical=False, iv_scale=1.0,
                 box=None):
        self.n = tuple(n)
        self.pwl = pwl
        self.res, self.freq = res, freq
        self.idxS, self.er, self.se = random_body(n, seed, box=box)
        self.emc = O.em_constants(freq)
        ep = O.em_assembly(self.er, self.se, self.emc["ce"])
        self.Mr, self.Mc = ep["Mr"], ep["Mc"]
        self.dims = O.geo_dims(*n, self.idxS, pwl, res)
        if physical:
            self.IV_N = O.assembly_op(*n, res, self.emc["k0"], pwl, "N")
            self.IV_K = O.assembly_op(*n, res, self.emc["k0"], pwl, "K")
        else:
            # iv_scale < 1 keeps A = I - chi invG N well conditioned for solver tests
            self.IV_N = synthetic_IV(n, pwl, "N", seed + 100) * iv_scale
            self.IV_K = synthetic_IV(n, pwl, "K", seed + 200) * iv_scale
        self.TN = O.assembly_fft_circ_tucker(self.IV_N if pwl else self.IV_N[:, :, :, 0, :], tucker_tol)
        self.TK = O.assembly_fft_circ_tucker(self.IV_K if pwl else self.IV_K[:, :, :, 0, :], tucker_tol)
        self.C = 12 if pwl else 3

    def gpu_operator(self, precisions=3, max_rhs=4, dense=False, mem_cap_bytes=0):
        from marie_gb300 import VieOperator
        N = self.IV_N if dense else self.TN
        K = self.IV_K if dense else self.TK
        return VieOperator(self.n, self.res, self.freq, self.dims["idx_solution"], self.Mr, N, K,
                           pwl=self.pwl, precisions=precisions, max_rhs=max_rhs, mem_cap_bytes=mem_cap_bytes)

    def random_grid(self, seed, nrhs=1):
        rng = np.random.default_rng(seed)
        shape = (nrhs,) + self.n + (self.C,)
        return rng.normal(size=shape) + 1j * rng.normal(size=shape)

    def random_body_vec(self, seed, nrhs=1):
        rng = np.random.default_rng(seed)
        Nb = self.dims["N_b"]
        return rng.normal(size=(nrhs, Nb)) + 1j * rng.normal(size=(nrhs, Nb))


def flat_F(a):
    """(n1,n2,n3,C) -> column-major flat vector (the C-ABI grid layout)."""
    return np.asarray(a).reshape(-1, order="F")


def unflat_F(v, n, C):
    return np.asarray(v).reshape(tuple(n) + (C,), order="F")


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))
