"""Generate the small committed fixtures under tests/golden/ with the CPU oracle.

Fixtures:
  iv_pwc_5.npz : I_V for N and K, PWC, 5x5x5 grid, 5 mm, 128 MHz
  iv_pwl_4.npz : I_V for N and K, PWL, 4x4x4 grid, 2 mm, 297.2 MHz
  mvp_*.npz    : a seeded input and the oracle's mvp_N / mvp_vie / GMRES
                 outputs on those operators (regression vectors)

The reference ships no golden vectors for this path (its MATLAB code has no
tests), so these pin the oracle against itself across changes; the oracle is
pinned to the reference's algorithm by the identities in test_oracle.py.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT), str(ROOT / "tests")]

from oracle import marie_oracle as O  # noqa: E402

CASES = {
    "pwc_5": dict(n=(5, 5, 5), pwl=False, res=5e-3, freq=128e6),
    "pwl_4": dict(n=(4, 4, 4), pwl=True, res=2e-3, freq=297.2e6),
}


def body(n, seed):
    rng = np.random.default_rng(seed)
    mask = rng.uniform(size=n) < 0.7
    mask[0, 0, 0] = True
    idxS = np.nonzero(mask.reshape(-1, order="F"))[0].astype(np.int64)
    er = np.where(mask, rng.uniform(5, 80, size=n), 1.0)
    se = np.where(mask, rng.uniform(0.02, 2.0, size=n), 0.0)
    return idxS, er, se


def make(name, n, pwl, res, freq):
    emc = O.em_constants(freq)
    ivN = O.assembly_op(*n, res, emc["k0"], pwl, "N")
    ivK = O.assembly_op(*n, res, emc["k0"], pwl, "K")
    np.savez_compressed(HERE / f"iv_{name}.npz", N=ivN, K=ivK, n=np.array(n), res=res, freq=freq,
                        pwl=pwl)
    idxS, er, se = body(n, 11)
    ep = O.em_assembly(er, se, emc["ce"])
    dims = O.geo_dims(*n, idxS, pwl, res)
    TN = O.assembly_fft_circ_tucker(ivN if pwl else ivN[:, :, :, 0, :], 1e-7)
    rng = np.random.default_rng(12)
    C = 12 if pwl else 3
    J = rng.normal(size=n + (C,)) + 1j * rng.normal(size=n + (C,))
    NJ = O.mvp_op_tucker(J, TN, "N")
    Jb = rng.normal(size=dims["N_b"]) + 1j * rng.normal(size=dims["N_b"])
    AJ = O.mvp_vie(Jb, ep["Mr"], ep["Mc"], dims, TN)
    b = O.vie_rhs(emc["ce"], ep["Mr"], ep["Mc"], idxS, dims["ql"], Jb)
    cache = {}
    x, it, rv = O.is_gmres_vie(lambda v: O.mvp_vie(v, ep["Mr"], ep["Mc"], dims, TN, cache), b, 50, 1e-8, 200,
                               np.zeros(dims["N_b"]))
    np.savez_compressed(HERE / f"mvp_{name}.npz", idxS=idxS, er=er, se=se, J=J, NJ=NJ, Jb=Jb, AJ=AJ, b=b, x=x,
                        it=it, resvec=rv, tucker_tol=1e-7)


if __name__ == "__main__":
    for name, kw in CASES.items():
        make(name, **kw)
        print("wrote", name)
