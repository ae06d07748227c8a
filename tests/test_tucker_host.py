"""Host Tucker compression of the product (marie_gb300.tucker.compress, the
reference's hosvd.m + assembly_fft_circ_tucker_pwl.m format) against the
oracle's restatement: the same ranks and the same expanded circulant spectra
(factors may differ by unit phases, which the product cancels)."""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import synthetic_IV


@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("tol", [1e-7, 1e-3])
def test_compress_matches_oracle(pwl, tol):
    from marie_gb300 import tucker
    n = (6, 5, 4)
    IV = synthetic_IV(n, pwl, "N", 3)
    Tp = tucker.compress(IV, tol)
    To = O.assembly_fft_circ_tucker(IV if pwl else IV[:, :, :, 0, :], tol)
    assert sorted(Tp) == sorted(To)
    for key in To:
        assert Tp[key][0].shape == To[key][0].shape, key
        a, b = O.tucker_block(Tp[key]), O.tucker_block(To[key])
        assert np.abs(a - b).max() <= 1e-12 * max(np.abs(b).max(), 1e-300), key
    for (j, k), t in Tp.items():
        assert all(u.shape[1] == 2 * n[d] for d, u in enumerate(t[1:]))


def test_compress_physical_operator_ranks():
    """The physical N operator of a 12^3 grid at 2 mm / 297.2 MHz compresses at
    the reference's tolerance 1e-7 (ranks 10-11 of 12 on so small a grid) and
    expands back to the dense operator's spectrum within it."""
    from marie_gb300 import tucker
    n, res, freq = (12, 12, 12), 2e-3, 297.2e6
    IV = O.assembly_op(*n, res, O.em_constants(freq)["k0"], True, "N", Np_medium=4)
    T = tucker.compress(IV, 1e-7)
    r = tucker.ranks(T)
    assert r.max() <= 12 and r.mean() < 11
    for key in [(0, 0), (4, 3), (9, 5)]:
        full = O.tucker_block(T[key])
        ref = O.block_spectrum_dense(IV, key, "N")
        assert np.abs(full - ref).max() <= 1e-5 * np.abs(ref).max(), key
