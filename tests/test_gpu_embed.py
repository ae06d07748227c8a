"""Grids embedded in a larger FFT grid on the GPU (through the C ABI).

A grid edge with a prime factor above 31 (the reference's inhomogeneous-
cylinder body is 73 x 73 x 84) is not an FFT length of the passes, so
marie_vie_create embeds the grid in one they cover, with the caller's Green's
tensor zero-padded (marie-tools_gb300/csrc/embed.h); with MARIE_EMBED=1 it
does the same for smooth grids with edges <= 128 (four-step passes).  The
results on the caller's body must equal the oracle's on the caller's grid:
complex128 <= 1e-12, complex64 <= 1e-5, float-float <= 1e-11 relative;
GMRES with the iteration counts and tolerances of test_gpu_gmres.py.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, rel_err, synthetic_IV, random_body

torch = pytest.importorskip("torch")
GOLD = Path(__file__).resolve().parent / "golden"
TOL = {"c128": 1e-12, "c64": 1e-5}


def _vie_parity(op, P, precs, nrhs=2):
    X = P.random_body_vec(seed=9, nrhs=nrhs)
    for prec in precs:
        dt = torch.complex128 if prec == "c128" else torch.complex64
        x = torch.from_numpy(X.reshape(-1)).to("cuda", dt)
        y = op.apply(x).cpu().numpy().reshape(nrhs, -1).astype(np.complex128)
        ya = op.apply_adjoint(x).cpu().numpy().reshape(nrhs, -1).astype(np.complex128)
        for r in range(nrhs):
            ref = O.mvp_vie(X[r], P.Mr, P.Mc, P.dims, P.TN, cache={})
            refa = O.mvp_vie_adjoint(X[r], P.Mr, P.Mc, P.dims, P.TN, cache={})
            assert rel_err(y[r], ref) <= TOL[prec], (prec, r)
            assert rel_err(ya[r], refa) <= TOL[prec], (prec, r)


@pytest.mark.gpu
@pytest.mark.parametrize("n,pwl,dense", [((37, 10, 9), False, False), ((37, 10, 9), False, True),
                                         ((5, 37, 6), True, False), ((6, 5, 41), True, True)],
                         ids=["pwc-37x10x9-tucker", "pwc-37x10x9-dense", "pwl-5x37x6-tucker", "pwl-6x5x41-dense"])
def test_prime_edge_grid_matches_oracle(n, pwl, dense):
    from marie_gb300._lib import MarieError
    P = Problem(n, pwl, seed=sum(n))
    op = P.gpu_operator(precisions=3, max_rhs=2, dense=dense)
    _vie_parity(op, P, ("c128", "c64"))
    # full-grid operators would see the embedded grid: refused
    with pytest.raises(MarieError, match="embedded"):
        op.apply_N(torch.zeros(P.C * int(np.prod(n)), dtype=torch.complex128, device="cuda"))
    op.close()


@pytest.mark.gpu
def test_prime_edge_grid_float_float():
    """Float-float complex128 needs four-step edges: available once the
    37 x 10 x 9 grid is embedded in 48 x 16 x 16."""
    n = (37, 10, 9)
    P = Problem(n, False, seed=5)
    op = P.gpu_operator(precisions=2 | 4, max_rhs=1)
    X = P.random_body_vec(seed=2)[0]
    y = op.apply(torch.from_numpy(X).cuda()).cpu().numpy()
    assert rel_err(y, O.mvp_vie(X, P.Mr, P.Mc, P.dims, P.TN, cache={})) <= 1e-11
    op.close()


@pytest.mark.gpu
def test_cylinder_body_grid_73x73x84():
    """The grid of the reference's inhomogeneous-cylinder body (73 x 73 x 84,
    2 mm), PWC, dense I_V: embedded in 80 x 80 x 96 (four-step passes)."""
    from marie_gb300 import VieOperator
    n, res, freq = (73, 73, 84), 2e-3, 128e6
    idxS, er, se = random_body(n, seed=73, density=0.4)
    IV = synthetic_IV(n, False, "N", seed=74)
    emc = O.em_constants(freq)
    ep = O.em_assembly(er, se, emc["ce"])
    dims = O.geo_dims(*n, idxS, False, res)
    T = O.assembly_fft_circ_tucker(IV[:, :, :, 0, :], 0.0)
    op = VieOperator(n, res, freq, dims["idx_solution"], ep["Mr"], IV, pwl=False, precisions=3, max_rhs=1)
    X = np.random.default_rng(3).normal(size=(dims["N_b"], 2)) @ np.array([1.0, 1j])
    ref = O.mvp_vie(X, ep["Mr"], ep["Mc"], dims, T, cache={})
    for prec, dt in (("c128", torch.complex128), ("c64", torch.complex64)):
        y = op.apply(torch.from_numpy(X).to("cuda", dt)).cpu().numpy().astype(np.complex128)
        assert rel_err(y, ref) <= TOL[prec], prec
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pwc_5", "pwl_4"])
def test_forced_embedding_gmres_matches_oracle(name, monkeypatch):
    """MARIE_EMBED=1 puts the golden 5^3 / 4^3 cases on 16^3 four-step
    grids; the complex128 GMRES still follows the oracle's is_gmres_vie on
    the caller's grid step for step."""
    from marie_gb300 import VieOperator
    monkeypatch.setenv("MARIE_EMBED", "1")
    iv = np.load(GOLD / f"iv_{name}.npz")
    mv = np.load(GOLD / f"mvp_{name}.npz")
    n = tuple(int(v) for v in iv["n"])
    pwl = bool(iv["pwl"])
    emc = O.em_constants(float(iv["freq"]))
    ep = O.em_assembly(mv["er"], mv["se"], emc["ce"])
    dims = O.geo_dims(*n, mv["idxS"], pwl, float(iv["res"]))
    T = O.assembly_fft_circ_tucker(iv["N"] if pwl else iv["N"][:, :, :, 0, :], float(mv["tucker_tol"]))
    op = VieOperator(n, float(iv["res"]), float(iv["freq"]), dims["idx_solution"], ep["Mr"], T, pwl=pwl,
                     precisions=3, max_rhs=1)
    cache = {}
    A = lambda v: O.mvp_vie(v, ep["Mr"], ep["Mc"], dims, T, cache)
    b = mv["b"]
    tol = 1e-8
    xr, itr, rvr = O.is_gmres_vie(A, b, 50, tol, 200, np.zeros(b.size))
    x, rep = op.gmres(torch.from_numpy(b).cuda(), restart=50, tol=tol, maxit=200, mode="fp64")
    assert rep.ok
    assert int(rep.outer[0]) == int(itr[1]) and int(rep.last_inner[0]) == int(itr[0])
    assert np.allclose(rep.resvec[0], rvr, rtol=1e-7, atol=1e-14)
    assert rel_err(x.cpu().numpy(), xr) < 1e-9
    op.close()
