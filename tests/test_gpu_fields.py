"""Field post-processing on the GPU against the oracle's restatement of
em_efield_vie_excitation.m, em_hfield_vie_excitation.m and em_ehfield_vie.m
(through the C ABI).  Tolerances as for the operator: complex128 1e-12,
complex64 1e-5, float-float complex128 1e-11 (relative 2-norm)."""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, rel_err

torch = pytest.importorskip("torch")

TOL = {"c128": 1e-12, "c64": 1e-5}


def _currents(P, seed, nport):
    rng = np.random.default_rng(seed)
    Nb = P.dims["N_b"]
    J = rng.normal(size=(Nb, nport)) + 1j * rng.normal(size=(Nb, nport))
    U = rng.normal(size=(Nb, nport)) + 1j * rng.normal(size=(Nb, nport))
    B = rng.normal(size=(Nb, nport)) + 1j * rng.normal(size=(Nb, nport))
    return J, U, B


def _dev(A, dt):
    return torch.from_numpy(np.ascontiguousarray(A.T).reshape(-1)).to("cuda", dt)


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("n", [(6, 5, 4), (16, 16, 16)], ids=["6x5x4", "16x16x16"])
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_fields_match_oracle(n, pwl, prec):
    P = Problem(n, pwl, seed=sum(n) + 3 * pwl)
    op = P.gpu_operator(precisions=3, max_rhs=4)
    J, U, B = _currents(P, 5, 3)
    dt = torch.complex128 if prec == "c128" else torch.complex64
    E, H = op.fields(_dev(J, dt), Ue=_dev(U, dt), Ub=_dev(B, dt))
    E = E.cpu().numpy().reshape(3, -1).astype(np.complex128)
    H = H.cpu().numpy().reshape(3, -1).astype(np.complex128)
    ce = P.emc["ce"]
    for r in range(3):
        Er = O.em_efield_vie_excitation(J[:, r], U[:, r], P.dims, P.TN, ce, cache={})
        Hr = O.em_hfield_vie_excitation(J[:, r], B[:, r], P.dims, P.TK, cache={})
        assert rel_err(E[r], Er) <= TOL[prec]
        assert rel_err(H[r], Hr) <= TOL[prec]
    # E alone, without an incident term
    E0, H0 = op.fields(_dev(J, dt), h=False)
    assert H0 is None
    E0 = E0.cpu().numpy().reshape(3, -1).astype(np.complex128)
    assert rel_err(E0[1], O.em_efield_vie_excitation(J[:, 1], 0 * U[:, 1], P.dims, P.TN, ce, cache={})) <= TOL[prec]
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_efield_float_float(pwl):
    P = Problem((32, 16, 16), pwl, seed=11 + pwl)
    op = P.gpu_operator(precisions=4 | 2, max_rhs=4)
    J, U, _ = _currents(P, 7, 2)
    E, _h = op.fields(_dev(J, torch.complex128), Ue=_dev(U, torch.complex128), h=False)
    E = E.cpu().numpy().reshape(2, -1)
    for r in range(2):
        assert rel_err(E[r], O.em_efield_vie_excitation(J[:, r], U[:, r], P.dims, P.TN, P.emc["ce"], cache={})) <= 1e-11
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_absorbed_power_and_b1(pwl):
    P = Problem((8, 8, 8), pwl, seed=21 + pwl)
    op = P.gpu_operator(precisions=1, max_rhs=8)
    J, _, B = _currents(P, 9, 7)
    phi = op.absorbed_power(_dev(J, torch.complex128))
    ref = O.em_noise_covariance(J, P.Mc, P.emc["ce"], P.dims)
    assert rel_err(phi, ref) <= 1e-12
    assert np.allclose(phi, phi.conj().T, rtol=1e-12, atol=0)     # Hermitian
    b1 = op.b1_plus(_dev(B, torch.complex128)).cpu().numpy().reshape(7, -1)
    for r in range(7):
        assert rel_err(b1[r], O.b1_plus(B[:, r], P.dims, P.emc["mu0"])) <= 1e-15
    op.close()
