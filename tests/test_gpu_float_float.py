"""The complex128 operator in float-float arithmetic (precisions bit 4).

Same inputs and outputs as the native complex128 operator; the FFTs and the
Green multiply run on pairs of FP32 numbers.  Tolerance against the oracle
and against the native FP64 kernels: 1e-11 relative (2-norm over the whole
output), a hundred times the native path's 1e-12 and six orders of magnitude
below the 1e-6 solver tolerance the residual serves.  GMRES with the float-
float operator must take the native FP64 iteration counts.
"""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, flat_F, unflat_F, rel_err

torch = pytest.importorskip("torch")

TOL_FF = 1e-11
SIZES = [(16, 16, 16), (32, 16, 48), (48, 32, 16)]


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("n", SIZES, ids=lambda n: "x".join(map(str, n)))
def test_float_float_matches_oracle_and_native(n, pwl):
    P = Problem(n, pwl, seed=sum(n) + 7 * pwl)
    opF = P.gpu_operator(precisions=4 | 2, max_rhs=4)
    opN = P.gpu_operator(precisions=1, max_rhs=4)
    assert opF.tiles(0)["float_float"] and not opN.tiles(0)["float_float"]
    J = P.random_grid(seed=8, nrhs=3)
    x = torch.from_numpy(np.concatenate([flat_F(J[r]) for r in range(3)])).to("cuda", torch.complex128)
    for name, adj, fF, fN in (("N", False, opF.apply_N, opN.apply_N), ("N", True, opF.apply_N_adj, opN.apply_N_adj)):
        y = fF(x).cpu().numpy()
        yn = fN(x).cpu().numpy()
        assert rel_err(y, yn) <= TOL_FF
        for r in range(3):
            ref = O.mvp_op_tucker(J[r], P.TN, name, adj, cache={})
            sl = slice(r * J[r].size, (r + 1) * J[r].size)
            assert rel_err(unflat_F(y[sl], n, P.C), ref) <= TOL_FF
    X = P.random_body_vec(seed=6, nrhs=5)
    xb = torch.from_numpy(X.reshape(-1)).to("cuda", torch.complex128)
    yb = opF.apply(xb).cpu().numpy().reshape(5, -1)
    ya = opF.apply_adjoint(xb).cpu().numpy().reshape(5, -1)
    yan = opN.apply_adjoint(xb).cpu().numpy().reshape(5, -1)
    for r in range(5):
        assert rel_err(yb[r], O.mvp_vie(X[r], P.Mr, P.Mc, P.dims, P.TN, cache={})) <= TOL_FF
        assert rel_err(ya[r], yan[r]) <= TOL_FF
    # the complex64 state of the same handle is unaffected
    y64 = opF.apply(xb.to(torch.complex64)).cpu().numpy().reshape(5, -1).astype(np.complex128)
    assert rel_err(y64[0], yb[0]) <= 1e-5
    opF.close()
    opN.close()


def _sphere_case(n, pwl, precisions):
    from marie_gb300 import VieOperator, assemble_green, phantoms
    res, freq = 5e-3, 128e6
    body = phantoms.sphere(n, res, 0.03, 50.0, 0.6)
    iv = assemble_green(body.n, res, freq, pwl, "N")
    op = VieOperator(body.n, res, freq, body.idx_solution(pwl), body.Mr(freq), iv, pwl=pwl, precisions=precisions,
                     max_rhs=4)
    U = op.incident_plane_wave(body.origin).reshape(-1)
    emc = O.em_constants(freq)
    Mr = body.Mr(freq).reshape(-1, order="F")[body.idxS]
    chi = np.tile((1.0 / Mr) * (Mr - 1.0), 12 if pwl else 3)
    b = emc["ce"] * torch.from_numpy(chi).cuda() * U
    return op, b


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_gmres_with_float_float_operator(pwl):
    """FP64 GMRES and the mixed solver's true residual on the float-float
    operator: native iteration counts, solutions within 1e-9."""
    opN, b = _sphere_case(16, pwl, 1 | 2)
    opF, _ = _sphere_case(16, pwl, 4 | 2)
    xN, rN = opN.gmres(b, restart=30, tol=1e-8, mode="fp64")
    xF, rF = opF.gmres(b, restart=30, tol=1e-8, mode="fp64")
    assert rN.ok and rF.ok
    assert int(rF.iters[0]) == int(rN.iters[0])
    assert rel_err(xF.cpu().numpy(), xN.cpu().numpy()) <= 1e-9
    assert abs(rF.true_resid[0] - rN.true_resid[0]) <= 1e-10
    xNm, rNm = opN.gmres(b, restart=30, tol=1e-6, mode="mixed")
    xFm, rFm = opF.gmres(b, restart=30, tol=1e-6, mode="mixed")
    assert rFm.ok and rFm.true_resid[0] <= 1e-6
    assert int(rFm.iters[0]) == int(rNm.iters[0]) and rFm.matvecs_c128 == rNm.matvecs_c128
    assert abs(rFm.true_resid[0] - rNm.true_resid[0]) <= 1e-10
    opN.close()
    opF.close()
