"""The Python mirror of the reference's VIE call surface (marie_gb300.vie)
against the oracle, through the C ABI.

The mirror keeps the reference's names and argument meaning:
parse_inputs.m:6-37 (the function-handle table), mvp_vie.m:1-19,
is_gmres_vie.m:1-30 (x, iter = [p outit], relative resvec), and
ie_solver_vie.m:1-32 (port right-hand sides, N_b x N_ports layout, and the
Zbb_hat_inv SVD when the excitation basis carries X).
"""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, rel_err

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def case():
    P = Problem((8, 7, 6), True, seed=41, iv_scale=0.3)
    op = P.gpu_operator(precisions=3, max_rhs=4)
    yield P, op
    op.close()


@pytest.mark.gpu
def test_function_handle_table(case):
    from marie_gb300 import vie
    P, op = case
    func = vie.parse_inputs(1)
    assert set(func) >= {"mvp_N", "mvp_K", "mvp_herm_adj_N", "mvp_herm_adj_K", "mvp_G", "mvp_invG",
                         "ie_solver_wsvie"}
    J = P.random_grid(seed=2)[0]            # (n1, n2, n3, 12), MATLAB order
    for name, T, opn, adj in [("mvp_N", P.TN, "N", False), ("mvp_herm_adj_N", P.TN, "N", True),
                              ("mvp_K", P.TK, "K", False), ("mvp_herm_adj_K", P.TK, "K", True)]:
        got = func[name](J, op)                       # numpy in, numpy out
        assert got.shape == J.shape
        assert rel_err(got, O.mvp_op_tucker(J, T, opn, adj, cache={})) <= 1e-12, name
        gt = func[name](torch.from_numpy(J).cuda(), op)     # gpuArray in, gpuArray out
        assert isinstance(gt, torch.Tensor) and gt.is_cuda
        assert rel_err(gt.cpu().numpy(), got) <= 1e-14
    Gs = O.G_scale(True, P.res)
    np.testing.assert_allclose(func["mvp_G"](J, P.res), J * Gs.reshape(1, 1, 1, -1), rtol=1e-15)
    np.testing.assert_allclose(func["mvp_invG"](J, P.res), J / Gs.reshape(1, 1, 1, -1), rtol=1e-15)


@pytest.mark.gpu
def test_mvp_vie_mirror(case):
    from marie_gb300 import vie
    P, op = case
    func = vie.parse_inputs(1)
    Jb = P.random_body_vec(seed=3)[0]
    ref = O.mvp_vie(Jb, P.Mr, P.Mc, P.dims, P.TN, cache={})
    got = vie.mvp_vie(Jb, None, func, P.dims, op)
    assert isinstance(got, np.ndarray) and rel_err(got, ref) <= 1e-12
    with pytest.raises(ValueError):
        vie.mvp_vie(Jb, None, func, {"N_b": P.dims["N_b"] + 1}, op)


@pytest.mark.gpu
def test_is_gmres_vie_mirror_batch_and_warm_start(case):
    from marie_gb300 import vie
    P, op = case
    B = P.random_body_vec(seed=4, nrhs=2).T                  # N_b x 2, columns = right-hand sides
    A = lambda v: O.mvp_vie(v, P.Mr, P.Mc, P.dims, P.TN, cache={})
    x, it, rv = vie.is_gmres_vie(op, B, 10, 1e-9, 30, None)
    assert x.shape == B.shape
    for c in range(2):
        xo, ito, rvo = O.is_gmres_vie(A, B[:, c], 10, 1e-9, 30, np.zeros(B.shape[0], complex))
        assert list(it[c]) == list(ito), (it[c], ito)
        assert rel_err(x[:, c], xo) <= 1e-9
        assert len(rv[c]) == len(rvo)
        np.testing.assert_allclose(rv[c], rvo, rtol=1e-7, atol=1e-14)
    # one right-hand side with a nonzero x0 (is_gmres_vie.m:5-9: r0 = b - A x0)
    x0 = 0.5 * x[:, 0]
    x1, it1, rv1 = vie.is_gmres_vie(op, B[:, 0], 10, 1e-9, 30, x0)
    xo, ito, rvo = O.is_gmres_vie(A, B[:, 0], 10, 1e-9, 30, x0)
    assert list(it1) == list(ito)
    assert rel_err(x1, xo) <= 1e-9
    np.testing.assert_allclose(rv1, rvo, rtol=1e-7, atol=1e-14)


@pytest.mark.gpu
def test_ie_solver_vie_mirror_with_basis(case):
    """Ports batched through the C ABI against the oracle's serial port loop;
    the MRGF factors from the Zbb_hat_inv SVD of ie_solver_vie.m:23-25."""
    from marie_gb300 import vie
    P, op = case
    rng = np.random.default_rng(8)
    nports = 3
    Ue = rng.normal(size=(P.dims["N_b"], nports)) + 1j * rng.normal(size=(P.dims["N_b"], nports))
    X = rng.normal(size=(nports, 2)) + 1j * rng.normal(size=(nports, 2))
    ce = P.emc["ce"]
    Jb, U, S, V = vie.ie_solver_vie(op, Ue, ce, P.Mr, P.Mc, P.idxS, 1e-10, X=X)
    Jo, out, (Uo, So, Vo) = O.ie_solver_vie(P.Mr, P.Mc, P.dims, P.TN, Ue, ce, 1e-10, X=X)
    assert Jb.shape == (P.dims["N_b"], nports)
    assert rel_err(Jb, Jo) <= 1e-9
    np.testing.assert_allclose(np.diag(S), np.diag(So), rtol=1e-8)
    assert rel_err(U @ S @ V.conj().T, Uo @ So @ Vo.conj().T) <= 1e-8
    # without a basis the factors are empty, as in ie_solver_vie.m:27-29
    Jb2, U2, S2, V2 = vie.ie_solver_vie(op, torch.from_numpy(Ue).cuda(), ce, P.Mr, P.Mc, P.idxS, 1e-10)
    assert isinstance(Jb2, torch.Tensor) and U2 == [] and S2 == [] and V2 == []
    assert rel_err(Jb2.cpu().numpy(), Jb) <= 1e-12
