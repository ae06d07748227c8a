"""Per-application Tucker expansion of the complex64 spectrum (precisions
bit 8, the reference's re-expansion in every product, mvp_N_pwl_tucker.m:31)
against the pre-expanded path and the oracle, through the C ABI.

* A synthetic 16 x 16 x 32 PWL operator (full-rank Tucker): mvp_vie, N and
  N^H in complex64 equal the pre-expanded handle's within complex64
  rounding (<= 2e-6) and the oracle's Tucker restatement (<= 1e-5).
* The physical operator of a 32^3 PWL sphere compressed at the reference's
  tolerance 1e-7 (marie_gb300.tucker.compress): the same, and the
  mixed-precision solve reaches 1e-6 with the float-float residual.
"""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, flat_F, unflat_F, rel_err

torch = pytest.importorskip("torch")


@pytest.mark.gpu
def test_per_apply_expansion_matches_pre_expanded():
    P = Problem((16, 16, 32), True, seed=4, tucker_tol=1e-14)
    a = P.gpu_operator(precisions=2 | 8, max_rhs=2)
    b = P.gpu_operator(precisions=2, max_rhs=2)
    J = P.random_grid(seed=2, nrhs=2)
    x = torch.from_numpy(np.concatenate([flat_F(J[r]) for r in range(2)])).to("cuda", torch.complex64)
    for name, adj in (("apply_N", False), ("apply_N_adj", True)):
        ya = getattr(a, name)(x).cpu().numpy().astype(np.complex128)
        yb = getattr(b, name)(x).cpu().numpy().astype(np.complex128)
        assert rel_err(ya, yb) <= 2e-6, name
        n = J[0].size
        for r in range(2):
            ref = O.mvp_op_tucker(J[r], P.TN, "N", adj, cache={})
            assert rel_err(unflat_F(ya[r * n:(r + 1) * n], P.n, 12), ref) <= 1e-5, (name, r)
    Jb = P.random_body_vec(seed=3)[0]
    xb = torch.from_numpy(Jb).to("cuda", torch.complex64)
    ref = O.mvp_vie(Jb, P.Mr, P.Mc, P.dims, P.TN, cache={})
    assert rel_err(a.apply(xb).cpu().numpy(), ref) <= 1e-5
    a.close()
    b.close()


@pytest.mark.gpu
def test_per_apply_expansion_physical_sphere_solve():
    from marie_gb300 import VieOperator, assemble_green, phantoms, tucker
    res, freq = 5e-3, 128e6
    body = phantoms.sphere(32, res, 0.06, 50.0, 0.6)
    iv = assemble_green(body.n, res, freq, True, "N")
    T = tucker.compress(iv, 1e-7)
    Mr = body.Mr(freq)
    op = VieOperator(body.n, res, freq, body.idx_solution(True), Mr, T, pwl=True, precisions=2 | 4 | 8, max_rhs=1)
    pre = VieOperator(body.n, res, freq, body.idx_solution(True), Mr, T, pwl=True, precisions=2 | 4, max_rhs=1)
    dims = O.geo_dims(*body.n, body.idxS, True, res)
    Jb = np.random.default_rng(1).normal(size=dims["N_b"]) + 0j
    x = torch.from_numpy(Jb).to("cuda", torch.complex64)
    ref = O.mvp_vie(Jb, Mr, Mr - 1, dims, T, cache={})
    ya = op.apply(x).cpu().numpy()
    assert rel_err(ya, ref) <= 1e-5
    assert rel_err(ya, pre.apply(x).cpu().numpy()) <= 2e-6
    b = op.incident_plane_wave(body.origin)
    emc = O.em_constants(freq)
    chi = np.tile((1.0 / Mr.reshape(-1, order="F")[body.idxS]) * (Mr.reshape(-1, order="F")[body.idxS] - 1), 12)
    b = (emc["ce"] * torch.from_numpy(chi).cuda() * b).contiguous()
    xa, repa = op.gmres(b, tol=1e-6, mode="mixed")
    xp, repp = pre.gmres(b, tol=1e-6, mode="mixed")
    assert repa.ok and repa.true_resid[0] <= 1e-6
    assert rel_err(xa.cpu().numpy(), xp.cpu().numpy()) <= 1e-5
    op.close()
    pre.close()
