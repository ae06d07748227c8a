"""Adjoint sensitivities of the B1+ objective J_obj = mean_ROI |B1+|^2 / P_abs
with respect to each body voxel's eps_r and sigma (GPU).

* 16^3 PWL sphere (physical N and K assembled on the GPU, one loop): the
  adjoint gradient against central finite differences (relative step 1e-4)
  of the objective recomputed with perturbed materials, complex128 solves
  to 1e-12, on 32 seeded voxels and both material parameters; per-voxel
  relative agreement within 1e-5 (measured 1e-9 to 1e-6).
* The configuration's full size (96^3) is checked in test_gpu_gradient96.py.
* torch.autograd through vie.b1_objective_autograd: backward returns the
  adjoint sensitivities, chained through a function of the materials.
"""
import numpy as np
import pytest

from oracle import marie_oracle as O

torch = pytest.importorskip("torch")


def _setup(body, res, freq, pwl, precisions, ivN, ivK):
    from marie_gb300 import VieOperator
    return VieOperator(body.n, res, freq, body.idx_solution(pwl), body.Mr(freq), ivN, ivK, pwl=pwl,
                       precisions=precisions, max_rhs=1)


def _rhs(op, body, freq, pwl, Ue):
    emc = O.em_constants(freq)
    Mr = body.Mr(freq).reshape(-1, order="F")[body.idxS]
    chi = np.tile((1.0 / Mr) * (Mr - 1.0), 12 if pwl else 3)
    return (emc["ce"] * torch.from_numpy(chi).cuda() * Ue).contiguous()


@pytest.mark.gpu
def test_b1_gradient_matches_finite_differences():
    from marie_gb300 import assemble_green, phantoms
    from marie_gb300 import vie
    res, freq, pwl = 5e-3, 297.2e6, True
    body = phantoms.sphere(16, res, 0.03, 50.0, 0.6)
    ivN = assemble_green(body.n, res, freq, pwl, "N")
    ivK = assemble_green(body.n, res, freq, pwl, "K")
    op = _setup(body, res, freq, pwl, 3, ivN, ivK)
    loops, radius = phantoms.loop_outside((0.03, 0.03, 0.03), gap=0.01, radius=0.02)
    Ue = op.incident_loops(body.origin, loops, radius, nseg=64)
    rng = np.random.default_rng(2)
    Ub = torch.from_numpy(1e-3 * (rng.normal(size=op.Nb) + 1j * rng.normal(size=op.Nb))).cuda()
    roi = np.arange(0, body.idxS.size, 7)
    kw = dict(tol=1e-12, mode="fp64")
    Jobj, de, ds, _J = vie.b1_objective_gradient(op, _rhs(op, body, freq, pwl, Ue), Ue, Ub, roi, **kw)
    de, ds = de.cpu().numpy(), ds.cpu().numpy()
    op.close()

    def objective(er, se):
        b2 = phantoms.Body(body.n, body.res, body.origin, er, se, body.idxS)
        o2 = _setup(b2, res, freq, pwl, 3, ivN, ivK)
        J, _r = o2.gmres(_rhs(o2, b2, freq, pwl, Ue), **kw)
        val = vie.b1_objective(o2, J, Ue, Ub, roi)[0]
        o2.close()
        return val

    vox = rng.choice(body.idxS.size, size=32, replace=False)
    scale_e, scale_s = np.abs(de).max(), np.abs(ds).max()
    for s in vox:
        g = np.unravel_index(body.idxS[s], body.n, order="F")
        for which in ("er", "se"):
            er, se = body.er.copy(), body.se.copy()
            arr = er if which == "er" else se
            h = 1e-4 * arr[g]
            arr[g] += h
            fp = objective(er, se)
            arr[g] -= 2 * h
            fm = objective(er, se)
            fd = (fp - fm) / (2 * h)
            adj = de[s] if which == "er" else ds[s]
            scale = scale_e if which == "er" else scale_s
            assert fd != 0 and abs(fd - adj) <= 1e-5 * abs(fd) + 1e-9 * scale, (which, s, fd, adj, scale)


@pytest.mark.gpu
def test_b1_objective_autograd_wrapper():
    """torch.autograd through vie.b1_objective_autograd returns the adjoint
    sensitivities (and the chain rule through a function of the materials)."""
    from marie_gb300 import assemble_green, phantoms
    from marie_gb300 import vie
    res, freq, pwl = 5e-3, 297.2e6, True
    body = phantoms.sphere(16, res, 0.03, 50.0, 0.6)
    ivN = assemble_green(body.n, res, freq, pwl, "N")
    ivK = assemble_green(body.n, res, freq, pwl, "K")
    loops, radius = phantoms.loop_outside((0.03, 0.03, 0.03), gap=0.01, radius=0.02)
    roi = np.arange(0, body.idxS.size, 5)
    cache = {}

    def build(er_s, se_s):
        er, se = body.er.copy(), body.se.copy()
        g = np.unravel_index(body.idxS, body.n, order="F")
        er[g], se[g] = er_s, se_s
        b2 = phantoms.Body(body.n, body.res, body.origin, er, se, body.idxS)
        op = _setup(b2, res, freq, pwl, 3, ivN, ivK)
        if "Ue" not in cache:
            cache["Ue"] = op.incident_loops(body.origin, loops, radius, nseg=64)
        Ue = cache["Ue"]
        return op, _rhs(op, b2, freq, pwl, Ue), Ue, torch.zeros_like(Ue)

    g = np.unravel_index(body.idxS, body.n, order="F")
    er0 = torch.tensor(body.er[g], dtype=torch.float64, device="cuda", requires_grad=True)
    se0 = torch.tensor(body.se[g], dtype=torch.float64, device="cuda", requires_grad=True)
    scale = torch.tensor(1.5, dtype=torch.float64, device="cuda")
    J = vie.b1_objective_autograd(er0 * scale, se0, build, roi, tol=1e-12, mode="fp64")
    J.backward()
    op, b, Ue, Ub = build(body.er[g] * 1.5, body.se[g])
    _J, de, ds, _ = vie.b1_objective_gradient(op, b, Ue, Ub, roi, tol=1e-12, mode="fp64")
    op.close()
    assert abs(float(J) - _J) <= 1e-12 * abs(_J)
    assert torch.allclose(er0.grad, 1.5 * de, rtol=1e-10, atol=0)
    assert torch.allclose(se0.grad, ds, rtol=1e-10, atol=0)
