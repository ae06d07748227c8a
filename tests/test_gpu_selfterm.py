"""The near-zone options of the GPU Green's-tensor assembly
(marie_assemble_green_ex, through the Python assemble_green).

* MARIE_GREEN_SELF_POINT_TERM (self_term="distributional") adds exactly the
  oracle's self_delta_term to I_V(0,0,0) of N and leaves every other entry,
  and K, as marie_assemble_green computes them.
* MARIE_GREEN_NEAR_EXACT (near="relative") gives the oracle's
  near_zone_relative on the offsets {0,1}^3 (N and K) and leaves the rest.
* Known answer: the GPU-assembled operator with it reproduces the internal
  field 3/(eps_r + 2) E0 of a quasi-static dielectric sphere (12^3 grid,
  1 cm voxels, r = 5 cm, 1 MHz) within the voxelisation error.
"""
import numpy as np
import pytest

from oracle import marie_oracle as O

torch = pytest.importorskip("torch")


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_self_point_term_flag(pwl):
    from marie_gb300 import assemble_green
    n, res, freq = (6, 5, 4), 2e-3, 297.2e6
    a = assemble_green(n, res, freq, pwl, "N", near="standin")
    b = assemble_green(n, res, freq, pwl, "N", self_term="distributional", near="standin")
    want = np.zeros_like(a)
    want[0, 0, 0] = O.self_delta_term(res, 10 if pwl else 1)
    assert np.allclose(b - a, want, rtol=0, atol=1e-12 * np.abs(a).max())
    k0 = assemble_green(n, res, freq, pwl, "K", near="standin")
    k1 = assemble_green(n, res, freq, pwl, "K", self_term="distributional", near="standin")
    assert np.allclose(k1, k0, rtol=0, atol=1e-12 * np.abs(k0).max())


@pytest.mark.gpu
@pytest.mark.parametrize("pwl,kernel", [(False, "N"), (True, "N"), (True, "K")], ids=["pwc-N", "pwl-N", "pwl-K"])
def test_near_exact_flag(pwl, kernel):
    from marie_gb300 import assemble_green
    n, res, freq = (5, 4, 3), 2e-3, 297.2e6
    a = assemble_green(n, res, freq, pwl, kernel, near="standin")
    b = assemble_green(n, res, freq, pwl, kernel, near="relative")
    near = [(x, y, z) for x in range(2) for y in range(2) for z in range(2)]
    ref = O.near_zone_relative(O.em_constants(freq)["k0"], res, 10 if pwl else 1, kernel, near)
    scale = np.abs(a).max()
    for m in near:
        assert np.abs(b[m] - ref[m]).max() <= 1e-12 * scale, m
        b[m] = a[m]
    assert np.allclose(b, a, rtol=0, atol=1e-13 * scale)


@pytest.mark.gpu
def test_quasi_static_sphere_field_gpu():
    from marie_gb300 import VieOperator, assemble_green, phantoms
    res, freq, er = 1e-2, 1e6, 50.0
    body = phantoms.sphere(12, res, 0.05, er, 0.0)
    emc = O.em_constants(freq)
    iv = assemble_green(body.n, res, freq, False, "N", near="relative")
    Mr = body.Mr(freq)
    op = VieOperator(body.n, res, freq, body.idx_solution(False), Mr, iv, pwl=False, precisions=3, max_rhs=1)
    Ns = body.idxS.size
    Ue = np.concatenate([np.ones(Ns), np.zeros(Ns), np.zeros(Ns)]).astype(complex)
    b = O.vie_rhs(emc["ce"], Mr, Mr - 1, body.idxS, 3, Ue)
    x, rep = op.gmres(torch.from_numpy(b).cuda(), restart=50, tol=1e-8, maxit=200, mode="fp64")
    assert rep.ok
    Mcb = Mr.reshape(-1, order="F")[body.idxS] - 1
    Ex = (x.cpu().numpy()[:Ns] / (emc["ce"] * Mcb)).real
    assert abs(Ex.mean() / (3.0 / (er + 2.0)) - 1.0) < 0.15, Ex.mean()
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("pwl,kernel", [(False, "N"), (True, "N"), (False, "K"), (True, "K")],
                         ids=["pwc-N", "pwl-N", "pwc-K", "pwl-K"])
def test_gpu_assembly_matches_oracle(pwl, kernel):
    """The GPU assembly (far and medium zones by the Gauss rules of
    assembly_N.m / assembly_K.m) against the oracle's restatement on the same
    grid, FP64 both sides: near zone by the stand-in (marie_assemble_green)
    and by the accurate cubature (the default of assemble_green, equal to the
    reference's DIRECTFN surface-surface near zone)."""
    from marie_gb300 import assemble_green
    n, res, freq = (5, 4, 3), 2e-3, 297.2e6
    k0 = O.em_constants(freq)["k0"]
    for near in ("standin", "relative"):
        got = assemble_green(n, res, freq, pwl, kernel, near=near)
        ref = O.assembly_op(*n, res, k0, pwl, kernel, near=near)
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max(), near
    assert np.array_equal(assemble_green(n, res, freq, pwl, kernel), got)
