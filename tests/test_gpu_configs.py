"""Parity at the benchmark configurations' sizes (GPU).

* Sphere, r = 6 cm, 32^3 at 5 mm, PWC, 128 MHz, plane wave: the GPU
  complex128 GMRES (four-step path) against the oracle's restatement of
  is_gmres_vie.m on the same operator (the GPU-assembled I_V through the
  oracle's Tucker compression): identical iteration counts and restart
  bookkeeping, solutions within 1e-9.
* Ellipsoid phantom, 96^3 at 2 mm, PWL, 297.2 MHz, one loop: full-size
  size-independent properties: the mixed solve and the complex128 solve
  (float-float operator) both reach 1e-6 true residual and agree within
  1e-5 (the field-error target), and the solution satisfies A x = b to the
  reported residual when re-applied through the complex128 operator.
* The PWC sweep: sixteen seeded phantoms with edges drawn from
  {48, 64, 80, 96, 112, 128} at 2 mm, f in {128, 297.2} MHz, 1-8 loops each,
  bodies scaled to the grid: mixed and complex128 solves of every loop.
"""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import rel_err

torch = pytest.importorskip("torch")


@pytest.mark.gpu
def test_sphere32_pwc_plane_wave_fp64_matches_oracle():
    from marie_gb300 import VieOperator, assemble_green, phantoms
    res, freq = 5e-3, 128e6
    body = phantoms.sphere(32, res, 0.06, 50.0, 0.6)
    iv = assemble_green(body.n, res, freq, False, "N")
    op = VieOperator(body.n, res, freq, body.idx_solution(False), body.Mr(freq), iv, pwl=False, precisions=3,
                     max_rhs=1)
    emc = O.em_constants(freq)
    Mr = body.Mr(freq)
    Ue = op.incident_plane_wave(body.origin).cpu().numpy()
    b = O.vie_rhs(emc["ce"], Mr, Mr - 1, body.idxS, 3, Ue)
    dims = O.geo_dims(*body.n, body.idxS, False, res)
    T = O.assembly_fft_circ_tucker(iv[:, :, :, 0, :], 1e-14)
    cache = {}
    A = lambda v: O.mvp_vie(v, Mr, Mr - 1, dims, T, cache)
    tol = 1e-6
    xr, itr, rvr = O.is_gmres_vie(A, b, 50, tol, 200, np.zeros(b.size))
    x, rep = op.gmres(torch.from_numpy(b).cuda(), restart=50, tol=tol, maxit=200, mode="fp64")
    assert rep.ok
    assert int(rep.outer[0]) == int(itr[1]) and int(rep.last_inner[0]) == int(itr[0])
    assert rel_err(x.cpu().numpy(), xr) < 1e-9
    true = np.linalg.norm(b - A(xr)) / np.linalg.norm(b)
    assert abs(rep.true_resid[0] - true) < 1e-9 and rep.true_resid[0] <= tol
    op.close()


@pytest.mark.gpu
def test_ellipsoid96_pwl_loop_full_size_properties():
    from marie_gb300 import VieOperator, assemble_green, phantoms
    res, freq = 2e-3, 297.2e6
    body = phantoms.ellipsoid_phantom(96, res, seed=0)
    iv = assemble_green(body.n, res, freq, True, "N")
    op = VieOperator(body.n, res, freq, body.idx_solution(True), body.Mr(freq), iv, pwl=True, precisions=2 | 4,
                     max_rhs=1)
    del iv
    loops, radius = phantoms.loop_outside((0.080, 0.065, 0.090), gap=0.01, radius=0.05)
    Ue = op.incident_loops(body.origin, loops, radius, nseg=64)
    emc = O.em_constants(freq)
    Mr = body.Mr(freq).reshape(-1, order="F")[body.idxS]
    chi = np.tile((1.0 / Mr) * (Mr - 1.0), 12)
    b = (emc["ce"] * torch.from_numpy(chi).cuda() * Ue).contiguous()
    xm, repm = op.gmres(b, restart=50, tol=1e-6, mode="mixed")
    xf, repf = op.gmres(b, restart=50, tol=1e-6, mode="fp64")
    assert repm.ok and repf.ok
    assert repm.true_resid[0] <= 1e-6 and repf.true_resid[0] <= 1e-6
    assert rel_err(xm.cpu().numpy(), xf.cpu().numpy()) <= 1e-5
    r = (b - op.apply(xf)).cpu().numpy()
    assert abs(np.linalg.norm(r) / np.linalg.norm(b.cpu().numpy()) - repf.true_resid[0]) < 1e-9
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n,freq", [(48, 128e6), (80, 297.2e6), (112, 128e6)], ids=["48", "80", "112"])
def test_pwc_phantoms_various_edges(n, freq):
    """PWC phantoms scaled to the grid (edges 48/80/112: four-step radices 3,
    5, 7), 2 mm, one loop: complex128 matvec against the oracle on the
    smallest grid; mixed and complex128 solves agree within 1e-5 at 1e-6."""
    from marie_gb300 import VieOperator, assemble_green, phantoms
    res = 2e-3
    scale = 0.9 * (n * res / 2) / 0.090
    body = phantoms.ellipsoid_phantom(n, res, seed=n, scale=scale)
    iv = assemble_green(body.n, res, freq, False, "N")
    op = VieOperator(body.n, res, freq, body.idx_solution(False), body.Mr(freq), iv, pwl=False, precisions=3,
                     max_rhs=2)
    if n == 48:
        dims = O.geo_dims(*body.n, body.idxS, False, res)
        T = O.assembly_fft_circ_tucker(iv[:, :, :, 0, :], 1e-14)
        rng = np.random.default_rng(1)
        J = rng.normal(size=dims["N_b"]) + 1j * rng.normal(size=dims["N_b"])
        Mr = body.Mr(freq)
        ref = O.mvp_vie(J, Mr, Mr - 1, dims, T)
        assert rel_err(op.apply(torch.from_numpy(J).cuda()).cpu().numpy(), ref) <= 1e-12
    del iv
    axes = np.array([0.080, 0.065, 0.090]) * scale
    loops, radius = phantoms.loop_outside(tuple(axes), gap=0.005, radius=0.25 * n * res)
    Ue = op.incident_loops(body.origin, loops, radius, nseg=64)
    emc = O.em_constants(freq)
    Mr = body.Mr(freq).reshape(-1, order="F")[body.idxS]
    chi = np.tile((1.0 / Mr) * (Mr - 1.0), 3)
    b = (emc["ce"] * torch.from_numpy(chi).cuda() * Ue).contiguous()
    xm, repm = op.gmres(b, restart=50, tol=1e-6, mode="mixed")
    xf, repf = op.gmres(b, restart=50, tol=1e-6, mode="fp64")
    assert repm.ok and repf.ok and repm.true_resid[0] <= 1e-6 and repf.true_resid[0] <= 1e-6
    assert rel_err(xm.cpu().numpy(), xf.cpu().numpy()) <= 1e-5
    op.close()


@pytest.mark.gpu
def test_pwc_sweep_sixteen_phantoms():
    """Sixteen seeded PWC phantoms (edges from {48, ..., 128}, 2 mm, 128 or
    297.2 MHz, 1-8 loops on a ring around the body, bodies scaled to the
    grid): for every loop the mixed solve and the complex128 solve
    (float-float operator) reach 1e-6 true residual and agree within 1e-5."""
    from marie_gb300 import VieOperator, assemble_green, phantoms
    rng = np.random.default_rng(44)
    res = 2e-3
    for i in range(16):
        n = int(rng.choice([48, 64, 80, 96, 112, 128]))
        freq = float(rng.choice([128e6, 297.2e6]))
        nl = int(rng.integers(1, 9))
        scale = 0.9 * (n * res / 2) / 0.090
        body = phantoms.ellipsoid_phantom(n, res, seed=100 + i, scale=scale)
        iv = assemble_green(body.n, res, freq, False, "N")
        op = VieOperator(body.n, res, freq, body.idx_solution(False), body.Mr(freq), iv, pwl=False,
                         precisions=2 | 4, max_rhs=nl)
        del iv
        loops = phantoms.loop_ring(nl, ring_radius=0.080 * scale + 0.01, z_extent=0.0, n_angles=nl, seed=200 + i)
        Ue = op.incident_loops(body.origin, loops, 0.25 * n * res / 2, nseg=64).reshape(nl, -1)
        emc = O.em_constants(freq)
        Mr = body.Mr(freq).reshape(-1, order="F")[body.idxS]
        chi = np.tile((1.0 / Mr) * (Mr - 1.0), 3)
        b = (emc["ce"] * torch.from_numpy(chi).cuda()[None, :] * Ue).reshape(-1).contiguous()
        xm, repm = op.gmres(b, restart=50, tol=1e-6, mode="mixed")
        xf, repf = op.gmres(b, restart=50, tol=1e-6, mode="fp64")
        assert repm.ok and repf.ok, (i, n, freq, nl)
        assert np.max(repm.true_resid) <= 1e-6 and np.max(repf.true_resid) <= 1e-6, (i, n)
        xm, xf = xm.cpu().numpy().reshape(nl, -1), xf.cpu().numpy().reshape(nl, -1)
        for r in range(nl):
            assert rel_err(xm[r], xf[r]) <= 1e-5, (i, n, freq, r)
        op.close()
