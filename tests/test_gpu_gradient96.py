"""The adjoint B1+ gradient at the full size of its configuration.

96^3 PWL ellipsoid phantom (2 mm, 297.2 MHz, accurate near zone), one 10 cm
loop 1 cm outside it whose incident E and H come from the wire kernels of
the reference's convention (marie_incident_wire: Assemble_tri_coupling_matrix
N and K), a seeded 20^3 ROI.  J_obj = mean_ROI |B1+|^2 / P_abs.

* Central finite differences, step 1e-4 relative, on 32 seeded body voxels
  (eps_r on 16, sigma on 16) against the adjoint gradient from FP64 solves:
  <= 1e-4 relative.  Each difference J_obj(p + h) - J_obj(p - h) is formed
  without cancellation: with J0 the base solution, the perturbed solution is
  J0 + dJ where A(p +- h) dJ = (b(p +- h) - b(p)) - (A(p +- h) - A(p)) J0 is
  solved for dJ itself (64 FP64 solves in all), and the changes of
  M = mean |B1+|^2 and P are expanded exactly in dJ (M and P are quadratic in
  J; H is affine in J).  Solving the two perturbed systems from scratch and
  subtracting the objectives would lose the ~1e-9 relative change of J_obj in
  the solver tolerance.
* The gradient from mixed-precision solves (tol 1e-8) against the FP64 one:
  <= 1e-4 relative (2-norm over all voxels).
"""
import numpy as np
import pytest

from oracle import marie_oracle as O

torch = pytest.importorskip("torch")


def _loop_bases(centre, normal, radius, nseg):
    normal = np.asarray(normal, float) / np.linalg.norm(normal)
    a = np.array([1.0, 0, 0]) if abs(normal[0]) < 0.9 else np.array([0, 1.0, 0])
    e1 = np.cross(normal, a)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(normal, e1)
    t = 2 * np.pi * np.arange(nseg) / nseg
    P = np.asarray(centre, float)[None, :] + radius * (np.cos(t)[:, None] * e1 + np.sin(t)[:, None] * e2)
    return np.roll(P, 1, axis=0), np.roll(P, -1, axis=0), P


@pytest.mark.gpu
def test_b1_gradient_96_finite_differences_and_mixed():
    from marie_gb300 import VieOperator, assemble_green, phantoms, vie
    res, freq, pwl = 2e-3, 297.2e6, True
    body = phantoms.ellipsoid_phantom(96, res, seed=0)
    emc = O.em_constants(freq)
    ce, mu0 = emc["ce"], emc["mu0"]
    ivN = assemble_green(body.n, res, freq, pwl, "N")
    ivK = assemble_green(body.n, res, freq, pwl, "K")
    idx = body.idx_solution(pwl)
    Mr0 = body.Mr(freq)
    # fields (K, native complex128) on one handle, solves (float-float N) on another
    opK = VieOperator(body.n, res, freq, idx, Mr0, ivN, ivK, pwl=pwl, precisions=1, max_rhs=2)
    opS = VieOperator(body.n, res, freq, idx, Mr0, ivN, pwl=pwl, precisions=2 | 4, max_rhs=1)
    del ivN, ivK
    r_p, r_n, r_2 = _loop_bases([0.080 + 0.01, 0.0, 0.0], [1.0, 0.0, 0.0], 0.05, 64)
    Ue = opK.incident_wire(body.origin, r_p, r_n, r_2, kind="E")
    Ub = opK.incident_wire(body.origin, r_p, r_n, r_2, kind="H")
    assert float(Ub.abs().max()) > 0
    rng = np.random.default_rng(5)
    ijk = np.stack(np.unravel_index(body.idxS, body.n, order="F"), 1)
    c0 = ijk[rng.integers(body.idxS.size)]
    lo = np.clip(c0 - 10, 0, np.array(body.n) - 20)
    roi = np.nonzero(np.all((ijk >= lo) & (ijk < lo + 20), axis=1))[0]
    assert roi.size > 1000
    g = np.unravel_index(body.idxS, body.n, order="F")
    er0, se0 = body.er[g].copy(), body.se[g].copy()
    Ns = er0.size

    def materials(er, se):
        mr = er + se / ce
        opK.set_materials(mr)
        opS.set_materials(mr)
        return mr

    def rhs(mr):
        chi = np.tile((1.0 / mr) * (mr - 1.0), 12)
        return (ce * torch.from_numpy(chi).cuda() * Ue).contiguous()

    mr0 = materials(er0, se0)
    b0 = rhs(mr0)
    Jobj, de, ds, J0 = vie.b1_objective_gradient(opK, b0, Ue, Ub, roi, tol=1e-12, mode="fp64", solve_op=opS)
    de, ds = de.cpu().numpy(), ds.cpu().numpy()
    r_roi = torch.as_tensor(roi, device="cuda")
    _E, H0 = opK.fields(J0, Ue=Ue, Ub=Ub)
    b10 = opK.b1_plus(H0)[r_roi]
    M0 = float((b10.abs() ** 2).mean())
    P0 = 0.5 * float(opK.absorbed_power(J0)[0, 0].real)
    assert abs(M0 / P0 - Jobj) <= 1e-12 * abs(Jobj)
    AJ0 = opK.apply(J0)

    def delta_obj(er, se):
        """J_obj(materials) - J_obj(base), formed without cancellation."""
        mr = materials(er, se)
        r = (rhs(mr) - b0) - (opK.apply(J0) - AJ0)
        dJ, rep = opS.gmres(r, tol=1e-10, mode="fp64")
        assert rep.ok, rep.status
        _e, Hd = opK.fields(dJ, h=True, e=False)
        db1 = opK.b1_plus(Hd)[r_roi]
        dM = float((2 * (b10.conj() * db1).real + db1.abs() ** 2).mean())
        phi = opK.absorbed_power(torch.cat([J0, dJ]))            # materials of this state
        dP = 0.5 * float(phi[0, 0].real - 2 * P0 + phi[0, 1].real + phi[1, 0].real + phi[1, 1].real)
        materials(er0, se0)
        return (dM * P0 - M0 * dP) / ((P0 + dP) * P0)

    vox = rng.choice(Ns, size=32, replace=False)
    scale_e, scale_s = np.abs(de).max(), np.abs(ds).max()
    for i, s in enumerate(vox):
        which = "er" if i < 16 else "se"
        base = er0 if which == "er" else se0
        h = 1e-4 * base[s]
        plus, minus = base.copy(), base.copy()
        plus[s] += h
        minus[s] -= h
        if which == "er":
            fd = (delta_obj(plus, se0) - delta_obj(minus, se0)) / (2 * h)
            adj, sc = de[s], scale_e
        else:
            fd = (delta_obj(er0, plus) - delta_obj(er0, minus)) / (2 * h)
            adj, sc = ds[s], scale_s
        assert abs(fd - adj) <= 1e-4 * abs(fd) + 1e-9 * sc, (which, int(s), fd, adj, sc)
    # mixed-precision solves against the FP64 gradient
    Jm, dem, dsm, _ = vie.b1_objective_gradient(opK, b0, Ue, Ub, roi, tol=1e-8, mode="mixed", solve_op=opS)
    assert abs(Jm - Jobj) <= 1e-6 * abs(Jobj)
    for a, ref in ((dem, de), (dsm, ds)):
        a = a.cpu().numpy()
        assert np.linalg.norm(a - ref) <= 1e-4 * np.linalg.norm(ref)
    opK.close()
    opS.close()
