"""Right-hand-side kernels against the oracle, through the C ABI.

marie_incident_loops (closed loops of straight segments with a uniform unit
current, E = -i omega mu0 sum_seg g(R) dl at the segment mid-points, tested
onto the PWC/PWL basis with a 3^3 Gauss rule) and marie_incident_plane_wave
(x-polarised, +z) against oracle.incident_moments with oracle.loop_field /
oracle.plane_wave_field, the same projections in numpy FP64.  Tolerance
1e-12 relative: both sides evaluate the same sums in FP64 in a different
order.  Cases: the 48^3 PWL benchmark phantom scaled to its grid with
three ring loops, the 32^3 PWC sphere with a plane wave, and every body
voxel of the full-size 96^3 PWL phantom for one loop 1 cm outside it
(oracle on a seeded sample of 4000 voxels).
"""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import rel_err

torch = pytest.importorskip("torch")

TOL = 1e-12


def _centres(body, res):
    c = O.voxel_centres(*body.n, res, origin=np.asarray(body.origin))
    return c.reshape(-1, 3, order="F")[body.idxS]


def _op(body, res, freq, pwl, nrhs):
    from marie_gb300 import VieOperator
    n = body.n
    iv = np.zeros(tuple(n) + ((10 if pwl else 1), 6), complex)
    iv[0, 0, 0, 0, 0] = 1e-12                     # the operator's values play no part here
    return VieOperator(n, res, freq, body.idx_solution(pwl), body.Mr(freq), iv, pwl=pwl,
                       precisions=2, max_rhs=nrhs)


def _oracle_loops(centres, res, pwl, loops, radius, nseg, freq):
    emc = O.em_constants(freq)
    out = []
    for L in loops:
        mid, dl = O.loop_points(L[:3], L[3:], radius, nseg)
        fn = lambda pts: O.loop_field(pts, mid, dl, emc["k0"], emc["omega"], emc["mu0"])
        out.append(O.incident_moments(centres, res, pwl, fn))
    return np.stack(out)


@pytest.mark.gpu
def test_loops_on_scaled_phantom_pwl():
    from marie_gb300 import phantoms
    n, res, freq = 48, 2e-3, 297.2e6
    body = phantoms.ellipsoid_phantom(n, res, seed=3, scale=0.5)
    loops = phantoms.loop_ring(3, ring_radius=0.07, z_extent=0.02, n_angles=3, seed=5)
    op = _op(body, res, freq, True, 3)
    got = op.incident_loops(body.origin, loops, 0.02, nseg=32).cpu().numpy().reshape(3, -1)
    ref = _oracle_loops(_centres(body, res), res, True, loops, 0.02, 32, freq)
    for l in range(3):
        assert rel_err(got[l], ref[l]) <= TOL, l
    op.close()


@pytest.mark.gpu
def test_plane_wave_sphere_pwc_and_pwl():
    from marie_gb300 import phantoms
    n, res, freq = 32, 5e-3, 128e6
    body = phantoms.sphere(n, res, 0.06, 50.0, 0.6)
    k0 = O.em_constants(freq)["k0"]
    for pwl in (False, True):
        op = _op(body, res, freq, pwl, 1)
        got = op.incident_plane_wave(body.origin).cpu().numpy()
        ref = O.incident_moments(_centres(body, res), res, pwl, lambda p: O.plane_wave_field(p, k0))
        assert rel_err(got, ref) <= TOL, pwl
        op.close()


@pytest.mark.gpu
def test_loop_full_size_phantom_sampled():
    """The 96^3 PWL phantom (244,976 body voxels) and the benchmark's 10 cm
    loop 1 cm outside it: every component and moment of a seeded sample of
    4000 body voxels."""
    from marie_gb300 import phantoms
    n, res, freq = 96, 2e-3, 297.2e6
    body = phantoms.ellipsoid_phantom(n, res, seed=0)
    loops, radius = phantoms.loop_outside((0.080, 0.065, 0.090), gap=0.01, radius=0.05)
    op = _op(body, res, freq, True, 1)
    got = op.incident_loops(body.origin, loops, radius, nseg=64).cpu().numpy()
    Ns = body.idxS.size
    assert got.size == 12 * Ns and np.all(np.isfinite(got))
    pick = np.sort(np.random.default_rng(0).choice(Ns, 4000, replace=False))
    ref = _oracle_loops(_centres(body, res)[pick], res, True, np.asarray(loops).reshape(-1, 6), radius, 64,
                        freq)[0].reshape(12, -1)
    assert rel_err(got.reshape(12, Ns)[:, pick], ref) <= TOL
    op.close()


def _loop_bases(centre, normal, radius, nseg):
    """Triangle bases of a closed regular nseg-gon: basis i spans nodes
    i-1 -> i -> i+1 (the wire layout of a closed loop)."""
    normal = np.asarray(normal, float) / np.linalg.norm(normal)
    a = np.array([1.0, 0, 0]) if abs(normal[0]) < 0.9 else np.array([0, 1.0, 0])
    e1 = np.cross(normal, a)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(normal, e1)
    t = 2 * np.pi * np.arange(nseg) / nseg
    P = np.asarray(centre, float)[None, :] + radius * (np.cos(t)[:, None] * e1 + np.sin(t)[:, None] * e2)
    return np.roll(P, 1, axis=0), np.roll(P, -1, axis=0), P


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_wire_fields_match_oracle(pwl):
    """marie_incident_wire (E and H, unit and complex wire currents, two
    right-hand sides) against oracle.wire_incident, the restatement of the
    reference's Assemble_tri_coupling_matrix_{N,K}_* kernels (which
    tests/test_loop_field_reference.py pins to those kernels compiled from
    source)."""
    from marie_gb300 import phantoms
    n, res, freq = 24, 2e-3, 297.2e6
    body = phantoms.ellipsoid_phantom(n, res, seed=2, scale=0.25)
    k0 = O.em_constants(freq)["k0"]
    op = _op(body, res, freq, pwl, 2)
    r_p, r_n, r_2 = _loop_bases([0.0, 0.0, 0.04], [0.1, 0.0, 1.0], 0.02, 16)
    rng = np.random.default_rng(7)
    coef = rng.normal(size=(2, 16)) + 1j * rng.normal(size=(2, 16))
    cen = _centres(body, res)
    for kind, kk in (("E", "N"), ("H", "K")):
        got = op.incident_wire(body.origin, r_p, r_n, r_2, kind=kind).cpu().numpy()
        ref = O.wire_incident(kk, cen, r_p, r_n, r_2, np.ones(16), res, k0, pwl)
        assert rel_err(got, ref) <= TOL, kind
        got2 = op.incident_wire(body.origin, r_p, r_n, r_2, coef, kind=kind).cpu().numpy().reshape(2, -1)
        for r in range(2):
            ref2 = O.wire_incident(kk, cen, r_p, r_n, r_2, coef[r], res, k0, pwl)
            assert rel_err(got2[r], ref2) <= TOL, (kind, r)
    op.close()
