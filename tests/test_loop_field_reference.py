"""The loop right-hand side against the reference's own wire-coupling kernels
(Assemble_tri_coupling_matrix_N_{x,y,z,y1,y2,y3}.cpp, compiled from the reference
checkout by oracle/Makefile; oracle/wire_ref.py).

The library's loop kernel (k_loops, checked against the oracle's
loop_field / incident_moments in the GPU tests) models a uniform unit
current.  The reference's kernels with unit coefficients carry a sawtooth
current of mean 1: its field component along the wire direction agrees with
the uniform one to 0.1% 1-4 cm from the wire, while the sawtooth's line and
point charges add radial and axial components that the uniform current does
not have (up to 2.4x the tangential one at 1 cm).  Skipped where the
reference checkout or g++ is absent.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import marie_oracle as O

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def wire():
    """oracle/_ref/libtri_N_x.so and its siblings, built from the reference's sources
    by oracle/Makefile (which finds the checkout); skipped without one."""
    if shutil.which("g++") and shutil.which("make"):
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    if not (ROOT / "oracle" / "_ref" / "libtri_N_x.so").exists():
        pytest.skip("oracle/_ref not built (no reference checkout or toolchain)")
    from oracle import wire_ref
    return wire_ref


def test_loop_field_along_the_wire_matches_reference(wire):
    freq, res, radius, nseg = 297.2e6, 2e-3, 0.05, 64
    emc = O.em_constants(freq)
    centre, normal = np.zeros(3), np.array([0.0, 0.0, 1.0])
    pts = np.array([[x, 0.0, -d] for d in (0.01, 0.02, 0.04) for x in (0.03, 0.05, 0.07)])
    ref = wire.loop_field_reference(pts, centre, normal, radius, nseg, res, emc["k0"])
    mid, dl = O.loop_points(centre, normal, radius, nseg)
    ours = O.incident_moments(pts, res, False,
                              lambda q: O.loop_field(q, mid, dl, emc["k0"], emc["omega"], emc["mu0"])).reshape(3, -1).T
    # in the plane y = 0 the wire direction is y: the uniform current's field is y only
    assert np.all(np.abs(ours[:, [0, 2]]) < 1e-9 * np.abs(ours[:, 1]).max())
    assert np.all(np.abs(ref[:, 1] / ours[:, 1] - 1) < 2e-3)
    # the sawtooth's charges: radial / axial components of the reference's field
    assert np.abs(ref[:, [0, 2]]).max() > 0.5 * np.abs(ref[:, 1]).max()


def test_loop_field_pwl_moments_match_reference(wire):
    """PWL moments of the wire-direction component (N_y, N_y1, N_y2, N_y3:
    the constant and the x-, y-, z-linear moments): the constant and the x-
    and z-moments agree to 2e-3 of the constant one; the y-moment, zero for
    the uniform current by symmetry, is the sawtooth's charge field."""
    freq, res, radius, nseg = 297.2e6, 2e-3, 0.05, 64
    emc = O.em_constants(freq)
    centre, normal = np.zeros(3), np.array([0.0, 0.0, 1.0])
    pts = np.array([[x, 0.0, -d] for d in (0.01, 0.02) for x in (0.03, 0.05, 0.07)])
    rp, rn, r2 = wire.loop_bases(centre, normal, radius, nseg)
    ref = np.stack([wire.tri_coupling(v, pts, rp, rn, r2, res, emc["k0"]).sum(axis=1)
                    for v in ("y", "y1", "y2", "y3")], axis=1)
    ref[:, 1:] *= 12                      # voxel average of E f_l -> coefficient (int f_l^2 = 1/12)
    mid, dl = O.loop_points(centre, normal, radius, nseg)
    ours = O.incident_moments(pts, res, True, lambda q: O.loop_field(q, mid, dl, emc["k0"], emc["omega"],
                                                                     emc["mu0"])).reshape(3, 4, -1)[1].T
    scale = np.abs(ours[:, 0])[:, None]
    assert np.all(np.abs(ours[:, [0, 1, 3]] - ref[:, [0, 1, 3]]) <= 2e-3 * scale)
    assert np.all(np.abs(ours[:, 2]) < 1e-9 * scale[:, 0]) and np.abs(ref[:, 2]).max() > 1e-3 * scale.max()


@pytest.mark.parametrize("kind", ["N", "K"])
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_wire_coupling_restatement_matches_reference(wire, kind, pwl):
    """oracle.wire_coupling (the restatement the GPU wire kernel is checked
    against) equals the reference's Assemble_tri_coupling_matrix_{N,K}_*
    kernels compiled from source, every component and moment, to 1e-13."""
    rng = np.random.default_rng(1)
    res, k0 = 2e-3, O.em_constants(297.2e6)["k0"]
    centres = rng.uniform(-0.02, 0.02, size=(9, 3))
    r_p, r_n, r_2 = wire.loop_bases([0.05, 0.01, -0.02], [1, 0.2, 0.1], 0.03, 12)
    Z = O.wire_coupling(kind, centres, r_p, r_n, r_2, res, k0, pwl)
    comps = ["x", "x1", "x2", "x3", "y", "y1", "y2", "y3", "z", "z1", "z2", "z3"] if pwl else ["x", "y", "z"]
    for i, v in enumerate(comps):
        ref = wire.tri_coupling(v, centres, r_p, r_n, r_2, res, k0, kind=kind) * res ** 3
        assert np.abs(Z[i] - ref).max() <= 1e-13 * np.abs(ref).max(), (kind, v)
