"""The near-zone cubature against the reference's own singular quadrature.

oracle/Makefile compiles the reference's DIRECTFN C++ (the singular
surface-surface integrals behind assembly_N.m:56-81) from the reference
checkout into oracle/_ref; oracle/directfn_ref.py restates the reference's
surface-surface near zone (surface_surface_kernels_Nop.m with
coefficients_Nop.m and kernels_Nop.m, singular face pairs through DIRECTFN
ST / EA / VA) and a short face-pair form of its PWC entries.  The oracle's
near_zone_relative (and hence the library's MARIE_GREEN_NEAR_EXACT cubature,
equal to it to 1e-14 in test_green_host.py) must agree: every near offset
of the PWC moment to 1e-12, the PWL moments (all ten pairs, six components)
on the self, face and vertex offsets to the accuracy of DIRECTFN at order
10.  Skipped where the reference checkout or g++ is absent.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import marie_oracle as O

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def directfn():
    """oracle/_ref/libdirectfn.so and its siblings, built from the reference's sources
    by oracle/Makefile (which finds the checkout); skipped without one."""
    if shutil.which("g++") and shutil.which("make"):
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    if not (ROOT / "oracle" / "_ref" / "libdirectfn.so").exists():
        pytest.skip("oracle/_ref not built (no reference checkout or toolchain)")
    from oracle import directfn_ref
    return directfn_ref


@pytest.mark.parametrize("freq,res", [(297.2e6, 2e-3), (128e6, 5e-3)])
def test_pwc_near_zone_matches_directfn(directfn, freq, res):
    k0 = O.em_constants(freq)["k0"]
    ref = directfn.pwc_near_entries(k0, res)
    nz = O.near_zone_relative(k0, res, 1, "N", [(0, 0, 0), (1, 0, 0)])
    for key, got in (("self_xx", nz[(0, 0, 0)][0, 0]), ("face_xx", nz[(1, 0, 0)][0, 0]),
                     ("face_yy", nz[(1, 0, 0)][0, 3])):
        assert abs(got - ref[key]) <= 1e-12 * abs(ref[key]), (key, got, ref[key])
    # the stand-in misses the point term (self) and is 13% low on the face neighbour
    st = O.near_zone_standin(k0, res, 1, "N", [(0, 0, 0), (1, 0, 0)])
    assert abs(st[(0, 0, 0)][0, 0]) < 1e-3 * abs(ref["self_xx"])
    assert abs(st[(1, 0, 0)][0, 0] / ref["face_xx"] - 1) > 0.05


NEAR = [(a, b, c) for a in range(2) for b in range(2) for c in range(2)]


def test_surface_form_pwc_all_offsets(directfn):
    k0 = O.em_constants(297.2e6)["k0"]
    nz = O.near_zone_relative(k0, 2e-3, 1, "N", NEAR)
    for m in NEAR:
        ref = directfn.surface_near_zone(k0, 2e-3, 1, m, N=16, qg=12)
        assert np.abs(nz[m] - ref).max() <= 1e-12 * np.abs(ref).max(), m


@pytest.mark.parametrize("m,tol", [((0, 0, 0), 1e-10), ((1, 0, 0), 1e-8), ((1, 1, 1), 1e-8)])
def test_surface_form_pwl(directfn, m, tol):
    k0 = O.em_constants(297.2e6)["k0"]
    ref = directfn.surface_near_zone(k0, 2e-3, 10, m, N=10, qg=8)
    got = O.near_zone_relative(k0, 2e-3, 10, "N", [m])[m]
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


def test_surface_form_K_pwc_all_offsets(directfn):
    """The K operator (surface_surface_kernels_Kop.m, DIRECTFN kernel types
    5-8): every near offset of the PWC moment (the self offset is zero on
    both sides)."""
    k0 = O.em_constants(297.2e6)["k0"]
    nz = O.near_zone_relative(k0, 2e-3, 1, "K", NEAR)
    ref = {m: directfn.surface_near_zone_K(k0, 2e-3, 1, m, N=12, qg=12) for m in NEAR}
    scale = max(np.abs(v).max() for v in ref.values())
    for m in NEAR:
        assert np.abs(nz[m] - ref[m]).max() <= 1e-10 * scale, m


@pytest.mark.parametrize("m", [(1, 0, 0), (1, 1, 1)])
def test_surface_form_K_pwl(directfn, m):
    k0 = O.em_constants(297.2e6)["k0"]
    ref = directfn.surface_near_zone_K(k0, 2e-3, 10, m, N=10, qg=10)
    got = O.near_zone_relative(k0, 2e-3, 10, "K", [m])[m]
    assert np.abs(got - ref).max() <= 1e-7 * np.abs(ref).max()
