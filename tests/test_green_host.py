"""The near zone of the Green's tensor on the CPU: the point term of the N
kernel at the self offset and the accurate near-zone cubature.

* The library's host helpers (marie-tools_gb300/csrc/green_host.h, through
  tests/host_shim.cpp) add exactly the oracle's self_delta_term to
  I_V(0,0,0), and reproduce the oracle's near_zone_relative (PWC and PWL,
  N and K) to rounding.
* near_zone_relative converges to rounding by order 12, agrees with the
  staggered cubature where that one converges (vertex neighbour; the PWC
  self offset plus the point term), and respects the axis symmetry.
* Known answer: a quasi-static dielectric sphere in a uniform field has the
  internal field 3/(eps_r + 2) E0.  The oracle's VIE solve with the
  distributional self term reproduces it within the voxelisation error
  (12^3 grid, 1 cm voxels, r = 5 cm, 1 MHz), which pins the operator
  generation to physics rather than to itself.
"""
import ctypes as ct
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import marie_oracle as O
from marie_gb300 import phantoms

HERE = Path(__file__).resolve().parent
D = ct.POINTER(ct.c_double)


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    so = tmp_path_factory.mktemp("green") / "libhost_shim.so"
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-o", str(so), str(HERE / "host_shim.cpp")],
                   check=True)
    lib = ct.CDLL(str(so))
    lib.shim_add_self_point_term.argtypes = [D, ct.c_longlong, ct.c_int, ct.c_double]
    lib.shim_near_zone_exact.argtypes = [D, ct.c_int, ct.c_int, ct.c_int, ct.c_double, ct.c_double, ct.c_int,
                                         ct.c_int, ct.c_int]
    lib.shim_gauss01.argtypes = [ct.c_int, D, D]
    return lib


@pytest.mark.parametrize("n", [1, 2, 5, 16, 24])
def test_host_gauss_rule(shim, n):
    """The host Gauss-Legendre rule on [0, 1] of the near-zone cubature equals
    numpy's and integrates polynomials of degree 2n-1 exactly."""
    x, w = np.zeros(n), np.zeros(n)
    shim.shim_gauss01(n, x.ctypes.data_as(D), w.ctypes.data_as(D))
    xr, wr = np.polynomial.legendre.leggauss(n)
    assert np.allclose(x, (xr + 1) / 2, atol=1e-15) and np.allclose(w, wr / 2, atol=1e-15)
    for deg in range(2 * n):
        assert abs(np.sum(w * x ** deg) - 1.0 / (deg + 1)) < 1e-14


@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_host_self_point_term_matches_oracle(shim, pwl):
    n, res = (3, 4, 2), 2e-3
    pwx = 10 if pwl else 1
    rng = np.random.default_rng(1)
    A = rng.normal(size=n + (pwx, 6)) + 1j * rng.normal(size=n + (pwx, 6))
    buf = np.ascontiguousarray(A.reshape(-1, order="F")).view(np.float64).copy()
    shim.shim_add_self_point_term(buf.ctypes.data_as(D), int(np.prod(n)), pwx, res)
    got = buf.view(np.complex128).reshape(n + (pwx, 6), order="F")
    want = A.copy()
    want[0, 0, 0] += O.self_delta_term(res, pwx)
    assert np.array_equal(got, want)


K0, RES = O.em_constants(297.2e6)["k0"], 2e-3
NEAR = [(a, b, c) for a in range(2) for b in range(2) for c in range(2)]


@pytest.mark.parametrize("kernel,pwx", [("N", 1), ("N", 10), ("K", 10)])
def test_host_near_zone_matches_oracle(shim, kernel, pwx):
    n = (3, 2, 2)
    nc = 6 if kernel == "N" else 3
    A = np.full(n + (pwx, nc), 7.0 + 1j)                        # far entries must stay untouched
    buf = np.ascontiguousarray(A.reshape(-1, order="F")).view(np.float64).copy()
    shim.shim_near_zone_exact(buf.ctypes.data_as(D), *n, RES, K0, pwx, int(kernel == "N"), 16)
    got = buf.view(np.complex128).reshape(n + (pwx, nc), order="F")
    ref = O.near_zone_relative(K0, RES, pwx, kernel, NEAR, order=16)
    scale = max(np.abs(v).max() for v in ref.values())
    for m in NEAR:
        assert np.abs(got[m] - ref[m]).max() <= 1e-12 * scale, m
    assert np.all(got[2] == 7.0 + 1j)


def test_near_zone_relative_convergence_and_checks():
    r12 = O.near_zone_relative(K0, RES, 10, "N", NEAR, order=12)
    r20 = O.near_zone_relative(K0, RES, 10, "N", NEAR, order=20)
    scale = np.abs(r20[(0, 0, 0)]).max()
    for m in NEAR:
        assert np.abs(r12[m] - r20[m]).max() <= 1e-12 * scale, m
    st = O.near_zone_standin(K0, RES, 10, "N", [(0, 0, 0), (1, 1, 1)])
    v = r20[(1, 1, 1)]
    assert np.abs(st[(1, 1, 1)] - v).max() <= 1e-3 * np.abs(v).max()          # vertex neighbour: converged there
    s0 = st[(0, 0, 0)][0] + O.self_delta_term(RES, 10)[0]                     # PWC moment of the self offset
    assert np.abs(s0 - r20[(0, 0, 0)][0]).max() <= 1e-5 * np.abs(s0).max()
    # axis symmetry of the PWC moment: xx of (1,0,0) = yy of (0,1,0) = zz of (0,0,1), etc.
    assert abs(r20[(1, 0, 0)][0, 0] - r20[(0, 1, 0)][0, 3]) <= 1e-13 * scale
    assert abs(r20[(1, 0, 0)][0, 0] - r20[(0, 0, 1)][0, 5]) <= 1e-13 * scale
    assert abs(r20[(1, 1, 0)][0, 1] - r20[(1, 0, 1)][0, 2]) <= 1e-13 * scale


def _sphere_field(er, self_term, near="standin"):
    res, freq = 1e-2, 1e6
    body = phantoms.sphere(12, res, 0.05, er, 0.0)
    emc = O.em_constants(freq)
    iv = O.assembly_op(*body.n, res, emc["k0"], False, "N", Np_medium=4, self_term=self_term, near=near)
    Mr = body.Mr(freq)
    Mc = Mr - 1
    dims = O.geo_dims(*body.n, body.idxS, False, res)
    Ns = body.idxS.size
    Ue = np.concatenate([np.ones(Ns), np.zeros(Ns), np.zeros(Ns)]).astype(complex)
    b = O.vie_rhs(emc["ce"], Mr, Mc, body.idxS, 3, Ue)
    T = O.assembly_fft_circ_tucker(iv[:, :, :, 0, :], 1e-14)
    cache = {}
    x, it, _ = O.is_gmres_vie(lambda v: O.mvp_vie(v, Mr, Mc, dims, T, cache), b, 50, 1e-8, 200, np.zeros(b.size))
    Mcb = Mr.reshape(-1, order="F")[body.idxS] - 1
    return (x[:Ns] / (emc["ce"] * Mcb)).real          # E_x / E0 in every body voxel (J = ce Mc E)


@pytest.mark.parametrize("er,near", [(50.0, "standin"), (10.0, "standin"), (50.0, "relative")])
def test_quasi_static_sphere_field(er, near):
    """Volume-averaged internal field within 10% of 3/(eps_r + 2) (measured:
    +6.2% at eps_r = 50, +3.5% at 10; the staircase surface of the 12^3
    sphere is the error).  The pointwise self term alone gives 0.35 / 0.40
    of the answer (the depolarising part of the voxel's own field is
    missing).  With the accurate near zone: +6.6% at 12^3, +5.6% at 16^3,
    +3.7% at 20^3 for eps_r = 50 (the staircase error shrinking)."""
    Ex = _sphere_field(er, "distributional", near)
    want = 3.0 / (er + 2.0)
    assert abs(Ex.mean() / want - 1.0) < 0.10, (Ex.mean(), want)
