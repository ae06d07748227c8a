"""The point term of the N kernel at the self offset, on the CPU.

* The library's host helper (marie-tools_gb300/csrc/green_host.h, through
  tests/host_shim.cpp) adds exactly the oracle's self_delta_term to
  I_V(0,0,0) (PWC and PWL).
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
    return lib


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


def _sphere_field(er, self_term):
    res, freq = 1e-2, 1e6
    body = phantoms.sphere(12, res, 0.05, er, 0.0)
    emc = O.em_constants(freq)
    iv = O.assembly_op(*body.n, res, emc["k0"], False, "N", Np_medium=4, self_term=self_term)
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


@pytest.mark.parametrize("er", [50.0, 10.0])
def test_quasi_static_sphere_field(er):
    """Volume-averaged internal field within 10% of 3/(eps_r + 2) (measured:
    +6.2% at eps_r = 50, +3.5% at 10; the staircase surface of the 12^3
    sphere is the error).  The pointwise self term alone gives 0.35 / 0.40
    of the answer (the depolarising part of the voxel's own field is
    missing)."""
    Ex = _sphere_field(er, "distributional")
    want = 3.0 / (er + 2.0)
    assert abs(Ex.mean() / want - 1.0) < 0.10, (Ex.mean(), want)
