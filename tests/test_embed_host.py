"""Grid embedding on the CPU: the host helpers that restate a grid's operator
data on a larger FFT grid (marie-tools_gb300/csrc/embed.h), and the
identity they rely on, checked with the oracle.

* embed_dims: which grids are embedded and in what.
* embed_factor: a Tucker factor of the n-grid circulant (FFT of
  [u, 0, s u(n-1..1)]) moved to the m-grid circulant equals the FFT of the
  zero-padded factor's extension, for both mirror signs.
* pad_grid / remap_voxel: layouts of I_V, Mr and idx_solution.
* The oracle's mvp_vie on the caller's grid equals mvp_vie on the embedded
  grid with the zero-padded I_V (PWC and PWL), i.e. embedding is exact.
"""
import ctypes as ct
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, rel_err

HERE = Path(__file__).resolve().parent
D = ct.POINTER(ct.c_double)
I3 = ct.c_int * 3


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    so = tmp_path_factory.mktemp("embed") / "libhost_shim.so"
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-o", str(so), str(HERE / "host_shim.cpp")],
                   check=True)
    lib = ct.CDLL(str(so))
    lib.shim_embed_factor.argtypes = [D, ct.c_int, ct.c_int, ct.c_int, D]
    lib.shim_pad_grid.argtypes = [D, ct.c_void_p, ct.c_void_p, ct.c_longlong, ct.c_double, D]
    lib.shim_remap.argtypes = [ct.c_longlong, ct.c_void_p, ct.c_void_p]
    lib.shim_remap.restype = ct.c_longlong
    return lib


def _dims(lib, n, force=False):
    m = I3()
    r = lib.shim_embed_dims(I3(*n), int(force), m)
    return bool(r), tuple(m)


def _p(a):
    return a.ctypes.data_as(D)


def test_embed_dims(shim):
    # edges with a prime factor above 31 force embedding; all edges <= 128 ->
    # multiples of 16 (the four-step grid), otherwise the next 31-smooth edge
    assert _dims(shim, (73, 73, 84)) == (True, (80, 80, 96))      # the reference's cylinder body
    assert _dims(shim, (37, 10, 9)) == (True, (48, 16, 16))
    assert _dims(shim, (200, 37, 64)) == (True, (200, 38, 64))
    assert _dims(shim, (1021, 8, 8)) == (True, (1023, 8, 8))
    # smooth grids run as given unless forced
    assert _dims(shim, (121, 121, 121)) == (False, (121, 121, 121))
    assert _dims(shim, (121, 121, 121), True) == (True, (128, 128, 128))
    assert _dims(shim, (5, 6, 7), True) == (True, (16, 16, 16))
    assert _dims(shim, (32, 48, 128), True)[0] is False
    assert _dims(shim, (300, 7, 5), True) == (False, (300, 7, 5))


@pytest.mark.parametrize("r,n,m,s", [(3, 5, 16, 1), (4, 37, 48, -1), (2, 73, 80, 1), (5, 7, 38, -1), (1, 1, 16, 1)])
def test_embed_factor_matches_zero_padded_extension(shim, r, n, m, s):
    rng = np.random.default_rng(n + m)
    u = rng.normal(size=(n, r)) + 1j * rng.normal(size=(n, r))
    U = np.fft.fft(np.concatenate([u, np.zeros((1, r)), s * u[n - 1:0:-1]], axis=0), axis=0).T   # r x 2n
    Uf = np.ascontiguousarray(U.reshape(-1, order="F")).view(np.float64)
    out = np.zeros(2 * r * 2 * m)
    shim.shim_embed_factor(_p(Uf), r, n, m, _p(out))
    got = out.view(np.complex128).reshape((r, 2 * m), order="F")
    up = np.concatenate([u, np.zeros((m - n, r))], axis=0)
    want = np.fft.fft(np.concatenate([up, np.zeros((1, r)), s * up[m - 1:0:-1]], axis=0), axis=0).T
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def test_pad_grid_and_remap(shim):
    rng = np.random.default_rng(2)
    n, m = (5, 4, 3), (16, 16, 8)
    A = rng.normal(size=n + (2,)) + 1j * rng.normal(size=n + (2,))
    Af = np.ascontiguousarray(A.reshape(-1, order="F")).view(np.float64)
    out = np.zeros(2 * int(np.prod(m)) * 2)
    shim.shim_pad_grid(_p(Af), I3(*n), I3(*m), 2, 1.0, _p(out))
    want = np.ones(m + (2,), complex)
    want[:5, :4, :3] = A
    assert np.array_equal(out.view(np.complex128).reshape(m + (2,), order="F"), want)
    for i, j, k in [(0, 0, 0), (4, 3, 2), (2, 1, 1), (4, 0, 2)]:
        assert shim.shim_remap(i + 5 * (j + 4 * k), I3(*n), I3(*m)) == i + 16 * (j + 16 * k)


@pytest.mark.parametrize("n,m,pwl", [((7, 5, 6), (16, 16, 16), False), ((5, 4, 3), (8, 16, 9), True)],
                         ids=["pwc", "pwl"])
def test_oracle_embedding_is_exact(n, m, pwl):
    """mvp_vie on the caller's grid == mvp_vie on the larger grid whose I_V
    is the caller's, zero-padded, with the body at the same (i, j, k)."""
    P = Problem(n, pwl, seed=11, tucker_tol=0.0)
    pad = np.zeros(m + P.IV_N.shape[3:], complex)
    pad[:n[0], :n[1], :n[2]] = P.IV_N
    Tm = O.assembly_fft_circ_tucker(pad if pwl else pad[:, :, :, 0, :], 0.0)
    i, j, k = np.unravel_index(P.idxS, n, order="F")
    idxm = np.ravel_multi_index((i, j, k), m, order="F").astype(np.int64)
    Mrm = np.ones(m, complex)
    Mrm[:n[0], :n[1], :n[2]] = P.Mr
    dm = O.geo_dims(*m, idxm, pwl, P.res)
    X = P.random_body_vec(seed=4)[0]
    ref = O.mvp_vie(X, P.Mr, P.Mc, P.dims, P.TN, cache={})
    got = O.mvp_vie(X, Mrm, Mrm - 1, dm, Tm, cache={})
    assert rel_err(got, ref) <= 1e-12
