"""Host algebra of the block GMRES solver (csrc/blocklsq.h) against numpy:
the per-column residual norms of min_Y ||[S0; 0] - Hbar_j Y||_F after every
block step j, the final Y and the residual block Z = [S0; 0] - Hbar Y, and
the Cholesky factor / triangular inverse used by the block QR.  Compiled with
the host compiler (no GPU); p = 64 runs the reflector updates on host threads."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "marie-tools_gb300", "csrc")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("blsq") / "block_lsq_driver")
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-I", CSRC, os.path.join(HERE, "block_lsq_driver.cpp"),
                    "-o", exe], check=True)
    return exe


def _case(p, m, seed, tiny_cols=()):
    rng = np.random.default_rng(seed)
    cz = lambda *s: rng.normal(size=s) + 1j * rng.normal(size=s)
    ld = (m + 1) * p
    H = np.zeros((ld, m * p), complex)
    for j in range(m):
        H[:(j + 1) * p, j * p:(j + 1) * p] = cz((j + 1) * p, p)
        H[(j + 1) * p:(j + 2) * p, j * p:(j + 1) * p] = np.triu(cz(p, p)) + 3 * np.eye(p)
    for c in tiny_cols:                      # nearly dependent directions (a converged column)
        H[(m) * p + c, (m - 1) * p + c] *= 1e-12
    S0 = np.triu(cz(p, p)) + 2 * np.eye(p)
    B = cz(3 * p, p)
    A = B.conj().T @ B
    return S0, H, A


def _run(driver, tmp_path, p, m, S0, H, A):
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fin, "wb") as f:
        np.array([p, m], np.int32).tofile(f)
        for a in (S0, H, A):
            np.asfortranarray(a).reshape(-1, order="F").astype(np.complex128).tofile(f)
    subprocess.run([driver, fin, fout], check=True)
    raw = open(fout, "rb").read()
    off = 0

    def take(dtype, n):
        nonlocal off
        a = np.frombuffer(raw, dtype, n, off)
        off += a.nbytes
        return a
    res = take(np.float64, m * p).reshape(m, p)
    Y = take(np.complex128, m * p * p).reshape(m * p, p, order="F")
    Z = take(np.complex128, (m + 1) * p * p).reshape((m + 1) * p, p, order="F")
    ok = int(take(np.int32, 1)[0])
    R = take(np.complex128, p * p).reshape(p, p, order="F")
    I = take(np.complex128, p * p).reshape(p, p, order="F")
    return res, Y, Z, ok, R, I


@pytest.mark.parametrize("p,m", [(1, 6), (3, 5), (8, 4), (16, 3), (64, 3)])
def test_block_least_squares_matches_numpy(driver, tmp_path, p, m):
    S0, H, A = _case(p, m, seed=10 * p + m)
    res, Y, Z, ok, R, I = _run(driver, tmp_path, p, m, S0, H, A)
    ld = (m + 1) * p
    E = np.zeros((ld, p), complex)
    E[:p] = S0
    for j in range(m):
        rows, cols = (j + 2) * p, (j + 1) * p
        Yj = np.linalg.lstsq(H[:rows, :cols], E[:rows], rcond=None)[0]
        rj = np.linalg.norm(E[:rows] - H[:rows, :cols] @ Yj, axis=0)
        np.testing.assert_allclose(res[j], rj, rtol=1e-9, atol=1e-12 * np.linalg.norm(S0))
    Yr = np.linalg.lstsq(H, E, rcond=None)[0]
    np.testing.assert_allclose(Y, Yr, rtol=1e-9, atol=1e-10 * np.abs(Yr).max())
    np.testing.assert_allclose(Z, E - H @ Yr, rtol=1e-8, atol=1e-10 * np.linalg.norm(S0))
    # Cholesky: A = R^H R, R upper; R R^{-1} = I
    assert ok == 1
    np.testing.assert_allclose(np.triu(R), R)
    np.testing.assert_allclose(R.conj().T @ R, A, rtol=1e-10, atol=1e-10 * np.abs(A).max())
    np.testing.assert_allclose(I, np.eye(p), atol=1e-10)


def test_nearly_dependent_block_and_indefinite_gram(driver, tmp_path):
    """A sub-diagonal entry at 1e-12 (a column whose residual has converged)
    keeps the residual norms finite and equal to numpy's; a Gram matrix that is
    not positive definite is refused."""
    p, m = 4, 3
    S0, H, A = _case(p, m, seed=3, tiny_cols=(1,))
    A = A - (np.linalg.eigvalsh(A).min() + 1.0) * np.eye(p)
    res, Y, Z, ok, R, I = _run(driver, tmp_path, p, m, S0, H, A)
    assert ok == 0
    ld = (m + 1) * p
    E = np.zeros((ld, p), complex)
    E[:p] = S0
    rj = np.linalg.norm(E - H @ np.linalg.lstsq(H, E, rcond=None)[0], axis=0)
    assert np.all(np.isfinite(res))
    np.testing.assert_allclose(res[-1], rj, rtol=1e-7, atol=1e-12)
