"""CPU checks of the oracle itself: the restatement is pinned by identities
that hold for the reference's algorithm, and by an independent direct-sum
evaluation of the convolution that mvp_N/mvp_K compute through FFTs."""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, rel_err


def direct_conv(J, IV, pwl, op, adjoint):
    """y_p(r) = sum_q sum_r' s_pq * A_blk(|r-r'|) * mirror signs * x_q(r'),
    evaluated as an explicit O(n^6) sum (no FFT, no Tucker)."""
    n1, n2, n3, C = J.shape
    tab = O.block_table(op, pwl, adjoint)
    nc = 6 if op == "N" else 3
    g1, g2, g3 = O.G_N_SIGNS[nc]
    bt = O.BT_SIGNS
    y = np.zeros_like(J, dtype=complex)
    X, Y, Z = np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3), indexing="ij")
    for p in range(C):
        for q in range(C):
            e = tab[p][q]
            if e is None:
                continue
            s, (j, k), cj = e
            A = IV[:, :, :, j, k] if pwl else IV[:, :, :, 0, k]
            s1 = g1[k] * (bt[0][j] if pwl else 1)
            s2 = g2[k] * (bt[1][j] if pwl else 1)
            s3 = g3[k] * (bt[2][j] if pwl else 1)
            for x in range(n1):
                for yy in range(n2):
                    for z in range(n3):
                        dx, dy, dz = x - X, yy - Y, z - Z
                        blk = A[np.abs(dx), np.abs(dy), np.abs(dz)]
                        if cj:
                            # conj(G_hat) is the spectrum of conj(A_ext(-d))
                            dx, dy, dz = -dx, -dy, -dz
                        sg = np.where(dx < 0, s1, 1) * np.where(dy < 0, s2, 1) * np.where(dz < 0, s3, 1)
                        g = blk * sg
                        if cj:
                            g = g.conj()
                        y[x, yy, z, p] += s * np.sum(g * J[..., q])
    return y


@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("op,adj", [("N", False), ("N", True), ("K", False), ("K", True)])
def test_fft_matvec_equals_direct_sum(pwl, op, adj):
    P = Problem((3, 4, 2), pwl, seed=1)
    J = P.random_grid(seed=4)[0]
    T = P.TN if op == "N" else P.TK
    IV = P.IV_N if op == "N" else P.IV_K
    got = O.mvp_op_tucker(J, T, op, adj)
    ref = direct_conv(J, IV, pwl, op, adj)
    assert rel_err(got, ref) < 1e-12


@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_tucker_exactness(pwl):
    """Reconstructed blocks equal the FFT of the circulant embedding of I_V
    within the HOSVD truncation (hosvd.m cut tol*s1/sqrt(3) per mode)."""
    P = Problem((5, 4, 6), pwl, seed=2)
    for tol in (1e-14, 1e-6):
        T = O.assembly_fft_circ_tucker(P.IV_N if pwl else P.IV_N[:, :, :, 0, :], tol)
        worst = 0.0
        for (j, k), t in T.items():
            s1 = O.G_N_SIGNS[6][0][k] * (O.BT_SIGNS[0][j] if pwl else 1)
            s2 = O.G_N_SIGNS[6][1][k] * (O.BT_SIGNS[1][j] if pwl else 1)
            s3 = O.G_N_SIGNS[6][2][k] * (O.BT_SIGNS[2][j] if pwl else 1)
            A = P.IV_N[:, :, :, j, k]
            ref = O.circ_spectrum_dense(A, s1, s2, s3)
            worst = max(worst, rel_err(O.tucker_block(t), ref))
        assert worst < max(10 * tol, 1e-12)


@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_adjoint_identity(pwl):
    """<A x, y> = <x, A^H y> for A = mvp_vie and A^H from the herm_adj files."""
    P = Problem((4, 5, 3), pwl, seed=3)
    X = P.random_body_vec(seed=1)[0]
    Y = P.random_body_vec(seed=2)[0]
    Ax = O.mvp_vie(X, P.Mr, P.Mc, P.dims, P.TN)
    AHy = O.mvp_vie_adjoint(Y, P.Mr, P.Mc, P.dims, P.TN)
    lhs = np.vdot(Y, Ax)
    rhs = np.vdot(AHy, X)
    assert abs(lhs - rhs) / abs(lhs) < 1e-12


@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_raw_adjoint_identities(pwl):
    P = Problem((4, 3, 5), pwl, seed=4)
    x = P.random_grid(seed=1)[0]
    y = P.random_grid(seed=2)[0]
    for op, T in (("N", P.TN), ("K", P.TK)):
        Ax = O.mvp_op_tucker(x, T, op, False)
        AHy = O.mvp_op_tucker(y, T, op, True)
        lhs = np.vdot(y, Ax)
        rhs = np.vdot(AHy, x)
        assert abs(lhs - rhs) / abs(lhs) < 1e-12, op


def test_physical_N_is_complex_symmetric_pwc():
    """With the physical Green's tensor, N is complex-symmetric (reciprocity):
    <N x, y> = <x, N y> without conjugation (PWC)."""
    n = (3, 3, 3)
    emc = O.em_constants(128e6)
    IV = O.assembly_op(*n, 5e-3, emc["k0"], False, "N")
    T = O.assembly_fft_circ_tucker(IV[:, :, :, 0, :], 1e-14)
    rng = np.random.default_rng(0)
    x = rng.normal(size=n + (3,)) + 1j * rng.normal(size=n + (3,))
    y = rng.normal(size=n + (3,)) + 1j * rng.normal(size=n + (3,))
    Nx = O.mvp_op_tucker(x, T, "N")
    Ny = O.mvp_op_tucker(y, T, "N")
    assert abs(np.sum(y * Nx) - np.sum(x * Ny)) / abs(np.sum(y * Nx)) < 1e-12


def test_gmres_converges_and_matches_direct_solve():
    P = Problem((4, 4, 3), False, seed=5, iv_scale=0.05 * 5e-3 ** 3)
    A = lambda v: O.mvp_vie(v, P.Mr, P.Mc, P.dims, P.TN, cache={})
    Nb = P.dims["N_b"]
    M = np.stack([A(e) for e in np.eye(Nb)], axis=1)
    b = P.random_body_vec(seed=6)[0]
    x, it, rv = O.is_gmres_vie(A, b, 50, 1e-10, 200, np.zeros(Nb))
    xd = np.linalg.solve(M, b)
    assert rv[-1] <= 1e-10
    assert rel_err(x, xd) < 1e-8
    assert it[1] >= 1


def _golden_problem(name):
    from pathlib import Path
    g = Path(__file__).resolve().parent / "golden"
    iv = np.load(g / f"iv_{name}.npz")
    mv = np.load(g / f"mvp_{name}.npz")
    n = tuple(int(v) for v in iv["n"])
    pwl = bool(iv["pwl"])
    emc = O.em_constants(float(iv["freq"]))
    ep = O.em_assembly(mv["er"], mv["se"], emc["ce"])
    dims = O.geo_dims(*n, mv["idxS"], pwl, float(iv["res"]))
    return iv, mv, n, pwl, emc, ep, dims


@pytest.mark.parametrize("name", ["pwc_5", "pwl_4"])
def test_golden_regression(name):
    """The oracle reproduces its committed vectors (tests/golden/make_golden.py)."""
    iv, mv, n, pwl, emc, ep, dims = _golden_problem(name)
    ivN = iv["N"]
    T = O.assembly_fft_circ_tucker(ivN if pwl else ivN[:, :, :, 0, :], float(mv["tucker_tol"]))
    assert rel_err(O.mvp_op_tucker(mv["J"], T, "N"), mv["NJ"]) < 1e-12
    assert rel_err(O.mvp_vie(mv["Jb"], ep["Mr"], ep["Mc"], dims, T), mv["AJ"]) < 1e-12
    cache = {}
    x, it, rv = O.is_gmres_vie(lambda v: O.mvp_vie(v, ep["Mr"], ep["Mc"], dims, T, cache), mv["b"], 50, 1e-8,
                               200, np.zeros(dims["N_b"]))
    assert np.array_equal(it, mv["it"])
    assert rel_err(x, mv["x"]) < 1e-10


def test_golden_assembly_tiny():
    """Green's tensor assembly reproduces the committed I_V (PWC 5^3 grid)."""
    iv = np.load(__import__("pathlib").Path(__file__).resolve().parent / "golden" / "iv_pwc_5.npz")
    emc = O.em_constants(float(iv["freq"]))
    A = O.assembly_op(3, 3, 3, float(iv["res"]), emc["k0"], False, "N")
    # grids of different size share every offset both contain except the medium rule
    # order (n <= 5 uses min(n)); compare the near zone and the 5^3 case directly
    ref = iv["N"]
    for m in [(0, 0, 0), (1, 0, 0), (1, 1, 0), (1, 1, 1)]:
        assert rel_err(A[m], ref[m]) < 1e-12


def test_gmres_restart_bookkeeping():
    """Small restart forces several cycles; the final residual estimate is
    below tol and the true residual agrees with it."""
    iv, mv, n, pwl, emc, ep, dims = _golden_problem("pwc_5")
    T = O.assembly_fft_circ_tucker(iv["N"][:, :, :, 0, :], 1e-7)
    cache = {}
    A = lambda v: O.mvp_vie(v, ep["Mr"], ep["Mc"], dims, T, cache=cache)
    b = mv["b"]
    x, it, rv = O.is_gmres_vie(A, b, 5, 1e-8, 400, np.zeros(b.size))
    assert it[1] > 1
    true = np.linalg.norm(b - A(x)) / np.linalg.norm(b)
    assert rv[-1] <= 1e-8
    assert abs(true - rv[-1]) < 1e-9


def test_field_postprocessing_oracle_identities():
    """E/H post-processing and the noise covariance of the oracle: zero
    currents return the incident fields, the fields are linear in J, and phi
    is Hermitian (em_ehfield_vie.m:44-52)."""
    P = Problem((6, 5, 4), True, seed=4)
    rng = np.random.default_rng(0)
    Nb = P.dims["N_b"]
    J1, J2, U = (rng.normal(size=Nb) + 1j * rng.normal(size=Nb) for _ in range(3))
    ce = P.emc["ce"]
    assert np.allclose(O.em_efield_vie_excitation(0 * J1, U, P.dims, P.TN, ce), U)
    e = lambda J: O.em_efield_vie_excitation(J, 0 * U, P.dims, P.TN, ce)
    h = lambda J: O.em_hfield_vie_excitation(J, 0 * U, P.dims, P.TK)
    assert rel_err(e(J1 + 2 * J2), e(J1) + 2 * e(J2)) < 1e-13
    assert rel_err(h(J1 - 3j * J2), h(J1) - 3j * h(J2)) < 1e-13
    phi = O.em_noise_covariance(np.stack([J1, J2, U], 1), P.Mc, ce, P.dims)
    assert np.allclose(phi, phi.conj().T, rtol=1e-13, atol=0)


@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_dense_block_products_equal_tucker_restatement(pwl):
    """mvp_op_dense (block spectra formed from dense I_V one at a time, the
    configuration-size checker) equals mvp_op_tucker on a full-rank Tucker
    form of the same blocks, for N, N^H, K, K^H and mvp_vie."""
    from helpers import Problem, rel_err
    P = Problem((6, 5, 4), pwl, seed=3)
    J = P.random_grid(seed=1)[0]
    for op, adj in [("N", False), ("N", True), ("K", False), ("K", True)]:
        IV, T = (P.IV_N, P.TN) if op == "N" else (P.IV_K, P.TK)
        assert rel_err(O.mvp_op_dense(J, IV, op, adj), O.mvp_op_tucker(J, T, op, adj)) <= 1e-13
    Jb = P.random_body_vec(seed=2)[0]
    spectra = {}
    a = O.mvp_vie_dense(Jb, P.Mr, P.Mc, P.dims, P.IV_N, spectra=spectra)
    assert len(spectra) == (60 if pwl else 6)
    assert rel_err(a, O.mvp_vie(Jb, P.Mr, P.Mc, P.dims, P.TN)) <= 1e-13
    assert rel_err(O.mvp_vie_dense(Jb, P.Mr, P.Mc, P.dims, P.IV_N, spectra=spectra), a) == 0.0


def test_mvp_svie_pfft_restatement_against_dense_matrices():
    """oracle.mvp_svie_pfft (mvp_svie_pfft.m:1-19) against the same formula
    written with dense matrices on a 3 x 3 x 2 PWC extended grid: N as the
    matrix of mvp_N on the grid's unit vectors, G as the Gram diagonal."""
    import scipy.sparse as sp
    from helpers import synthetic_IV, rel_err
    rng = np.random.default_rng(0)
    n, ql, n_sie, res, ce = (3, 3, 2), 3, 4, 5e-3, 1j * 0.01
    nvox = 18
    ng = nvox * ql
    idxS = np.array([4, 5, 13])
    N_b = ql * idxS.size
    IV = synthetic_IV(n, False, "N", 3)
    Nmat = np.zeros((ng, ng), complex)
    for j in range(ng):
        e = np.zeros(ng, complex)
        e[j] = 1
        Nmat[:, j] = O.mvp_op_dense(e.reshape(n + (ql,), order="F"), IV, "N").reshape(-1, order="F")
    PSd = np.zeros((ng, n_sie + N_b), complex)
    PSd[np.concatenate([c * nvox + idxS for c in range(ql)]), n_sie + np.arange(N_b)] = 1
    PSd[:, :n_sie] = (rng.uniform(size=(ng, n_sie)) < 0.2) * (rng.normal(size=(ng, n_sie)) + 1j)
    Zcc = rng.normal(size=(n_sie, n_sie)) + 1j * rng.normal(size=(n_sie, n_sie))
    Zbc = rng.normal(size=(N_b, n_sie)) + 1j * rng.normal(size=(N_b, n_sie))
    mc = np.zeros(n, complex)
    mc.reshape(-1, order="F")[idxS] = rng.normal(size=idxS.size) + 1j * rng.normal(size=idxS.size)
    M1 = np.r_[np.ones(n_sie), -np.ones(N_b)]
    M2 = np.r_[np.zeros(n_sie), np.ones(N_b)]
    x = rng.normal(size=n_sie + N_b) + 1j * rng.normal(size=n_sie + N_b)
    got = O.mvp_svie_pfft(x, sp.csr_matrix(PSd), sp.csr_matrix(Zcc), sp.csr_matrix(Zbc), mc, IV, M1, M2, ce,
                          n_sie, res, n + (ql,))
    G = res ** 3 * np.eye(ng)
    Mcd = np.diag(np.tile(mc.reshape(-1, order="F"), ql))
    xb = np.r_[np.zeros(n_sie), x[n_sie:]]
    want = (M1 * (PSd.T @ ((Nmat - G) @ (PSd @ x))) + M2 * (PSd.T @ (G @ (Mcd @ (PSd @ xb))))) / ce
    want += np.r_[Zcc @ x[:n_sie] + Zbc.T @ x[n_sie:], -(Zbc @ x[:n_sie])]
    assert rel_err(got, want) <= 1e-13
