"""Limits and failure paths of the C ABI on the GPU.

* Grids whose generic passes need narrower row tiles to fit one CTA's shared
  memory still run (and agree with the oracle); grids that cannot fit at all
  are refused by marie_vie_create with MARIE_ERR_BAD_ARG before any launch.
* The device-memory cap (marie_vie_desc.mem_cap_bytes) turns an allocation
  beyond it into MARIE_ERR_OOM, at create and for the GMRES workspace.
* An Arnoldi step whose new vector is exactly zero (the Krylov space closes:
  is_iter_gmres_vie.m:19-21 divides by H(k+1,k) = 0) ends the cycle with the
  exact solution and no non-finite value, as the oracle's restatement does.
"""
import ctypes as ct

import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, flat_F, unflat_F, rel_err

torch = pytest.importorskip("torch")


@pytest.mark.gpu
def test_wide_x_edge_runs_with_narrowed_tiles():
    """864 x 16 x 2 PWC in complex64: the x pass' default 16-row tile would
    need 240 KB of shared memory; the tile is narrowed and the result equals
    the oracle's mvp_N.  The allocation-free entry agrees with it."""
    from marie_gb300 import _lib
    n = (864, 16, 2)
    P = Problem(n, False, seed=3)
    op = P.gpu_operator(precisions=2, max_rhs=1)
    J = P.random_grid(seed=4)[0]
    x = torch.from_numpy(flat_F(J)).to("cuda", torch.complex64)
    y = op.apply_N(x).cpu().numpy().astype(np.complex128)
    ref = O.mvp_op_tucker(J, P.TN, "N", False, cache={})
    assert rel_err(unflat_F(y, n, 3), ref) <= 1e-5
    op.close()
    # the same grid through marie_vie_apply_N_noalloc (octant spectrum input)
    M = 8.0 * n[0] * n[1] * n[2]
    blocks = [np.transpose(O.tucker_block(P.TN[(0, k)])[: n[0] + 1, : n[1] + 1, : n[2] + 1], (1, 0, 2)) / M
              for k in range(6)]
    G = torch.from_numpy(np.ascontiguousarray(np.stack(blocks)).astype(np.complex64)).cuda()
    yn = torch.empty_like(x)
    lib = _lib.load()
    st = lib.marie_vie_apply_N_noalloc(*n, 0, ct.c_void_p(G.data_ptr()), ct.c_void_p(x.data_ptr()),
                                       ct.c_void_p(yn.data_ptr()), ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, _lib.last_error()
    assert rel_err(unflat_F(yn.cpu().numpy().astype(np.complex128), n, 3), ref) <= 1e-5


@pytest.mark.gpu
def test_create_refuses_grid_beyond_shared_memory():
    """complex128 PWL with n3 = 600: the z pass holds 12 components x 600
    points x 2 halves of 16 bytes per column (> 227 KB) even with a one-column
    tile, so create refuses it with MARIE_ERR_BAD_ARG and a message."""
    from marie_gb300 import VieOperator, _lib
    n = (2, 2, 600)
    idx = np.arange(4)       # voxel 0..3 of slice 0, PWL: 12 blocks of N_s
    idxS = idx.astype(np.int64)
    dims = O.geo_dims(*n, idxS, True, 5e-3)
    Mr = np.ones(n, complex) * (10 - 1j)
    IV = np.zeros(n + (10, 6), complex)
    IV[0, 0, 0, 0, 0] = 1e-9
    with pytest.raises(_lib.MarieError) as ei:
        VieOperator(n, 5e-3, 128e6, dims["idx_solution"], Mr, IV, pwl=True, precisions=1, max_rhs=1)
    assert ei.value.status == 1
    assert "shared memory" in str(ei.value)
    # complex64 fits (8-byte elements)
    op = VieOperator(n, 5e-3, 128e6, dims["idx_solution"], Mr, IV, pwl=True, precisions=2, max_rhs=1)
    op.close()


@pytest.mark.gpu
def test_memory_cap_gives_oom():
    from marie_gb300 import _lib
    P = Problem((8, 8, 8), False, seed=2, iv_scale=0.02)
    with pytest.raises(_lib.MarieError) as ei:
        P.gpu_operator(precisions=1, max_rhs=1, mem_cap_bytes=1024)
    assert ei.value.status == 2 and "cap" in str(ei.value)
    # smallest cap (to 4 KB) that admits create: the GMRES workspace is beyond it
    lo, hi = 1024, 1 << 30
    while hi - lo > 4096:
        mid = (lo + hi) // 2
        try:
            P.gpu_operator(precisions=1, max_rhs=1, mem_cap_bytes=mid).close()
            hi = mid
        except _lib.MarieError as e:
            assert e.status == 2
            lo = mid
    op = P.gpu_operator(precisions=1, max_rhs=1, mem_cap_bytes=hi)
    b = torch.from_numpy(P.random_body_vec(seed=1)[0]).cuda()
    with pytest.raises(_lib.MarieError) as ei:
        op.gmres(b, restart=20, tol=1e-8, maxit=5, mode="fp64")
    assert ei.value.status == 2 and "cap" in str(ei.value)
    op.close()
    # without the cap the same solve runs (allocates its workspace and iterates)
    op = P.gpu_operator(precisions=1, max_rhs=1)
    x, rep = op.gmres(b, restart=20, tol=1e-8, maxit=3, mode="fp64")
    assert rep.status[0] in (0, 4) and rep.iters[0] > 0 and np.isfinite(rep.true_resid[0])
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_arnoldi_breakdown_is_exact(mode):
    """Zero Green's tensor: mvp_vie is the identity on the body; with a unit
    right-hand side the first Arnoldi vector is mapped onto itself and
    H(2,1) = ||w - H(1,1) v_1|| is exactly 0.  The cycle ends after one
    iteration with x = b, residual 0 and no NaN, like the oracle."""
    n = (6, 5, 4)
    P = Problem(n, True, seed=9)
    Z = np.zeros_like(P.IV_N)
    from marie_gb300 import VieOperator
    op = VieOperator(n, P.res, P.freq, P.dims["idx_solution"], P.Mr, Z, pwl=True,
                     precisions=3, max_rhs=2)
    Nb = P.dims["N_b"]
    B = np.zeros((2, Nb), complex)
    B[0, 7] = 1.0
    B[1, Nb - 1] = 0.5j
    b = torch.from_numpy(B.reshape(-1)).cuda()
    x, rep = op.gmres(b, restart=10, tol=1e-6, maxit=5, mode=mode)
    X = x.cpu().numpy().reshape(2, Nb)
    assert rep.ok, rep.status
    assert np.all(np.isfinite(X))
    np.testing.assert_array_equal(rep.iters, [1, 1])
    assert np.max(rep.true_resid) == 0.0
    np.testing.assert_allclose(X, B, rtol=0, atol=1e-15)
    # the oracle's restatement of is_gmres_vie on the same (identity) operator
    T = O.assembly_fft_circ_tucker(Z, 1e-14)
    A = lambda v: O.mvp_vie(v, P.Mr, P.Mc, P.dims, T, cache={})
    with np.errstate(invalid="ignore", divide="ignore"):
        xo, it, rv = O.is_gmres_vie(A, B[0], 10, 1e-6, 5, np.zeros(Nb, complex))
    assert rel_err(X[0], xo) <= 1e-15
    assert list(it) == [1, 1]
    op.close()
