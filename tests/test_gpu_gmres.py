"""GPU GMRES against the oracle's restatement of is_gmres_vie.m.

FP64 path: same iteration counts and restart bookkeeping as the oracle, x
within 1e-9 relative, resvec within 1e-7 (Krylov recurrences amplify the
1e-16 per-matvec differences).  Mixed path: FP64 true residual <= tol and
field error <= 1e-5 against the FP64 oracle solution.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import rel_err

torch = pytest.importorskip("torch")
GOLD = Path(__file__).resolve().parent / "golden"


def _case(name):
    from marie_gb300 import VieOperator
    iv = np.load(GOLD / f"iv_{name}.npz")
    mv = np.load(GOLD / f"mvp_{name}.npz")
    n = tuple(int(v) for v in iv["n"])
    pwl = bool(iv["pwl"])
    emc = O.em_constants(float(iv["freq"]))
    ep = O.em_assembly(mv["er"], mv["se"], emc["ce"])
    dims = O.geo_dims(*n, mv["idxS"], pwl, float(iv["res"]))
    T = O.assembly_fft_circ_tucker(iv["N"] if pwl else iv["N"][:, :, :, 0, :], float(mv["tucker_tol"]))
    op = VieOperator(n, float(iv["res"]), float(iv["freq"]), dims["idx_solution"], ep["Mr"], T, pwl=pwl,
                     precisions=3, max_rhs=4)
    cache = {}
    A = lambda v: O.mvp_vie(v, ep["Mr"], ep["Mc"], dims, T, cache)
    return op, A, mv, dims, emc, ep


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pwc_5", "pwl_4"])
@pytest.mark.parametrize("restart", [50, 7])
def test_fp64_matches_oracle(name, restart):
    op, A, mv, dims, emc, ep = _case(name)
    b = mv["b"]
    tol = 1e-8
    xr, itr, rvr = O.is_gmres_vie(A, b, restart, tol, 200, np.zeros(b.size))
    x, rep = op.gmres(torch.from_numpy(b).cuda(), restart=restart, tol=tol, maxit=200, mode="fp64")
    assert rep.ok
    assert int(rep.outer[0]) == int(itr[1])
    assert int(rep.last_inner[0]) == int(itr[0])
    assert len(rep.resvec[0]) == len(rvr)
    assert np.allclose(rep.resvec[0], rvr, rtol=1e-7, atol=1e-14)
    assert rel_err(x.cpu().numpy(), xr) < 1e-9
    true = np.linalg.norm(b - A(xr)) / np.linalg.norm(b)
    assert abs(rep.true_resid[0] - true) < 1e-9
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pwc_5", "pwl_4"])
def test_mixed_reaches_tol_with_field_error(name):
    op, A, mv, dims, emc, ep = _case(name)
    b = mv["b"]
    xr, itr, rvr = O.is_gmres_vie(A, b, 50, 1e-12, 200, np.zeros(b.size))
    x, rep = op.gmres(torch.from_numpy(b).cuda(), restart=50, tol=1e-6, maxit=200, mode="mixed")
    assert rep.ok and rep.status[0] == 0
    assert rep.true_resid[0] <= 1e-6
    assert rep.matvecs_c64 > 0 and rep.matvecs_c128 >= 1
    assert rel_err(x.cpu().numpy(), xr) <= 1e-5
    op.close()


@pytest.mark.gpu
def test_batched_rhs_equal_single():
    op, A, mv, dims, emc, ep = _case("pwl_4")
    rng = np.random.default_rng(3)
    B = np.stack([mv["b"], rng.normal(size=mv["b"].size) + 1j * rng.normal(size=mv["b"].size), 0.5 * mv["b"]])
    xb, repb = op.gmres(torch.from_numpy(B.reshape(-1)).cuda(), restart=20, tol=1e-8, mode="fp64")
    xb = xb.cpu().numpy().reshape(3, -1)
    for r in range(3):
        xs, reps = op.gmres(torch.from_numpy(B[r]).cuda(), restart=20, tol=1e-8, mode="fp64")
        assert np.array_equal(xs.cpu().numpy(), xb[r])
        assert repb.iters[r] == reps.iters[0]
    op.close()


@pytest.mark.gpu
def test_warm_start_and_maxit():
    op, A, mv, dims, emc, ep = _case("pwc_5")
    b = mv["b"]
    x0 = 0.9 * mv["x"]
    xr, itr, rvr = O.is_gmres_vie(A, b, 10, 1e-9, 200, x0)
    x, rep = op.gmres(torch.from_numpy(b).cuda(), torch.from_numpy(x0).cuda(), restart=10, tol=1e-9, mode="fp64")
    assert int(rep.outer[0]) == int(itr[1]) and rel_err(x.cpu().numpy(), xr) < 1e-9
    # maxit = 1 cycle of 3 iterations cannot reach 1e-12: status NOT_CONVERGED, residual reported
    x, rep = op.gmres(torch.from_numpy(b).cuda(), restart=3, tol=1e-12, maxit=1, mode="fp64")
    assert not rep.ok and rep.status[0] == 4 and rep.iters[0] == 3
    assert 0 < rep.true_resid[0] < 1
    op.close()


@pytest.mark.gpu
def test_nonfinite_rhs_is_rejected():
    from marie_gb300._lib import MarieError
    op, A, mv, dims, emc, ep = _case("pwc_5")
    b = mv["b"].copy()
    b[3] = np.nan
    with pytest.raises(MarieError, match="NONFINITE"):
        op.gmres(torch.from_numpy(b).cuda(), restart=10, tol=1e-8, mode="fp64")
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [None, "1", "2", "3"], ids=["default", "c1", "c2", "c3"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_host_buffer_solve_equals_device_solve(mode, chunk, monkeypatch):
    """marie_gmres_vie_host (chunked, copies overlapped) returns the device
    solve's result for every right-hand side, with and without x0, and with
    more right-hand sides than one chunk; MARIE_HOST_CHUNK 1-3 gives the
    uneven schedules (7 right-hand sides in chunks of 3: 1 + 3 + 2 + 1)."""
    if chunk is not None:
        monkeypatch.setenv("MARIE_HOST_CHUNK", chunk)
    op, A, mv, dims, emc, ep = _case("pwl_4")
    rng = np.random.default_rng(5)
    nrhs = 7
    B = np.stack([mv["b"] * (1 + 0.1 * r) + 0.01 * (rng.normal(size=mv["b"].size) + 1j * rng.normal(size=mv["b"].size))
                  for r in range(nrhs)])
    bd = torch.from_numpy(B.reshape(-1)).cuda()
    xd, repd = op.gmres(bd, restart=20, tol=1e-8, mode=mode)
    bh = torch.from_numpy(B.reshape(-1)).pin_memory()
    xh, reph = op.gmres_host(bh, restart=20, tol=1e-8, mode=mode)
    assert np.array_equal(xh.numpy(), xd.cpu().numpy())
    assert np.array_equal(reph.iters, repd.iters) and np.array_equal(reph.true_resid, repd.true_resid)
    x0 = (0.5 * xd).cpu().contiguous()
    xh2, _ = op.gmres_host(bh, x0.clone(), restart=20, tol=1e-8, mode=mode)
    xd2, _ = op.gmres(bd, (0.5 * xd).contiguous(), restart=20, tol=1e-8, mode=mode)
    assert np.array_equal(xh2.numpy(), xd2.cpu().numpy())
    op.close()
