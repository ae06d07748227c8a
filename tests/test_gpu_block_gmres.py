"""Block GMRES (mode "block", MARIE_SOLVE_MIXED_BLOCK) against the oracle.

The reference solves the ports one at a time with is_gmres_vie
(ie_solver_vie.m:16-21); the block solver lets the right-hand sides of each
refinement step share one block Krylov space (complex64, FP64 refinement),
so its iteration history differs by design.  Parity is that of the solve:
the oracle's own FP64 residual ||b - A x|| / ||b|| of the GPU solution is
<= tol and equals the GPU-reported true residual to 1e-9, and the solution
is within 1e-5 of the oracle's FP64 GMRES solution (run to 1e-12).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import rel_err

torch = pytest.importorskip("torch")
GOLD = Path(__file__).resolve().parent / "golden"


def _case(name, max_rhs=4):
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
                     precisions=3, max_rhs=max_rhs)
    cache = {}
    A = lambda v: O.mvp_vie(v, ep["Mr"], ep["Mc"], dims, T, cache)
    return op, A, mv


def _rhs(mv, nrhs, seed):
    rng = np.random.default_rng(seed)
    b = mv["b"]
    cols = [b, rng.normal(size=b.size) + 1j * rng.normal(size=b.size), 0.5 * b + 0.1 * rng.normal(size=b.size)]
    while len(cols) < nrhs:
        cols.append(rng.normal(size=b.size) + 1j * rng.normal(size=b.size))
    return np.stack(cols[:nrhs])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pwc_5", "pwl_4"])
@pytest.mark.parametrize("block_steps", [20, 3])
def test_block_solve_matches_oracle(name, block_steps):
    op, A, mv = _case(name)
    B = _rhs(mv, 4, seed=1)
    x, rep = op.gmres(torch.from_numpy(B.reshape(-1)).cuda(), restart=50, tol=1e-6, maxit=200, mode="block",
                      block_steps=block_steps)
    assert rep.ok and np.all(rep.status == 0)
    assert rep.matvecs_c64 > 0 and rep.matvecs_c128 >= 1
    X = x.cpu().numpy().reshape(4, -1)
    for r in range(4):
        xr, _, _ = O.is_gmres_vie(A, B[r], 50, 1e-12, 200, np.zeros(B.shape[1]))
        true = np.linalg.norm(B[r] - A(X[r])) / np.linalg.norm(B[r])
        assert true <= 1e-6, (r, true)
        assert abs(rep.true_resid[r] - true) <= 1e-9
        assert rel_err(X[r], xr) <= 1e-5, r
        assert rep.resvec[r][-1] <= 1e-6
    if block_steps == 3:
        assert np.all(rep.outer >= 2)          # restarted block cycles
    op.close()


@pytest.mark.gpu
def test_block_single_rhs_host_buffers_and_adjoint():
    """One right-hand side (the block solver with p = 1), the host-buffer
    entry (one chunk holding every right-hand side) and the adjoint solve
    A^H x = b against the complex128 GPU solve of the same system."""
    op, A, mv = _case("pwl_4")
    B = _rhs(mv, 3, seed=2)
    x1, rep1 = op.gmres(torch.from_numpy(B[0]).cuda(), tol=1e-6, mode="block")
    xr, _, _ = O.is_gmres_vie(A, B[0], 50, 1e-12, 200, np.zeros(B.shape[1]))
    assert rep1.ok and rel_err(x1.cpu().numpy(), xr) <= 1e-5
    bd = torch.from_numpy(B.reshape(-1)).cuda()
    xd, repd = op.gmres(bd, tol=1e-6, mode="block", block_steps=10)
    hb = torch.from_numpy(B.reshape(-1)).pin_memory()
    xh, reph = op.gmres_host(hb, tol=1e-6, mode="block", block_steps=10)
    assert reph.ok and rel_err(xh.numpy(), xd.cpu().numpy()) <= 1e-12
    assert list(reph.iters) == list(repd.iters)
    xa, repa = op.gmres(bd, tol=1e-6, mode="block", adjoint=True)
    xf, repf = op.gmres(bd, tol=1e-10, mode="fp64", adjoint=True)
    assert repa.ok and repf.ok
    Xa, Xf = xa.cpu().numpy().reshape(3, -1), xf.cpu().numpy().reshape(3, -1)
    for r in range(3):
        assert rel_err(Xa[r], Xf[r]) <= 1e-5, r
    op.close()


@pytest.mark.gpu
def test_block_bad_args():
    from marie_gb300 import _lib
    op, A, mv = _case("pwc_5")
    b = torch.from_numpy(mv["b"]).cuda()
    for kw in ({"block_steps": -1}, {"block_steps": 201}):
        with pytest.raises(_lib.MarieError) as ei:
            op.gmres(b, mode="block", raise_on_fail=True, **kw)
        assert ei.value.status == 1
    op.close()


@pytest.mark.gpu
def test_block_solves_on_concurrent_streams():
    """Two handles solving in block mode at once from two host threads, each
    on its own stream (each handle's pinned staging area and GEMM handle are
    its own): every solve converges and matches the same solve run alone."""
    import threading
    cases = [_case("pwl_4"), _case("pwc_5")]
    rhs = [torch.from_numpy(_rhs(mv, 3, seed=5 + k).reshape(-1)).cuda() for k, (_, _, mv) in enumerate(cases)]
    seq = [op.gmres(b, tol=1e-6, mode="block", block_steps=4)[0].cpu() for (op, _, _), b in zip(cases, rhs)]
    out, errs = [None, None], []

    def work(k):
        try:
            st = torch.cuda.Stream()
            with torch.cuda.stream(st):
                for _ in range(3):
                    x, rep = cases[k][0].gmres(rhs[k], tol=1e-6, mode="block", block_steps=4)
                    assert rep.ok
                st.synchronize()
                out[k] = x.cpu()
        except Exception as e:
            errs.append(e)

    th = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs, errs
    for k in range(2):     # cuBLAS may pick other GEMM algorithms with several streams active
        assert rel_err(out[k].numpy(), seq[k].numpy()) <= 1e-5, k
    for op, _, _ in cases:
        op.close()


@pytest.mark.gpu
def test_block_warm_start_and_not_converged():
    """A warm start (x0 near the solution) needs fewer block steps than a cold
    one and still meets tol by the oracle's residual; one short cycle per
    refinement step and one refinement step end with MARIE_ERR_NOT_CONVERGED
    per right-hand side, reported, not raised."""
    op, A, mv = _case("pwl_4")
    B = _rhs(mv, 2, seed=9)
    bd = torch.from_numpy(B.reshape(-1)).cuda()
    xc, repc = op.gmres(bd, tol=1e-6, mode="block", block_steps=8)
    X = np.stack([O.is_gmres_vie(A, B[r], 50, 1e-12, 200, np.zeros(B.shape[1]))[0] for r in range(2)])
    x0 = torch.from_numpy((0.999 * X).reshape(-1)).cuda()
    xw, repw = op.gmres(bd, x=x0.clone(), tol=1e-6, mode="block", block_steps=8)
    assert repc.ok and repw.ok
    assert repw.matvecs_c64 < repc.matvecs_c64
    Xw = xw.cpu().numpy().reshape(2, -1)
    for r in range(2):
        assert np.linalg.norm(B[r] - A(Xw[r])) / np.linalg.norm(B[r]) <= 1e-6
    xn, repn = op.gmres(bd, tol=1e-10, maxit=1, max_refine=1, mode="block", block_steps=2)
    assert not repn.ok and np.all(repn.status == 4)
    assert np.all(repn.true_resid > 1e-10)
    op.close()


@pytest.mark.gpu
def test_block_solve_with_tensor_core_projections(tmp_path):
    """The block solver with its projections on the tcgen05 kernel
    (MARIE_BLOCK_PROJ=tcgen05, read once per process: run in a child
    process) reaches tol by the oracle's residual."""
    import os
    import subprocess
    import sys
    root = Path(__file__).resolve().parent.parent
    script = tmp_path / "solve.py"
    script.write_text(
        "import sys, numpy as np, torch\n"
        f"sys.path[:0] = [{str(root)!r}, {str(root / 'marie-tools_gb300')!r}, {str(root / 'tests')!r}]\n"
        "from test_gpu_block_gmres import _case, _rhs\n"
        "op, A, mv = _case('pwl_4')\n"
        "B = _rhs(mv, 4, seed=1)\n"
        "x, rep = op.gmres(torch.from_numpy(B.reshape(-1)).cuda(), tol=1e-6, mode='block', block_steps=6)\n"
        "X = x.cpu().numpy().reshape(4, -1)\n"
        "r = max(np.linalg.norm(B[k] - A(X[k])) / np.linalg.norm(B[k]) for k in range(4))\n"
        "print('RESULT', int(rep.ok), r)\n")
    env = dict(os.environ, MARIE_BLOCK_PROJ="tcgen05")
    out = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, env=env, timeout=600,
                         cwd=str(root / "tests"))
    assert out.returncode == 0, out.stderr[-2000:]
    line = [l for l in out.stdout.splitlines() if l.startswith("RESULT")][-1].split()
    assert int(line[1]) == 1 and float(line[2]) <= 1e-6, line


@pytest.mark.gpu
def test_block_solve_more_than_64_rhs():
    """70 right-hand sides in one block (above the tensor-core kernel's 64:
    the cuBLAS path for every GEMM), two block steps per cycle."""
    op, A, mv = _case("pwl_4", max_rhs=70)
    n = mv["b"].size
    assert n > 140
    rng = np.random.default_rng(12)
    B = rng.normal(size=(70, n)) + 1j * rng.normal(size=(70, n))
    x, rep = op.gmres(torch.from_numpy(B.reshape(-1)).cuda(), tol=1e-6, mode="block", block_steps=2)
    assert rep.ok and np.all(rep.status == 0)
    X = x.cpu().numpy().reshape(70, -1)
    for r in (0, 33, 69):
        assert np.linalg.norm(B[r] - A(X[r])) / np.linalg.norm(B[r]) <= 1e-6, r
    op.close()
