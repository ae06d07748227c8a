"""GPU parity of the FFT-VIE operator against the CPU oracle (through the C ABI).

Tolerances: complex128 path <= 1e-12 relative (2-norm over the whole output);
complex64 path <= 1e-5 relative.
"""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, flat_F, unflat_F, rel_err

torch = pytest.importorskip("torch")

TOL = {"c128": 1e-12, "c64": 1e-5}
SIZES = [(6, 5, 4), (8, 8, 8), (12, 10, 7), (11, 6, 13), (1, 4, 3)]
OPS = [("N", False), ("N", True), ("K", False), ("K", True)]


def _dt(prec):
    return torch.complex128 if prec == "c128" else torch.complex64


_CACHE = {}


def _problem(n, pwl):
    key = (n, pwl)
    if key not in _CACHE:
        _CACHE[key] = Problem(n, pwl, seed=sum(n) + 7 * pwl)
    return _CACHE[key]


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("n", SIZES, ids=lambda n: "x".join(map(str, n)))
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_grid_operators(n, pwl, prec):
    P = _problem(n, pwl)
    op = P.gpu_operator()
    J = P.random_grid(seed=3, nrhs=2)
    x = torch.from_numpy(np.concatenate([flat_F(J[r]) for r in range(2)])).to("cuda", _dt(prec))
    for name, adj in OPS:
        T = P.TN if name == "N" else P.TK
        fn = {("N", False): op.apply_N, ("N", True): op.apply_N_adj,
              ("K", False): op.apply_K, ("K", True): op.apply_K_adj}[(name, adj)]
        y = fn(x).cpu().numpy().astype(np.complex128)
        for r in range(2):
            ref = O.mvp_op_tucker(J[r], T, name, adj, cache={})
            got = unflat_F(y[r * J[r].size:(r + 1) * J[r].size], n, P.C)
            e = rel_err(got, ref)
            assert e <= TOL[prec], f"{name}{'_adj' if adj else ''} rhs {r}: rel err {e:.3e}"
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_vie_apply_and_adjoint(pwl, prec):
    n = (8, 7, 6)
    P = _problem(n, pwl)
    op = P.gpu_operator()
    X = P.random_body_vec(seed=5, nrhs=3)
    x = torch.from_numpy(X.reshape(-1)).to("cuda", _dt(prec))
    y = op.apply(x).cpu().numpy().reshape(3, -1).astype(np.complex128)
    ya = op.apply_adjoint(x).cpu().numpy().reshape(3, -1).astype(np.complex128)
    for r in range(3):
        ref = O.mvp_vie(X[r], P.Mr, P.Mc, P.dims, P.TN, cache={})
        refa = O.mvp_vie_adjoint(X[r], P.Mr, P.Mc, P.dims, P.TN, cache={})
        assert rel_err(y[r], ref) <= TOL[prec]
        assert rel_err(ya[r], refa) <= TOL[prec]
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
def test_dense_equals_tucker(pwl):
    """Operator built from dense I_V (no truncation) equals the Tucker path
    built with a full-rank truncation tolerance."""
    n = (6, 6, 5)
    P = _problem(n, pwl)
    opT = P.gpu_operator(precisions=1)
    opD = P.gpu_operator(precisions=1, dense=True)
    x = torch.from_numpy(P.random_body_vec(seed=9).reshape(-1)).to("cuda")
    assert rel_err(opT.apply(x).cpu().numpy(), opD.apply(x).cpu().numpy()) <= 1e-12
    opT.close()
    opD.close()


@pytest.mark.gpu
def test_batched_equals_single():
    P = _problem((8, 8, 8), True)
    op = P.gpu_operator(max_rhs=2)   # workspace for 2 -> 5 rhs run in 3 chunks
    X = P.random_body_vec(seed=11, nrhs=5)
    x = torch.from_numpy(X.reshape(-1)).to("cuda")
    yb = op.apply(x).cpu().numpy().reshape(5, -1)
    for r in range(5):
        ys = op.apply(torch.from_numpy(X[r]).to("cuda")).cpu().numpy()
        assert np.array_equal(ys, yb[r])      # same kernels, same order: bit-identical
    op.close()


@pytest.mark.gpu
def test_rerun_bit_identical():
    P = _problem((12, 10, 7), True)
    op = P.gpu_operator()
    x = torch.from_numpy(P.random_body_vec(seed=2).reshape(-1)).to("cuda", torch.complex64)
    a = op.apply(x).cpu().numpy()
    b = op.apply(x).cpu().numpy()
    assert np.array_equal(a, b)
    op.close()


@pytest.mark.gpu
def test_rejects_operator_without_circulant_parity():
    from marie_gb300 import VieOperator
    from marie_gb300._lib import MarieError
    P = _problem((6, 5, 4), True)
    rng = np.random.default_rng(0)
    bad = rng.normal(size=P.IV_N.shape) + 1j * rng.normal(size=P.IV_N.shape)
    with pytest.raises(MarieError, match="parity"):
        VieOperator(P.n, P.res, P.freq, P.dims["idx_solution"], P.Mr, bad, pwl=True, precisions=1)
    Tbad = O.assembly_fft_circ_tucker(bad, 1e-14)
    with pytest.raises(MarieError, match="parity"):
        VieOperator(P.n, P.res, P.freq, P.dims["idx_solution"], P.Mr, Tbad, pwl=True, precisions=1)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pwc_5", "pwl_4"])
def test_physical_operator_parity(name):
    """Assembled (physical) Green's tensors from the committed fixtures."""
    from pathlib import Path
    from marie_gb300 import VieOperator
    g = Path(__file__).resolve().parent / "golden"
    iv = np.load(g / f"iv_{name}.npz")
    mv = np.load(g / f"mvp_{name}.npz")
    n = tuple(int(v) for v in iv["n"])
    pwl = bool(iv["pwl"])
    emc = O.em_constants(float(iv["freq"]))
    ep = O.em_assembly(mv["er"], mv["se"], emc["ce"])
    dims = O.geo_dims(*n, mv["idxS"], pwl, float(iv["res"]))
    T = O.assembly_fft_circ_tucker(iv["N"] if pwl else iv["N"][:, :, :, 0, :], float(mv["tucker_tol"]))
    op = VieOperator(n, float(iv["res"]), float(iv["freq"]), dims["idx_solution"], ep["Mr"], T, pwl=pwl)
    for prec, dt in (("c128", torch.complex128), ("c64", torch.complex64)):
        y = op.apply(torch.from_numpy(mv["Jb"]).to("cuda", dt)).cpu().numpy()
        assert rel_err(y, mv["AJ"]) <= TOL[prec]
        yN = op.apply_N(torch.from_numpy(flat_F(mv["J"])).to("cuda", dt)).cpu().numpy()
        assert rel_err(unflat_F(yN, n, 12 if pwl else 3), mv["NJ"]) <= TOL[prec]
    op.close()


FAST_SIZES = [(16, 16, 16), (32, 16, 48), (48, 32, 16)]


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("n", FAST_SIZES, ids=lambda n: "x".join(map(str, n)))
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_four_step_path(n, pwl, prec, monkeypatch):
    """Grids with edges 16*NB take the four-step register FFT path for N and
    N^H; it must match the oracle and the generic shared-memory path."""
    P = _problem(n, pwl)
    op = P.gpu_operator(max_rhs=4)
    J = P.random_grid(seed=8, nrhs=3)
    x = torch.from_numpy(np.concatenate([flat_F(J[r]) for r in range(3)])).to("cuda", _dt(prec))
    for name, adj, fn in (("N", False, op.apply_N), ("N", True, op.apply_N_adj)):
        y = fn(x).cpu().numpy().astype(np.complex128)
        monkeypatch.setenv("MARIE_GENERIC_FFT", "1")
        yg = fn(x).cpu().numpy().astype(np.complex128)
        monkeypatch.delenv("MARIE_GENERIC_FFT")
        for r in range(3):
            ref = O.mvp_op_tucker(J[r], P.TN, name, adj, cache={})
            sl = slice(r * J[r].size, (r + 1) * J[r].size)
            assert rel_err(unflat_F(y[sl], n, P.C), ref) <= TOL[prec]
            assert rel_err(y[sl], yg[sl]) <= TOL[prec]
    X = P.random_body_vec(seed=6, nrhs=5)
    xb = torch.from_numpy(X.reshape(-1)).to("cuda", _dt(prec))
    yb = op.apply(xb).cpu().numpy().reshape(5, -1).astype(np.complex128)
    for r in range(5):
        assert rel_err(yb[r], O.mvp_vie(X[r], P.Mr, P.Mc, P.dims, P.TN, cache={})) <= TOL[prec]
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("n3", [64, 80, 96, 112, 128])
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_four_step_z_lengths(n3, pwl, prec):
    """z lengths 16*NB for NB = 4..8 (the z pass is compiled per NB): N and
    N^H on a 16 x 16 x n3 grid against the oracle, 3 right-hand sides."""
    n = (16, 16, n3)
    P = _problem(n, pwl)
    op = P.gpu_operator(max_rhs=4)
    J = P.random_grid(seed=9, nrhs=3)
    x = torch.from_numpy(np.concatenate([flat_F(J[r]) for r in range(3)])).to("cuda", _dt(prec))
    for name, adj, fn in (("N", False, op.apply_N), ("N", True, op.apply_N_adj)):
        y = fn(x).cpu().numpy().astype(np.complex128)
        for r in range(3):
            ref = O.mvp_op_tucker(J[r], P.TN, name, adj, cache={})
            sl = slice(r * J[r].size, (r + 1) * J[r].size)
            assert rel_err(unflat_F(y[sl], n, P.C), ref) <= TOL[prec], (name, adj, r)
    op.close()
    _CACHE.pop((n, pwl), None)


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("precisions,prec", [(3, "c128"), (3, "c64"), (6, "c128")], ids=["c128", "c64", "c128ff"])
def test_pruned_passes_on_a_partial_body(pwl, precisions, prec, monkeypatch):
    """A body inside a sub-box leaves grid rows and z slices without body
    voxels: the four-step passes skip them (inputs are zero there, outputs
    are not needed).  Results equal the unpruned passes and the oracle."""
    n = (32, 16, 48)
    P = Problem(n, pwl, seed=31 + pwl, box=((3, 21), (2, 11), (6, 40)))
    # a hole: slices 15..19 and rows y = 5 hold no body voxel either
    keep = []
    for s_ in P.idxS:
        x, r = s_ % n[0], s_ // n[0]
        y, z = r % n[1], r // n[1]
        keep.append(not (15 <= z < 20 or y == 5))
    P2 = Problem.__new__(Problem)
    P2.__dict__.update(P.__dict__)
    P2.idxS = P.idxS[np.array(keep)]
    P2.dims = O.geo_dims(*n, P2.idxS, pwl, P.res)
    op = P2.gpu_operator(precisions=precisions, max_rhs=4)
    X = P2.random_body_vec(seed=2, nrhs=3)
    x = torch.from_numpy(X.reshape(-1)).to("cuda", _dt(prec))
    y = op.apply(x).cpu().numpy()
    ya = op.apply_adjoint(x).cpu().numpy()
    monkeypatch.setenv("MARIE_NO_PRUNE", "1")
    yu = op.apply(x).cpu().numpy()
    yau = op.apply_adjoint(x).cpu().numpy()
    monkeypatch.delenv("MARIE_NO_PRUNE")
    assert np.array_equal(y, yu) and np.array_equal(ya, yau)
    tol = 1e-11 if precisions == 6 else TOL[prec]
    y = y.reshape(3, -1).astype(np.complex128)
    for r in range(3):
        ref = O.mvp_vie(X[r], P2.Mr, P2.Mc, P2.dims, P2.TN, cache={})
        assert rel_err(y[r], ref) <= tol
    op.close()
