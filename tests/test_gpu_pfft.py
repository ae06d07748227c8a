"""The coupled coil/body matvec of the pFFT formulation
(marie_svie_pfft_*, mvp_svie_pfft.m:1-19) against the oracle's restatement,
through the C ABI.

Operands are seeded stand-ins with the reference's shapes and structure
(pfft_projection_*_assembly.m and pfft_assemble_voxel_*.m are outside this
library): an extended grid with a body in a sub-box; PS maps each body
unknown onto its own grid unknown (weight 1) and each coil unknown onto a
stencil of 8 grid unknowns with complex weights; Z_cc dense, Z_bc_N sparse;
ext_Mc_inv nonzero on the body voxels only.  The extended grid's N operator
is a synthetic I_V with the physical kernel's circulant parity.
Tolerances: complex128 <= 1e-12, complex64 <= 1e-5 relative.
"""
import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import synthetic_IV, rel_err

torch = pytest.importorskip("torch")
sp = pytest.importorskip("scipy.sparse")


def _operands(n, pwl, n_sie, seed):
    rng = np.random.default_rng(seed)
    n1, n2, n3 = n
    ql = 12 if pwl else 3
    nvox = n1 * n2 * n3
    mask = np.zeros(n, bool)
    mask[1:n1 - 1, 1:n2 - 1, 1:n3 - 1] = rng.uniform(size=(n1 - 2, n2 - 2, n3 - 2)) < 0.7
    idxS = np.nonzero(mask.reshape(-1, order="F"))[0]
    Ns = idxS.size
    N_b = ql * Ns
    idx_solution = np.concatenate([c * nvox + idxS for c in range(ql)])
    ng = nvox * ql
    # body columns: identity embedding; coil columns: 8-point stencils
    rows = list(idx_solution)
    cols = list(n_sie + np.arange(N_b))
    vals = list(np.ones(N_b, complex))
    for c in range(n_sie):
        r = rng.choice(ng, 8, replace=False)
        rows += list(r)
        cols += [c] * 8
        vals += list(rng.normal(size=8) + 1j * rng.normal(size=8))
    PS = sp.csr_matrix((np.array(vals), (np.array(rows), np.array(cols))), shape=(ng, n_sie + N_b))
    Zcc = sp.csr_matrix(rng.normal(size=(n_sie, n_sie)) + 1j * rng.normal(size=(n_sie, n_sie)))
    nz = max(1, int(0.05 * N_b * n_sie))
    Zbc = sp.csr_matrix((rng.normal(size=nz) + 1j * rng.normal(size=nz),
                         (rng.integers(0, N_b, nz), rng.integers(0, n_sie, nz))), shape=(N_b, n_sie))
    mc = np.zeros(n, complex)
    mc[mask] = rng.uniform(0.01, 0.2, Ns) + 1j * rng.uniform(-0.2, 0.0, Ns)
    IV = synthetic_IV(n, pwl, "N", seed + 7)
    Mr = np.where(mask, 40 - 5j, 1.0 + 0j)
    return dict(PS=PS, Zcc=Zcc, Zbc=Zbc, mc=mc, IV=IV, idxS=idxS, idx_solution=idx_solution, Mr=Mr, N_b=N_b,
                ql=ql)


def _grid_op(n, pwl, d, res=5e-3, freq=128e6, precisions=3):
    from marie_gb300 import VieOperator
    return VieOperator(n, res, freq, d["idx_solution"], d["Mr"], d["IV"] if pwl else d["IV"][:, :, :, :1, :],
                       pwl=pwl, precisions=precisions, max_rhs=8)


@pytest.mark.gpu
@pytest.mark.parametrize("pwl", [False, True], ids=["pwc", "pwl"])
@pytest.mark.parametrize("nrhs", [1, 10])
def test_svie_pfft_matches_oracle(pwl, nrhs):
    from marie_gb300.pfft import SviePfftOperator
    n, n_sie, res, freq = (10, 9, 8), 37, 5e-3, 128e6
    d = _operands(n, pwl, n_sie, seed=11 + pwl)
    g = _grid_op(n, pwl, d, res, freq)
    op = SviePfftOperator(g, n_sie, d["PS"], d["Zcc"], d["Zbc"], d["mc"])
    ntot = n_sie + d["N_b"]
    rng = np.random.default_rng(3)
    X = rng.normal(size=(nrhs, ntot)) + 1j * rng.normal(size=(nrhs, ntot))
    ce = O.em_constants(freq)["ce"]
    M1 = np.r_[np.ones(n_sie), -np.ones(d["N_b"])]
    M2 = np.r_[np.zeros(n_sie), np.ones(d["N_b"])]
    IV = d["IV"] if pwl else d["IV"][:, :, :, :1, :]
    spectra = {}
    ref = [O.mvp_svie_pfft(X[r], d["PS"], d["Zcc"], d["Zbc"], d["mc"], IV, M1, M2, ce, n_sie, res,
                           n + (d["ql"],), spectra) for r in range(nrhs)]
    x = torch.from_numpy(X.reshape(-1)).cuda()
    y = op.apply(x).cpu().numpy().reshape(nrhs, ntot)
    y32 = op.apply(x.to(torch.complex64)).cpu().numpy().reshape(nrhs, ntot)
    for r in range(nrhs):
        assert rel_err(y[r], ref[r]) <= 1e-12, r
        assert rel_err(y32[r], ref[r]) <= 1e-5, r
    op.close()
    g.close()


@pytest.mark.gpu
def test_svie_pfft_mirror_and_multipliers():
    """The signature mirror of mvp_svie_pfft.m (numpy in, numpy out), and
    caller-given multipliers."""
    from marie_gb300.pfft import SviePfftOperator, mvp_svie_pfft
    n, n_sie, res, freq = (8, 8, 6), 20, 5e-3, 128e6
    d = _operands(n, True, n_sie, seed=5)
    g = _grid_op(n, True, d, res, freq)
    ntot = n_sie + d["N_b"]
    rng = np.random.default_rng(9)
    Jcb = rng.normal(size=ntot) + 1j * rng.normal(size=ntot)
    M1 = rng.uniform(-1, 1, ntot)
    M2 = rng.uniform(-1, 1, ntot)
    ce = O.em_constants(freq)["ce"]
    ref = O.mvp_svie_pfft(Jcb, d["PS"], d["Zcc"], d["Zbc"], d["mc"], d["IV"], M1, M2, ce, n_sie, res,
                          n + (12,))
    got = mvp_svie_pfft(Jcb, d["PS"], d["Zcc"], d["Zbc"], d["mc"], None, g, M1, M2, None, n_sie, res, n + (12,))
    assert isinstance(got, np.ndarray) and rel_err(got, ref) <= 1e-12
    op = SviePfftOperator(g, n_sie, d["PS"], d["Zcc"], d["Zbc"], d["mc"], M1, M2)
    assert rel_err(op.apply(torch.from_numpy(Jcb).cuda()).cpu().numpy(), ref) <= 1e-12
    op.close()
    g.close()


@pytest.mark.gpu
def test_svie_pfft_four_step_grid_and_bad_args():
    """A 32 x 32 x 48 extended grid (four-step passes, float-float
    complex128) with 400 coil unknowns; and descriptors the create call must
    refuse (shape mismatch, column index out of range)."""
    from marie_gb300 import _lib
    from marie_gb300.pfft import SviePfftOperator
    n, n_sie, res, freq = (32, 32, 48), 400, 2e-3, 297.2e6
    d = _operands(n, False, n_sie, seed=21)
    g = _grid_op(n, False, d, res, freq, precisions=2 | 4)
    op = SviePfftOperator(g, n_sie, d["PS"], d["Zcc"], d["Zbc"], d["mc"])
    ntot = n_sie + d["N_b"]
    rng = np.random.default_rng(4)
    Jcb = rng.normal(size=ntot) + 1j * rng.normal(size=ntot)
    ce = O.em_constants(freq)["ce"]
    M1 = np.r_[np.ones(n_sie), -np.ones(d["N_b"])]
    M2 = np.r_[np.zeros(n_sie), np.ones(d["N_b"])]
    ref = O.mvp_svie_pfft(Jcb, d["PS"], d["Zcc"], d["Zbc"], d["mc"], d["IV"][:, :, :, :1, :], M1, M2, ce, n_sie,
                          res, n + (3,))
    x = torch.from_numpy(Jcb).cuda()
    assert rel_err(op.apply(x).cpu().numpy(), ref) <= 1e-11
    assert rel_err(op.apply(x.to(torch.complex64)).cpu().numpy(), ref) <= 1e-5
    op.close()
    with pytest.raises(_lib.MarieError) as ei:
        SviePfftOperator(g, n_sie, d["PS"][:-1], d["Zcc"], d["Zbc"], d["mc"])
    assert ei.value.status == 1
    with pytest.raises(_lib.MarieError):
        SviePfftOperator(g, n_sie, d["PS"], d["Zcc"][:, :-1], d["Zbc"], d["mc"])
    g.close()
