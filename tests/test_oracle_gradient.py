"""The adjoint sensitivities of the B1+ objective J_obj = mean_ROI |B1+|^2 /
P_abs, restated in the oracle (b1_objective_gradient), against central
finite differences of the oracle objective (CPU; dense solves on a 4^3 PWL
grid with synthetic operators; relative step 1e-4, eight voxels, both
parameters; measured agreement 2e-9 to 2e-7 relative).  Finite differences
do not use the adjoint formula, so this checks the derivation the GPU
kernels implement."""
import numpy as np

from oracle import marie_oracle as O
from helpers import Problem

MU0 = 4e-7 * np.pi


def _dense(fn, n):
    cols = []
    for i in range(n):
        e = np.zeros(n, dtype=complex)
        e[i] = 1.0
        cols.append(fn(e))
    return np.stack(cols, axis=1)


def test_oracle_b1_gradient_matches_finite_differences():
    P = Problem((4, 4, 4), True, seed=3, iv_scale=0.3)
    dims, TN, TK = P.dims, P.TN, P.TK
    ce = P.emc["ce"]
    nb, ns, ql = dims["N_b"], dims["N_scat"], dims["ql"]
    cache = {}
    invg = np.repeat(O.invG_scale(True, dims["res"]), ns)
    # B = invG N on the body; mvp_vie(J) = J - chi * (B J) (mvp_vie.m:12-18)
    B = _dense(lambda x: invg * O.gather(O.mvp_op_tucker(O.scatter(x, dims), TN, "N", False, cache), dims), nb)
    rng = np.random.default_rng(11)
    Ue = rng.normal(size=nb) + 1j * rng.normal(size=nb)
    Ub = 1e-3 * (rng.normal(size=nb) + 1j * rng.normal(size=nb))
    roi = np.arange(0, ns, 3)
    g_body = np.unravel_index(dims["idxS"], P.n, order="F")

    def state(er, se):
        ep = O.em_assembly(er, se, ce)
        Mr, Mc = ep["Mr"], ep["Mc"]
        mr = Mr.reshape(-1, order="F")[dims["idxS"]]
        chi = np.tile((Mr.reshape(-1, order="F")[dims["idxS"]] - 1.0) / mr, ql)
        A = np.eye(nb) - chi[:, None] * B
        b = O.vie_rhs(ce, Mr, Mc, dims["idxS"], ql, Ue)
        return Mr, Mc, A, np.linalg.solve(A, b)

    er0, se0 = P.er.copy(), P.se.copy()
    Mr, Mc, A, J = state(er0, se0)
    x = rng.normal(size=nb) + 1j * rng.normal(size=nb)
    assert np.allclose(A @ x, O.mvp_vie(x, Mr, Mc, dims, TN, cache), rtol=1e-12, atol=1e-12 * np.abs(x).max())
    Jobj, M, Pabs, E, H, b1 = O.b1_objective(J, Ue, Ub, dims, TN, TK, Mc, ce, roi, MU0, cache)
    de, ds, lam = O.b1_objective_gradient(J, E, b1, M, Pabs, Mr, Mc, ce, dims, TK, roi, MU0,
                                          lambda g: np.linalg.solve(A.conj().T, g), cache)

    def objective(er, se):
        Mr2, Mc2, _A2, J2 = state(er, se)
        return O.b1_objective(J2, Ue, Ub, dims, TN, TK, Mc2, ce, roi, MU0, cache)[0]

    vox = rng.choice(ns, size=min(8, ns), replace=False)
    for s in vox:
        g = tuple(int(a[s]) for a in g_body)
        for which, ref in (("er", de), ("se", ds)):
            er, se = er0.copy(), se0.copy()
            arr = er if which == "er" else se
            h = 1e-4 * arr[g]
            arr[g] += h
            fp = objective(er, se)
            arr[g] -= 2 * h
            fm = objective(er, se)
            fd = (fp - fm) / (2 * h)
            assert abs(fd - ref[s]) <= 1e-6 * abs(fd) + 1e-9 * np.abs(ref).max(), (which, s, fd, ref[s])
