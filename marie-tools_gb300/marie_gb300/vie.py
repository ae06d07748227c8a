"""Mirror of MARIE's VIE operator/solver call surface on the GB300 library.

The reference builds a table of function handles (parse_inputs.m:6-37) and
calls them from its solver driver:

    func.mvp_N(Jin, fN), func.mvp_K, func.mvp_herm_adj_N/K, func.mvp_G(T,res),
    func.mvp_invG(T,res)
    Jout = mvp_vie(Jb, EP, func, dim, fN)                    (mvp_vie.m:1)
    [x, iter, resvec] = is_gmres_vie(A, b, restart, tol, maxit, x0)
                                                            (is_gmres_vie.m:1)
    [Jb, ...] = ie_solver_vie(MREDM, gpu_flag)               (ie_solver_vie.m:1)

Here the same names take the same arguments, with ``fN`` a
:class:`VieOperator` (the operator handle that replaces ``to_GPU(N)``) and
arrays as CUDA tensors (gpuArray) or numpy arrays (host double); outputs
follow the input, like MATLAB's ``'like'``.  Grids are (n1, n2, n3, C) arrays
in MATLAB (column-major) order.  Errors raise ``MarieError`` (the reference
raises MATLAB errors); there is no CPU fallback.
"""
from __future__ import annotations

import numpy as np

from .operator import VieOperator


def _to_cuda(a, dtype=None):
    import torch
    if isinstance(a, torch.Tensor):
        t = a
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.complex128)))
    if dtype is not None:
        t = t.to(dtype)
    return t.to("cuda")


def _grid_flat(Jin):
    """(n1,n2,n3,C) MATLAB-ordered array -> flat column-major CUDA vector."""
    import torch
    if isinstance(Jin, torch.Tensor):
        t = Jin.permute(*reversed(range(Jin.dim()))).contiguous().reshape(-1)
        return t.to("cuda"), Jin.shape, True
    a = np.asarray(Jin)
    return _to_cuda(a.reshape(-1, order="F")), a.shape, False


def _grid_back(y, shape, was_torch, like):
    if was_torch:
        return y.reshape(tuple(reversed(shape))).permute(*reversed(range(len(shape)))).to(like.device)
    return y.cpu().numpy().reshape(shape, order="F")


def _grid_op(name):
    def fn(Jin, fN: VieOperator):
        flat, shape, was_torch = _grid_flat(Jin)
        y = getattr(fN, name)(flat)
        return _grid_back(y, shape, was_torch, Jin)
    fn.__name__ = name
    return fn


mvp_N = _grid_op("apply_N")
mvp_K = _grid_op("apply_K")
mvp_herm_adj_N = _grid_op("apply_N_adj")
mvp_herm_adj_K = _grid_op("apply_K_adj")


def _gram(pwl, res):
    if not pwl:
        return np.full(3, res ** 3)
    return np.tile(np.array([res ** 3, res ** 3 / 12, res ** 3 / 12, res ** 3 / 12]), 3)


def mvp_G_pwc(T, res):
    """mvp_G_pwc.m:3."""
    return res ** 3 * T


def mvp_invG_pwc(T, res):
    """mvp_invG_pwc.m:3."""
    return (1 / res ** 3) * T


def mvp_G_pwl(T, res):
    """mvp_G_pwl.m:5-9: per-component Gram diagonal on (n1,n2,n3,12)."""
    return T * _gram(True, res).reshape((1,) * (T.ndim - 1) + (-1,))


def mvp_invG_pwl(T, res):
    """mvp_invG_pwl.m:3-7."""
    return T / _gram(True, res).reshape((1,) * (T.ndim - 1) + (-1,))


def assembly_N(n1, n2, n3, res, freq, PWX: int, near: str = "relative"):
    """I_V = assembly_N(MREDM, n1, n2, n3) (assembly_N.m:1-83) on the GPU:
    (n1, n2, n3, pwx, 6) complex, far and medium zones by the reference's
    Gauss rules, near zone by the accurate cubature that matches its DIRECTFN
    surface-surface terms ("standin": the staggered stand-in)."""
    from .operator import assemble_green
    return assemble_green((n1, n2, n3), res, freq, PWX == 1, "N", near=near)


def assembly_K(n1, n2, n3, res, freq, PWX: int, near: str = "relative"):
    """I_V = assembly_K(MREDM, n1, n2, n3) (assembly_K.m) on the GPU:
    (n1, n2, n3, pwx, 3) complex, as :func:`assembly_N`."""
    from .operator import assemble_green
    return assemble_green((n1, n2, n3), res, freq, PWX == 1, "K", near=near)


def parse_inputs(PWX: int) -> dict:
    """The VIE entries of the function-handle table of parse_inputs.m:6-37."""
    pwl = PWX == 1
    return dict(mvp_N=mvp_N, mvp_K=mvp_K, mvp_herm_adj_N=mvp_herm_adj_N, mvp_herm_adj_K=mvp_herm_adj_K,
                mvp_G=mvp_G_pwl if pwl else mvp_G_pwc, mvp_invG=mvp_invG_pwl if pwl else mvp_invG_pwc,
                ie_solver_wsvie=ie_solver_vie)


def mvp_vie(Jb, EP, func, dim, fN: VieOperator):
    """Jout = Jp - (Mc./Mr) .* invG(N Jp) on the body (mvp_vie.m:1-19).

    EP and dim are accepted for signature parity; the contrast and index map
    were bound into ``fN`` when it was created, and dim['N_b'] is checked.
    """
    import torch
    if dim is not None and int(dim.get("N_b", fN.Nb)) != fN.Nb:
        raise ValueError("dim.N_b does not match the operator handle")
    was_torch = isinstance(Jb, torch.Tensor)
    x = _to_cuda(Jb)
    if x.dtype not in (torch.complex64, torch.complex128):
        x = x.to(torch.complex128)
    y = fN.apply(x.reshape(-1)).reshape(x.shape)
    return y if was_torch else y.cpu().numpy()


def is_gmres_vie(A, b, restart, tol, maxit, x0, mode="fp64"):
    """[x, iter, resvec] = is_gmres_vie(A, b, restart, tol, maxit, x0).

    ``A`` is the operator handle (the reference passes the closure
    @(J) mvp_vie(J, EP, func, dims, fN), ie_solver_vie.m:15); ``b`` may hold
    several right-hand sides as columns (N_b x nrhs), solved in one batch.
    Returns x (like b), iter = [p, outit] per rhs and the relative residual
    history (a list per rhs, or one array for a single rhs).  ``mode``:
    "fp64" (the reference's arithmetic), "mixed" (complex64 GMRES per rhs
    inside FP64 refinement) or "block" (the same refinement with one block
    Krylov space for all columns of b; iter then counts block steps).
    """
    import torch
    if not isinstance(A, VieOperator):
        raise TypeError("A must be a VieOperator (the GPU operator handle)")
    was_torch = isinstance(b, torch.Tensor)
    bb = _to_cuda(b, torch.complex128)
    single = bb.dim() == 1
    B = bb.reshape(A.Nb, -1) if not single else bb.reshape(A.Nb, 1)
    nrhs = B.shape[1]
    Bc = B.t().contiguous().reshape(-1)      # rhs-major for the C ABI
    X0 = None
    if x0 is not None:
        xx = _to_cuda(x0, torch.complex128).reshape(A.Nb, nrhs)
        if torch.count_nonzero(xx) > 0:
            X0 = xx.t().contiguous().reshape(-1)
    x, rep = A.gmres(Bc, X0, restart=restart, tol=tol, maxit=maxit, mode=mode)
    X = x.reshape(nrhs, A.Nb).t()
    it = np.stack([rep.last_inner, rep.outer], axis=1)
    if single:
        X = X.reshape(-1)
        it, resvec = it[0], rep.resvec[0]
    else:
        resvec = rep.resvec
    return (X if was_torch else X.cpu().numpy()), it, resvec


def ie_solver_vie(fN: VieOperator, Ue, ce, Mr, Mc, idxS, tol, restart=50, maxit=200, mode="fp64", X=None):
    """[Jb, U_hat_inv, S_hat_inv, V_hat_inv] = ie_solver_vie(MREDM, gpu_flag)
    (ie_solver_vie.m:1-32) with the port loop batched:
    rhs = ce * repmat((1./Mr(idxS)).*Mc(idxS), ql, 1) .* Ue(:, i) for all i,
    solved from Jb = 0 (:16-21).  ``X`` is MREDM.BASIS.X (N_ports x r) when
    the excitation basis carries one: then Zbb_hat_inv = X.'*((Ue.'*Jb)*X)
    (plain transposes) and its economy SVD are returned as (U, S, V) with S
    diagonal (:23-25), as numpy arrays; otherwise three empty lists (:27-29).
    Jb follows Ue ((N_b, N_ports); CUDA tensor or numpy)."""
    import torch
    ql = fN.C
    mr = np.asarray(Mr).reshape(-1, order="F")[idxS]
    mc = np.asarray(Mc).reshape(-1, order="F")[idxS]
    chi = np.tile((1.0 / mr) * mc, ql)
    U = _to_cuda(Ue, torch.complex128).reshape(fN.Nb, -1)
    rhs = ce * _to_cuda(chi, torch.complex128)[:, None] * U
    Jd, _it, _rv = is_gmres_vie(fN, rhs, restart, tol, maxit, None, mode=mode)
    Jd = Jd.reshape(fN.Nb, -1)
    Jb = Jd if isinstance(Ue, torch.Tensor) else Jd.cpu().numpy()     # Jb follows Ue
    if X is None:
        return Jb, [], [], []
    UJ = (U.t() @ Jd).cpu().numpy()                # Ue.' * Jb: N_ports x N_ports
    Xn = np.asarray(X, dtype=np.complex128)
    Z = Xn.T @ (UJ @ Xn)
    Uh, S, Vh = np.linalg.svd(Z, full_matrices=False)
    return Jb, Uh, np.diag(S), Vh.conj().T


def _ports(a, op, dtype):
    """(N_b, N_ports) array (MATLAB layout) -> contiguous (N_ports*N_b) CUDA vector."""
    import torch
    A = _to_cuda(a, dtype).reshape(op.Nb, -1)
    return A.t().contiguous().reshape(-1), A.shape[1]


def em_efield_vie_excitation(op: VieOperator, Jb, Ue):
    """em_efield_vie_excitation.m:17-23 for every port at once:
    Ue + mask.*invG((1/ce)(mvp_N(Jb) - mvp_G(Jb))) on the body.  Jb, Ue:
    (N_b, N_ports); returns (N_b, N_ports) complex128 on the GPU."""
    import torch
    J, npt = _ports(Jb, op, torch.complex128)
    U, _ = _ports(Ue, op, torch.complex128)
    E, _h = op.fields(J, Ue=U, e=True, h=False)
    return E.reshape(npt, op.Nb).t()


def em_hfield_vie_excitation(op: VieOperator, Jb, Ub):
    """em_hfield_vie_excitation.m:16-22: Ub + mask.*invG(mvp_K(Jb)) on the body."""
    import torch
    J, npt = _ports(Jb, op, torch.complex128)
    U, _ = _ports(Ub, op, torch.complex128)
    _e, H = op.fields(J, Ub=U, e=False, h=True)
    return H.reshape(npt, op.Nb).t()


def em_ehfield_vie(op: VieOperator, Jb, Ue, Ub):
    """Field part of em_ehfield_vie.m:31-52: total E and H fields per port and
    the noise-covariance matrix phi; the ultimate-SNR/TXE metrics that follow
    (em_ehfield_vie.m:54-) are outside this library."""
    import torch
    J, npt = _ports(Jb, op, torch.complex128)
    Ut, _ = _ports(Ue, op, torch.complex128)
    Bt, _ = _ports(Ub, op, torch.complex128)
    E, H = op.fields(J, Ue=Ut, Ub=Bt)
    phi = op.absorbed_power(J)
    return E.reshape(npt, op.Nb).t(), H.reshape(npt, op.Nb).t(), phi


def b1_objective(op: VieOperator, J, Ue, Ub, roi):
    """J_obj = mean_ROI |B1+|^2 / P_abs of one solved current J (complex128
    CUDA, N_b): B1+ = mu0 (H_x + i H_y) (em_ehfield_vie.m:68), P_abs =
    phi(1,1)/2 (em_ehfield_vie.m:44-52).  roi: body-voxel indices (0-based,
    into idxS).  Returns (J_obj, M, P, E, H, b1)."""
    import torch
    E, H = op.fields(J, Ue=Ue, Ub=Ub)
    b1 = op.b1_plus(H)
    r = torch.as_tensor(np.asarray(roi), device="cuda")
    M = float((b1[r].abs() ** 2).mean())
    P = 0.5 * float(op.absorbed_power(J)[0, 0].real)
    return M / P, M, P, E, H, b1


def b1_objective_gradient(op: VieOperator, b, Ue, Ub, roi, *, tol=1e-6, mode="mixed", J=None, solve_op=None):
    """Adjoint gradient of J_obj = mean_ROI |B1+|^2 / P_abs with respect to
    eps_r and sigma of every body voxel, for the solution J of A J = b (one
    right-hand side; J is solved here unless given).  Steps: forward solve,
    fields, B1+ and P; adjoint source g = dJ_obj/dconj(J) (the B1+ part
    through marie_vie_apply_hfield_adjoint); adjoint solve A^H lam = g;
    per-voxel sensitivities (marie_vie_gradient).  ``solve_op`` (default
    ``op``) runs the two GMRES solves: a handle on the same body and
    materials, e.g. one with the float-float complex128 N operator while
    ``op`` holds native complex128 with K.  Returns (J_obj, d_eps, d_sigma,
    J)."""
    import torch
    sop = op if solve_op is None else solve_op
    if J is None:
        J, _rep = sop.gmres(b, tol=tol, mode=mode)
    Jobj, M, P, E, H, b1 = b1_objective(op, J, Ue, Ub, roi)
    Ns, l = op.Ns, 4 if op.pwl else 1
    r = torch.as_tensor(np.asarray(roi), device="cuda")
    w = torch.zeros(op.Nb, dtype=torch.complex128, device="cuda")
    w[r] = b1[r]
    w[l * Ns + r] = -1j * b1[r]
    mu0 = 4e-7 * np.pi
    gM = op.apply_hfield_adjoint(w) * (mu0 / len(roi))
    g = op.gradient_source(J, gM, M, P)
    lam, _repa = sop.gmres(g, tol=tol, mode=mode, adjoint=True)
    de, ds = op.gradient(J, lam, E, M, P)
    return Jobj, de, ds, J


def _b1_objective_function():
    import torch

    class B1Objective(torch.autograd.Function):
        """J_obj = mean_ROI |B1+|^2 / P_abs as a differentiable function of the
        body voxels' eps_r and sigma (float64 tensors of length N_s).  `build`
        (eps_r, sigma as numpy) -> (VieOperator, b, Ue, Ub) creates the
        operator for given materials; backward uses the adjoint sensitivities
        of b1_objective_gradient."""

        @staticmethod
        def forward(ctx, eps_r, sigma, build, roi, tol, mode):
            op, b, Ue, Ub = build(eps_r.detach().cpu().numpy(), sigma.detach().cpu().numpy())
            try:
                Jobj, de, ds, _J = b1_objective_gradient(op, b, Ue, Ub, roi, tol=tol, mode=mode)
            finally:
                op.close()
            ctx.save_for_backward(de.to(eps_r.device), ds.to(sigma.device))
            return torch.tensor(Jobj, dtype=torch.float64, device=eps_r.device)

        @staticmethod
        def backward(ctx, grad_out):
            de, ds = ctx.saved_tensors
            return grad_out * de, grad_out * ds, None, None, None, None

    return B1Objective


def b1_objective_autograd(eps_r, sigma, build, roi, *, tol=1e-6, mode="mixed"):
    """torch.autograd entry point of the B1+ objective (see _b1_objective_function)."""
    return _b1_objective_function().apply(eps_r, sigma, build, roi, tol, mode)
