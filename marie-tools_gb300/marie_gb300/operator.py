"""VieOperator: a handle on the GB300 FFT-VIE operator (libmarie_gb300.so).

Device memory is plain ``torch`` CUDA tensors (plumbing only); every operator
application and solve runs in the library's CUDA kernels.  Grids are flat
column-major (x fastest) vectors of length n1*n2*n3*C per right-hand side;
body vectors have length N_b = C*N_s in idx_solution order.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import C128, C64, PWC, PWL, SOLVE_FP64, SOLVE_MIXED, SOLVE_MIXED_BLOCK, check


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_lib.c_double_p)


def _cplx_f(a) -> np.ndarray:
    """Complex128 array in column-major order, viewed as interleaved doubles."""
    a = np.asarray(a, dtype=np.complex128)
    return np.ascontiguousarray(a.reshape(-1, order="F")).view(np.float64)


@dataclass
class SolveReport:
    iters: np.ndarray
    outer: np.ndarray
    last_inner: np.ndarray
    true_resid: np.ndarray
    resvec: list
    status: np.ndarray
    matvecs_c128: int
    matvecs_c64: int
    ok: bool = field(default=True)


class VieOperator:
    """Operator handle: body map, contrast, Green's-tensor spectra, workspaces.

    Parameters mirror the reference's operator data: grid edges, basis
    (PWC/PWL), voxel edge ``res``, frequency, ``idx_solution`` (0-based,
    component-major), the relative permittivity map ``Mr`` (em_assembly.m:14)
    and the N (and optionally K) operator either as Tucker blocks
    {(j, k): (G, U1, U2, U3)} (assembly_fft_circ_tucker_*.m output) or as a
    dense I_V array (n1, n2, n3, pwx, 6|3).

    ``precisions`` is a bit mask of the device states to build: 1 native
    complex128, 2 complex64, 4 complex128 evaluated in float-float arithmetic
    (grid edges 16*NB with NB <= 8, N and N^H only; exclusive with 1).
    complex128 calls run on whichever complex128 state was built.
    """

    def __init__(self, dims, res, freq, idx_solution, Mr, N, K=None, *, pwl: bool,
                 precisions: int = 3, max_rhs: int = 1, mem_cap_bytes: int = 0):
        self._lib = _lib.load()
        self.n1, self.n2, self.n3 = (int(v) for v in dims)
        self.pwl = bool(pwl)
        self.C = 12 if self.pwl else 3
        self.res, self.freq = float(res), float(freq)
        idx = np.ascontiguousarray(np.asarray(idx_solution, dtype=np.int64))
        self.Nb = int(idx.size)
        self.Ns = self.Nb // self.C
        self.nD = self.n1 * self.n2 * self.n3
        self._keep = []          # host arrays that must outlive create()
        d = _lib.VieDesc()
        d.n1, d.n2, d.n3 = self.n1, self.n2, self.n3
        d.basis = PWL if self.pwl else PWC
        d.res, d.freq = self.res, self.freq
        d.n_b = self.Nb
        d.idx_solution = idx.ctypes.data_as(ct.POINTER(ct.c_int64))
        mr = _cplx_f(np.asarray(Mr).reshape(self.n1, self.n2, self.n3, order="F"))
        d.Mr = _dptr(mr)
        self._keep += [idx, mr]
        tN, dN = self._op_arg(N, 6)
        d.tucker_N, d.dense_N = tN, dN
        if K is not None:
            tK, dK = self._op_arg(K, 3)
            d.tucker_K, d.dense_K = tK, dK
        d.precisions, d.max_rhs, d.mem_cap_bytes = int(precisions), int(max_rhs), int(mem_cap_bytes)
        h = ct.c_void_p()
        check(self._lib.marie_vie_create(ct.byref(h), ct.byref(d)))
        self._h = h
        self._keep = None
        self.precisions = precisions

    def _op_arg(self, op, ncomp):
        pwx = 10 if self.pwl else 1
        if isinstance(op, dict):
            arr = (_lib.TuckerBlock * (pwx * ncomp))()
            for j in range(pwx):
                for k in range(ncomp):
                    G, U1, U2, U3 = op[(j, k)]
                    t = arr[j * ncomp + k]
                    t.r1, t.r2, t.r3 = G.shape
                    bufs = [_cplx_f(G), _cplx_f(U1), _cplx_f(U2), _cplx_f(U3)]
                    self._keep += bufs
                    t.G, t.U1, t.U2, t.U3 = (_dptr(b) for b in bufs)
            self._keep.append(arr)
            return ct.cast(arr, ct.POINTER(_lib.TuckerBlock)), None
        A = np.asarray(op)
        if A.shape != (self.n1, self.n2, self.n3, pwx, ncomp) and not (
                not self.pwl and A.shape == (self.n1, self.n2, self.n3, ncomp)):
            raise ValueError(f"dense operator has shape {A.shape}")
        buf = _cplx_f(A)
        self._keep.append(buf)
        return None, _dptr(buf)

    # -- lifetime ---------------------------------------------------------
    def release_workspace(self):
        """Free the GMRES workspace kept between solves."""
        check(self._lib.marie_vie_release_workspace(self._h))

    def set_materials(self, Mr_body):
        """Replace the body's Mr = eps_r + sigma/ce (N_s complex values, body
        voxels in idx_solution order); the Green's tensor stays."""
        mr = np.ascontiguousarray(np.asarray(Mr_body, dtype=np.complex128).reshape(-1))
        if mr.size != self.Ns:
            raise ValueError(f"Mr_body must have N_s = {self.Ns} entries")
        check(self._lib.marie_vie_set_materials(self._h, _dptr(mr.view(np.float64))))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.marie_vie_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- applications -------------------------------------------------------
    @staticmethod
    def _stream():
        import torch
        return ct.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _apply(self, fn, x, length, out=None):
        import torch
        if x.device.type != "cuda":
            raise ValueError("x must be a CUDA tensor")
        prec = C128 if x.dtype == torch.complex128 else (C64 if x.dtype == torch.complex64 else None)
        if prec is None:
            raise ValueError("x must be complex64 or complex128")
        x = x.contiguous()
        if x.numel() % length:
            raise ValueError(f"x length {x.numel()} is not a multiple of {length}")
        nrhs = x.numel() // length
        y = torch.empty_like(x) if out is None else out
        check(fn(self._h, prec, ct.c_void_p(x.data_ptr()), ct.c_void_p(y.data_ptr()), nrhs, self._stream()))
        return y

    def apply(self, x, out=None):
        """mvp_vie (mvp_vie.m:1-19) on body vectors."""
        return self._apply(self._lib.marie_vie_apply, x, self.Nb, out)

    def apply_adjoint(self, x, out=None):
        return self._apply(self._lib.marie_vie_apply_adjoint, x, self.Nb, out)

    def apply_N(self, x, out=None):
        return self._apply(self._lib.marie_vie_apply_N, x, self.C * self.nD, out)

    def apply_N_adj(self, x, out=None):
        return self._apply(self._lib.marie_vie_apply_N_adj, x, self.C * self.nD, out)

    def apply_K(self, x, out=None):
        return self._apply(self._lib.marie_vie_apply_K, x, self.C * self.nD, out)

    def apply_K_adj(self, x, out=None):
        return self._apply(self._lib.marie_vie_apply_K_adj, x, self.C * self.nD, out)

    def profile(self, x, reps=5):
        """Per-pass device times [ms] of mvp_vie on x (CUDA events on the
        current stream): x-fwd, y-fwd, z, y-inv, x-inv, whole application."""
        import torch
        prec = C128 if x.dtype == torch.complex128 else C64
        y = torch.empty_like(x)
        ms = np.zeros(6)
        check(self._lib.marie_vie_profile(self._h, prec, ct.c_void_p(x.data_ptr()), ct.c_void_p(y.data_ptr()),
                                          x.numel() // self.Nb, int(reps), _dptr(ms), self._stream()))
        return ms

    def autotune(self, x, reps=3):
        """Time mvp_vie on x (CUDA, nrhs*N_b; its dtype selects the precision)
        for every z-pass tile width that fits, keep the fastest; returns
        {width: mean ms}."""
        import torch
        prec = C128 if x.dtype == torch.complex128 else C64
        x = x.contiguous()
        y = torch.empty_like(x)
        w = np.zeros(8, np.int32)
        ms = np.zeros(8, np.float64)
        cnt = np.zeros(1, np.int32)
        check(self._lib.marie_vie_autotune(self._h, prec, ct.c_void_p(x.data_ptr()), ct.c_void_p(y.data_ptr()),
                                           x.numel() // self.Nb, int(reps), w.ctypes.data_as(_lib.c_int32_p),
                                           _dptr(ms), 8, cnt.ctypes.data_as(_lib.c_int32_p), self._stream()))
        return {int(w[i]): float(ms[i]) for i in range(min(int(cnt[0]), 8))}

    def tiles(self, prec=C64):
        out = np.zeros(4, np.int32)
        check(self._lib.marie_vie_tiles(self._h, prec, out.ctypes.data_as(_lib.c_int32_p)))
        return dict(chunk=int(out[0]), width=int(out[1]), float_float=bool(out[2]))

    # -- field post-processing -------------------------------------------------
    def fields(self, J, Ue=None, Ub=None, *, e=True, h=True):
        """Total fields of solved body currents J (nrhs*N_b, complex64/128 CUDA):
        E = Ue + invG((1/ce)(N J - G J)) (em_efield_vie_excitation.m:21) and
        H = Ub + invG(K J) (em_hfield_vie_excitation.m:20) on the body."""
        import torch
        if J.device.type != "cuda" or J.dtype not in (torch.complex64, torch.complex128):
            raise ValueError("J must be a complex64 or complex128 CUDA tensor")
        J = J.contiguous()
        prec = C128 if J.dtype == torch.complex128 else C64
        nrhs = J.numel() // self.Nb
        ptr = lambda t: ct.c_void_p(t.data_ptr()) if t is not None else None
        for t in (Ue, Ub):
            if t is not None and (t.dtype != J.dtype or t.numel() != J.numel() or not t.is_contiguous()):
                raise ValueError("Ue/Ub must match J in dtype and length and be contiguous")
        E = torch.empty_like(J) if e else None
        H = torch.empty_like(J) if h else None
        check(self._lib.marie_vie_fields(self._h, prec, ptr(J), ptr(Ue), ptr(Ub), ptr(E), ptr(H), nrhs,
                                         self._stream()))
        return E, H

    def absorbed_power(self, J):
        """phi = conj(J^H (real(Mc_inv/ce) .* G J)) (em_ehfield_vie.m:44-52); J: complex128 CUDA,
        nrhs*N_b with nrhs <= 64; returns an (nrhs, nrhs) complex128 numpy array."""
        import torch
        if J.device.type != "cuda" or J.dtype != torch.complex128:
            raise ValueError("J must be a complex128 CUDA tensor")
        J = J.contiguous()
        nrhs = J.numel() // self.Nb
        phi = np.zeros(2 * nrhs * nrhs, np.float64)
        check(self._lib.marie_vie_absorbed_power(self._h, ct.c_void_p(J.data_ptr()), nrhs, _dptr(phi),
                                                 self._stream()))
        return phi.view(np.complex128).reshape(nrhs, nrhs)

    def b1_plus(self, H):
        """B1+ = mu0 (H_x + i H_y) per body voxel (em_ehfield_vie.m:68); H: complex128 CUDA nrhs*N_b."""
        import torch
        if H.device.type != "cuda" or H.dtype != torch.complex128:
            raise ValueError("H must be a complex128 CUDA tensor")
        H = H.contiguous()
        nrhs = H.numel() // self.Nb
        out = torch.empty(nrhs * self.Ns, dtype=torch.complex128, device="cuda")
        check(self._lib.marie_vie_b1_plus(self._h, ct.c_void_p(H.data_ptr()), nrhs, ct.c_void_p(out.data_ptr()),
                                          self._stream()))
        return out

    def apply_hfield_adjoint(self, x, out=None):
        """K^H(invG x) on body vectors: the adjoint of the H-field map."""
        return self._apply(self._lib.marie_vie_apply_hfield_adjoint, x, self.Nb, out)

    def gradient_source(self, J, gM, M, P):
        """Adjoint source g = gM/P - (M/P^2)(1/2) D J of J_obj = M/P (one right-hand side)."""
        import torch
        g = torch.empty_like(J)
        check(self._lib.marie_vie_gradient_source(self._h, ct.c_void_p(J.data_ptr()), ct.c_void_p(gM.data_ptr()),
                                                  float(M), float(P), ct.c_void_p(g.data_ptr()), self._stream()))
        return g

    def gradient(self, J, lam, E, M, P):
        """dJ_obj/d eps_r and dJ_obj/d sigma per body voxel (two float64 CUDA tensors of length N_s)."""
        import torch
        de = torch.empty(self.Ns, dtype=torch.float64, device="cuda")
        ds = torch.empty_like(de)
        check(self._lib.marie_vie_gradient(self._h, ct.c_void_p(J.data_ptr()), ct.c_void_p(lam.data_ptr()),
                                           ct.c_void_p(E.data_ptr()), float(M), float(P),
                                           ct.c_void_p(de.data_ptr()), ct.c_void_p(ds.data_ptr()), self._stream()))
        return de, ds

    # -- solve ----------------------------------------------------------------
    def _run_gmres(self, fn, bptr, xptr, nrhs, x0, restart, tol, maxit, mode, inner_tol, max_refine, resvec_cap,
                   raise_on_fail, inner_safety=0.0, adjoint=False, block_steps=0):
        modes = {"fp64": SOLVE_FP64, "mixed": SOLVE_MIXED, "block": SOLVE_MIXED_BLOCK}
        if mode not in modes:
            raise ValueError(f"mode must be one of {sorted(modes)}")
        o = _lib.GmresOpts(restart=restart, maxit=maxit, tol=tol, mode=modes[mode],
                           x0_present=1 if x0 else 0, inner_tol=inner_tol, max_refine=max_refine,
                           inner_safety=inner_safety, adjoint=1 if adjoint else 0, block_steps=block_steps)
        it = np.zeros(nrhs, np.int32); ou = np.zeros(nrhs, np.int32); li = np.zeros(nrhs, np.int32)
        tr = np.zeros(nrhs, np.float64); st = np.zeros(nrhs, np.int32); rl = np.zeros(nrhs, np.int32)
        rv = np.zeros((nrhs, resvec_cap), np.float64)
        ip = lambda a: a.ctypes.data_as(_lib.c_int32_p)
        rep = _lib.GmresReport(iters=ip(it), outer=ip(ou), last_inner=ip(li), true_resid=_dptr(tr),
                               resvec=_dptr(rv), resvec_cap=resvec_cap, resvec_len=ip(rl), status=ip(st))
        s = fn(self._h, bptr, xptr, nrhs, ct.byref(o), ct.byref(rep), self._stream())
        if s not in (0, 4) or (raise_on_fail and s != 0):
            check(s)
        return SolveReport(it, ou, li, tr, [rv[r, :rl[r]].copy() for r in range(nrhs)], st,
                           rep.matvecs_c128, rep.matvecs_c64, ok=(s == 0))

    def gmres(self, b, x=None, *, restart=50, tol=1e-6, maxit=200, mode="fp64", inner_tol=1e-7,
              max_refine=10, resvec_cap=4096, raise_on_fail=False, inner_safety=0.0, adjoint=False, block_steps=0):
        """Batched is_gmres_vie (is_gmres_vie.m:1-30); b: (nrhs*N_b) complex128 CUDA.
        mode: "fp64" (the drop-in), "mixed" (complex64 GMRES per right-hand
        side inside FP64 refinement) or "block" (the same refinement with one
        block Krylov space for all right-hand sides, block_steps block
        Arnoldi steps per cycle).  adjoint=True solves A^H x = b."""
        import torch
        b = b.contiguous()
        if b.dtype != torch.complex128 or b.device.type != "cuda":
            raise ValueError("b must be a complex128 CUDA tensor")
        nrhs = b.numel() // self.Nb
        x0 = x is not None
        if x is None:
            x = torch.zeros_like(b)
        report = self._run_gmres(self._lib.marie_gmres_vie, ct.c_void_p(b.data_ptr()), ct.c_void_p(x.data_ptr()),
                                 nrhs, x0, restart, tol, maxit, mode, inner_tol, max_refine, resvec_cap,
                                 raise_on_fail, inner_safety, adjoint, block_steps)
        return x, report

    def gmres_host(self, b, x=None, *, out=None, restart=50, tol=1e-6, maxit=200, mode="fp64", inner_tol=1e-7,
                   max_refine=10, resvec_cap=4096, raise_on_fail=False, inner_safety=0.0, block_steps=0):
        """is_gmres_vie on host buffers (marie_gmres_vie_host): b is a CPU
        complex128 tensor (nrhs*N_b), page-locked for copy/compute overlap.
        x (optional) holds x0 and receives the solution; otherwise the
        solution goes to `out` (or a new tensor) from x0 = 0."""
        import torch
        if b.dtype != torch.complex128 or b.device.type != "cpu" or not b.is_contiguous():
            raise ValueError("b must be a contiguous complex128 CPU tensor")
        nrhs = b.numel() // self.Nb
        x0 = x is not None
        if x is None:
            x = out if out is not None else torch.empty_like(b, pin_memory=b.is_pinned())
        if x.dtype != torch.complex128 or x.device.type != "cpu" or not x.is_contiguous() or x.numel() != b.numel():
            raise ValueError("x / out must match b")
        report = self._run_gmres(self._lib.marie_gmres_vie_host, ct.c_void_p(b.data_ptr()),
                                 ct.c_void_p(x.data_ptr()), nrhs, x0, restart, tol, maxit, mode, inner_tol,
                                 max_refine, resvec_cap, raise_on_fail, inner_safety, False, block_steps)
        return x, report

    # -- right-hand sides -----------------------------------------------------
    def incident_loops(self, origin, loops, radius, nseg=64):
        """Loop incident fields tested onto the basis: (nloop*N_b) complex128 CUDA."""
        import torch
        loops = np.ascontiguousarray(np.asarray(loops, dtype=np.float64).reshape(-1, 6))
        org = np.ascontiguousarray(np.asarray(origin, dtype=np.float64))
        out = torch.empty(loops.shape[0] * self.Nb, dtype=torch.complex128, device="cuda")
        check(self._lib.marie_incident_loops(self._h, _dptr(org), _dptr(loops), loops.shape[0], float(radius),
                                             int(nseg), ct.c_void_p(out.data_ptr()), self._stream()))
        return out

    def incident_wire(self, origin, r_p, r_n, r_2, coef=None, *, kind="E", q_wire=4, q_vox=2):
        """Incident E (kind "E") or H (kind "H") field coefficients on the body
        of wire currents in the reference's wire-basis convention
        (Assemble_tri_coupling_matrix_{N,K}_*.cpp, wvie_mrgf_assembly.m):
        r_p / r_n / r_2 (n_tri, 3) basis nodes, coef (nrhs, n_tri) complex wire
        currents or None for all ones.  Returns (nrhs*N_b) complex128 CUDA."""
        import torch
        pts = [np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, 3)) for a in (r_p, r_n, r_2)]
        ntri = pts[0].shape[0]
        if coef is None:
            cf, nrhs = None, 1
        else:
            c = np.ascontiguousarray(np.asarray(coef, dtype=np.complex128).reshape(-1, ntri))
            nrhs = c.shape[0]
            cf = c.view(np.float64)
        org = np.ascontiguousarray(np.asarray(origin, dtype=np.float64))
        out = torch.empty(nrhs * self.Nb, dtype=torch.complex128, device="cuda")
        check(self._lib.marie_incident_wire(self._h, 0 if kind == "E" else 1, _dptr(org), *(_dptr(a) for a in pts),
                                            ntri, None if cf is None else _dptr(cf), nrhs, int(q_wire), int(q_vox),
                                            ct.c_void_p(out.data_ptr()), self._stream()))
        return out

    def incident_plane_wave(self, origin):
        import torch
        org = np.ascontiguousarray(np.asarray(origin, dtype=np.float64))
        out = torch.empty(self.Nb, dtype=torch.complex128, device="cuda")
        check(self._lib.marie_incident_plane_wave(self._h, _dptr(org), ct.c_void_p(out.data_ptr()),
                                                  self._stream()))
        return out


def assemble_green(dims, res, freq, pwl: bool, kernel: str = "N", self_term: str = "pointwise",
                   near: str = "relative") -> np.ndarray:
    """I_V (n1,n2,n3,pwx,6|3) computed on the GPU (assembly_N.m / assembly_K.m).

    near="relative" (default): the near offsets {0,1}^3 by an accurate host
    cubature of the same integrals (the point term of N included), equal to
    the reference's surface-surface near zone with its DIRECTFN singular
    quadrature (assembly_N.m:56-81) to ~1e-13; far and medium zones by the
    GPU Gauss rules.  near="standin": the staggered GPU cubature everywhere,
    which lacks N's point term and is 13% low on face neighbours; with it,
    self_term="distributional" adds the point term of the N kernel at the
    self offset ((2/3) Gram on the diagonal components)."""
    if self_term not in ("pointwise", "distributional") or near not in ("standin", "relative"):
        raise ValueError(f"bad self_term {self_term!r} or near {near!r}")
    lib = _lib.load()
    n1, n2, n3 = (int(v) for v in dims)
    pwx = 10 if pwl else 1
    nc = 6 if kernel == "N" else 3
    out = np.empty(n1 * n2 * n3 * pwx * nc * 2, dtype=np.float64)
    args = (n1, n2, n3, float(res), float(freq), PWL if pwl else PWC, 0 if kernel == "N" else 1)
    flags = (2 if near == "relative" else 0) | (1 if self_term == "distributional" else 0)   # MARIE_GREEN_*
    if flags:
        check(lib.marie_assemble_green_ex(*args, flags, _dptr(out)))
    else:
        check(lib.marie_assemble_green(*args, _dptr(out)))
    return out.view(np.complex128).reshape((n1, n2, n3, pwx, nc), order="F")
