"""Timed CPU baseline: the FP64 reference algorithm on the host cores.

TEST AND CPU-BASELINE INFRASTRUCTURE ONLY (used by bench.py's cpu_baseline leg and
its reference arm).  The reference path is MATLAB (fftn, elementwise MACs,
mldivide); MATLAB is unavailable, so the same algorithm is timed as a
numpy/scipy port using every host core:

  one GMRES iteration = one mvp_vie (mvp_vie.m:12-18 with
  mvp_N_pwl_tucker.m:15-41: C zero-padded 3D FFTs, C x C block products with
  the circulant Green spectra, C inverse FFTs + crop, contrast epilogue)
  + one classical Gram-Schmidt Arnoldi step (is_iter_gmres_vie.m:15-19).

Two variants: "pre-expanded" Green blocks (the fastest CPU form of the
algorithm), and "reference" (tucker_ranks given), which re-expands a Tucker
block inside every block product as mvp_N_pwl_tucker.m:31 does (three mode
products, nmp.m:1-21, of an r1 x r2 x r3 core with r x 2n factors).  Values
are seeded synthetic arrays: the timing of FFTs, GEMMs and elementwise
products does not depend on them.  Sizes, layouts and operation counts are
the workload's.
"""
from __future__ import annotations

import os
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.fft as sfft

from . import marie_oracle as O


def _chunks(n, k):
    step = (n + k - 1) // k
    return [(i, min(n, i + step)) for i in range(0, n, step)]


def _expand(G, U1, U2, U3):
    """Tucker block G x1 U1^T x2 U2^T x3 U3^T on the (2n)^3 grid (nmp.m:1-21
    applied three times, as mvp_N_pwl_tucker.m:31)."""
    A = np.tensordot(G, U1, axes=([0], [0]))       # r2 r3 m
    A = np.tensordot(A, U2, axes=([0], [0]))       # r3 m m
    return np.tensordot(A, U3, axes=([0], [0]))    # m m m


def time_iteration(n: int, pwl: bool, steps: int = 1, warmup: int = 0, budget_s: float = 30.0,
                   body_fraction: float = 0.117, k_arnoldi: int = 25, restart: int = 50, seed: int = 0,
                   tucker_ranks=None):
    """tucker_ranks: None (pre-expanded blocks) or (r1, r2, r3) of the Tucker
    blocks that every block product re-expands (the reference's form)."""
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    C = 12 if pwl else 3
    m = 2 * n
    M = m ** 3
    # distinct synthetic spectra (one per dyadic component); 60 PWL blocks map onto them
    nspec = 6
    spec = [(rng.standard_normal(M) + 1j * rng.standard_normal(M)).reshape(m, m, m) for _ in range(nspec)]
    tab = O.block_table("N", pwl, False)
    Ns = int(body_fraction * n ** 3)
    idxS = np.sort(rng.choice(n ** 3, Ns, replace=False))
    Nb = C * Ns
    chi = rng.standard_normal(Ns) + 1j * rng.standard_normal(Ns)
    invg = O.invG_scale(pwl, 2e-3)
    x = rng.standard_normal(Nb) + 1j * rng.standard_normal(Nb)
    V = rng.standard_normal((Nb, k_arnoldi + 1)) + 1j * rng.standard_normal((Nb, k_arnoldi + 1))
    pool = ThreadPoolExecutor(max_workers=cores)
    parts = _chunks(M, cores)
    tk = None
    if tucker_ranks is not None:
        r1, r2, r3 = (int(v) for v in tucker_ranks)
        tk = [((rng.standard_normal((r1, r2, r3)) + 1j * rng.standard_normal((r1, r2, r3))),
               *(rng.standard_normal((r, m)) + 1j * rng.standard_normal((r, m)) for r in (r1, r2, r3)))
              for _ in range(nspec)]

    def matvec(xb):
        Jp = np.zeros(n ** 3 * C, complex)
        for c in range(C):
            Jp[c * n ** 3 + idxS] = xb[c * Ns:(c + 1) * Ns]
        Jp = Jp.reshape((n, n, n, C), order="F")
        fJ = [sfft.fftn(Jp[..., q], s=(m, m, m), axes=(0, 1, 2), workers=cores).reshape(-1) for q in range(C)]
        out = np.empty_like(Jp)
        acc = np.empty(M, complex)
        for p in range(C):
            if tk is None:
                terms = [(tab[p][q][0], spec[tab[p][q][1][1] % nspec].reshape(-1), fJ[q])
                         for q in range(C) if tab[p][q] is not None]
            else:
                # the reference re-expands the block of every product (mvp_N_pwl_tucker.m:31)
                terms = [(tab[p][q][0], _expand(*tk[tab[p][q][1][1] % nspec]).reshape(-1), fJ[q])
                         for q in range(C) if tab[p][q] is not None]

            def work(lohi):
                lo, hi = lohi
                a = acc[lo:hi]
                a[:] = 0
                tmp = np.empty(hi - lo, complex)
                for s, g, f in terms:
                    np.multiply(g[lo:hi], f[lo:hi], out=tmp)
                    if s < 0:
                        a -= tmp
                    else:
                        a += tmp

            list(pool.map(work, parts))
            out[..., p] = sfft.ifftn(acc.reshape(m, m, m), workers=cores)[:n, :n, :n]
        NJ = out.reshape(-1, order="F")
        y = np.empty(Nb, complex)
        for c in range(C):
            blk = NJ[c * n ** 3 + idxS]
            y[c * Ns:(c + 1) * Ns] = xb[c * Ns:(c + 1) * Ns] - chi * (invg[c] * blk)
        return y

    def arnoldi(w):
        h = V.conj().T @ w
        w = w - V @ h
        return np.linalg.norm(w)

    for _ in range(warmup):
        arnoldi(matvec(x))
    times = []
    t_start = time.perf_counter()
    for i in range(max(1, steps)):
        t0 = time.perf_counter()
        arnoldi(matvec(x))
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > budget_s:
            break
    pool.shutdown()
    return {"sec_per_iter": float(np.mean(times)), "iters_timed": len(times), "cores": cores, "k": k_arnoldi,
            "Nb": Nb, "variant": "reference (Tucker re-expanded per product)" if tk is not None else "pre-expanded"}
