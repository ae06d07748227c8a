"""The block solver's tensor-core GEMM (marie_block_gemm_cn: H = V^H W,
tcgen05 kind::tf32 with three split products) against a complex128 product
of the same complex64 data.

Tolerance: every entry within 5e-7 of ||V_a|| ||W_c|| (the Cauchy-Schwarz
bound of the entry; measured 5.5e-8 - 2.3e-7, FP32 level): the split products carry
~2^-23 of each product, the tensor core sums chains of 256 chunks in FP32,
the chains and the contraction slices are added in FP32 / FP64.
Cases: one and several 512-column tiles, ragged column counts (1, 17, 300,
1100), p = 1 / 7 / 64, an odd number of complex rows, leading dimensions
larger than the row count, and misaligned arguments refused.
"""
import ctypes as ct

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _gemm(V, W, K, M, p, ldv, ldw):
    from marie_gb300 import _lib
    lib = _lib.load()
    H = torch.zeros(M * p, dtype=torch.complex64, device="cuda")
    nf = lib.marie_block_gemm_part_floats(K, M)
    part = torch.empty(nf, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = lib.marie_block_gemm_cn(ct.c_void_p(V.data_ptr()), ldv, ct.c_void_p(W.data_ptr()), ldw, K, M, p,
                                 ct.c_void_p(H.data_ptr()), M, ct.c_void_p(part.data_ptr()), nf,
                                 ct.c_void_p(err.data_ptr()), ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, H.reshape(p, M).T, int(err.item())


@pytest.mark.gpu
@pytest.mark.parametrize("K,M,p,pad", [(4096, 1, 1, 0), (10000, 17, 7, 2), (200001, 300, 64, 1),
                                       (65536, 1100, 64, 0), (131072, 64, 64, 0)])
def test_block_gemm_matches_complex128(K, M, p, pad):
    g = torch.Generator(device="cuda").manual_seed(K + M + p)
    ldv = K + pad + (K + pad) % 2          # even leading dimensions
    ldw = ldv
    V = torch.randn(M * ldv, dtype=torch.complex64, device="cuda", generator=g)
    W = torch.randn(p * ldw, dtype=torch.complex64, device="cuda", generator=g)
    st, H, err = _gemm(V, W, K, M, p, ldv, ldw)
    assert st == 0 and err == 0
    Vm = V.reshape(M, ldv)[:, :K].to(torch.complex128)          # rows = columns of V
    Wm = W.reshape(p, ldw)[:, :K].to(torch.complex128)
    ref = Vm.conj() @ Wm.T                                       # (M, p) = V^H W
    bound = torch.linalg.norm(Vm, dim=1)[:, None] * torch.linalg.norm(Wm, dim=1)[None, :]
    rel = ((H.to(torch.complex128) - ref).abs() / bound).max().item()
    assert rel <= 5e-7, rel


@pytest.mark.gpu
def test_block_gemm_gram_and_bad_args():
    """W^H W of one block (the Gram matrix of the block QR) is Hermitian
    positive definite to the tolerance; p > 64 and odd leading dimensions
    are refused before any launch."""
    K, p = 50000, 64
    g = torch.Generator(device="cuda").manual_seed(7)
    W = torch.randn(p * K, dtype=torch.complex64, device="cuda", generator=g)
    st, G, err = _gemm(W, W, K, p, p, K, K)
    assert st == 0 and err == 0
    Gd = G.to(torch.complex128)
    assert (Gd - Gd.conj().T).abs().max().item() <= 5e-7 * Gd.diagonal().real.max().item()
    assert torch.linalg.eigvalsh(0.5 * (Gd + Gd.conj().T)).min().item() > 0
    st, _, _ = _gemm(W, W, K, p, 65, K, K)
    assert st == 1
    st, _, _ = _gemm(W, W, K - 1, p, p, K - 1, K - 1)
    assert st == 1
