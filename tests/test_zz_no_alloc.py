"""The allocation-free N apply (marie_vie_apply_N_noalloc) against the handle
path (marie_vie_apply_N), through the C ABI.

The no-alloc entry point serves callers that cannot allocate device memory
(allocator-free regions, real-time loops, processes that reserved all device
memory): it takes every buffer from the caller and keeps its FFT work arrays
in a fixed 64 MiB device array.  This file is collected last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes as ct

import numpy as np
import pytest

from oracle import marie_oracle as O
from helpers import Problem, flat_F, rel_err

torch = pytest.importorskip("torch")

TOL_C64 = 1e-5


def _octant(P):
    """Green octant spectrum in the entry point's layout [blk][ky][kx][kz]."""
    n1, n2, n3 = P.n
    M = 8.0 * n1 * n2 * n3
    pwx = 10 if P.pwl else 1
    blocks = []
    for j in range(pwx):
        for k in range(6):
            full = O.tucker_block(P.TN[(j, k)])
            blocks.append(np.transpose(full[: n1 + 1, : n2 + 1, : n3 + 1], (1, 0, 2)) / M)
    return np.ascontiguousarray(np.stack(blocks)).astype(np.complex64)


@pytest.mark.gpu
@pytest.mark.parametrize("n,pwl", [((8, 7, 6), False), ((6, 5, 4), True), ((12, 10, 7), True)],
                         ids=["pwc-8x7x6", "pwl-6x5x4", "pwl-12x10x7"])
def test_noalloc_matches_handle_path_twice(n, pwl):
    from marie_gb300 import _lib
    lib = _lib.load()
    P = Problem(n, pwl, seed=31)
    op = P.gpu_operator(precisions=2, max_rhs=1)
    J = P.random_grid(seed=5)[0]
    x = torch.from_numpy(flat_F(J)).to("cuda", torch.complex64)
    ref = op.apply_N(x).cpu().numpy()
    G = torch.from_numpy(_octant(P)).cuda()
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = []
    free = []
    for _ in range(2):
        y = torch.full_like(x, complex(float("nan"), float("nan")))
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        st = lib.marie_vie_apply_N_noalloc(*P.n, 1 if pwl else 0, ct.c_void_p(G.data_ptr()),
                                           ct.c_void_p(x.data_ptr()), ct.c_void_p(y.data_ptr()), stream)
        assert st == 0, _lib.last_error()
        torch.cuda.synchronize()
        outs.append(y.cpu().numpy())
    free.append(torch.cuda.mem_get_info()[0])
    for y in outs:
        assert np.all(np.isfinite(y))
        assert rel_err(y, ref) <= TOL_C64
    # the second call runs on the scratch the first call left behind
    assert rel_err(outs[1], outs[0]) <= TOL_C64
    # no device memory taken by the calls after the first one's set-up
    assert free[2] == free[1]
    op.close()


@pytest.mark.gpu
def test_noalloc_rejects_grids_beyond_scratch():
    from marie_gb300 import _lib
    lib = _lib.load()
    null = ct.c_void_p(1)
    st = lib.marie_vie_apply_N_noalloc(64, 64, 64, 1, null, null, null, None)
    assert st == 1 and "64 MiB" in _lib.last_error()
    st = lib.marie_vie_apply_N_noalloc(0, 4, 4, 0, null, null, null, None)
    assert st == 1
