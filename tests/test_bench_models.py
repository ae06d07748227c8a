"""The benchmark's fixed byte models (bench.solve_alg_bytes), by hand on
small cases: per-RHS GMRES (Arnoldi step k reads/writes (2k + 4) N_b words)
and block GMRES (block step j: (2(j + 1) + 10) N_b words per right-hand
side), plus the per-matvec bytes 26 n^3 C s and the Green spectrum shared
by a launch's right-hand sides."""
import numpy as np

import bench


def _mv(n, C, U, s, chunk):
    return 26 * n ** 3 * C * s + U * (n + 1) ** 3 * s / chunk


def test_per_rhs_model():
    n, Nb, chunk = 8, 1000, 4
    iters = [7, 12]                    # restart 5: cycles 5+2 and 5+5+2
    got = bench.solve_alg_bytes(n, True, Nb, iters, 2, chunk, restart=5)
    want = 0.0
    for it in iters:
        steps = sum(2 * (k % 5 + 1) + 4 for k in range(it))      # k of the cycle is 1-based in the model
        want += it * _mv(n, 12, 60, 8, chunk) + steps * Nb * 8 + 2 * _mv(n, 12, 60, 16, chunk)
    assert np.isclose(got, want, rtol=1e-12)


def test_block_model():
    n, Nb, chunk = 8, 1000, 16
    iters, cycles = [60, 60], [2, 2]   # two cycles of 30 block steps
    got = bench.solve_alg_bytes(n, False, Nb, iters, 2, chunk, block_steps=30, cycles=cycles)
    per = 2 * sum(2 * (j + 1) + 10 for j in range(30))
    want = 2 * (60 * _mv(n, 3, 6, 8, chunk) + per * Nb * 8 + 2 * _mv(n, 3, 6, 16, chunk))
    assert np.isclose(got, want, rtol=1e-12)


def test_metric_names():
    wl = bench.WORKLOADS["ellipsoid128"]
    assert bench.metric_of(wl) == bench.METRIC
    assert "96^3 PWL" in bench.metric_of(bench.WORKLOADS["ellipsoid96"])
