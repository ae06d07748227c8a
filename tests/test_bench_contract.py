"""bench.py's command-line contract on the CPU: the reference arm (the FP64
algorithm timed on the host cores) prints one JSON line with the keys the
benchmark contract names, and the uneven-size batch generator draws the
configuration's instances."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--workload", "sphere32", "--impl", "reference",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "solves/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]


def test_uneven_batch_instances():
    sys.path.insert(0, str(ROOT))
    import bench
    inst = bench.uneven_instances()
    assert len(inst) == 16
    assert all(d["n"] in (48, 64, 80, 96, 112, 128) and 1 <= d["nloops"] <= 8 for d in inst)
    assert {d["freq"] for d in inst} <= {128e6, 297.2e6}
    assert inst == bench.uneven_instances()           # seeded


def test_solve_alg_bytes_formula():
    """One iteration, no residual: one matvec of 26 n^3 C s bytes plus the
    Green spectrum over the chunk, and Arnoldi step 1 (6 N_b s bytes); the
    128^3 PWL complex64 matvec is 5.234 GB + 1.030 GB of Green spectrum."""
    sys.path.insert(0, str(ROOT))
    import bench
    n, Nb = 128, 2939712
    one = bench.solve_alg_bytes(n, True, Nb, [1], 0, 1)
    assert abs(one - (26 * n ** 3 * 12 * 8 + 60 * (n + 1) ** 3 * 8 + 6 * Nb * 8)) < 1.0
    assert abs(26 * n ** 3 * 12 * 8 / 1e9 - 5.234) < 1e-3 and abs(60 * (n + 1) ** 3 * 8 / 1e9 - 1.030) < 1e-3
    # k = 1..13 in one cycle: sum (2k + 4) = 234; restart 5: cycles 5 + 5 + 3
    assert abs(bench.solve_alg_bytes(n, True, Nb, [13], 0, 1) - 13 * (one - 6 * Nb * 8) - 234 * Nb * 8) < 1.0
    assert abs(bench.solve_alg_bytes(n, True, Nb, [13], 0, 1, restart=5)
               - 13 * (one - 6 * Nb * 8) - (2 * 50 + 24) * Nb * 8) < 1.0
    # a complex128 residual matvec moves twice the complex64 bytes
    assert abs(bench.solve_alg_bytes(n, True, Nb, [0], 1, 1) - 2 * (one - 6 * Nb * 8)) < 1.0
