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
