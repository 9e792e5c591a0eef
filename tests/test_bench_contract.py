"""The reference arm of bench.py on the host cores: one JSON line with the
keys the driver reads (CPU only, a tiny bounded sample)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup",
                        "0", "--cpu-scale", "0.05", "--cpu-threads", "2"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["unit"] == "s" and d["higher_is_better"] is False and d["value"] > 0
    assert d["config"]["workload"] == "block337_mixed_L6" and d["config"]["dofs"] == 153245634
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 2 and cb["value"] == d["value"] and cb["sample"]
    # the headline figure is an extrapolation and says so; the measured sample is beside it
    assert d["extrapolated"] is True and cb["extrapolated"] is True
    m = d["measured"]
    assert m["threads"] == 2 and m["thread_env"]["OPENBLAS_NUM_THREADS"] == "2"
    assert len(m["iteration_s"]) == 1 and m["iteration_s_median"] > 0 and m["sample_dofs"] < d["config"]["dofs"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
