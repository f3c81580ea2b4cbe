"""The reference arm of bench.py runs on the CPU (the oracle's APGD on the host cores): one step of it must
print one JSON line with the keys and meanings the benchmark contract fixes. The run here uses a short
iteration budget (--max-iters) so that the calibration solve and the sample stay short on CPU."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--max-iters", "300"], cwd=REPO, capture_output=True, text=True, timeout=900, check=True)
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "ms" and d["higher_is_better"] is False
    assert d["steps"] == 1 and d["warmup"] == 0 and d["n_gpus"] == 1 and d["dtype"] == "f64"
    assert d["value"] > 0 and d["ms_per_step"] == d["value"]
    assert d["config"]["workload"] == "fp64_apgd_200k_contacts_to_1e-6" and d["config"]["contacts"] == 200_000
    assert d["config"]["max_iters"] == 300 and d["config"]["iterations"] == 300
    assert d["config"]["reached_tol"] is False
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
