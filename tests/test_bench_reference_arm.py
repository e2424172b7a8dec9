"""bench.py's reference arm runs on the host cores alone (no GPU): it prints
one JSON line with the headline's metric, config and unit, timed on the
oracle's FP64 restatement of the reference walker, and a cpu_baseline and
e2e block describing that run."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line(orc):
    env = dict(os.environ, AXX_REF_SAMPLE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "walker-steps/s"
    assert d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["workload"] == "gamma_pack_400_cylinders_permeable_64seq"
    assert d["config"]["walkers"] == 4194304 and d["config"]["sample_walkers_per_step"] == 2
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
