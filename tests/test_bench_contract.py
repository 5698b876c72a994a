"""bench.py's reference arm runs on the host (the oracle on all cores) and
prints the JSON line the benchmark contract asks for; no GPU needed."""

import json
import os
import subprocess
import sys

from conftest import REPO


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0", "--clusters", "64"],
                         capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    # a finite step time, and the workload the GPU arm prints
    assert isinstance(d["ms_per_step"], float) and d["ms_per_step"] > 0
    assert d["config"]["clusters"] == 64 and d["config"]["healpix_order"] == 7
    assert d["config"]["n_sky"] == 196608 and d["config"]["total_pix"] > 0
