"""bench.py --impl reference on CPU at a small size: the oracle timed on the
host cores on a slab of the workload, printed as one JSON line with the
reference arm's keys (impl, cpu_baseline, an e2e without copies)."""
from __future__ import annotations

import json
import os

import bench


def test_reference_arm_prints_one_line(capsys):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    bench.main(["--impl", "reference", "--n", "32", "--n3", "8", "--steps", "2", "--warmup", "1",
                "--reference-budget-s", "5"])
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "cell-steps/s" and d["unit"] == "cell-steps/s"
    assert d["steps"] == 2 and d["warmup"] == 3           # at least 3 warm-up steps
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["value"] > 0
    assert ":slab_32x32x" in d["config"]["workload"] and 2 <= d["config"]["sample_levels"] <= 8
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
