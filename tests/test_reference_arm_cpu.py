"""The reference arm of the benchmark (`bench.py --impl reference`) runs the
reference algorithm on the host cores: the oracle's FP32 C restatement over a
row sample of the CT-scan workload.  It needs no GPU, so it runs here once and
its JSON line is checked against the benchmark contract."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup",
                          "3"], capture_output=True, text=True, timeout=600, cwd=ROOT, check=True).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Mrays/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert set(d["per_traversal"]) == {"dda", "svo-naive", "esvo", "svo-df", "svo-rope"}
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert d["config"]["volume"] == [512, 361, 512] and d["config"]["resolution"] == [1920, 1080]


def test_committed_profile_figures_cover_every_traversal():
    """The DRAM traffic and the issue/ALU figures the bench line carries come
    from the committed ncu summaries; every traversal has both, and the
    values are plausible (bytes per launch, fractions of peak)."""
    sys.path.insert(0, str(ROOT))
    import bench
    traffic, issue = bench.load_traffic(), bench.load_issue()
    trav = {"dda", "svo-naive", "esvo", "svo-df", "svo-rope"}
    assert set(traffic) == trav and set(issue) == trav
    assert all(1e6 < v < 1e10 for v in traffic.values())
    for v in issue.values():
        assert 0.0 < v["issue_active_frac"] <= 1.0 and 0.0 < v["alu_pipe_frac"] <= 1.0


def test_cpu_sample_bands_stay_inside_the_frame():
    sys.path.insert(0, str(ROOT))
    import bench
    for bands, rows in ((16, 64), (4, 64), (1, 8), (40, 64)):
        offs = bench.band_offsets(bands, rows)
        assert offs == sorted(offs) and offs[0] >= 0 and offs[-1] + rows <= bench.HEIGHT
        assert all(b - a >= rows for a, b in zip(offs, offs[1:]))
