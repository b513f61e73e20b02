"""The bench's reference arm runs on the CPU (the oracle restatement) and prints the JSON
line the measurement contract asks for: one line, the metric, unit and direction of the
GPU arm, a cpu_baseline block and a zero-copy e2e block."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "cavity", "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "cell-iterations/s" and d["unit"] == "cell-iterations/s"
    assert d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 2 and d["warmup"] >= 3  # the contract's minimum warm-up
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["nproc"] == os.cpu_count()
    # whether the reference's own runtime (warp-lang) is importable on this host, and why not
    assert "warp_available" in d["reference_runtime"]
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["cells"] == 4096


def test_stratified_sample_keeps_kind_shares_and_size_spread():
    sys.path.insert(0, ROOT)
    import numpy as np

    from bench import stratified_sample
    from warpcfd_gb300.serve import make_request_mix

    mix = make_request_mix(1024, seed=0, rate=2000.0)
    s = stratified_sample(mix, 48)
    assert len(s) == 48 and len({r.rid for r in s}) == 48
    share_mix = np.mean([r.kind == "cavity" for r in mix])
    share_s = np.mean([r.kind == "cavity" for r in s])
    assert abs(share_mix - share_s) < 0.05
    for kind in ("cavity", "channel"):
        cm = np.array([r.cells for r in mix if r.kind == kind])
        cs = np.array([r.cells for r in s if r.kind == kind])
        # the sample's sizes span the kind's range and sit near its median
        assert cs.min() <= np.percentile(cm, 5) and cs.max() >= np.percentile(cm, 95)
        assert abs(np.log(np.median(cs) / np.median(cm))) < 0.2
