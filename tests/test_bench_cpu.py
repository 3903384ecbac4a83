"""bench.py's reference arm (the CPU oracle port on the host's cores) keeps
the JSON contract: one line with the metric, unit and config of the GPU arm,
impl "reference", a cpu_baseline describing the run and an e2e object with
no host<->device bytes. It imports no product module (the import trace shows
none). The reference arm needs no GPU, so this runs here on a small sample."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "-X", "importtime", "bench.py", "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--ref-rays", "4096"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "rays/s (full 800x800 frames)" and d["unit"] == "rays/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"].startswith("c2:")
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "4096" in cb["sample"] and cb["cores"] == (os.cpu_count() or 1)
    assert d["config"]["rays_per_step"] == 4096 and d["config"]["full_frames"] is False
    # the arm runs the oracle only: no product module is imported
    assert "nsvf_gb300" not in r.stderr
    assert d["e2e"] == {"value": d["value"], "unit": "rays/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
