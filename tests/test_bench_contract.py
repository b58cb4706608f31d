"""The reference arm of bench.py end to end on the CPU (it needs no GPU): one JSON
line with the GB300 arm's metric string, unit and direction, a whole first SIMP
iteration of the CPU restatement behind the projection, and the e2e / cpu_baseline
objects the line must carry."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    sys.path.insert(0, ROOT)
    import bench

    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "cantilever48", "--steps", "2", "--warmup", "1"], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "SIMP iters/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] >= 1 and d["value"] > 0
    assert d["config"]["workload"] == "cantilever48" and d["config"]["shape"] == [48, 24, 12]
    # iteration 1 run whole: its PCG count drives the projection of every step
    assert d["projected"] is True and d["whole_iteration_1"]["pcg_iterations"] == d["pcg_iterations_per_solve"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_ku_traffic_uses_the_workload_capture():
    """The K*u roofline's DRAM traffic: the committed ncu capture of the workload's
    own grid where there is one (the cantilever and the bracket), else the largest
    capture scaled by nodes; every capture names the command that made it."""
    sys.path.insert(0, ROOT)
    import bench

    with open(os.path.join(ROOT, "profiles", "ku_pcg_fp32_traffic.json")) as f:
        caps = json.load(f)["captures"]
    for name, c in caps.items():
        assert c["source"].startswith("ncu ") and "--clock-control none" in c["source"], name
        assert c["dram_bytes_per_launch"] == c["dram_bytes_read"] + c["dram_bytes_write"] or \
            abs(c["dram_bytes_per_launch"] - (c["dram_bytes_read"] + c["dram_bytes_write"])) < 1e3, name
        assert bench.ku_traffic_per_launch(None, c["nodes"], c["elements"]) == c["dram_bytes_per_launch"]
    big = max(caps.values(), key=lambda c: c["nodes"])
    assert bench.ku_traffic_per_launch(None, big["nodes"] // 2, 1) == big["dram_bytes_per_launch"] * (
        big["nodes"] // 2) / big["nodes"]
