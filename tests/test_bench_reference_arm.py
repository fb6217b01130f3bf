"""bench.py's reference arm (--impl reference) runs on the host cores only:
its JSON line carries the metric, unit, direction and config of the GPU arm,
a cpu_baseline describing the run (with the one-thread figure beside it) and
an e2e object without host<->device traffic; the process never maps the
product library (scene, agents and paths come from Python and the oracle)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RUN = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "boxes_1k", "--steps", "2", "--warmup", "3",
            "--cpu-budget", "2"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("MAPPED_PRODUCT_LIBRARY" if "libecmg" in maps else "PRODUCT_LIBRARY_NOT_MAPPED")
"""


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, "-c", RUN], capture_output=True, text=True, timeout=900, cwd=ROOT,
                         check=True)
    assert "PRODUCT_LIBRARY_NOT_MAPPED" in out.stdout, out.stdout[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "agent-steps/s" and d["higher_is_better"] is True
    assert d["metric"].startswith("agent-steps/s")
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] >= 3
    assert set(d["config"]) == {"workload", "agents", "max_neighbors", "neighbor_dist_m", "time_horizon_s", "dt_s",
                                "scene", "l2", "parallelism", "seed", "planner"}
    assert d["config"]["workload"] == "boxes_1k" and d["config"]["planner"] == "reference"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"].startswith("port") and cb["cores"] >= 1 and cb["sample"]
    assert d["one_thread"]["cores"] == 1 and d["one_thread"]["value"] > 0
    assert len(d["tick_ms"]) == 2
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
