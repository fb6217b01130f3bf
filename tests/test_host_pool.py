"""The planner thread pool (ecmgenerator_gb300/csrc/host_pool.h) under
stress on the CPU: 12,000 runs of 1-40 jobs from three callers; every job
runs exactly once and every run returns (a lost wake-up would hang it, so
the run has a time limit)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_host_pool_runs_every_job_once(tmp_path):
    exe = str(tmp_path / "pool_stress")
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "ecmgenerator_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "pool_stress.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
