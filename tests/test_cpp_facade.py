"""The header-only C++ facade compiles against the C ABI and behaves like the
reference Simulator class (construct, SpawnAgent, Update, raw getters)."""
import os
import subprocess

import pytest

from ecmgenerator_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def facade_exe(tmp_path_factory):
    lib = B.build()
    out = str(tmp_path_factory.mktemp("facade") / "facade_main")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_main.cpp"), "-o", out, lib,
                    f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    return out


def test_facade_without_gpu_reports_no_device(facade_exe):
    r = subprocess.run([facade_exe], capture_output=True, text=True, env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode == 2, r.stdout + r.stderr


@pytest.mark.gpu
def test_facade_on_gpu(facade_exe):
    r = subprocess.run([facade_exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
