"""CPU checks of the host construction of the multigrid's rigid-body deflation
space (csrc/defl_space.h): passive-solid components, the merge radius that keeps
their supports disjoint, the rigid-body mode values, padded node strides and the
limits beyond which no deflation is built."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_deflation_space_construction(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "defl_space_check"
    src = os.path.join(ROOT, "tests", "defl_space_check.cpp")
    inc = os.path.join(ROOT, "am_ml_suite_gb300", "csrc")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-I", inc, src, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
