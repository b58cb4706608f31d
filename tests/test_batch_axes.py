"""CPU checks of the batch's axis order (csrc/batch_axes.h): the order chosen for
a problem's grid, never worse than the caller's, and index maps between the
caller's order and the stored one that are bijections inverting one another."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_batch_axis_order_maps(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "batch_axes_check"
    src = os.path.join(ROOT, "tests", "batch_axes_check.cpp")
    inc = os.path.join(ROOT, "am_ml_suite_gb300", "csrc")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-I", inc, src, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
