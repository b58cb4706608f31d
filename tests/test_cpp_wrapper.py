"""The header-only C++ wrapper (include/am_gpu.hpp), compiled with g++ against
the C ABI: the reference's TopologyOptimizer interface, its structs and its
exception types (tests/cpp/wrapper_check.cpp)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "am_ml_suite_gb300", "lib")
ORACLE = os.path.join(ROOT, "oracle")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    from am_ml_suite_gb300 import _build
    import oracle

    _build.build()
    oracle.build()
    out = str(tmp_path_factory.mktemp("cpp") / "wrapper_check")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "wrapper_check.cpp"), "-o", out,
           "-L", LIB, "-lamgpu", f"-Wl,-rpath,{LIB}", "-L", ORACLE, "-loracle", f"-Wl,-rpath,{ORACLE}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_wrapper_errors_without_a_device(exe):
    r = subprocess.run([exe, "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    # the ctypes mirrors of the ABI structs have the C compiler's sizes
    import ctypes

    from am_ml_suite_gb300 import _native as nat

    sizes = dict(zip(r.stdout.split()[0::2], r.stdout.split()[1::2]))
    assert int(sizes["sizeof(am_simp_config)"]) == ctypes.sizeof(nat.SimpConfig)
    assert int(sizes["sizeof(am_iteration_result)"]) == ctypes.sizeof(nat.IterationResult)
    assert int(sizes["sizeof(am_solve_stats)"]) == ctypes.sizeof(nat.SolveStats)


@pytest.mark.gpu
def test_wrapper_runs_against_the_oracle(exe):
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
