"""CPU checks of the native library: it loads, exports every entry point that
include/am_gpu.h declares, and its host-only functions agree with the oracle.
No compute call needs a GPU here."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O
from am_ml_suite_gb300 import _build, _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    out = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", name)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            out |= set(re.findall(r"\b(am_[a-z0-9_]+)\s*\(", txt))
    return out


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return nat.load()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in sorted(syms):
        assert hasattr(lib, s), s
    # the ctypes signature table covers the same set
    assert syms == set(nat.SIGNATURES)


def test_element_stiffness_host(lib, golden):
    k = nat.element_stiffness(1.0, 0.3, 1.0)
    assert np.abs(k - golden["ke_E1_nu03_h1"]).max() < 1e-15
    k2 = nat.element_stiffness(113.8e9, 0.342, 0.002)
    assert np.abs(k2 - golden["ke_ti_h2mm"]).max() < 1e-14 * np.abs(k2).max()
    assert np.abs(k2 - O.ke(113.8e9, 0.342, 0.002)).max() < 1e-14 * np.abs(k2).max()
    with pytest.raises(nat.AmError):
        nat.element_stiffness(1.0, 0.5, 1.0)


def test_config_defaults(lib):
    c = nat.default_config(nat.VARIANT_CPP)
    # SIMPConfig defaults (topology_optimizer.hpp:49-59)
    assert (c.volume_fraction, c.penalty, c.filter_radius, c.move_limit, c.rho_min, c.E_min,
            c.max_iterations, c.convergence_tol) == (0.25, 3.0, 2.0, 0.2, 0.01, 1e-6, 100, 0.01)
    p = nat.default_config(nat.VARIANT_PY)
    assert p.E_min == 1e-9 and p.variant == nat.VARIANT_PY
    assert ctypes.sizeof(nat.SimpConfig) == 120  # sizeof(am_simp_config) on LP64 (wrapper_check prints it)


def test_status_strings(lib):
    for code, name in nat.STATUS.items():
        assert lib.am_status_string(code).decode() == name


def test_no_device_is_loud(lib):
    if nat.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(nat.AmError) as e:
        nat.Problem((2, 2, 2))
    assert e.value.name == "AM_ERR_NO_DEVICE"
