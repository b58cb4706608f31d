"""am_residual_noalloc: the residual entry point for callers that cannot allocate
device memory once they run (code inside another framework's fixed memory pool,
allocation-free real-time or certified loops, plugins whose host owns every
buffer).  The tests own the device buffers (allocated with torch, as such a
caller's host would) and call the entry point through the C ABI.

Its results are checked against the FP64 oracle's K*u and against the
handle-based am_ku_apply, on two calls in a row (the second on a non-default
stream), and once more as the very first call into the library in a fresh
process, which is how a fixed-pool caller uses it.

Collected last (file name) so that a failure here does not hide the others."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from am_ml_suite_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHAPE = (37, 9, 13)
H, E0, NU = 0.5, 2.0, 0.3


def _compact_from_reference(v, shape):
    """Reference DOF order -> three component planes, x fastest."""
    nx, ny, nz = shape
    a = np.asarray(v).reshape(nx + 1, ny + 1, nz + 1, 3)       # [i][j][k][d]
    return np.ascontiguousarray(a.transpose(3, 2, 1, 0)).ravel()  # [d][k][j][i]


def _case(shape, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    rho = rng.uniform(0.05, 1.0, size=shape)                     # C-order (nx, ny, nz)
    u = rng.normal(size=3 * nn)                                   # reference order
    f = rng.normal(size=3 * nn)
    fixed_node = rng.uniform(size=nn) < 0.1
    return rho, u, f, fixed_node


def _oracle_residual(shape, rho, u, f, fixed_node):
    """r = mask(f - K(rho) u) from the FP64 CPU oracle, compact layout."""
    import oracle as O

    y = O.ku(shape, O.ke(E0, NU, H), rho.ravel(), u)
    r = f - y
    r.reshape(-1, 3)[fixed_node] = 0.0
    return _compact_from_reference(r, shape)


def _call_noalloc(torch, shape, rho, u, f, fixed_node, stream=None):
    """Device buffers owned by the caller; returns (r, |r|^2) on the host."""
    nx, ny, nz = shape
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    dev = torch.device("cuda:0")
    scale_d = torch.tensor(np.ascontiguousarray(rho.transpose(2, 1, 0)).ravel(), dtype=torch.float64, device=dev)
    u_d = torch.tensor(_compact_from_reference(u, shape), dtype=torch.float64, device=dev)
    f_d = torch.tensor(_compact_from_reference(f, shape), dtype=torch.float64, device=dev)
    mask_nodes = np.ascontiguousarray(
        (fixed_node.reshape(nx + 1, ny + 1, nz + 1).transpose(2, 1, 0).ravel() * 7).astype(np.uint8))
    mask_d = torch.tensor(mask_nodes, dtype=torch.uint8, device=dev)
    r_d = torch.full((3 * nn,), float("nan"), dtype=torch.float64, device=dev)
    rr_d = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    handle = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
    st = nat.load().am_residual_noalloc(
        nx, ny, nz, H, E0, NU, ctypes.c_void_p(scale_d.data_ptr()), ctypes.c_void_p(u_d.data_ptr()),
        ctypes.c_void_p(f_d.data_ptr()), ctypes.c_void_p(mask_d.data_ptr()), ctypes.c_void_p(r_d.data_ptr()),
        ctypes.c_void_p(rr_d.data_ptr()), handle)
    assert st == nat.AM_OK, nat.load().am_last_error()
    if stream is None:
        torch.cuda.synchronize()
    else:
        stream.synchronize()
    return r_d.cpu().numpy(), float(rr_d.cpu().numpy()[0])


def _check(r, rr, r_ref):
    scale = np.abs(r_ref).max()
    assert np.abs(r - r_ref).max() <= 1e-12 * scale
    assert rr == pytest.approx(float(np.sum(r_ref * r_ref)), rel=1e-12)


@pytest.mark.gpu
def test_residual_noalloc_matches_oracle_and_ku_apply():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    nat.load()
    side = torch.cuda.Stream()
    results = []
    for call, seed in enumerate((1, 2)):
        rho, u, f, fixed_node = _case(SHAPE, seed)
        r, rr = _call_noalloc(torch, SHAPE, rho, u, f, fixed_node, stream=None if call == 0 else side)
        _check(r, rr, _oracle_residual(SHAPE, rho, u, f, fixed_node))
        results.append((rho, u, f, fixed_node, r))
    # the handle-based entry point on the same inputs (created after the
    # allocation-free calls): y = K u, then r = mask(f - y)
    p = nat.Problem(SHAPE, H, E0, NU)
    # scale = rho exactly: C++ rule with E_min = 0, p = 1, rho_min = 0
    cfg = nat.default_config(nat.VARIANT_CPP, E_min=0.0, penalty=1.0, rho_min=0.0)
    for rho, u, f, fixed_node, r in results:
        y = p.ku(cfg, rho, u, nat.PREC_FP64)
        r_ref = f - y
        r_ref.reshape(-1, 3)[fixed_node] = 0.0
        r_ref_c = _compact_from_reference(r_ref, SHAPE)
        assert np.abs(r - r_ref_c).max() <= 1e-13 * np.abs(r_ref_c).max()
    p.close()


_FIRST_CALL = r"""
import sys
sys.path.insert(0, {root!r})
import numpy as np, torch
sys.path.insert(0, {root!r} + "/tests")
import test_zz_no_alloc as T
rho, u, f, fixed_node = T._case(T.SHAPE, 3)
x = torch.zeros(1, device="cuda:0")  # the caller's own context; the library is not called yet
r, rr = T._call_noalloc(torch, T.SHAPE, rho, u, f, fixed_node)
T._check(r, rr, T._oracle_residual(T.SHAPE, rho, u, f, fixed_node))
r2, rr2 = T._call_noalloc(torch, T.SHAPE, rho, u, f, fixed_node)
assert np.array_equal(r, r2) and rr == rr2
print("first-call ok")
"""


@pytest.mark.gpu
def test_residual_noalloc_as_first_library_call():
    """A fresh process whose first (and only) calls into the library are the
    allocation-free ones: no problem handle was ever created."""
    pytest.importorskip("torch")
    out = subprocess.run([sys.executable, "-c", _FIRST_CALL.format(root=ROOT)], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "first-call ok" in out.stdout


def test_residual_noalloc_rejects_oversized_grid():
    L = nat.load()
    # ceil(2049/32) * ceil(2049/4) tiles exceed the fixed scratch; rejected before
    # any device work
    args = [ctypes.c_void_p(16)] * 6 + [None]
    st = L.am_residual_noalloc(2048, 2048, 4, 1.0, 1.0, 0.3, *args)
    assert nat.STATUS[st] == "AM_ERR_SIZE_MISMATCH"
    assert b"too large" in L.am_last_error()
    # dimensions whose +1 would overflow an int are refused outright
    st = L.am_residual_noalloc(2**31 - 1, 1, 1, 1.0, 1.0, 0.3, *args)
    assert nat.STATUS[st] == "AM_ERR_INVALID_ARG"
    st = L.am_residual_noalloc(1, 2**31 - 1, 1, 1.0, 1.0, 0.3, *args)
    assert nat.STATUS[st] == "AM_ERR_INVALID_ARG"
