"""am_residual_noalloc: the residual entry point for callers that cannot allocate
device memory (fixed memory pools, allocation-free real-time loops, plugins whose
host owns every buffer).  The test owns the device buffers (allocated with torch,
as such a caller's host would), calls the entry point through the C ABI twice in
a row, and checks each result against the handle-based am_ku_apply.

Collected last (file name) so that a failure here does not hide the others."""
import ctypes

import numpy as np
import pytest

from am_ml_suite_gb300 import _native as nat

pytestmark = pytest.mark.gpu


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


def test_residual_noalloc_matches_ku_apply():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    L = nat.load()
    shape = (37, 9, 13)
    nx, ny, nz = shape
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    h, E0, nu = 0.5, 2.0, 0.3
    fn = L.am_residual_noalloc
    p = nat.Problem(shape, h, E0, nu)
    # scale = rho exactly: C++ rule with E_min = 0, p = 1, rho_min = 0
    cfg = nat.default_config(nat.VARIANT_CPP, E_min=0.0, penalty=1.0, rho_min=0.0)
    for call, seed in enumerate((1, 2)):
        rho, u, f, fixed_node = _case(shape, seed)
        # the existing entry point: y = K u, then r = mask(f - y)
        y = p.ku(cfg, rho, u, nat.PREC_FP64)
        r_ref = f - y
        r_ref.reshape(-1, 3)[fixed_node] = 0.0
        r_ref_c = _compact_from_reference(r_ref, shape)
        # caller-owned device buffers in the compact layout
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
        st = fn(nx, ny, nz, h, E0, nu, ctypes.c_void_p(scale_d.data_ptr()), ctypes.c_void_p(u_d.data_ptr()),
                ctypes.c_void_p(f_d.data_ptr()), ctypes.c_void_p(mask_d.data_ptr()), ctypes.c_void_p(r_d.data_ptr()),
                ctypes.c_void_p(rr_d.data_ptr()), None)
        assert st == nat.AM_OK, (call, nat.load().am_last_error())
        torch.cuda.synchronize()
        r = r_d.cpu().numpy()
        rr = float(rr_d.cpu().numpy()[0])
        scale = np.abs(r_ref_c).max()
        assert np.abs(r - r_ref_c).max() <= 1e-13 * scale, call
        assert rr == pytest.approx(float(np.sum(r_ref_c * r_ref_c)), rel=1e-12), call


def test_residual_noalloc_rejects_oversized_grid():
    L = nat.load()
    # ceil(2049/32) * ceil(2049/4) tiles exceed the fixed scratch; rejected before
    # any device work
    st = L.am_residual_noalloc(2048, 2048, 4, 1.0, 1.0, 0.3, ctypes.c_void_p(16), ctypes.c_void_p(16),
                               ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
                               None)
    assert nat.STATUS[st] == "AM_ERR_SIZE_MISMATCH"
    assert b"too large" in L.am_last_error()
