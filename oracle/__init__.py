"""FP64 CPU oracle for the SIMP inner loop -- TEST INFRASTRUCTURE ONLY.

This package is the oracle the CUDA path is tested against.  Only ``tests/``,
``__graft_entry__.smoke()`` and the cpu_baseline / reference arm of
``bench.py`` may import it; the product package ``am_ml_suite_gb300`` never
does, and has no CPU fallback.

The numpy wrappers below call ``liboracle.so`` (built from ``oracle.c`` by
``oracle/Makefile``).  Arrays use the reference layout: elements C-order
``(nx, ny, nz)`` (z fastest), DOFs ``3*(i*(ny+1)*(nz+1) + j*(nz+1) + k) + d``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_i8p = ctypes.POINTER(ctypes.c_int8)
_ip = ctypes.POINTER(ctypes.c_int)


class SimpParams(ctypes.Structure):
    """Mirror of ``orc_simp_params`` (oracle.h)."""

    _fields_ = [
        ("volume_fraction", ctypes.c_double),
        ("penalty", ctypes.c_double),
        ("filter_radius", ctypes.c_double),
        ("move_limit", ctypes.c_double),
        ("rho_min", ctypes.c_double),
        ("E_min", ctypes.c_double),
        ("convergence_tol", ctypes.c_double),
        ("max_iterations", ctypes.c_int),
        ("cg_tol", ctypes.c_double),
        ("cg_maxit", ctypes.c_int),
        ("bug_d1", ctypes.c_int),
        ("warm_start", ctypes.c_int),
        ("use_csr", ctypes.c_int),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile next to this file."""
    so = os.path.join(_HERE, "liboracle.so")
    src = os.path.join(_HERE, "oracle.c")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE, "-B" if force else "liboracle.so"])
    return so


def lib():
    global _LIB
    if _LIB is None:
        so = build()
        L = ctypes.CDLL(so)
        L.orc_ke.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_element_dofs.argtypes = [ctypes.c_int] * 6 + [_i64p]
        L.orc_scales.argtypes = [ctypes.c_int, ctypes.c_int64, _i8p, _dp, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_ku.argtypes = [ctypes.c_int] * 3 + [_dp, _dp, _dp, _dp]
        L.orc_csr_nnz.argtypes = [ctypes.c_int] * 3
        L.orc_csr_nnz.restype = ctypes.c_int64
        L.orc_csr_build.argtypes = [ctypes.c_int] * 3 + [_dp, _dp, _i64p, _i32p, _dp]
        L.orc_csr_spmv.argtypes = [ctypes.c_int64, _i64p, _i32p, _dp, _dp, _dp]
        L.orc_diag.argtypes = [ctypes.c_int] * 3 + [_dp, _dp, _dp]
        L.orc_pcg.argtypes = [ctypes.c_int] * 3 + [_dp, _dp, _u8p, _dp, _dp, ctypes.c_double,
                                                   ctypes.c_int, ctypes.c_int, _dp]
        L.orc_pcg.restype = ctypes.c_int
        L.orc_element_energy.argtypes = [ctypes.c_int] * 3 + [_dp, _dp, _dp]
        L.orc_filter_cpp.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double, _dp, _dp, _dp]
        L.orc_filter_py.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double, _dp, _dp]
        L.orc_oc_cpp.argtypes = [ctypes.c_int64, _dp, _dp, _u8p, ctypes.c_int64, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, _ip]
        L.orc_oc_cpp.restype = ctypes.c_double
        L.orc_oc_py.argtypes = [ctypes.c_int64, _dp, _dp, _u8p, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double, _dp]
        L.orc_oc_py.restype = ctypes.c_int
        L.orc_simp_cpp.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_double] * 3 +
                                   [ctypes.POINTER(SimpParams), _dp, _dp, _i64p, ctypes.c_int64,
                                    _dp, _dp, _dp, _dp, _ip, _ip])
        L.orc_simp_cpp.restype = ctypes.c_int
        L.orc_simp_py.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_double] * 3 +
                                  [ctypes.POINTER(SimpParams), _i8p, ctypes.c_int, _dp, _i64p, _i64p,
                                   _dp, _dp, _dp, _dp, _ip])
        L.orc_simp_py.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(t)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def ke(E=1.0, nu=0.3, h=1.0):
    out = np.zeros((24, 24))
    lib().orc_ke(E, nu, h, _p(out, _dp))
    return out


def element_dofs(ijk, shape):
    out = np.zeros(24, dtype=np.int64)
    lib().orc_element_dofs(*[int(v) for v in ijk], *[int(v) for v in shape], _p(out, _i64p))
    return out


def scales(variant, rho, grid=None, p=3.0, emin=1e-9, rho_min=0.0, E=1.0):
    rho = _f64(rho)
    out = np.zeros_like(rho)
    g = None if grid is None else np.ascontiguousarray(grid, dtype=np.int8)
    lib().orc_scales(int(variant), rho.size, None if g is None else _p(g, _i8p), _p(rho, _dp),
                     p, emin, rho_min, E, _p(out, _dp))
    return out


def ku(shape, kmat, s, u):
    nx, ny, nz = shape
    kmat, s, u = _f64(kmat), _f64(s), _f64(u)
    y = np.zeros_like(u)
    lib().orc_ku(nx, ny, nz, _p(kmat, _dp), _p(s, _dp), _p(u, _dp), _p(y, _dp))
    return y


def csr(shape, kmat, s):
    """(rowptr, col, val) of K(s)."""
    nx, ny, nz = shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    nnz = lib().orc_csr_nnz(nx, ny, nz)
    rowptr = np.zeros(N + 1, dtype=np.int64)
    col = np.zeros(nnz, dtype=np.int32)
    val = np.zeros(nnz)
    kmat, s = _f64(kmat), _f64(s)
    lib().orc_csr_build(nx, ny, nz, _p(kmat, _dp), _p(s, _dp), _p(rowptr, _i64p), _p(col, _i32p),
                        _p(val, _dp))
    return rowptr, col, val


def diag(shape, kmat, s):
    nx, ny, nz = shape
    out = np.zeros(3 * (nx + 1) * (ny + 1) * (nz + 1))
    kmat, s = _f64(kmat), _f64(s)
    lib().orc_diag(nx, ny, nz, _p(kmat, _dp), _p(s, _dp), _p(out, _dp))
    return out


def pcg(shape, kmat, s, constrained, F, u0=None, tol=1e-12, maxit=100000, use_csr=False):
    """Returns (u, iterations, relres)."""
    nx, ny, nz = shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    cons = np.zeros(N, dtype=np.uint8)
    if constrained is not None:
        c = np.asarray(constrained)
        if c.dtype == np.bool_ or (c.size == N and c.dtype == np.uint8):
            cons[:] = c.astype(np.uint8)
        else:
            cons[c.astype(np.int64)] = 1
    F = _f64(F)
    u = np.zeros(N) if u0 is None else _f64(u0).copy()
    rr = ctypes.c_double(0.0)
    kmat, s = _f64(kmat), _f64(s)
    it = lib().orc_pcg(nx, ny, nz, _p(kmat, _dp), _p(s, _dp), _p(cons, _u8p), _p(F, _dp), _p(u, _dp),
                       tol, maxit, int(use_csr), ctypes.byref(rr))
    return u, it, rr.value


def element_energy(shape, kmat, u):
    nx, ny, nz = shape
    out = np.zeros(nx * ny * nz)
    kmat, u = _f64(kmat), _f64(u)
    lib().orc_element_energy(nx, ny, nz, _p(kmat, _dp), _p(u, _dp), _p(out, _dp))
    return out


def filter_cpp(shape, r, dc, rho):
    nx, ny, nz = shape
    dc, rho = _f64(dc).ravel(), _f64(rho).ravel()
    out = np.zeros_like(dc)
    lib().orc_filter_cpp(nx, ny, nz, r, _p(dc, _dp), _p(rho, _dp), _p(out, _dp))
    return out


def filter_py(shape, r, x):
    nx, ny, nz = shape
    x = _f64(x).ravel()
    out = np.zeros_like(x)
    lib().orc_filter_py(nx, ny, nz, r, _p(x, _dp), _p(out, _dp))
    return out


def oc_cpp(rho, dc, design, vf, move, rho_min, n_design=None):
    """Returns (rho_new, max_change, passes)."""
    rho = _f64(rho).ravel().copy()
    dc = _f64(dc).ravel()
    d = np.ascontiguousarray(design, dtype=np.uint8).ravel()
    nd = int(d.sum()) if n_design is None else int(n_design)
    passes = ctypes.c_int(0)
    mc = lib().orc_oc_cpp(rho.size, _p(rho, _dp), _p(dc, _dp), _p(d, _u8p), nd, vf, move, rho_min,
                          ctypes.byref(passes))
    return rho, mc, passes.value


def oc_py(rho, dc, design, vf, move, rho_min):
    """Returns (rho_new, passes)."""
    rho = _f64(rho).ravel()
    dc = _f64(dc).ravel()
    d = np.ascontiguousarray(design, dtype=np.uint8).ravel()
    out = rho.copy()
    passes = lib().orc_oc_py(rho.size, _p(rho, _dp), _p(dc, _dp), _p(d, _u8p), vf, move, rho_min,
                             _p(out, _dp))
    return out, passes


def make_params(**kw):
    prm = SimpParams(volume_fraction=0.25, penalty=3.0, filter_radius=2.0, move_limit=0.2,
                     rho_min=0.01, E_min=1e-9, convergence_tol=0.01, max_iterations=100,
                     cg_tol=1e-12, cg_maxit=100000, bug_d1=0, warm_start=0, use_csr=0)
    for k, v in kw.items():
        setattr(prm, k, v)
    return prm


def simp_cpp(shape, h, E, nu, prm, rho0, F, fixed):
    nx, ny, nz = shape
    nel = nx * ny * nz
    m = prm.max_iterations
    rho0 = _f64(rho0).ravel()
    F = _f64(F)
    fixed = np.ascontiguousarray(fixed, dtype=np.int64)
    out = np.zeros(nel)
    ch, vh, dh = np.zeros(m), np.zeros(m), np.zeros(m)
    cg = np.zeros(m, dtype=np.int32)
    conv = ctypes.c_int(0)
    it = lib().orc_simp_cpp(nx, ny, nz, h, E, nu, ctypes.byref(prm), _p(rho0, _dp), _p(F, _dp),
                            _p(fixed, _i64p), fixed.size, _p(out, _dp), _p(ch, _dp), _p(vh, _dp),
                            _p(dh, _dp), cg.ctypes.data_as(_ip), ctypes.byref(conv))
    return dict(density=out.reshape(shape), compliance=ch[:it], volume=vh[:it], change=dh[:it],
                cg_iters=cg[:it], iterations=it, converged=bool(conv.value))


def simp_py(shape, h, E, nu, prm, grid, F_list, fixed_list):
    nx, ny, nz = shape
    nel = nx * ny * nz
    m = prm.max_iterations
    grid = np.ascontiguousarray(grid, dtype=np.int8).ravel()
    F = np.ascontiguousarray(np.stack([_f64(f) for f in F_list]))
    fx = [np.asarray(f, dtype=np.int64) for f in fixed_list]
    fixed = np.ascontiguousarray(np.concatenate(fx) if fx else np.zeros(0, np.int64))
    nf = np.array([f.size for f in fx], dtype=np.int64)
    out = np.zeros(nel)
    ch, vh, dh = np.zeros(m), np.zeros(m), np.zeros(m)
    conv = ctypes.c_int(0)
    it = lib().orc_simp_py(nx, ny, nz, h, E, nu, ctypes.byref(prm), _p(grid, _i8p), len(F_list),
                           _p(F, _dp), _p(fixed, _i64p), _p(nf, _i64p), _p(out, _dp), _p(ch, _dp),
                           _p(vh, _dp), _p(dh, _dp), ctypes.byref(conv))
    return dict(density=out.reshape(shape), compliance=ch[:it], volume=vh[:it], change=dh[:it],
                iterations=it, converged=bool(conv.value))


def baseline_sample(shape, prm, rho, F, fixed, pcg_iters=20):
    """Times one C++-variant SIMP iteration of the CPU restatement (CSR assembly,
    `pcg_iters` Jacobi-PCG iterations, sensitivities, filter, OC).  Returns
    (times dict in seconds, threads)."""
    L = lib()
    if not hasattr(L, "_bs_set"):
        L.orc_baseline_sample.argtypes = ([ctypes.c_int] * 3 + [ctypes.POINTER(SimpParams), _dp, _dp, _i64p,
                                          ctypes.c_int64, ctypes.c_int, _dp])
        L.orc_baseline_sample.restype = ctypes.c_int
        L._bs_set = True
    nx, ny, nz = shape
    rho = _f64(rho).ravel()
    F = _f64(F)
    fixed = np.ascontiguousarray(fixed, dtype=np.int64)
    t = np.zeros(6)
    th = L.orc_baseline_sample(nx, ny, nz, ctypes.byref(prm), _p(rho, _dp), _p(F, _dp), _p(fixed, _i64p),
                               fixed.size, int(pcg_iters), _p(t, _dp))
    keys = ["assembly", "pcg_setup", "pcg_iteration", "sensitivities", "filter", "oc"]
    return dict(zip(keys, t.tolist())), th
