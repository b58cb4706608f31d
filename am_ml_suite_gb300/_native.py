"""ctypes binding of the C ABI in include/am_gpu.h (libamgpu.so).

There is no CPU fallback: if the library is missing or no CUDA device is
present, the calls raise.  Host arrays are numpy float64 / int8 / int64 in the
reference layouts (see include/am_gpu.h).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libamgpu.so")

AM_OK = 0
STATUS = {0: "AM_OK", 1: "AM_ERR_INVALID_ARG", 2: "AM_ERR_SIZE_MISMATCH", 3: "AM_ERR_DOF_OUT_OF_RANGE",
          4: "AM_ERR_NOT_CONVERGED", 5: "AM_ERR_NAN_DETECTED", 6: "AM_ERR_SINGULAR", 7: "AM_ERR_CUDA",
          8: "AM_ERR_TIMEOUT", 9: "AM_ERR_OOM", 10: "AM_ERR_NO_DEVICE"}

LAYOUT_ZFASTEST, LAYOUT_XFASTEST = 0, 1
VARIANT_CPP, VARIANT_PY = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
MIXED_RELIABLE, MIXED_FLEXIBLE = 0, 1
PRECOND_JACOBI, PRECOND_LEARNED, PRECOND_MG = 0, 1, 2


class AmError(RuntimeError):
    """A non-OK status returned by the native library."""

    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        self.name = STATUS.get(status, str(status))
        super().__init__(f"{where}: {self.name}: {detail}")


class SimpConfig(ctypes.Structure):
    """Mirror of ``am_simp_config``."""

    _fields_ = [
        ("volume_fraction", ctypes.c_double),
        ("penalty", ctypes.c_double),
        ("filter_radius", ctypes.c_double),
        ("move_limit", ctypes.c_double),
        ("rho_min", ctypes.c_double),
        ("E_min", ctypes.c_double),
        ("convergence_tol", ctypes.c_double),
        ("max_iterations", ctypes.c_int),
        ("variant", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("preconditioner", ctypes.c_int),
        ("cg_tol", ctypes.c_double),
        ("cg_max_iterations", ctypes.c_int),
        ("warm_start", ctypes.c_int),
        ("inner_tol", ctypes.c_double),
        ("max_outer", ctypes.c_int),
        ("layout", ctypes.c_int),
        ("verbose", ctypes.c_int),
        ("mixed_solver", ctypes.c_int),
        ("mg_deflation", ctypes.c_int),
        ("cpp_assembly_index", ctypes.c_int),
    ]


class SolveStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("outer_iterations", ctypes.c_int),
        ("residual", ctypes.c_double),
        ("converged", ctypes.c_int),
        ("solve_time_s", ctypes.c_double),
        ("max_displacement", ctypes.c_double),
        ("min_displacement", ctypes.c_double),
        ("learned_applications", ctypes.c_int),
    ]


class IterationResult(ctypes.Structure):
    _fields_ = [
        ("compliance", ctypes.c_double),
        ("compliance_energy", ctypes.c_double),
        ("volume_fraction", ctypes.c_double),
        ("max_density_change", ctypes.c_double),
        ("solver_iterations", ctypes.c_int),
        ("solver_outer_iterations", ctypes.c_int),
        ("solver_residual", ctypes.c_double),
        ("solver_converged", ctypes.c_int),
        ("oc_passes", ctypes.c_int),
        ("assembly_time_s", ctypes.c_double),
        ("solve_time_s", ctypes.c_double),
        ("sensitivity_time_s", ctypes.c_double),
        ("update_time_s", ctypes.c_double),
        ("solver_learned_applications", ctypes.c_int),
    ]


class TrainConfig(ctypes.Structure):
    """Mirror of ``am_train_config``."""

    _fields_ = [
        ("epochs", ctypes.c_int),
        ("batch", ctypes.c_int),
        ("lr", ctypes.c_float),
        ("beta1", ctypes.c_float),
        ("beta2", ctypes.c_float),
        ("eps", ctypes.c_float),
        ("seed", ctypes.c_uint64),
        ("verbose", ctypes.c_int),
        ("loss", ctypes.c_int),
    ]


class RunMetadata(ctypes.Structure):
    """Mirror of ``am_run_metadata``."""

    _fields_ = [
        ("case_name", ctypes.c_char_p), ("mode", ctypes.c_char_p), ("provenance", ctypes.c_char_p),
        ("resolution_mm", ctypes.c_double),
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("n_elements", ctypes.c_longlong), ("n_design", ctypes.c_longlong), ("n_fixed", ctypes.c_longlong),
        ("n_void", ctypes.c_longlong),
        ("volume_fraction_target", ctypes.c_double),
        ("has_history", ctypes.c_int),
        ("volume_fraction_final", ctypes.c_double), ("compliance_final", ctypes.c_double),
        ("iterations", ctypes.c_int), ("converged", ctypes.c_int),
        ("elapsed_time_s", ctypes.c_double),
        ("threads", ctypes.c_int),
        ("filter_radius", ctypes.c_double), ("E_min", ctypes.c_double), ("penalty", ctypes.c_double),
        ("move_limit", ctypes.c_double),
    ]


class BracketParams(ctypes.Structure):
    """Mirror of ``am_bracket_params``."""

    _fields_ = [
        ("size_mm", ctypes.c_double * 3),
        ("resolution_mm", ctypes.c_double),
        ("base_thickness_mm", ctypes.c_double),
        ("hole_diameter_mm", ctypes.c_double),
        ("hole_offset_mm", ctypes.c_double),
        ("eyelet_diameter_mm", ctypes.c_double),
        ("eyelet_offset_mm", ctypes.c_double),
        ("eyelet_z_offset_mm", ctypes.c_double),
        ("eyelet_height_mm", ctypes.c_double),
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
    ]


_dp = ctypes.POINTER(ctypes.c_double)
_i8p = ctypes.POINTER(ctypes.c_int8)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_i64p = ctypes.POINTER(ctypes.c_int64)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p

# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "am_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "am_last_error": (ctypes.c_char_p, []),
    "am_is_available": (ctypes.c_int, []),
    "am_device_info": (ctypes.c_int, [_ip, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]),
    "am_simp_config_default": (None, [ctypes.POINTER(SimpConfig), ctypes.c_int]),
    "am_element_stiffness": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp]),
    "am_problem_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, _i8p, ctypes.c_int,
                                         ctypes.POINTER(_vp)]),
    "am_problem_destroy": (ctypes.c_int, [_vp]),
    "am_problem_set_loads": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _i64p, _i64p]),
    "am_ku_apply": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp, _dp, _dp, ctypes.c_int]),
    "am_ku_pcg_step": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp, ctypes.c_int, _dp, _dp, ctypes.c_double,
                                      ctypes.c_int, _dp, _dp, _dp]),
    "am_solve": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp, ctypes.c_int, _dp,
                                ctypes.POINTER(SolveStats)]),
    "am_sensitivities": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp, _dp, _dp, _dp, _dp]),
    "am_filter": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), ctypes.c_int, _dp, _dp, _dp]),
    "am_oc_update": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp, _dp, _u8p, _dp, _dp, _ip]),
    "am_simp_run": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp, _dp, _dp, _dp, _dp, _ip, _ip]),
    "am_simp_begin": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp]),
    "am_simp_step": (ctypes.c_int, [_vp, ctypes.POINTER(IterationResult)]),
    "am_simp_get_density": (ctypes.c_int, [_vp, _dp]),
    "am_launch_count": (ctypes.c_longlong, []),
    "am_selftest_copy_wait": (ctypes.c_int, [ctypes.c_double, _ip, _dp]),
    "am_selftest_solve_timeout": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp, ctypes.c_int, _ip]),
    "am_bench_kernel": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "am_problem_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "am_precond_create": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_longlong, ctypes.POINTER(_vp)]),
    "am_precond_destroy": (ctypes.c_int, [_vp]),
    "am_precond_num_params": (ctypes.c_longlong, [_vp]),
    "am_precond_num_samples": (ctypes.c_longlong, [_vp]),
    "am_precond_get_params": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "am_precond_set_params": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "am_precond_forward": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "am_precond_param_grad": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                             ctypes.POINTER(ctypes.c_float)]),
    "am_precond_bench_forward": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, _dp, _dp]),
    "am_precond_harvest": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(SimpConfig), _dp, ctypes.c_int, _ip,
                                          ctypes.c_int]),
    "am_precond_train": (ctypes.c_int, [_vp, ctypes.POINTER(TrainConfig), ctypes.POINTER(ctypes.c_float)]),
    "am_precond_eval": (ctypes.c_int, [_vp, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int, _dp]),
    "am_problem_set_preconditioner": (ctypes.c_int, [_vp, _vp]),
    "am_problem_set_device_loop": (ctypes.c_int, [_vp, ctypes.c_int]),
    "am_problem_set_ku_plan": (ctypes.c_int, [_vp, ctypes.c_int]),
    "am_problem_get_ku_plan": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_int)]),
    "am_problem_set_residual_arithmetic": (ctypes.c_int, [_vp, ctypes.c_int]),
    "am_batch_set_device_loop": (ctypes.c_int, [_vp, ctypes.c_int]),
    "am_batch_set_plan": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "am_batch_axes": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "am_batch_set_staged": (ctypes.c_int, [_vp, ctypes.c_int]),
    "am_batch_bench_ku": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "am_precond_set_kernels": (ctypes.c_int, [ctypes.c_int]),
    "am_unet_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                      ctypes.POINTER(_vp)]),
    "am_unet_destroy": (ctypes.c_int, [_vp]),
    "am_unet_num_params": (ctypes.c_longlong, [_vp]),
    "am_unet_get_params": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "am_unet_set_params": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "am_unet_forward": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
    "am_unet_param_grad": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                          ctypes.POINTER(ctypes.c_float)]),
    "am_unet_set_data": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), _u8p]),
    "am_unet_train": (ctypes.c_int, [_vp, ctypes.POINTER(TrainConfig), ctypes.POINTER(ctypes.c_float)]),
    "am_unet_eval": (ctypes.c_int, [_vp, _dp]),
    "am_bracket_params_default": (None, [ctypes.POINTER(BracketParams), ctypes.c_double]),
    "am_bracket_build": (ctypes.c_int, [ctypes.POINTER(BracketParams), _dp, ctypes.c_int, _i8p, _dp, _i64p, _i64p,
                                        _i64p, _i64p, ctypes.c_int64]),
    "am_write_density_npy": (ctypes.c_int, [ctypes.c_char_p, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int]),
    "am_write_history_csv": (ctypes.c_int, [ctypes.c_char_p, _dp, _dp, ctypes.c_int]),
    "am_write_metadata_json": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(RunMetadata)]),
    "am_batch_create": (ctypes.c_int, [ctypes.c_int, _ip, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.POINTER(_vp)]),
    "am_batch_destroy": (ctypes.c_int, [_vp]),
    "am_batch_set_loads": (ctypes.c_int, [_vp, _dp, _i64p, _i64p]),
    "am_batch_autotune": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _ip, _ip, _dp]),
    "am_batch_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "am_batch_simp_begin": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp]),
    "am_batch_simp_step": (ctypes.c_int, [_vp, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_longlong), _ip]),
    "am_batch_get_density": (ctypes.c_int, [_vp, _dp]),
    "am_batch_simp_run": (ctypes.c_int, [_vp, ctypes.POINTER(SimpConfig), _dp, _dp, _dp, _dp, _ip, _ip,
                                         ctypes.POINTER(ctypes.c_longlong)]),
    "am_problem_layout": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                                         ctypes.POINTER(ctypes.c_longlong), _ip]),
    # device pointers are passed as c_void_p
    "am_residual_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
}

_LIB = None


def load(path: str = LIB_PATH):
    """Loads libamgpu.so (raises if it is absent: there is no fallback)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(path):
            raise ImportError(f"native library not built: {path} (run am_ml_suite_gb300._build.build())")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status: int, where: str):
    if status != AM_OK:
        detail = load().am_last_error()
        raise AmError(status, where, detail.decode() if detail else "")


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def ptr(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


def default_config(variant: int = VARIANT_CPP, **kw) -> SimpConfig:
    cfg = SimpConfig()
    load().am_simp_config_default(ctypes.byref(cfg), int(variant))
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise AttributeError(f"unknown config field {k}")
        setattr(cfg, k, v)
    return cfg


def is_available() -> bool:
    try:
        return bool(load().am_is_available())
    except (ImportError, OSError):
        return False


def element_stiffness(E: float = 1.0, nu: float = 0.3, h: float = 1.0) -> np.ndarray:
    out = np.zeros((24, 24))
    check(load().am_element_stiffness(E, nu, h, ptr(out)), "am_element_stiffness")
    return out


class Problem:
    """Owns an ``am_problem`` handle (one voxel domain on the current device)."""

    def __init__(self, shape, h=1.0, E0=1.0, nu=0.3, grid=None, layout=LAYOUT_ZFASTEST):
        L = load()
        self.shape = tuple(int(s) for s in shape)
        nx, ny, nz = self.shape
        self.nel = nx * ny * nz
        self.N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
        self.layout = layout
        g = None if grid is None else np.ascontiguousarray(grid, dtype=np.int8).ravel()
        if g is not None and g.size != self.nel:
            raise ValueError("grid size mismatch")
        self._grid = g
        h_ = _vp()
        check(L.am_problem_create(nx, ny, nz, float(h), float(E0), float(nu), ptr(g, _i8p), int(layout),
                                  ctypes.byref(h_)), "am_problem_create")
        self.handle = h_
        self.n_cases = 0

    def close(self):
        if getattr(self, "handle", None):
            load().am_problem_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_loads(self, F_list, fixed_list):
        F = np.ascontiguousarray(np.stack([f64(f).ravel() for f in F_list]))
        if F.shape[1] != self.N:
            raise ValueError("force vector size mismatch")
        fx = [np.asarray(f, dtype=np.int64).ravel() for f in fixed_list]
        fixed = np.ascontiguousarray(np.concatenate(fx) if fx else np.zeros(0, np.int64))
        nf = np.array([f.size for f in fx], dtype=np.int64)
        check(load().am_problem_set_loads(self.handle, F.shape[0], ptr(F), ptr(fixed, _i64p), ptr(nf, _i64p)),
              "am_problem_set_loads")
        self.n_cases = F.shape[0]

    def _rho(self, rho):
        r = f64(rho).ravel()
        if r.size != self.nel:
            raise ValueError("density size mismatch")
        return r

    def ku(self, cfg, rho, u, precision=PREC_FP64):
        u = f64(u).ravel()
        y = np.zeros(self.N)
        check(load().am_ku_apply(self.handle, ctypes.byref(cfg), ptr(self._rho(rho)), ptr(u), ptr(y),
                                 int(precision)), "am_ku_apply")
        return y

    def ku_pcg_step(self, cfg, rho, r, p_prev, beta, impl=3, load_case=0):
        """One FP32 inner-PCG K*u step: returns (p, q, p.q) with p = D^-1 r + beta p_prev
        and q = mask(K p) (impl 3: the staged kernel the solver runs, 2: the
        register-direct kernel it replaced)."""
        r = f64(r).ravel()
        pp = f64(p_prev).ravel()
        if r.size != self.N or pp.size != self.N:
            raise ValueError("vector size mismatch")
        p_out = np.zeros(self.N)
        q_out = np.zeros(self.N)
        pq = ctypes.c_double(0.0)
        check(load().am_ku_pcg_step(self.handle, ctypes.byref(cfg), ptr(self._rho(rho)), int(load_case), ptr(r),
                                    ptr(pp), float(beta), int(impl), ptr(p_out), ptr(q_out), ctypes.byref(pq)),
              "am_ku_pcg_step")
        return p_out, q_out, pq.value

    def selftest_solve_timeout(self, cfg, rho, load_case=0):
        """Status (an int) that am_solve returns when a kernel of its PCG reports a
        copy wait that ran out; the flag is set on the host, no wait runs out."""
        st = ctypes.c_int(-1)
        check(load().am_selftest_solve_timeout(self.handle, ctypes.byref(cfg), ptr(self._rho(rho)), int(load_case),
                                               ctypes.byref(st)), "am_selftest_solve_timeout")
        return st.value

    def solve(self, cfg, rho, load_case=0):
        u = np.zeros(self.N)
        st = SolveStats()
        check(load().am_solve(self.handle, ctypes.byref(cfg), ptr(self._rho(rho)), int(load_case), ptr(u),
                              ctypes.byref(st)), "am_solve")
        return u, st

    def sensitivities(self, cfg, rho, u):
        dc = np.zeros(self.nel)
        ce = np.zeros(self.nel)
        c = ctypes.c_double(0.0)
        check(load().am_sensitivities(self.handle, ctypes.byref(cfg), ptr(self._rho(rho)), ptr(f64(u).ravel()),
                                      ptr(dc), ptr(ce), ctypes.byref(c)), "am_sensitivities")
        return dc, ce, c.value

    def filter(self, cfg, which, x, rho=None):
        out = np.zeros(self.nel)
        r = None if rho is None else self._rho(rho)
        check(load().am_filter(self.handle, ctypes.byref(cfg), int(which), ptr(self._rho(x)), ptr(r), ptr(out)),
              "am_filter")
        return out

    def oc_update(self, cfg, rho, dc, design):
        out = np.zeros(self.nel)
        d = np.ascontiguousarray(design, dtype=np.uint8).ravel()
        mc = ctypes.c_double(0.0)
        passes = ctypes.c_int(0)
        check(load().am_oc_update(self.handle, ctypes.byref(cfg), ptr(self._rho(rho)), ptr(self._rho(dc)),
                                  ptr(d, _u8p), ptr(out), ctypes.byref(mc), ctypes.byref(passes)),
              "am_oc_update")
        return out, mc.value, passes.value

    def simp_run(self, cfg, rho0=None):
        m = max(int(cfg.max_iterations), 1)
        rho = np.zeros(self.nel)
        ch, vh, dh = np.zeros(m), np.zeros(m), np.zeros(m)
        it, conv = ctypes.c_int(0), ctypes.c_int(0)
        r0 = None if rho0 is None else self._rho(rho0)
        check(load().am_simp_run(self.handle, ctypes.byref(cfg), ptr(r0), ptr(rho), ptr(ch), ptr(vh), ptr(dh),
                                 ctypes.byref(it), ctypes.byref(conv)), "am_simp_run")
        n = it.value
        return dict(density=rho, compliance=ch[:n], volume=vh[:n], change=dh[:n], iterations=n,
                    converged=bool(conv.value))

    def simp_begin(self, cfg, rho0=None):
        r0 = None if rho0 is None else self._rho(rho0)
        check(load().am_simp_begin(self.handle, ctypes.byref(cfg), ptr(r0)), "am_simp_begin")

    def simp_step(self) -> IterationResult:
        res = IterationResult()
        check(load().am_simp_step(self.handle, ctypes.byref(res)), "am_simp_step")
        return res

    def simp_density(self):
        out = np.zeros(self.nel)
        check(load().am_simp_get_density(self.handle, ptr(out)), "am_simp_get_density")
        return out

    def bench_kernel(self, which: int, reps: int = 20, flush_l2: bool = True):
        avg, mn = ctypes.c_double(0.0), ctypes.c_double(0.0)
        check(load().am_bench_kernel(self.handle, int(which), int(reps), int(flush_l2), ctypes.byref(avg),
                                     ctypes.byref(mn)), "am_bench_kernel")
        return avg.value, mn.value

    def stream(self) -> int:
        """The cudaStream_t of this problem's kernels, as an integer."""
        st = _vp()
        check(load().am_problem_stream(self.handle, ctypes.byref(st)), "am_problem_stream")
        return int(st.value or 0)

    def set_preconditioner(self, pre):
        check(load().am_problem_set_preconditioner(self.handle, None if pre is None else pre.handle),
              "am_problem_set_preconditioner")
        self._pre = pre

    def set_device_loop(self, on=True):
        """True (default): each inner PCG solve is one CUDA-graph launch with a
        device-side loop; False: the host launches and checks chunk by chunk."""
        check(load().am_problem_set_device_loop(self.handle, int(bool(on))), "am_problem_set_device_loop")

    def set_ku_plan(self, warps=0):
        """Tile height of the FP32 PCG's staged K*u: 0 (chosen by grid), 7 or 8 warps."""
        check(load().am_problem_set_ku_plan(self.handle, int(warps)), "am_problem_set_ku_plan")

    def ku_plan(self):
        """The staged K*u's plan: dict(warps, tiles, z_chunk)."""
        w, t, z = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        check(load().am_problem_get_ku_plan(self.handle, ctypes.byref(w), ctypes.byref(t), ctypes.byref(z)),
              "am_problem_get_ku_plan")
        return {"warps": w.value, "tiles": t.value, "z_chunk": z.value}

    def set_residual_arithmetic(self, mode):
        """RESID_DOUBLE_FLOAT (default) or RESID_FP64: the arithmetic of the mixed
        solvers' residual replacements and acceptance test."""
        check(load().am_problem_set_residual_arithmetic(self.handle, int(mode)), "am_problem_set_residual_arithmetic")

    def layout_info(self):
        n, e, cs = ctypes.c_longlong(0), ctypes.c_longlong(0), ctypes.c_longlong(0)
        t = ctypes.c_int(0)
        check(load().am_problem_layout(self.handle, ctypes.byref(n), ctypes.byref(e), ctypes.byref(cs),
                                       ctypes.byref(t)), "am_problem_layout")
        return dict(nodes=n.value, elements=e.value, vector_stride=cs.value, ku_tiles=t.value)


_fp = ctypes.POINTER(ctypes.c_float)


class Preconditioner:
    """Owns an ``am_precond`` handle: the learned conv3d preconditioner."""

    def __init__(self, seed=0, capacity=4096):
        h = _vp()
        check(load().am_precond_create(int(seed), int(capacity), ctypes.byref(h)), "am_precond_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            load().am_precond_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return int(load().am_precond_num_params(self.handle))

    @property
    def num_samples(self) -> int:
        return int(load().am_precond_num_samples(self.handle))

    def get_params(self) -> np.ndarray:
        w = np.zeros(self.num_params, np.float32)
        check(load().am_precond_get_params(self.handle, w.ctypes.data_as(_fp)), "am_precond_get_params")
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        if w.size != self.num_params:
            raise ValueError("parameter count mismatch")
        check(load().am_precond_set_params(self.handle, w.ctypes.data_as(_fp)), "am_precond_set_params")

    def forward(self, x):
        """x: (n, gz, gy, gx, 4) float32 -> (n, gz, gy, gx, 3)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        n, gz, gy, gx, c = x.shape
        if c != 4:
            raise ValueError("input has 4 channels")
        out = np.zeros((n, gz, gy, gx, 3), np.float32)
        check(load().am_precond_forward(self.handle, n, gz, gy, gx, x.ctypes.data_as(_fp),
                                        out.ctypes.data_as(_fp)), "am_precond_forward")
        return out

    def param_grad(self, x, dout):
        x = np.ascontiguousarray(x, dtype=np.float32)
        dout = np.ascontiguousarray(dout, dtype=np.float32)
        n, gz, gy, gx, _ = x.shape
        g = np.zeros(self.num_params, np.float32)
        check(load().am_precond_param_grad(self.handle, n, gz, gy, gx, x.ctypes.data_as(_fp),
                                           dout.ctypes.data_as(_fp), g.ctypes.data_as(_fp)), "am_precond_param_grad")
        return g

    def bench_forward(self, n, gz, gy, gx, reps=5):
        """(ms per forward pass, convolution flops per pass) on a device tensor."""
        ms, fl = ctypes.c_double(0.0), ctypes.c_double(0.0)
        check(load().am_precond_bench_forward(self.handle, int(n), int(gz), int(gy), int(gx), int(reps),
                                              ctypes.byref(ms), ctypes.byref(fl)), "am_precond_bench_forward")
        return ms.value, fl.value

    def harvest(self, problem, cfg, rho, iters, load_case=0):
        it = np.ascontiguousarray(iters, dtype=np.int32)
        check(load().am_precond_harvest(self.handle, problem.handle, ctypes.byref(cfg), ptr(problem._rho(rho)),
                                        int(load_case), ptr(it, _ip), it.size), "am_precond_harvest")

    LOSS_RESIDUAL, LOSS_ENERGY = 0, 1

    def train(self, epochs=20, batch=8, lr=1e-3, seed=0, verbose=0, loss=0):
        c = TrainConfig(int(epochs), int(batch), float(lr), 0.9, 0.999, 1e-8, int(seed), int(verbose), int(loss))
        losses = np.zeros(max(int(epochs), 1), np.float32)
        check(load().am_precond_train(self.handle, ctypes.byref(c), losses.ctypes.data_as(_fp)), "am_precond_train")
        return losses[:int(epochs)]

    def eval(self, first=0, count=None, loss=0):
        count = self.num_samples - first if count is None else count
        v = ctypes.c_double(0.0)
        check(load().am_precond_eval(self.handle, int(first), int(count), int(loss), ctypes.byref(v)),
              "am_precond_eval")
        return v.value


class UNet:
    """Owns an ``am_unet`` handle: the density-predicting 3-D U-Net."""

    def __init__(self, in_channels=4, out_channels=1, f0=32, seed=0):
        h = _vp()
        check(load().am_unet_create(int(in_channels), int(out_channels), int(f0), int(seed), ctypes.byref(h)),
              "am_unet_create")
        self.handle = h
        self.in_channels, self.out_channels, self.f0 = int(in_channels), int(out_channels), int(f0)

    def close(self):
        if getattr(self, "handle", None):
            load().am_unet_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return int(load().am_unet_num_params(self.handle))

    def get_params(self) -> np.ndarray:
        w = np.zeros(self.num_params, np.float32)
        check(load().am_unet_get_params(self.handle, w.ctypes.data_as(_fp)), "am_unet_get_params")
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        if w.size != self.num_params:
            raise ValueError("parameter count mismatch")
        check(load().am_unet_set_params(self.handle, w.ctypes.data_as(_fp)), "am_unet_set_params")

    def forward(self, x, sigmoid=True):
        """x: (n, gz, gy, gx, in_channels) -> (n, gz, gy, gx, out_channels)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        n, gz, gy, gx, c = x.shape
        if c != self.in_channels:
            raise ValueError("input channel count mismatch")
        out = np.zeros((n, gz, gy, gx, self.out_channels), np.float32)
        check(load().am_unet_forward(self.handle, n, gz, gy, gx, x.ctypes.data_as(_fp), out.ctypes.data_as(_fp),
                                     int(bool(sigmoid))), "am_unet_forward")
        return out

    def param_grad(self, x, dout):
        x = np.ascontiguousarray(x, dtype=np.float32)
        dout = np.ascontiguousarray(dout, dtype=np.float32)
        n, gz, gy, gx, _ = x.shape
        g = np.zeros(self.num_params, np.float32)
        check(load().am_unet_param_grad(self.handle, n, gz, gy, gx, x.ctypes.data_as(_fp), dout.ctypes.data_as(_fp),
                                        g.ctypes.data_as(_fp)), "am_unet_param_grad")
        return g

    def set_data(self, inputs, targets, mask):
        x = np.ascontiguousarray(inputs, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        S, gz, gy, gx, c = x.shape
        if c != self.in_channels or t.shape != (S, gz, gy, gx) or m.shape != t.shape:
            raise ValueError("training tensors have inconsistent shapes")
        check(load().am_unet_set_data(self.handle, S, gz, gy, gx, x.ctypes.data_as(_fp), t.ctypes.data_as(_fp),
                                      m.ctypes.data_as(_u8p)), "am_unet_set_data")

    def train(self, epochs=50, batch=4, lr=1e-3, seed=0, verbose=0):
        c = TrainConfig(int(epochs), int(batch), float(lr), 0.9, 0.999, 1e-8, int(seed), int(verbose), 0)
        losses = np.zeros(max(int(epochs), 1), np.float32)
        check(load().am_unet_train(self.handle, ctypes.byref(c), losses.ctypes.data_as(_fp)), "am_unet_train")
        return losses[:int(epochs)]

    def eval(self) -> float:
        v = ctypes.c_double(0.0)
        check(load().am_unet_eval(self.handle, ctypes.byref(v)), "am_unet_eval")
        return v.value


CONV_MMA_SYNC, CONV_TCGEN05 = 0, 1
RESID_DOUBLE_FLOAT, RESID_FP64 = 0, 1


def set_conv_kernels(impl: int):
    """Kernels of the network's convolutions: CONV_TCGEN05 (default) or the legacy
    CONV_MMA_SYNC baseline."""
    check(load().am_precond_set_kernels(int(impl)), "am_precond_set_kernels")


class Batch:
    """Owns an ``am_batch`` handle: independent C++-variant problems of uneven
    sizes solved together (one kernel launch per family for the whole batch)."""

    def __init__(self, shapes, h=1.0, E0=1.0, nu=0.3):
        L = load()
        self.shapes = [tuple(int(v) for v in s) for s in shapes]
        self.n = len(self.shapes)
        sh = np.ascontiguousarray(np.array(self.shapes, dtype=np.int32).ravel())
        h_ = _vp()
        check(L.am_batch_create(self.n, ptr(sh, _ip), float(h), float(E0), float(nu), ctypes.byref(h_)),
              "am_batch_create")
        self.handle = h_
        self.nel = [nx * ny * nz for nx, ny, nz in self.shapes]
        self.N = [3 * (nx + 1) * (ny + 1) * (nz + 1) for nx, ny, nz in self.shapes]

    def close(self):
        if getattr(self, "handle", None):
            load().am_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_loads(self, F_list, fixed_list):
        if len(F_list) != self.n or len(fixed_list) != self.n:
            raise ValueError("one force vector and one fixed-DOF list per problem")
        for f, N in zip(F_list, self.N):
            if np.asarray(f).size != N:
                raise ValueError("force vector size mismatch")
        F = np.ascontiguousarray(np.concatenate([f64(f).ravel() for f in F_list]))
        fx = [np.asarray(f, dtype=np.int64).ravel() for f in fixed_list]
        fixed = np.ascontiguousarray(np.concatenate(fx) if fx else np.zeros(0, np.int64))
        nf = np.array([f.size for f in fx], dtype=np.int64)
        check(load().am_batch_set_loads(self.handle, ptr(F), ptr(fixed, _i64p), ptr(nf, _i64p)),
              "am_batch_set_loads")

    def autotune(self, reps=3):
        w, z, c = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        ms = ctypes.c_double(0.0)
        check(load().am_batch_autotune(self.handle, int(reps), ctypes.byref(w), ctypes.byref(z), ctypes.byref(c),
                                       ctypes.byref(ms)), "am_batch_autotune")
        return dict(warps=w.value, z_chunk=z.value, ctas_per_sm=c.value, ms=ms.value)

    def stream(self) -> int:
        st = _vp()
        check(load().am_batch_stream(self.handle, ctypes.byref(st)), "am_batch_stream")
        return int(st.value or 0)

    def set_device_loop(self, on=True):
        check(load().am_batch_set_device_loop(self.handle, int(bool(on))), "am_batch_set_device_loop")

    def set_staged(self, on=True):
        """True (default): the FP32 PCG K*u runs the tensor-copy staged kernel;
        False: the warp-row kernel with the autotuned / pinned plan."""
        check(load().am_batch_set_staged(self.handle, int(bool(on))), "am_batch_set_staged")

    def bench_ku(self, reps=10):
        """Average ms of one batched FP32 PCG K*u launch (every problem active), on
        the state the last simp_step left."""
        ms = ctypes.c_double(0.0)
        check(load().am_batch_bench_ku(self.handle, int(reps), ctypes.byref(ms)), "am_batch_bench_ku")
        return ms.value

    def axes(self, i):
        """The caller's axis (0 = x, 1 = y, 2 = z) that problem i stores as each of its
        internal axes (the first is the K*u tiles' 30-column axis)."""
        a = (ctypes.c_int * 3)()
        check(load().am_batch_axes(self.handle, int(i), a), "am_batch_axes")
        return tuple(a)

    def set_plan(self, warps, z_chunk=0, ctas_per_sm=2):
        """Pins the batched K*u plan: warps 0 (per problem), 4 or 8."""
        check(load().am_batch_set_plan(self.handle, int(warps), int(z_chunk), int(ctas_per_sm)), "am_batch_set_plan")

    def simp_begin(self, cfgs, rho0_list=None):
        if len(cfgs) != self.n:
            raise ValueError("one config per problem")
        self._cfgs = (SimpConfig * self.n)(*cfgs)
        r0 = None
        if rho0_list is not None:
            r0 = np.ascontiguousarray(np.concatenate([f64(r).ravel() for r in rho0_list]))
            if r0.size != sum(self.nel):
                raise ValueError("density size mismatch")
        check(load().am_batch_simp_begin(self.handle, self._cfgs, ptr(r0)), "am_batch_simp_begin")

    def simp_step(self):
        """One SIMP iteration of every running problem: (compliance, volume,
        change) arrays (NaN for problems that did not step) and the number still
        running; ``self.pcg_iterations`` holds each problem's PCG iterations so far."""
        c, v, d = (np.full(self.n, np.nan) for _ in range(3))
        pcg = np.zeros(self.n, np.int64)
        act = ctypes.c_int(0)
        check(load().am_batch_simp_step(self.handle, ptr(c), ptr(v), ptr(d),
                                        pcg.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), ctypes.byref(act)),
              "am_batch_simp_step")
        self.pcg_iterations = pcg
        return c, v, d, act.value

    def densities(self):
        rho = np.zeros(sum(self.nel))
        check(load().am_batch_get_density(self.handle, ptr(rho)), "am_batch_get_density")
        out, o = [], 0
        for ne in self.nel:
            out.append(rho[o:o + ne].copy())
            o += ne
        return out

    def simp_run(self, cfgs, rho0_list=None):
        if len(cfgs) != self.n:
            raise ValueError("one config per problem")
        arr = (SimpConfig * self.n)(*cfgs)
        H = max(max(int(c.max_iterations) for c in cfgs), 1)
        r0 = None
        if rho0_list is not None:
            r0 = np.ascontiguousarray(np.concatenate([f64(r).ravel() for r in rho0_list]))
            if r0.size != sum(self.nel):
                raise ValueError("density size mismatch")
        rho = np.zeros(sum(self.nel))
        ch, vh = np.zeros(self.n * H), np.zeros(self.n * H)
        it, conv = np.zeros(self.n, np.int32), np.zeros(self.n, np.int32)
        pcg = np.zeros(self.n, np.int64)
        check(load().am_batch_simp_run(self.handle, arr, ptr(r0), ptr(rho), ptr(ch), ptr(vh), ptr(it, _ip),
                                       ptr(conv, _ip), pcg.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))),
              "am_batch_simp_run")
        out, o = [], 0
        for p, (nx, ny, nz) in enumerate(self.shapes):
            k = int(it[p])
            out.append(dict(density=rho[o:o + self.nel[p]].copy(), compliance=ch[p * H:p * H + k].copy(),
                            volume=vh[p * H:p * H + k].copy(), iterations=k, converged=bool(conv[p]),
                            pcg_iterations=int(pcg[p])))
            o += self.nel[p]
        return out


def write_density_npy(path, rho, shape, layout=LAYOUT_ZFASTEST):
    nx, ny, nz = (int(v) for v in shape)
    r = f64(rho).ravel()
    if r.size != nx * ny * nz:
        raise ValueError("density size mismatch")
    check(load().am_write_density_npy(os.fsencode(path), ptr(r), nx, ny, nz, int(layout)), "am_write_density_npy")


def write_history_csv(path, compliance, volume):
    c, v = f64(compliance).ravel(), f64(volume).ravel()
    if c.size != v.size:
        raise ValueError("history lengths differ")
    check(load().am_write_history_csv(os.fsencode(path), ptr(c), ptr(v), c.size), "am_write_history_csv")


def write_metadata_json(path, **fields):
    m = RunMetadata()
    for k, v in fields.items():
        if not hasattr(m, k):
            raise AttributeError(f"unknown metadata field {k}")
        setattr(m, k, v.encode() if isinstance(v, str) else v)
    check(load().am_write_metadata_json(os.fsencode(path), ctypes.byref(m)), "am_write_metadata_json")


def launch_count() -> int:
    return int(load().am_launch_count())


def selftest_copy_wait(limit_ms: float = 5.0):
    """Runs the bounded copy-wait self-test: (timed_out, waited_ms)."""
    t = ctypes.c_int(0)
    w = ctypes.c_double(0.0)
    check(load().am_selftest_copy_wait(float(limit_ms), ctypes.byref(t), ctypes.byref(w)), "am_selftest_copy_wait")
    return bool(t.value), w.value
