"""Python host side of sclet_gb300: ctypes bindings of the C ABI
(include/sclet_gb300.h) and a small object wrapper.

The CUDA library must be built (energy-stability_gb300/build_ext.py); if it
is missing or fails to load, every entry point raises: there is no CPU path.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsclet_gb300.so")

AC, CH = 0, 1
FP64, MIXED = 0, 1
PHYSICS_LANDAU246, PHYSICS_FORMULA234 = 0, 1

_c_dp = ctypes.POINTER(ctypes.c_double)


class Params(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("px", ctypes.c_int), ("py", ctypes.c_int), ("pz", ctypes.c_int),
        ("nghost", ctypes.c_int),
        ("work_dir", ctypes.c_char * 1024), ("data_dir", ctypes.c_char * 1024),
        ("dt", ctypes.c_double), ("t_total", ctypes.c_double),
        ("epn2", ctypes.c_double),
        ("periodic", ctypes.c_int),
        ("nac", ctypes.c_int), ("nch", ctypes.c_int),
        ("restart", ctypes.c_int), ("restart_iter", ctypes.c_int),
        ("restart_dir", ctypes.c_char * 1024),
        ("xmin", ctypes.c_double), ("ymin", ctypes.c_double), ("zmin", ctypes.c_double),
        ("xmax", ctypes.c_double), ("ymax", ctypes.c_double), ("zmax", ctypes.c_double),
        ("etd2", ctypes.c_int), ("elastic", ctypes.c_int), ("anisotropic", ctypes.c_int),
        ("kkx", ctypes.c_double), ("kky", ctypes.c_double), ("kkz", ctypes.c_double),
        ("variable_mobility", ctypes.c_int),
        ("elastic_scale", ctypes.c_double),
        ("voigt", ctypes.c_double * 36),
        ("eigenstrain", ctypes.c_double * 36),
        ("lambda_file", ctypes.c_double * 36),
        ("landau", ctypes.c_double * 11),
        ("physics", ctypes.c_int),
    ]


class LearnedStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_longlong), ("fallbacks", ctypes.c_longlong),
                ("energy_fail", ctypes.c_longlong), ("mass_fail", ctypes.c_longlong),
                ("deviation_fail", ctypes.c_longlong), ("deviation_checks", ctypes.c_longlong),
                ("max_deviation", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Diag(ctypes.Structure):
    _fields_ = [("max", ctypes.c_double), ("min", ctypes.c_double), ("vol", ctypes.c_double),
                ("energy", ctypes.c_double)]


# Every entry point of include/sclet_gb300.h with its ctypes signature.
SIGNATURES = {
    "sclet_params_default": (None, [ctypes.c_void_p]),
    "sclet_read_ini": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p]),
    "sclet_read_elastic_input": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p]),
    "sclet_read_anisotropic_input": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p]),
    "sclet_read_landau_input": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p]),
    "sclet_read_case": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p]),
    "sclet_read_eigen": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _c_dp, _c_dp, _c_dp]),
    "sclet_eigen_dirichlet": (None, [ctypes.c_int, _c_dp, _c_dp, _c_dp]),
    "sclet_seeded_value": (ctypes.c_double, [ctypes.c_ulonglong, ctypes.c_int, ctypes.c_longlong,
                                             ctypes.c_double, ctypes.c_double]),
    "sclet_write_restart": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _c_dp]),
    "sclet_read_restart": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _c_dp]),
    "sclet_write_chk_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _c_dp]),
    "sclet_read_chk_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _c_dp]),
    "sclet_chk_path": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]),
    "sclet_field2b_path": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int]),
    "sclet_set_fields": (ctypes.c_int, [ctypes.c_void_p, _c_dp]),
    "sclet_get_fields": (ctypes.c_int, [ctypes.c_void_p, _c_dp]),
    "sclet_set_fields_async": (ctypes.c_int, [ctypes.c_void_p, _c_dp]),
    "sclet_get_fields_async": (ctypes.c_int, [ctypes.c_void_p, _c_dp]),
    "sclet_write_vtk_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_dp]),
    "sclet_write_vtk": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]),
    "sclet_append_soln_log": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_dp, _c_dp]),
    "sclet_log_soln": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]),
    "sclet_write_chk": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]),
    "sclet_read_chk": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "sclet_field_u16": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "sclet_write_field2b": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]),
    "sclet_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "sclet_create_runs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "sclet_destroy": (None, [ctypes.c_void_p]),
    "sclet_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "sclet_set_eigen": (ctypes.c_int, [ctypes.c_void_p, _c_dp, _c_dp, _c_dp]),
    "sclet_block_edge": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_field_count": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "sclet_set_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _c_dp]),
    "sclet_get_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _c_dp]),
    "sclet_load_restart": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]),
    "sclet_transfer": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_elastic_calculate": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_calc_rhs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "sclet_etd_update": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_etd2_correct": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "sclet_check_soln": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "sclet_set_step_diagnostics": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "sclet_last_diagnostics": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "sclet_set_energy_tensors": (ctypes.c_int, [ctypes.c_void_p, _c_dp]),
    "sclet_get_rhs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_dp]),
    "sclet_get_felas": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _c_dp]),
    "sclet_mode_product": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _c_dp, _c_dp]),
    "sclet_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_time_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "sclet_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "sclet_stage_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float),
                                         ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    "sclet_launch_count": (ctypes.c_longlong, [ctypes.c_void_p]),
    "sclet_host_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "sclet_host_free": (None, [ctypes.c_void_p]),
    "sclet_net_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_ulonglong, ctypes.c_float,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "sclet_net_destroy": (None, [ctypes.c_void_p]),
    "sclet_net_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "sclet_net_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "sclet_net_param_count": (ctypes.c_longlong, []),
    "sclet_net_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "sclet_net_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "sclet_net_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "sclet_net_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_net_set_conv_runs": (ctypes.c_int, [ctypes.c_int]),
    "sclet_net_gradient": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
    "sclet_net_train_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_float, ctypes.POINTER(ctypes.c_double)]),
    "sclet_learned_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_void_p]),
    "sclet_selftest_wait_timeout": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_measure_fp64_rate": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "sclet_graph_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "sclet_tune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "sclet_ensemble_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "sclet_ensemble_destroy": (None, [ctypes.c_void_p]),
    "sclet_ensemble_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "sclet_ensemble_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "sclet_ensemble_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "sclet_ensemble_time_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "sclet_check_soln_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
}

_LIB = None


def lib():
    """Loads the CUDA library (raises OSError if it is not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is not built; run energy-stability_gb300/build_ext.py")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


class ScletError(RuntimeError):
    pass


class PinnedArray:
    """numpy view of page-locked host memory (sclet_host_alloc)."""

    def __init__(self, shape, dtype=np.float64):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = lib().sclet_host_alloc(self.nbytes)
        if not self.ptr:
            raise MemoryError("sclet_host_alloc failed")
        buf = (ctypes.c_char * self.nbytes).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            lib().sclet_host_free(self.ptr)
            self.ptr = None


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_c_dp)


def read_case(case_dir: str, suffix: str) -> Params:
    p = Params()
    rc = lib().sclet_read_case(case_dir.encode(), suffix.encode(), ctypes.byref(p))
    if rc != 0:
        raise ScletError(f"sclet_read_case({case_dir}, {suffix}) failed with status {rc}")
    return p


def fp64_rate(device: int = 0) -> float:
    """Measured FP64 FMA rate of the device in TFLOP/s (sclet_measure_fp64_rate)."""
    t = ctypes.c_double()
    rc = lib().sclet_measure_fp64_rate(device, ctypes.byref(t))
    if rc != 0:
        raise ScletError(f"sclet_measure_fp64_rate failed ({rc})")
    return t.value


def default_params() -> Params:
    p = Params()
    lib().sclet_params_default(ctypes.byref(p))
    return p


class Solver:
    """One device-resident ETD state (a sclet_ctx)."""

    def __init__(self, params: Params, precision: int = FP64, device: int = 0, runs: int = 1,
                 krun: Optional[np.ndarray] = None):
        """runs > 1: that many independent runs side by side (sclet_create_runs),
        krun their per-run plugin constant 0; arrays then hold runs * F blocks."""
        self.L = lib()
        h = ctypes.c_void_p()
        if runs == 1 and krun is None:
            rc = self.L.sclet_create(ctypes.byref(params), precision, device, ctypes.byref(h))
        else:
            kr = None if krun is None else np.ascontiguousarray(krun, dtype=np.float64)
            rc = self.L.sclet_create_runs(ctypes.byref(params), runs, None if kr is None else kr.ctypes.data, precision,
                                          device, ctypes.byref(h))
        if rc != 0:
            raise ScletError(f"sclet_create failed ({rc}): {self.L.sclet_last_error(None).decode()}")
        self.h = h
        self.params = params
        self.runs = runs
        self.n = self.L.sclet_block_edge(h)
        self.F = self.L.sclet_field_count(h)
        self.nac = params.nac
        self.nch = params.nch

    def close(self):
        if getattr(self, "h", None):
            self.L.sclet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc: int, what: str):
        if rc != 0:
            raise ScletError(f"{what} failed ({rc}): {self.L.sclet_last_error(self.h).decode()}")

    def _kind(self, f: int):
        return (AC, f) if f < self.nac else (CH, f - self.nac)

    def _fields_arg(self, u: np.ndarray) -> np.ndarray:
        if u.shape != (self.F, self.n, self.n, self.n) or u.dtype != np.float64 or not u.flags.c_contiguous:
            raise ValueError(f"expected a C-contiguous float64 array of shape {(self.F, self.n, self.n, self.n)}")
        return u

    def set_fields(self, u: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64)
        self._ck(self.L.sclet_set_fields(self.h, _dp(self._fields_arg(u))), "set_fields")

    def get_fields(self) -> np.ndarray:
        out = np.zeros((self.F, self.n, self.n, self.n))
        self._ck(self.L.sclet_get_fields(self.h, _dp(out)), "get_fields")
        return out

    def set_fields_async(self, u: np.ndarray):
        """Queues the state's replacement by u (kept alive and unchanged by the
        caller until sync); page-locked u (PinnedArray) overlaps the steps."""
        self._ck(self.L.sclet_set_fields_async(self.h, _dp(self._fields_arg(u))), "set_fields_async")

    def get_fields_async(self, out: np.ndarray):
        """Queues the copy of the state into out, complete after sync."""
        self._ck(self.L.sclet_get_fields_async(self.h, _dp(self._fields_arg(out))), "get_fields_async")

    def load_restart_dir(self, case_dir: str, restart_iter: int = 0):
        """init_field with restart = 1: ./input/field_iter{it}_{ac|ch}{m}_000.txt"""
        for f in range(self.F):
            k, m = self._kind(f)
            name = f"field_iter{restart_iter}_{'ac' if k == AC else 'ch'}{m}_000.txt"
            path = os.path.join(case_dir, "input", name)
            self._ck(self.L.sclet_load_restart(self.h, k, m, path.encode()), "load_restart")

    def set_eigen(self, d: np.ndarray, v: np.ndarray, vi: np.ndarray):
        self._ck(self.L.sclet_set_eigen(self.h, _dp(np.ascontiguousarray(d)), _dp(np.ascontiguousarray(v)),
                                        _dp(np.ascontiguousarray(vi))), "set_eigen")

    def transfer(self):
        self._ck(self.L.sclet_transfer(self.h), "transfer")

    def elastic(self):
        self._ck(self.L.sclet_elastic_calculate(self.h), "elastic_calculate")

    def calc_rhs(self, slot: int = 1):
        self._ck(self.L.sclet_calc_rhs(self.h, slot), "calc_rhs")

    def get_rhs(self, slot: int = 1) -> np.ndarray:
        out = np.zeros((self.F, self.n, self.n, self.n))
        for f in range(self.F):
            k, m = self._kind(f)
            self._ck(self.L.sclet_get_rhs(self.h, slot, k, m, _dp(out[f])), "get_rhs")
        return out

    def get_felas(self) -> np.ndarray:
        out = np.zeros((self.nac, self.n, self.n, self.n))
        for m in range(self.nac):
            self._ck(self.L.sclet_get_felas(self.h, m, _dp(out[m])), "get_felas")
        return out

    def step(self, k: int = 1):
        self._ck(self.L.sclet_step(self.h, k), "step")

    def graph_step(self, k: int = 1):
        """k steps replayed from one captured CUDA graph (sclet_graph_step)."""
        self._ck(self.L.sclet_graph_step(self.h, k), "graph_step")

    def tune(self, trials: int = 3):
        """Autotuned launch shapes (sclet_tune): (RHS z-planes, tensor-core CTAs)."""
        c = (ctypes.c_int * 2)()
        self._ck(self.L.sclet_tune(self.h, trials, c), "tune")
        return c[0], c[1]

    def sync(self):
        self._ck(self.L.sclet_sync(self.h), "sync")

    def check_soln(self, form: int = 1) -> np.ndarray:
        d = (Diag * self.F)()
        self._ck(self.L.sclet_check_soln(self.h, form, d), "check_soln")
        return np.array([[x.max, x.min, x.vol, x.energy] for x in d])

    def write_chk(self, directory: str, chk: int, irun: int):
        """write_chk of the alpha driver: one checkpoint file per order parameter."""
        self._ck(self.L.sclet_write_chk(self.h, directory.encode(), chk, irun), "write_chk")

    def read_chk(self, directory: str, chk: int) -> int:
        irun = ctypes.c_int()
        self._ck(self.L.sclet_read_chk(self.h, directory.encode(), chk, ctypes.byref(irun)), "read_chk")
        return irun.value

    def field_u16(self, f: int) -> np.ndarray:
        """16-bit codes of field f (AC fields first), as Dtype2B_E / Dtype2B_CI."""
        k, m = self._kind(f)
        out = np.zeros((self.n, self.n, self.n), dtype=np.uint16)
        self._ck(self.L.sclet_field_u16(self.h, k, m, out.ctypes.data_as(ctypes.c_void_p)), "field_u16")
        return out

    def log_soln(self, work_dir: str, iter_: int, energy_form: int = 1):
        self._ck(self.L.sclet_log_soln(self.h, work_dir.encode(), iter_, energy_form), "log_soln")

    def write_vtk(self, path: str, istep: int):
        self._ck(self.L.sclet_write_vtk(self.h, path.encode(), istep), "write_vtk")

    def write_field2b(self, data_dir: str, irun: int, mode: int = 0):
        self._ck(self.L.sclet_write_field2b(self.h, data_dir.encode(), irun, mode), "write_field2b")

    def set_step_diagnostics(self, form: int = 1):
        """Queue check_soln_new after every step (form -1: none)."""
        self._ck(self.L.sclet_set_step_diagnostics(self.h, form), "set_step_diagnostics")

    def last_diagnostics(self) -> np.ndarray:
        d = (Diag * self.F)()
        self._ck(self.L.sclet_last_diagnostics(self.h, d), "last_diagnostics")
        return np.array([[x.max, x.min, x.vol, x.energy] for x in d])

    def set_energy_tensors(self, lam: np.ndarray):
        self._ck(self.L.sclet_set_energy_tensors(self.h, _dp(np.ascontiguousarray(lam, dtype=np.float64))),
                 "set_energy_tensors")

    def mode_product(self, a: np.ndarray, inverse: bool = False) -> np.ndarray:
        out = np.zeros_like(a)
        self._ck(self.L.sclet_mode_product(self.h, int(inverse), _dp(np.ascontiguousarray(a)), _dp(out)),
                 "mode_product")
        return out

    def time_steps(self, k: int) -> float:
        ms = ctypes.c_float()
        self._ck(self.L.sclet_time_steps(self.h, k, ctypes.byref(ms)), "time_steps")
        return ms.value

    def set_profiling(self, on: bool):
        self._ck(self.L.sclet_set_profiling(self.h, int(on)), "set_profiling")

    def stage_times(self, nclasses: int = 5):
        ms = (ctypes.c_float * nclasses)()
        ln = (ctypes.c_int * nclasses)()
        self._ck(self.L.sclet_stage_times(self.h, ms, ln, nclasses), "stage_times")
        return list(ms), list(ln)

    def launch_count(self) -> int:
        return int(self.L.sclet_launch_count(self.h))


class Ensemble:
    """Contexts advanced together by one captured graph (sclet_ensemble_*)."""

    def __init__(self, solvers: List["Solver"]):
        self.L = lib()
        self.solvers = solvers
        arr = (ctypes.c_void_p * len(solvers))(*[s.h.value for s in solvers])
        h = ctypes.c_void_p()
        rc = self.L.sclet_ensemble_create(arr, len(solvers), ctypes.byref(h))
        self.h = h
        if rc != 0:
            msg = self.L.sclet_ensemble_last_error(h).decode() if h else ""
            self.close()
            raise ScletError(f"sclet_ensemble_create failed ({rc}): {msg}")

    def _ck(self, rc, what):
        if rc != 0:
            raise ScletError(f"{what} failed ({rc}): {self.L.sclet_ensemble_last_error(self.h).decode()}")

    def step(self, k: int = 1):
        self._ck(self.L.sclet_ensemble_step(self.h, k), "ensemble_step")

    def sync(self):
        self._ck(self.L.sclet_ensemble_sync(self.h), "ensemble_sync")

    def time_steps(self, k: int) -> float:
        ms = ctypes.c_float()
        self._ck(self.L.sclet_ensemble_time_steps(self.h, k, ctypes.byref(ms)), "ensemble_time_steps")
        return ms.value

    def close(self):
        if getattr(self, "h", None):
            self.L.sclet_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
