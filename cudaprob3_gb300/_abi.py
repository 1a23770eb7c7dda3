"""ctypes binding of libcp3gb300.so (the C ABI in include/cudaprob3_gb300.h).

The library is built in-tree by ``cudaprob3_gb300.build``.  There is no CPU fallback: if the
library is missing or cannot be loaded, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

# C ABI symbols, in header order; the CPU test-suite checks the library exports each one.
EXPORTS = (
    "cp3_atmos_create", "cp3_beam_create", "cp3_destroy", "cp3_last_error", "cp3_get_info",
    "cp3_set_energies", "cp3_set_cosines", "cp3_set_mns", "cp3_set_masses", "cp3_set_layers",
    "cp3_set_layers_poly", "cp3_set_density_file", "cp3_set_chemical_composition",
    "cp3_get_n_layer_boundaries",
    "cp3_set_production_height", "cp3_set_beam_density", "cp3_set_beam_path_length",
    "cp3_set_production_height_averaging", "cp3_calculate", "cp3_calculate_async",
    "cp3_calculate_to_host_async",
    "cp3_synchronize", "cp3_get_probability", "cp3_get_probability_beam",
    "cp3_get_probability_arr", "cp3_device_result", "cp3_copy_result_async",
    "cp3_trajectory_table", "cp3_set_profiling", "cp3_kernel_times", "cp3_atmos_mixed_noalloc",
    "cp3_batch_create", "cp3_batch_destroy", "cp3_batch_last_error", "cp3_batch_set_earth",
    "cp3_batch_add_atmos", "cp3_batch_add_beam", "cp3_batch_set_params", "cp3_batch_commit",
    "cp3_batch_set_shape", "cp3_batch_get_shape", "cp3_batch_set_split_tables",
    "cp3_batch_get_split_tables", "cp3_batch_debug_withhold_tables",
    "cp3_batch_tune", "cp3_batch_run", "cp3_batch_run_to_host",
    "cp3_batch_synchronize", "cp3_batch_result", "cp3_batch_copy_result", "cp3_batch_info",
    "cp3_batch_result_offset", "cp3_batch_copy_results",
    "cp3_batch_parameter_bytes",
    "cp3_server_create", "cp3_server_destroy", "cp3_server_last_error", "cp3_server_set_earth",
    "cp3_server_add_atmos_grid", "cp3_server_add_beam_grid", "cp3_server_start",
    "cp3_server_submit", "cp3_server_wait", "cp3_server_result", "cp3_server_copy_result",
    "cp3_server_release",
    "cp3_server_stats", "cp3_server_poll", "cp3_server_debug_fail_launches",
)

CP3_OK = 0
FP64 = 0
MIXED = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_h = C.c_void_p

_SIGS = {
    "cp3_atmos_create": ([C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_h)], C.c_int),
    "cp3_beam_create": ([C.c_int, C.c_int, C.c_int, C.POINTER(_h)], C.c_int),
    "cp3_destroy": ([_h], C.c_int),
    "cp3_last_error": ([_h], C.c_char_p),
    "cp3_get_info": ([_h, _ip, _ip, _ip, _ip], C.c_int),
    "cp3_set_energies": ([_h, _dp, C.c_int], C.c_int),
    "cp3_set_cosines": ([_h, _dp, C.c_int], C.c_int),
    "cp3_set_mns": ([_h, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int], C.c_int),
    "cp3_set_masses": ([_h, C.c_double, C.c_double], C.c_int),
    "cp3_set_layers": ([_h, _dp, _dp, _dp, C.c_int], C.c_int),
    "cp3_set_layers_poly": ([_h, _dp, _dp, _dp, _dp, _dp, C.c_int], C.c_int),
    "cp3_set_density_file": ([_h, C.c_char_p, C.c_double, C.c_double], C.c_int),
    "cp3_set_chemical_composition": ([_h, _dp, C.c_int], C.c_int),
    "cp3_get_n_layer_boundaries": ([_h, C.POINTER(C.c_int)], C.c_int),
    "cp3_set_production_height": ([_h, C.c_double], C.c_int),
    "cp3_set_beam_density": ([_h, C.c_double], C.c_int),
    "cp3_set_beam_path_length": ([_h, C.c_double], C.c_int),
    "cp3_set_production_height_averaging": ([_h, C.c_int, _dp, _dp], C.c_int),
    "cp3_calculate": ([_h, C.c_int], C.c_int),
    "cp3_calculate_async": ([_h, C.c_int, C.c_void_p], C.c_int),
    "cp3_calculate_to_host_async": ([_h, C.c_int, C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "cp3_synchronize": ([_h], C.c_int),
    "cp3_get_probability": ([_h, C.c_int, C.c_int, C.c_int, _dp], C.c_int),
    "cp3_get_probability_beam": ([_h, C.c_int, C.c_int, _dp], C.c_int),
    "cp3_get_probability_arr": ([_h, C.c_int, _dp], C.c_int),
    "cp3_device_result": ([_h, C.POINTER(C.c_void_p), _ip, C.POINTER(C.c_size_t)], C.c_int),
    "cp3_copy_result_async": ([_h, C.c_void_p, C.c_void_p], C.c_int),
    "cp3_trajectory_table": ([_dp, _dp, _dp, _dp, _dp, C.c_int, C.c_int, _dp, C.c_int, C.c_double,
                              _ip, _ip, _ip, _dp, _dp, _ip, _dp], C.c_int),
    "cp3_set_profiling": ([_h, C.c_int], C.c_int),
    "cp3_batch_create": ([C.c_int, C.POINTER(_h)], C.c_int),
    "cp3_batch_destroy": ([_h], C.c_int),
    "cp3_batch_last_error": ([_h], C.c_char_p),
    "cp3_batch_set_earth": ([_h, _dp, _dp, _dp, C.c_int, C.c_double], C.c_int),
    "cp3_batch_add_atmos": ([_h, _dp, C.c_int, _dp, C.c_int, _ip], C.c_int),
    "cp3_batch_add_beam": ([_h, _dp, C.c_int, C.c_double, _dp, C.c_int, _ip], C.c_int),
    "cp3_batch_set_params": ([_h, C.c_int] + [C.c_double] * 4 + [C.c_int, C.c_double, C.c_double,
                                                                    C.c_int], C.c_int),
    "cp3_batch_commit": ([_h], C.c_int),
    "cp3_batch_set_shape": ([_h, C.c_int, C.c_int, C.c_int], C.c_int),
    "cp3_batch_get_shape": ([_h, _ip, _ip, _ip], C.c_int),
    "cp3_batch_set_split_tables": ([_h, C.c_int], C.c_int),
    "cp3_batch_get_split_tables": ([_h, _ip], C.c_int),
    "cp3_batch_debug_withhold_tables": ([_h, C.c_int], C.c_int),
    "cp3_batch_tune": ([_h, C.c_int], C.c_int),
    "cp3_batch_run": ([_h, C.c_void_p], C.c_int),
    "cp3_batch_run_to_host": ([_h, C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "cp3_batch_synchronize": ([_h, _dp], C.c_int),
    "cp3_batch_result": ([_h, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)], C.c_int),
    "cp3_batch_copy_result": ([_h, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "cp3_batch_result_offset": ([_h, C.c_int, C.POINTER(C.c_size_t)], C.c_int),
    "cp3_batch_copy_results": ([_h, C.c_size_t, C.c_size_t, C.c_void_p, C.c_void_p], C.c_int),
    "cp3_batch_parameter_bytes": ([], C.c_size_t),
    "cp3_batch_info": ([_h, _ip, C.POINTER(C.c_longlong), C.POINTER(C.c_size_t),
                        C.POINTER(C.c_longlong)], C.c_int),
    "cp3_server_create": ([C.c_int, C.c_size_t, C.c_int, C.c_longlong, C.POINTER(_h)], C.c_int),
    "cp3_server_destroy": ([_h], C.c_int),
    "cp3_server_last_error": ([_h], C.c_char_p),
    "cp3_server_set_earth": ([_h, _dp, _dp, _dp, C.c_int, C.c_double], C.c_int),
    "cp3_server_add_atmos_grid": ([_h, _dp, C.c_int, _dp, C.c_int, _ip], C.c_int),
    "cp3_server_add_beam_grid": ([_h, _dp, C.c_int, C.c_double, _dp, C.c_int, _ip], C.c_int),
    "cp3_server_start": ([_h], C.c_int),
    "cp3_server_submit": ([_h, C.c_int] + [C.c_double] * 4 + [C.c_int, C.c_double, C.c_double,
                                                                C.c_int, C.POINTER(C.c_ulonglong)],
                          C.c_int),
    "cp3_server_wait": ([_h, C.c_ulonglong, C.c_double, _ip], C.c_int),
    "cp3_server_result": ([_h, C.c_ulonglong, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t), _dp],
                          C.c_int),
    "cp3_server_copy_result": ([_h, C.c_ulonglong, C.c_void_p], C.c_int),
    "cp3_server_release": ([_h, C.c_ulonglong], C.c_int),
    "cp3_server_stats": ([_h, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                          C.POINTER(C.c_longlong)], C.c_int),
    "cp3_server_poll": ([_h, C.POINTER(C.c_ulonglong), C.c_int, C.c_double, _ip], C.c_int),
    "cp3_server_debug_fail_launches": ([_h, C.c_int], C.c_int),
    "cp3_atmos_mixed_noalloc": ([C.c_int, C.c_void_p, C.c_int, _ip, _dp, _ip, C.c_int, _dp, C.c_int]
                                + [C.c_double] * 4 + [C.c_int, C.c_double, C.c_double, C.c_int,
                                                      C.c_void_p, C.c_void_p, C.c_char_p,
                                                      C.c_size_t], C.c_int),
    "cp3_kernel_times": ([_h, _dp, _dp], C.c_int),
}

_LIB = None


def library_path() -> str:
    """The in-tree library, or the one CP3GB300_LIB names (e.g. the debug build with device
    bounds checks, `python -m cudaprob3_gb300.build --device-checks`)."""
    return os.environ.get("CP3GB300_LIB") or _build.LIB


def lib(build_if_missing: bool = False):
    """Load the library once.  Raises if it is missing (no fallback exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libcp3gb300.so not built ({path}); run "
                               "`python -m cudaprob3_gb300.build` or __graft_entry__.build()")
        _build.build()
    L = C.CDLL(path)
    for name, (args, res) in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _LIB = L
    return L


class CP3Error(RuntimeError):
    """A non-zero status of the C ABI; the message is cp3_last_error()."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def trajectory_table(radii, c1, ye, cosines, height_km, c2=None, c3=None, poly=False):
    """Host-side geometry of the atmospheric kernels (no GPU needed): returns a dict with
    seg_offset, seg_len_km, seg_rho_e, seg_class, class_rho_e."""
    import numpy as np

    L = lib()
    f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    r, a1, a2, a3, y, cz = f(radii), f(c1), f(c2), f(c3), f(ye), f(cosines)
    p = lambda a: None if a is None else a.ctypes.data_as(_dp)  # noqa: E731
    ns, ncl = C.c_int(), C.c_int()
    args = (p(r), p(a1), p(a2), p(a3), p(y), len(r), int(poly), p(cz), len(cz), float(height_km))
    check(L.cp3_trajectory_table(*args, C.byref(ns), C.byref(ncl), None, None, None, None, None))
    off = np.empty(len(cz) + 1, dtype=np.int32)
    ln, rho = np.empty(ns.value), np.empty(ns.value)
    cls = np.empty(ns.value, dtype=np.int32)
    crho = np.empty(max(ncl.value, 1))
    ip = lambda a: a.ctypes.data_as(_ip)  # noqa: E731
    check(L.cp3_trajectory_table(*args, C.byref(ns), C.byref(ncl), ip(off), p(ln), p(rho),
                                 ip(cls), p(crho)))
    return dict(seg_offset=off, seg_len_km=ln, seg_rho_e=rho, seg_class=cls,
                class_rho_e=crho[:ncl.value])


def check(rc: int, handle=None):
    if rc != CP3_OK:
        msg = lib().cp3_last_error(handle)
        raise CP3Error(rc, msg.decode() if msg else f"status {rc}")
