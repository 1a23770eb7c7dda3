"""Continuous-batching server over the persistent kernel (C ABI cp3_server_*)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import CP3Error
from .types import Mixing

_dp = C.POINTER(C.c_double)


def _f64(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    return a, a.ctypes.data_as(_dp)


class Server:
    """Register grids, start(), then submit requests from any thread."""

    def __init__(self, device=0, pool_bytes=8 << 30, max_batch=256, max_bins_per_launch=8_000_000):
        self._lib = _abi.lib()
        h = C.c_void_p()
        rc = self._lib.cp3_server_create(int(device), int(pool_bytes), int(max_batch),
                                         int(max_bins_per_launch), C.byref(h))
        if rc:
            raise CP3Error(rc, self._lib.cp3_server_last_error(None).decode())
        self._h = h
        self.grids = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.cp3_server_destroy(h)
            self._h = None

    def close(self):
        self.__del__()

    def _check(self, rc):
        if rc:
            raise CP3Error(rc, self._lib.cp3_server_last_error(self._h).decode())

    def set_earth(self, radii, rho, ye, production_height_km):
        (r, pr), (d, pd), (y, py) = _f64(radii), _f64(rho), _f64(ye)
        self._check(self._lib.cp3_server_set_earth(self._h, pr, pd, py, len(r),
                                                   float(production_height_km)))

    def add_atmos_grid(self, cosines, energies) -> int:
        (c, pc), (e, pe) = _f64(cosines), _f64(energies)
        g = C.c_int()
        self._check(self._lib.cp3_server_add_atmos_grid(self._h, pc, len(c), pe, len(e), C.byref(g)))
        self.grids.append(("atmos", len(c), len(e)))
        return g.value

    def add_beam_grid(self, energies, rho, baselines_km) -> int:
        (e, pe), (L, pL) = _f64(energies), _f64(np.atleast_1d(baselines_km))
        g = C.c_int()
        self._check(self._lib.cp3_server_add_beam_grid(self._h, pe, len(e), float(rho), pL, len(L),
                                                       C.byref(g)))
        self.grids.append(("beam", len(L), len(e)))
        return g.value

    def start(self):
        self._check(self._lib.cp3_server_start(self._h))

    def submit(self, grid: int, m: Mixing, antineutrino: bool) -> int:
        i = C.c_ulonglong()
        self._check(self._lib.cp3_server_submit(self._h, int(grid), m.theta12, m.theta13, m.theta23,
                                                m.dcp, -1 if antineutrino else 1, m.dm12sq,
                                                m.dm23sq, int(bool(antineutrino)), C.byref(i)))
        return i.value

    def wait(self, rid: int, timeout_s: float = 30.0) -> bool:
        d = C.c_int()
        self._check(self._lib.cp3_server_wait(self._h, C.c_ulonglong(rid), float(timeout_s),
                                              C.byref(d)))
        return bool(d.value)

    def latency_ms(self, rid: int) -> float:
        lat = C.c_double()
        self._check(self._lib.cp3_server_result(self._h, C.c_ulonglong(rid), None, None,
                                                C.byref(lat)))
        return lat.value

    def result_ptr(self, rid: int):
        p, n = C.c_void_p(), C.c_size_t()
        self._check(self._lib.cp3_server_result(self._h, C.c_ulonglong(rid), C.byref(p), C.byref(n),
                                                None))
        return p.value, n.value

    def result(self, rid: int, grid: int) -> np.ndarray:
        """Copy of a finished request's result (atmospheric [9][nc][ne], beam [nL][9][ne])."""
        _, n = self.result_ptr(rid)
        kind, rows, ne = self.grids[grid]
        out = np.empty(n, dtype=np.float32)
        self._check(self._lib.cp3_server_copy_result(self._h, C.c_ulonglong(rid),
                                                     C.c_void_p(out.ctypes.data)))
        return out.reshape((9, rows, ne) if kind == "atmos" else (rows, 9, ne))

    def release(self, rid: int):
        self._check(self._lib.cp3_server_release(self._h, C.c_ulonglong(rid)))

    def poll(self, max_ids: int = 4096, timeout_s: float = 0.0):
        """Ids of requests finished since the previous poll, in completion order (waits up to
        timeout_s while there is none).  Call once before the first submit: recording starts
        with the first poll."""
        n = C.c_int()
        if max_ids <= 0:
            self._check(self._lib.cp3_server_poll(self._h, None, 0, 0.0, C.byref(n)))
            return []
        buf = (C.c_ulonglong * max_ids)()  # per call: poll may be called from any thread
        self._check(self._lib.cp3_server_poll(self._h, buf, int(max_ids), float(timeout_s),
                                              C.byref(n)))
        return list(buf[:n.value])

    def debug_fail_launches(self, count: int):
        """Testing aid: the next ``count`` launches fail on the host before any GPU work."""
        self._check(self._lib.cp3_server_debug_fail_launches(self._h, int(count)))

    def stats(self):
        a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong()
        self._check(self._lib.cp3_server_stats(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return dict(launches=a.value, completed=b.value, queued=c.value)

